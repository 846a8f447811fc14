// a3d_kvti_ms.cu — VTI multi-shot sweeps: one launch advances L.nshot shots of one
// model (kernels in a3d_kvti.cuh with MS = true: 4-D wavefield maps, the shot as
// the fastest part of the tile index).  Built for float and 2-byte storage, tile
// shapes 32x8 and 32x16 with one or two rows per lane (2-byte: not 32x8 with two),
// ring depths 0 and 2.
#include "a3d_kvti.cuh"

namespace a3d {

template <class S>
static cudaError_t launch_vti_ms_t(const K1Launch &L, cudaStream_t st) {
    if (L.depth == 1 || L.rows == 4) return cudaErrorInvalidConfiguration;
#define A3D_MS(TX_, R_) \
    return L.depth == 2 ? launch_vti_s<TX_, S, 2, R_, true>(L, st) : launch_vti_s<TX_, S, 0, R_, true>(L, st)
    if (L.tx == 16) {
        if (L.rows == 1) A3D_MS(16, 1);
        A3D_MS(16, 2);
    }
    if (L.rows == 1) A3D_MS(8, 1);
    if constexpr (sizeof(S) == 2) return cudaErrorInvalidConfiguration;
    else A3D_MS(8, 2);
#undef A3D_MS
}

cudaError_t launch_vti_ms(const K1Launch &L, cudaStream_t st) {
    if (L.fp64) return cudaErrorInvalidConfiguration;
    if (L.half == 1) return launch_vti_ms_t<__nv_bfloat16>(L, st);
    if (L.half == 2) return launch_vti_ms_t<__half>(L, st);
    return launch_vti_ms_t<float>(L, st);
}

}  // namespace a3d
