// a3d_kvti.cu — 1st-order pseudo-acoustic VTI engine, one shot per launch
// (kernels in a3d_kvti.cuh; multi-shot sweeps in a3d_kvti_ms.cu).
#include "a3d_kvti.cuh"

namespace a3d {

template <int TX, class S, int D, int R>
static cudaError_t launch_vti_t(const K1Launch &L, cudaStream_t st) {
    return launch_vti_s<TX, S, D, R, false>(L, st);
}

// configurations: (tile width, rows per lane) in (8, 1), (16, 1), (8, 2), (16, 2), three ring depths
// 2-byte storage: tile shapes (8, 1), (16, 1), (16, 2) at ring depths 0 and 2
template <class S>
static cudaError_t launch_vti_half(const K1Launch &L, cudaStream_t st) {
    if (L.depth == 1 || L.rows == 4 || (L.tx == 8 && L.rows != 1)) return cudaErrorInvalidConfiguration;
    if (L.tx == 8) return L.depth ? launch_vti_t<8, S, 2, 1>(L, st) : launch_vti_t<8, S, 0, 1>(L, st);
    if (L.rows == 1) return L.depth ? launch_vti_t<16, S, 2, 1>(L, st) : launch_vti_t<16, S, 0, 1>(L, st);
    return L.depth ? launch_vti_t<16, S, 2, 2>(L, st) : launch_vti_t<16, S, 0, 2>(L, st);
}

cudaError_t launch_vti(const K1Launch &L, cudaStream_t st) {
    if (L.pf) return launch_vti_pf(L, st);
    if (L.ms) return launch_vti_ms(L, st);
    if (L.fp64) return launch_vti_t<8, double, 0, 2>(L, st);
    if (L.half == 1) return launch_vti_half<__nv_bfloat16>(L, st);
    if (L.half == 2) return launch_vti_half<__half>(L, st);
    if (L.rows == 4) return cudaErrorInvalidConfiguration;
#define A3D_BY_DEPTH(TX_, R_)                                                   \
    return L.depth == 2 ? launch_vti_t<TX_, float, 2, R_>(L, st)                \
         : L.depth == 1 ? launch_vti_t<TX_, float, 1, R_>(L, st)                \
                        : launch_vti_t<TX_, float, 0, R_>(L, st)
    if (L.tx == 16) {
        if (L.rows == 1) A3D_BY_DEPTH(16, 1);
        A3D_BY_DEPTH(16, 2);
    }
    if (L.rows == 1) A3D_BY_DEPTH(8, 1);
    A3D_BY_DEPTH(8, 2);
#undef A3D_BY_DEPTH
}

}  // namespace a3d
