// a3d_ktti.cu — the TTI kernels (a3d_ktti.cuh) for FP32, the FP64 error-reference
// run and 2-byte storage.
#include "a3d_ktti.cuh"

namespace a3d {

// 2-byte storage: tile widths 8 and 16, ring depths 0 and 2
template <class S>
static cudaError_t launch_tti_half(const K1Launch &L, cudaStream_t st) {
    if (L.depth == 1) return cudaErrorInvalidConfiguration;
    if (L.tx == 16) return L.depth ? launch_tti_t<16, S, 2, 1>(L, st) : launch_tti_t<16, S, 0, 1>(L, st);
    return L.depth ? launch_tti_t<8, S, 2, 1>(L, st) : launch_tti_t<8, S, 0, 1>(L, st);
}

// configurations: (tile width, rows per lane) (8, 1), (16, 1), three ring depths
cudaError_t launch_tti(const K1Launch &L, cudaStream_t st) {
    if (L.pf) return launch_tti_pf(L, st);
    if (L.fp64) return launch_tti_t<8, double, 0, 1>(L, st);
    if (L.rows != 1) return cudaErrorInvalidConfiguration;
    if (L.half == 1) return launch_tti_half<__nv_bfloat16>(L, st);
    if (L.half == 2) return launch_tti_half<__half>(L, st);
    if (L.tx == 16)
        return L.depth == 2 ? launch_tti_t<16, float, 2, 1>(L, st)
             : L.depth == 1 ? launch_tti_t<16, float, 1, 1>(L, st)
                            : launch_tti_t<16, float, 0, 1>(L, st);
    return L.depth == 2 ? launch_tti_t<8, float, 2, 1>(L, st)
         : L.depth == 1 ? launch_tti_t<8, float, 1, 1>(L, st)
                        : launch_tti_t<8, float, 0, 1>(L, st);
}

}  // namespace a3d
