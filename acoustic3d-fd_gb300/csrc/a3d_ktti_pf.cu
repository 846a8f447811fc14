// a3d_ktti_pf.cu — TTI with float16 velocities and float pressures (A3D_FP16V): u, v,
// w stored as scaled float16, P, Q and their split components as float (kernels in
// a3d_ktti.cuh with PF = true).  Built for tile widths 8 and 16 at ring depths 0
// and 2, as the 2-byte forms.
#include "a3d_ktti.cuh"

namespace a3d {

cudaError_t launch_tti_pf(const K1Launch &L, cudaStream_t st) {
    if (L.half != 2 || L.fp64 || L.rows != 1 || L.depth == 1) return cudaErrorInvalidConfiguration;
    if (L.tx == 16)
        return L.depth ? launch_tti_t<16, __half, 2, 1, true>(L, st) : launch_tti_t<16, __half, 0, 1, true>(L, st);
    return L.depth ? launch_tti_t<8, __half, 2, 1, true>(L, st) : launch_tti_t<8, __half, 0, 1, true>(L, st);
}

}  // namespace a3d
