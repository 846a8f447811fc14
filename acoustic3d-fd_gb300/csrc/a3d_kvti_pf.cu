// a3d_kvti_pf.cu — VTI with float16 velocities and float pressures (A3D_FP16V): u, v,
// w stored as scaled float16, P, Q and their split components as float (kernels in
// a3d_kvti.cuh with PF = true), one shot per launch or multi-shot sweeps.  Built for
// tile shapes (8, 1), (16, 1), (16, 2) at ring depths 0 and 2, as the 2-byte forms.
#include "a3d_kvti.cuh"

namespace a3d {

template <bool MS>
static cudaError_t launch_vti_pf_t(const K1Launch &L, cudaStream_t st) {
    if (L.depth == 1 || L.rows == 4 || (L.tx == 8 && L.rows != 1)) return cudaErrorInvalidConfiguration;
    if (L.tx == 8)
        return L.depth ? launch_vti_s<8, __half, 2, 1, MS, true>(L, st)
                       : launch_vti_s<8, __half, 0, 1, MS, true>(L, st);
    if (L.rows == 1)
        return L.depth ? launch_vti_s<16, __half, 2, 1, MS, true>(L, st)
                       : launch_vti_s<16, __half, 0, 1, MS, true>(L, st);
    return L.depth ? launch_vti_s<16, __half, 2, 2, MS, true>(L, st) : launch_vti_s<16, __half, 0, 2, MS, true>(L, st);
}

cudaError_t launch_vti_pf(const K1Launch &L, cudaStream_t st) {
    if (L.half != 2 || L.fp64) return cudaErrorInvalidConfiguration;
    return L.ms ? launch_vti_pf_t<true>(L, st) : launch_vti_pf_t<false>(L, st);
}

}  // namespace a3d
