// a3d_k1.cuh — parameter block and launch entry points of the 1st-order
// (staggered-grid) engines: isotropic, VTI and TTI.
#pragma once
#include "a3d_kernels.cuh"

namespace a3d {

struct K1Params {
    Sweep sw;
    int nnz, nnx, nny, ldz;
    int nx, ny, npml;
    float dtx, dty, dtz;                              // dt/dx, dt/dy, dt/dz (float, as the reference)
    const float *cx1, *cx2, *cy1, *cy2, *cz1, *cz2;   // velocity PML coefficients (half cell)
    const float *ax1, *ax2, *ay1, *ay2, *az1, *az2;   // pressure PML coefficients (integer cell)
    // source cell in padded coordinates; the isotropic dipole's second pole is s_z + 2
    int s_x, s_y, s_z;
    int inj;                 // inject this step (t <= 2/fm)
    float amp0, amp1;        // isotropic: added at s_z and at s_z+2; VTI/TTI: added to P and Q
    const float2 *taper;     // SV ball: hi/lo of the epsilon/delta factor for r^2 = 0..225
    // split (PML) components, touched only on damped axes; pressure-undamped
    // interval per axis (x, y, z): index i is undamped iff ulo <= i < uhi
    void *px, *py, *pz, *qx, *qy, *qz;
    int ulo[3], uhi[3];
    // record at model depth 0 (padded z = npml)
    float *rec;
    const int *mute_nt;
    int it, nt;
    int *err;
    // 2-byte storage: fields hold sigma * value with power-of-two scales (sigma_v for
    // u, v, w; sigma_P for P and its split components), so scaling is exact and is
    // folded into coefficients: svp = sigma_v / sigma_P multiplies the velocity
    // terms, spv = sigma_P / sigma_v the pressure terms, rec_scale = 1 / sigma_P
    // the recorded P.  All 1 for 4- and 8-byte storage.
    float svp, spv, rec_scale;
    // multi-shot sweeps (sw.nshot > 1, VTI): source cell of each shot in padded
    // coordinates (x, y, z, unused) instead of s_x, s_y, s_z; the shots' wavefields
    // and split components lie fstride elements apart, their records rstride floats
    // apart and their mute tables nx * ny ints apart
    const int4 *shots;
    size_t fstride, rstride;
    size_t fstride_p;  // the same for P, Q and the split components (elements of their type)
};

enum K1Kind { K1_ISO_VEL = 0, K1_ISO_STR, K1_VTI_VEL, K1_VTI_STR, K1_TTI_VEL, K1_TTI_STR, K1_ISO_STEP };

// tensor-map box shapes: core {32,TX}, x-halo {32,TX+8}, z-halo {40,TX}, both {40,TX+8},
// both doubled {48,TX+16} (the fused isotropic step's P tile)
enum Box { BOX_CORE = 0, BOX_HX = 1, BOX_HZ = 2, BOX_H = 3, BOX_H2 = 4 };

struct K1Launch {
    int kind;
    const CUtensorMap *maps;  // in the order the kernel documents
    int nmaps;
    void *out0, *out1, *out2, *out3;  // fields written (vel: u,v,w; stress: P[,Q]; fused step: u,v,w,P)
    K1Params p;
    int tx, grid;
    bool fp64;
    int half;   // 2-byte wavefield storage: 0 none, 1 bfloat16, 2 float16
    int depth;  // TMA ring depth (0, 1, 2: see Ring in a3d_pipe.cuh; VTI/TTI: 0, 1)
    int mode;   // sweep plan (plan_sweep)
    int rows;   // tile rows per consumer warp (iso: 2 or 4; VTI/TTI: 1)
    int rot;    // 1: rotated z-tile order of the sweep (Sweep::rot)
    int ms;     // 1: multi-shot kernels (VTI: 4-D wavefield maps, p.shots, p.fstride, p.rstride)
    int nshot;  // multi-shot kernels: shots this launch advances (1 .. the maps' shot count)
    int sblk;   // multi-shot kernels: grid tiles per block of the tile order (Sweep::sblk)
    int pf;     // VTI / TTI with half == 2: P, Q and split components stored as float (A3D_FP16V)
};

cudaError_t launch_k1(const K1Launch &L, cudaStream_t st);

}  // namespace a3d

namespace a3d {
cudaError_t launch_iso(const K1Launch &L, cudaStream_t st);
cudaError_t launch_iso_step(const K1Launch &L, cudaStream_t st);  // fused isotropic step (FP32)
cudaError_t launch_vti(const K1Launch &L, cudaStream_t st);
cudaError_t launch_vti_ms(const K1Launch &L, cudaStream_t st);  // L.ms (launch_vti forwards)
cudaError_t launch_vti_pf(const K1Launch &L, cudaStream_t st);  // L.pf (launch_vti forwards)
cudaError_t launch_tti(const K1Launch &L, cudaStream_t st);
cudaError_t launch_tti_pf(const K1Launch &L, cudaStream_t st);  // L.pf (launch_tti forwards)
}  // namespace a3d
