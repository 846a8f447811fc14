// a3d_kernels.cuh — parameter blocks and launch entry points of the stencil
// kernels, shared between the kernel translation units and the host engine.
#pragma once
#include <cudaTypedefs.h>

#include <atomic>

#include "a3d_common.cuh"

namespace a3d {

// 8th-order second-derivative coefficients (Toa_3dfd_cuda.cu:32), float-rounded
constexpr float S8_0 = (float)(-205.0 / 72.0), S8_1 = (float)(8.0 / 5.0),
                S8_2 = (float)(-1.0 / 5.0), S8_3 = (float)(8.0 / 315.0),
                S8_4 = (float)(-1.0 / 560.0);
// 8th-order staggered first-derivative coefficients (..iso..:37), float-rounded
constexpr float C8_0 = 1.196289f, C8_1 = -0.0797526f, C8_2 = 0.009570313f,
                C8_3 = -0.0006975447f;

__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }

// sponge multiply on the y, x, z faces in that order (Toa_3dfd_cuda.cu:138-151);
// a face factor is stored as hi+lo floats of the double factor, hi == 0: no face
template <class T> __device__ __forceinline__ T sponge1(T v, float2 f);
template <> __device__ __forceinline__ float sponge1<float>(float v, float2 f) {
    return f.x != 0.0f ? mul_df(v, f.x, f.y) : v;
}
template <> __device__ __forceinline__ double sponge1<double>(double v, float2 f) {
    return f.x != 0.0f ? ((double)f.x + (double)f.y) * v : v;
}
template <class T>
__device__ __forceinline__ T sponge3(T v, float2 fy, float2 fx, float2 fz) {
    return sponge1<T>(sponge1<T>(sponge1<T>(v, fy), fx), fz);
}

// ---------------------------------------------------------------------------
// 2nd-order step
struct K2OParams {
    Sweep sw;
    int nnz, nnx, nny, ldz;
    int nx, ny;           // model (receiver grid) size
    int gz, rx0, ry0;     // receiver depth and first receiver column/row (padded coords)
    const float2 *fz, *fx, *fy;  // sponge factors per axis
    float dz2, dx2, dy2;  // 1/d^2
    int s_x, s_y, s_z;    // dipole cell (padded coords); the second pole is s_z + 2
    float w_next;         // dipole amplitude of the next step (0 after the last)
    float *rec;           // record [ny][nx][nt]
    const int *mute_nt;   // first unmuted sample per trace, or null
    int it, nt;
    int *err;
};

struct K2OLaunch {
    CUtensorMap tm_cur, tm_prev, tm_vv;
    void *ybuf;  // previous-level buffer, overwritten with the next level
    K2OParams p;
    int tx;      // tile width along x (8, 16)
    int grid;    // CTAs (0: planned from the occupancy)
    bool fp64;
    int depth;   // TMA ring depth (0, 1, 2: see Ring in a3d_pipe.cuh)
    int mode;    // sweep plan (plan_sweep)
    int rows;    // tile rows per consumer warp (2 or 4)
};

cudaError_t launch_k2o(const K2OLaunch &L, cudaStream_t st);
size_t k2o_smem_bytes(int tx, bool fp64);

// Pick gridDim.x and the y-chunk length of a sweep (ntz, ntx, NY already set)
// for occ_per_sm resident CTAs per SM.  Mode 0 (lockstep): if every tile fits
// in one wave, one CTA per (tile, chunk) with as many chunks as the wave holds
// (each >= 16 planes), otherwise one wave over whole-y segments.  Mode 1 (fill):
// one full wave of CTAs, the chunk count rounded to the nearest fit.  Mode 2
// (wave): one wave of CTAs sweeping whole tile columns b, b + G, ... (Sweep::wave).
// Fills sw.Yc, sw.W and sw.wave.
int plan_sweep(Sweep &sw, int occ_per_sm, int mode);

// does a CTA with this much dynamic shared memory fit on the current device?
// (launchers return cudaErrorInvalidConfiguration for shapes that do not, which
// the autotuner skips)
inline bool smem_fits(size_t bytes) {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return false;
    return bytes <= (size_t)optin;
}

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) applies to the device that is
// current when it is called, so a launcher records it per device: one bit per
// device ordinal in an atomic word (ordinals >= 64 set it on every launch).
struct SmemAttr {
    std::atomic<unsigned long long> done{0};
};
template <class Kern>
inline cudaError_t ensure_smem_attr(Kern kern, size_t bytes, SmemAttr &a) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
    if (bit && (a.done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess && bit) a.done.fetch_or(bit, std::memory_order_acq_rel);
    return e;
}

}  // namespace a3d
