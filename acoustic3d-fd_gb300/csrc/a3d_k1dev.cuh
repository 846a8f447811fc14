// a3d_k1dev.cuh — device helpers shared by the 1st-order kernels.
#pragma once
#include "a3d_k1.cuh"
#include "a3d_pipe.cuh"

namespace a3d {

template <int N> struct Maps { CUtensorMap m[N]; };

__device__ __forceinline__ bool damped(float a1, float a2) { return !(a1 == 1.0f && a2 == 1.0f); }

// does the tile [a0, a0+len) of an axis touch its damped region?
__device__ __forceinline__ bool range_damped(int a0, int len, int lo, int hi) {
    return a0 < lo || a0 + len > hi;
}


// launch helper: sets the smem attribute once per device, launches
template <class Kern, class... Args>
static cudaError_t k1_launch(Kern kern, int nthreads, size_t smem, long long W, int grid,
                             cudaStream_t st, SmemAttr &attr, Args... args) {
    if (!smem_fits(smem)) return cudaErrorInvalidConfiguration;
    cudaError_t e = ensure_smem_attr(kern, smem, attr);
    if (e != cudaSuccess) return e;
    (void)W;
    kern<<<grid, nthreads, smem, st>>>(args...);
    return cudaGetLastError();
}

// sweep of the updated region [4, nn-4)^3 in 32 x TX tiles; returns gridDim.x
template <int TX, class Kern>
static int k1_sweep(K1Params &p, Kern kern, int nthreads, size_t smem, int grid, int mode, int rot) {
    p.sw.ntz = (p.nnz - 2 * MM + 31) / 32;
    if (p.sw.nshot < 1) p.sw.nshot = 1;  // multi-shot sweeps set it before the launch
    p.sw.ntx = (p.nnx - 2 * MM + TX - 1) / TX;
    p.sw.y_begin = MM;
    p.sw.NY = p.nny - 2 * MM;
    int occ = 0;
    // a ring larger than a CTA's shared memory is refused by k1_launch; do not let the
    // attribute call fail here and leave its error pending for a later launch check
    if (smem_fits(smem)) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, nthreads, smem);
    }
    const int g = plan_sweep(p.sw, occ, mode);
    p.sw.rot = rot ? 1 : 0;
    return grid > 0 ? grid : g;
}

// TMA load of a wavefield tile: 3-D, or 4-D with the shot as 4th coordinate in a
// multi-shot sweep
template <bool MS>
__device__ __forceinline__ void tma_field(void *dst, const CUtensorMap *map, uint64_t *bar, int z, int x, int y,
                                          int shot) {
    if constexpr (MS) tma_load_4d(dst, map, bar, z, x, y, shot);
    else tma_load_3d(dst, map, bar, z, x, y);
}

// source cell of the segment's shot (padded coordinates)
template <bool MS>
__device__ __forceinline__ int3 shot_cell(const K1Params &p, int shot) {
    if constexpr (MS) {
        const int4 c = p.shots[shot];
        return make_int3(c.x, c.y, c.z);
    } else {
        return make_int3(p.s_x, p.s_y, p.s_z);
    }
}

// loads of a stored field value / smem tile element as the arithmetic type
template <class T, class S> __device__ __forceinline__ T ld(const S *a, int i) { return from_store<T, S>(a[i]); }

// Wavefield tensor maps of 2-byte storage start 4 elements before the field base
// (the field base is only 8-byte aligned; base - 4 elements is 16-byte aligned), so
// their z coordinates are shifted by 4.  That puts both the core box start z0 and
// the halo box start z0 - 4 on 16-byte boundaries.
template <class S> struct WFieldZShift { static constexpr int v = sizeof(S) == 2 ? 4 : 0; };
// Halo'd-in-z wavefield boxes: 4-, 8-byte storage load 40 cells from z0 - 4; with
// 2-byte storage z0 - 4 and z0 cannot both be 16-byte aligned (they are 8 bytes
// apart), so those boxes load 48 cells from z0 - 8, which is aligned whenever the
// core box start z0 is.  ZH = offset of the tile's first z cell inside a halo'd row.
template <class S> struct ZHalo {
    static constexpr int ZH = sizeof(S) == 2 ? 8 : 4;
    static constexpr int W = 32 + 2 * ZH;
};

// exact power-of-two rescaling of a value for 2-byte storage; identity otherwise
template <class S, class T> __device__ __forceinline__ T scl(T x, float f) {
    if constexpr (sizeof(S) == 2) return x * (T)f;
    else return x;
}

// Two z-adjacent cells per lane: elements i, i+1 (i even, so the pair is aligned)
// move as one 8-byte (float) or 16-byte (double) access.
template <class T> struct Two { T a, b; };
template <class S> struct Vec2;
template <> struct Vec2<float> { using t = float2; };
template <> struct Vec2<double> { using t = double2; };
template <> struct Vec2<__nv_bfloat16> { using t = __nv_bfloat162; };
template <> struct Vec2<__half> { using t = __half2; };
__device__ __forceinline__ float2 to_f2(float2 v) { return v; }
__device__ __forceinline__ double2 to_f2(double2 v) { return v; }
__device__ __forceinline__ float2 to_f2(__nv_bfloat162 v) { return __bfloat1622float2(v); }
__device__ __forceinline__ float2 to_f2(__half2 v) { return __half22float2(v); }
template <class T, class S> __device__ __forceinline__ Two<T> ld2(const S *p, int i) {
    const auto v = to_f2(*reinterpret_cast<const typename Vec2<S>::t *>(p + i));
    return Two<T>{(T)v.x, (T)v.y};
}
template <class S, class T> __device__ __forceinline__ void st2(S *p, uint32_t i, T a, T b) {
    typename Vec2<S>::t v;
    if constexpr (sizeof(S) == 2) {  // round to nearest, as the scalar conversions
        v.x = to_store<S, float>((float)a);
        v.y = to_store<S, float>((float)b);
    } else {
        v.x = to_store<S, T>(a);
        v.y = to_store<S, T>(b);
    }
    *reinterpret_cast<typename Vec2<S>::t *>(p + i) = v;
}
// store the pair, or only its first element when the second lies past the sweep
template <class S, class T> __device__ __forceinline__ void st2m(S *p, uint32_t i, T a, T b, bool both) {
    if (both) st2<S, T>(p, i, a, b);
    else p[i] = to_store<S, T>(a);
}

}  // namespace a3d
