// a3d_common.cuh — device building blocks shared by the stencil engines:
// mbarrier + TMA (cp.async.bulk.tensor) primitives with bounded waits, the
// float helpers that reproduce the reference's double-precision steps with
// float operations, storage-type conversions, and the work split.
//
// Grid convention (all engines, as the reference): z fastest, then x, then y;
// padded sizes nnz, nnx, nny; element (iz, ix, iy) lives at
//     iz + ldz * (ix + nnx * iy)            ldz = nnz rounded up to 4 elements
// so that every row starts on a 16-byte boundary (a TMA requirement).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace a3d {

constexpr int MM = 4;  // stencil half-width (8th order)

// error codes a kernel writes into its error word (first error wins)
enum : int {
    KERR_NONE = 0,
    KERR_FULL_TIMEOUT = 1,   // consumer gave up waiting for a tile
    KERR_EMPTY_TIMEOUT = 2,  // producer gave up waiting for a free stage
    KERR_DRAIN_TIMEOUT = 3,  // exit-time wait for in-flight copies gave up
};

// a bounded mbarrier wait gives up after this many SM clock cycles (~1 s)
constexpr long long WAIT_CYCLES = 2000000000LL;

// ---------------------------------------------------------------------------
// float helpers (identical on host and device; compile with --fmad=false)

__host__ __device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    float x = a + b;
    float bv = x - a;
    float av = x - bv;
    e = (a - av) + (b - bv);
    s = x;
}

// (float)((2.0*cur - prev) + (double)m) with float operations only
__host__ __device__ __forceinline__ float upd2o(float cur, float prev, float m) {
    float s, e, t, f;
    two_sum(2.0f * cur, -prev, s, e);
    two_sum(s, m, t, f);
    return t + (f + e);
}

// (float)(F * (double)v) for a double factor F = fhi + flo
__host__ __device__ __forceinline__ float mul_df(float v, float fhi, float flo) {
    float p = fhi * v;
    float err = fmaf(fhi, v, -p);
    return p + fmaf(flo, v, err);
}

// ---------------------------------------------------------------------------
// storage types: fields may be stored as float, bf16, half or double; the
// arithmetic type is float except for double storage (the FP64 oracle run).

template <class S> struct Arith { using T = float; };
template <> struct Arith<double> { using T = double; };

__device__ __forceinline__ float ld_as_float(float v) { return v; }
__device__ __forceinline__ float ld_as_float(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float ld_as_float(__half v) { return __half2float(v); }

template <class S, class T> __device__ __forceinline__ S to_store(T v);
template <> __device__ __forceinline__ float to_store<float, float>(float v) { return v; }
template <> __device__ __forceinline__ double to_store<double, double>(double v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 to_store<__nv_bfloat16, float>(float v) {
    return __float2bfloat16_rn(v);
}
template <> __device__ __forceinline__ __half to_store<__half, float>(float v) {
    return __float2half_rn(v);
}

template <class T, class S> __device__ __forceinline__ T from_store(S v);
template <> __device__ __forceinline__ float from_store<float, float>(float v) { return v; }
template <> __device__ __forceinline__ double from_store<double, double>(double v) { return v; }
template <> __device__ __forceinline__ float from_store<float, __nv_bfloat16>(__nv_bfloat16 v) {
    return __bfloat162float(v);
}
template <> __device__ __forceinline__ float from_store<float, __half>(__half v) {
    return __half2float(v);
}

// ---------------------------------------------------------------------------
// shared-memory / mbarrier / TMA primitives (sm_90+ PTX, used on sm_103a)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false (and records `code` in *err) if the phase does not
// complete within WAIT_CYCLES, or if another role already aborted (*abort != 0).
// With abort == nullptr (the exit-time drain of in-flight copies) only the time
// limit ends the wait: copies already issued must land before the CTA exits.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, int code,
                                          volatile int *abort) {
    // fast path: plain retries (try_wait suspends the warp for a while on each)
    for (int i = 0; i < 64; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (abort && *abort) return false;
        if (clock64() - t0 > WAIT_CYCLES) {
            atomicCAS(err, 0, code);
            if (abort) *abort = 1;
            return false;
        }
    }
}

// 4-D tiled TMA load (box {b0,b1,1,1}): a field of several shots, the 4th
// coordinate selecting the shot
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int c0, int c1, int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// 3-D tiled TMA load of box {b0,b1,1} at coordinates (c0,c1,c2) into smem,
// completing on `bar` (CTA-local destination address).
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar,
                                            int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// named barrier among the consumer warps only (id 1; id 0 is __syncthreads)
__device__ __forceinline__ void consumer_sync(int nthreads) {
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// ---------------------------------------------------------------------------
// work split: the (tile, plane) space of a sweep is cut along y into chunks of
// Yc planes (the last one may be shorter) and linearised chunk-major:
//     w = c * (ntiles * Yc) + tile * len_c + (y - y_begin - c * Yc),
//     tile = shot + nshot * (tz + ntz * tx),  len_c = planes of chunk c,
// then split into gridDim.x contiguous ranges of nearly equal length.  With one
// chunk-segment per CTA (the host picks Yc so), CTAs that run concurrently march
// the same y range and neighbouring tiles read each other's halos from L2.
// A sweep over several shots of one model (nshot > 1) orders its tiles in blocks
// of sblk grid tiles, each block visited for every shot before the next block:
//     tile = t_in_block + sblk * (shot + nshot * block)
// (the last block may hold fewer tiles).  With sblk = 1 the shot is the fastest
// part, so the CTAs that hold one grid tile for the different shots run at the
// same time and read its model parameters once from HBM, the others from L2; with
// larger blocks the CTAs that run together also hold neighbouring tiles of one
// shot and share their halo rows through L2.  The autotuner picks sblk.

struct Sweep {
    int ntz, ntx;    // tiles along z and x
    int nshot;       // shots advanced together (>= 1)
    int sblk;        // multi-shot sweeps: grid tiles per block of the tile order (<= 1: one)
    int y_begin;     // first output plane
    int NY;          // output planes per tile
    int Yc;          // planes per y chunk
    long long W;     // ntz * ntx * nshot * NY
    // 1: column (chunk c, x tile xt) visits its z tiles rotated by
    // ntz * (c * ntx + xt) / (chunks * ntx), so CTAs far apart in the sweep (those that
    // share an SM) start from different z tiles
    int rot;
    // 1 (wave plan, one y chunk): with T tiles and G CTAs, CTA b sweeps the whole
    // columns of tiles b, b + G, ..., b + (P-1) G (P = T / G), so the CTAs of a wave
    // hold consecutive tiles and march y in step; the last R = T - P G tiles are cut
    // into G equal runs of (tile, plane) units, one more run per CTA.  The units of a
    // CTA form one contiguous range of a virtual order that make_seg decodes.
    int wave;
};

__device__ __forceinline__ void cta_range(const Sweep &s, long long &w0, long long &w1) {
    const long long G = gridDim.x, b = blockIdx.x;
    if (s.wave) {
        const long long T = (long long)s.ntz * s.ntx * s.nshot, P = T / G, R = T - P * G, NY = s.NY;
        w0 = b * P * NY + (b * R * NY) / G;
        w1 = (b + 1) * P * NY + ((b + 1) * R * NY) / G;
        return;
    }
    w0 = (s.W * b) / G;
    w1 = (s.W * (b + 1)) / G;
}

}  // namespace a3d
