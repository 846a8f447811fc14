// a3d_closure_tc.cu — the learned rim's inference on the 5th-generation tensor
// cores: both 3x3x3 convolutions of a face-box block as tcgen05 MMAs (bfloat16
// operands in shared memory, float accumulators in tensor memory), fused so the
// hidden activations never leave the SM.
//
// A CTA block is the full normal depth of a face box (7 cells: depth -1..5) by
// 16 x 8 cells of its two tangential axes.  Its input tile (block + 2 cells of halo,
// 8 bfloat16 channels = 16 bytes per cell) and hidden tile (block + 1, 32 channels
// as four 16-byte chunks per cell) sit in shared memory with cells linear in the
// tile's own (l0, l1, l2) order, l0 following global z.  A 3x3x3 convolution is
// then a sum over taps of GEMMs whose A operand is the tile shifted by the tap's
// linear offset: an MMA row r reads cell p0 + r + offset, so every operand is a
// plain no-swizzle K-major descriptor (8-row core matrices 128 bytes apart) whose
// start address moves with the tap.  Rows that fall on halo cells compute values
// nobody stores.
//
//   layer 1: M 128 rows, N 32, K 16 = two taps along l0 of 8 channels each
//            (18 MMAs: 9 (l1, l2) rows x {(-1, 0), (+1, zero weights)})
//   layer 2: M 128 rows, N 16 (4 outputs + 12 zero columns), K 16 = 16 channels
//            (54 MMAs: 27 taps x 2 channel halves)
//
// One thread issues the MMAs; the accumulators are double-buffered in tensor
// memory so the epilogue of one 128-row slice overlaps the MMAs of the next.
// Every mbarrier wait is bounded; on a timeout the kernel records an error, stops
// issuing, drains the MMAs it issued and frees its tensor memory.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/acoustic3d.h"
#include "a3d_closure_dev.cuh"
#include "a3d_common.cuh"

namespace a3d {

namespace tc {

constexpr int B1 = 16, B2 = 8;                 // tangential block extents
constexpr int XC = 11 * 20 * 12;               // input-tile cells (block + 2)
constexpr int XS = XC + 64;                    // with zero slack for shifted rows
constexpr int HC = 9 * 18 * 10;                // hidden-tile cells (block + 1)
constexpr int HS = HC + 64;                    // cells per 16-byte channel chunk
constexpr int NK1 = 18, NK2 = 54;              // MMAs per 128-row slice
constexpr uint32_t W1_BYTES = NK1 * 1024;      // [step][chunk 2][n 32][8 ch]
constexpr uint32_t W2_BYTES = NK2 * 512;       // [tap][half][chunk 2][n 16][8 ch]
constexpr uint32_t OFF_W1 = 0, OFF_W2 = W1_BYTES, OFF_X = OFF_W2 + W2_BYTES;
constexpr uint32_t OFF_H = OFF_X + XS * 16, OFF_BAR = OFF_H + 4 * HS * 16;
constexpr uint32_t SMEM = OFF_BAR + 64;
constexpr int THREADS = 256;
constexpr uint32_t TM_COLS = 128;              // layer-1 buffers at columns 0, 32; layer 2 at 64, 80
constexpr int IMAGE = (W1_BYTES + W2_BYTES) / 2;  // bfloat16 values of one face's weight image
constexpr int KERR_CLOSURE = 4;                // error word: a closure wait gave up
static_assert(SMEM <= 227 * 1024, "tile exceeds shared memory");

// instruction descriptor of kind::f16: D float, A and B bfloat16, both K-major
__host__ __device__ constexpr uint32_t idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// shared-memory matrix descriptor, no swizzle: start address, leading (K-chunk)
// and stride (8-row group) byte offsets, descriptor version 1
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 lanes x 16 columns of the warp's lane quarter
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&p);
}

// compile-time tile geometry of face F: z faces run (l0, l1, l2) = (a, t1, t2),
// x and y faces (t1, a, t2); O = output block, H = O + 2 and X = O + 4 cells per
// axis; tap offsets are tile-linear constants, so descriptors step by immediates
template <int F> struct Face {
    static constexpr int A = F >> 1, SG = (F & 1) ? 1 : -1;
    static constexpr int T1A = A == 0 ? 1 : 0, T2A = A == 2 ? 1 : 2;
    static constexpr int O0 = A == 0 ? 7 : B1, O1 = A == 0 ? B1 : 7, O2 = B2;
    static constexpr int H0 = O0 + 2, H1 = O1 + 2, H2 = O2 + 2;
    static constexpr int X0 = O0 + 4, X1 = O1 + 4, X2 = O2 + 4;
    static constexpr int P1 = 1 + X0 * (1 + X1);                               // first layer-1 row
    static constexpr int Q1 = (X0 - 2) + X0 * ((X1 - 2) + X1 * (X2 - 2));      // last
    static constexpr int M1 = (Q1 - P1 + 128) / 128;
    static constexpr int P2 = 1 + H0 * (1 + H1);
    static constexpr int Q2 = (H0 - 2) + H0 * ((H1 - 2) + H1 * (H2 - 2));
    static constexpr int M2 = (Q2 - P2 + 128) / 128;
    static_assert(X0 * X1 * X2 == XC && H0 * H1 * H2 == HC, "tile sizes");
    // layer-1 step s: taps (l0 = -1, 0) or (+1, zero weights) at (l1, l2) row s / 2
    static __host__ __device__ constexpr int off1(int s) {
        return ((s & 1) ? 1 : -1) + X0 * (((s >> 1) % 3 - 1) + X1 * ((s >> 1) / 3 - 1));
    }
    // global tap t = ((dy+1)*3 + (dx+1))*3 + (dz+1) in block-local axes
    static __host__ __device__ constexpr int d0(int t) { return A == 0 ? SG * (t % 3 - 1) : t % 3 - 1; }
    static __host__ __device__ constexpr int d1(int t) {
        return A == 0 ? (t / 3) % 3 - 1 : (A == 1 ? SG * ((t / 3) % 3 - 1) : SG * (t / 9 - 1));
    }
    static __host__ __device__ constexpr int d2(int t) { return A == 2 ? (t / 3) % 3 - 1 : t / 9 - 1; }
    static __host__ __device__ constexpr int off2(int t) { return d0(t) + H0 * (d1(t) + H1 * d2(t)); }
    // block-local cell -> face coordinates (a = depth + 1, t1, t2)
    static __device__ __forceinline__ void face(int l0, int l1, int l2, int t10, int t20, int &a, int &t1,
                                                int &t2) {
        if (A == 0) { a = l0; t1 = t10 + l1; } else { t1 = t10 + l0; a = l1; }
        t2 = t20 + l2;
    }
};

struct Geo {
    ClGeom g;
    int toff[7];  // first tile of face f; toff[6] = tiles
    int nb1[6];   // blocks along t1 of face f
};

struct Ctx {
    unsigned char *smem;
    uint32_t s_x, s_h, s_w1, s_w2, tm;
    uint64_t *bar;
    volatile int *abort;
    int *err;
    int tid, warp, lane;
};

// one 7 x 16 x 8 block of face F: input tile, layer 1 into the hidden tile, layer 2
// into y; returns false once the CTA has aborted
template <int F>
__device__ __noinline__ bool tile_pass(const ClGeom &g, int t10, int t20, const float *__restrict__ u,
                                       const float *__restrict__ v, const float *__restrict__ w,
                                       const float *__restrict__ P, const float *__restrict__ zinv,
                                       const float *__restrict__ kap, float4 *__restrict__ y, const Ctx &cx,
                                       uint32_t (&ph)[4]) {
    using K = Face<F>;
    const int T1 = g.T1[F], T2 = g.T2[F];
    unsigned char *smem = cx.smem;
    for (int i = cx.tid; i < XC; i += THREADS) {
        const int m0 = i % K::X0, m1 = (i / K::X0) % K::X1, m2 = i / (K::X0 * K::X1);
        int a, t1, t2;
        K::face(m0 - 2, m1 - 2, m2 - 2, t10, t20, a, t1, t2);
        int c[3];
        c[K::A] = (F & 1) ? g.nn[K::A] - CL_PAD - 1 + a : CL_PAD - a;
        c[K::T1A] = 4 + t1;
        c[K::T2A] = 4 + t2;
        uint4 q = make_uint4(0, 0, 0, 0);
        if (c[K::T1A] < g.nn[K::T1A] && c[K::T2A] < g.nn[K::T2A]) {  // the other bounds hold by construction
            float x[8];
            load_x(u, v, w, P, zinv, kap, gidx(g, c[0], c[1], c[2]), x);
            q = make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]),
                           pack_bf16(x[6], x[7]));
        }
        *reinterpret_cast<uint4 *>(smem + OFF_X + i * 16) = q;
    }
    fence_proxy_async();
    __syncthreads();

    // ---- layer 1: h = relu(W1 * x) on the hidden tile
    auto issue1 = [&](int m, int b) {
        const uint64_t a0 = sdesc(cx.s_x + (K::P1 + 128 * m) * 16, 16, 128), b0 = sdesc(cx.s_w1, 512, 128);
#pragma unroll
        for (int s = 0; s < NK1; ++s)
            mma(cx.tm + 32 * b, a0 + (uint64_t)(int64_t)K::off1(s), b0 + (uint64_t)(s * 64), idesc(128, 32), s > 0);
        commit(&cx.bar[b]);
    };
    if (cx.tid == 0) {
        fence_after();
        issue1(0, 0);
    }
    for (int m = 0; m < K::M1; ++m) {
        const int b = m & 1;
        if (cx.tid == 0 && m + 1 < K::M1) {
            fence_after();
            issue1(m + 1, b ^ 1);
        }
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&cx.bar[b], ph[b], cx.err, KERR_CLOSURE, cx.abort));
        ph[b] ^= 1;
        fence_after();
        if (ok) {
            const int qd = cx.warp & 3, hf = cx.warp >> 2;
            float val[16];
            ld16(cx.tm + 32 * b + 16 * hf + ((uint32_t)(32 * qd) << 16), val);
            const int p = K::P1 + 128 * m + 32 * qd + cx.lane;
            const int k0 = p % K::X0 - 1, k1 = (p / K::X0) % K::X1 - 1, k2 = p / (K::X0 * K::X1) - 1;
            if (p <= K::Q1 && k0 >= 0 && k0 < K::H0 && k1 >= 0 && k1 < K::H1 && k2 >= 0 && k2 < K::H2) {
                int a, t1, t2;
                K::face(k0 - 1, k1 - 1, k2 - 1, t10, t20, a, t1, t2);
                const bool in = a >= 0 && a < 7 && t1 >= 0 && t1 < T1 && t2 >= 0 && t2 < T2;
                const int hk = k0 + K::H0 * (k1 + K::H1 * k2);
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const float *vv = val + 8 * c;
                    uint4 q;
                    q.x = in ? pack_bf16(fmaxf(vv[0], 0.0f), fmaxf(vv[1], 0.0f)) : 0u;
                    q.y = in ? pack_bf16(fmaxf(vv[2], 0.0f), fmaxf(vv[3], 0.0f)) : 0u;
                    q.z = in ? pack_bf16(fmaxf(vv[4], 0.0f), fmaxf(vv[5], 0.0f)) : 0u;
                    q.w = in ? pack_bf16(fmaxf(vv[6], 0.0f), fmaxf(vv[7], 0.0f)) : 0u;
                    *reinterpret_cast<uint4 *>(smem + OFF_H + ((2 * hf + c) * HS + hk) * 16) = q;
                }
            }
        }
        fence_before();
        __syncthreads();
        if (*cx.abort) return false;
    }
    fence_proxy_async();
    __syncthreads();

    // ---- layer 2: y_f = W2_f * h on the block's rim cells
    auto issue2 = [&](int m, int b) {
        const uint64_t a0 = sdesc(cx.s_h + (K::P2 + 128 * m) * 16, HS * 16, 128), b0 = sdesc(cx.s_w2, 256, 128);
#pragma unroll
        for (int t = 0; t < 27; ++t)
#pragma unroll
            for (int q = 0; q < 2; ++q)
                mma(cx.tm + 64 + 16 * b, a0 + (uint64_t)(int64_t)(K::off2(t) + 2 * q * HS),
                    b0 + (uint64_t)((t * 2 + q) * 32), idesc(128, 16), (t | q) != 0);
        commit(&cx.bar[2 + b]);
    };
    if (cx.tid == 0) {
        fence_after();
        issue2(0, 0);
    }
    for (int m = 0; m < K::M2; ++m) {
        const int b = m & 1;
        if (cx.tid == 0 && m + 1 < K::M2) {
            fence_after();
            issue2(m + 1, b ^ 1);
        }
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&cx.bar[2 + b], ph[2 + b], cx.err, KERR_CLOSURE, cx.abort));
        ph[2 + b] ^= 1;
        fence_after();
        if (ok && cx.warp < 4) {
            float val[16];
            ld16(cx.tm + 64 + 16 * b + ((uint32_t)(32 * cx.warp) << 16), val);
            const int p = K::P2 + 128 * m + 32 * cx.warp + cx.lane;
            const int l0 = p % K::H0 - 1, l1 = (p / K::H0) % K::H1 - 1, l2 = p / (K::H0 * K::H1) - 1;
            if (p <= K::Q2 && l0 >= 0 && l0 < K::O0 && l1 >= 0 && l1 < K::O1 && l2 >= 0 && l2 < K::O2) {
                int a, t1, t2;
                K::face(l0, l1, l2, t10, t20, a, t1, t2);
                if (a >= 1 && a < 7 && t1 < T1 && t2 < T2) {
                    const long long lin = K::A == 0 ? a + 7LL * (t1 + (long long)T1 * t2)
                                                    : t1 + (long long)T1 * (a + 7LL * t2);
                    y[g.hoff[F] + lin] = make_float4(val[0], val[1], val[2], val[3]);
                }
            }
        }
        fence_before();
        __syncthreads();
        if (*cx.abort) return false;
    }
    return true;
}

__global__ void __launch_bounds__(THREADS, 1)
    closure_tc(const __grid_constant__ Geo G, const float *__restrict__ u, const float *__restrict__ v,
               const float *__restrict__ w, const float *__restrict__ P, const float *__restrict__ zinv,
               const float *__restrict__ kap, const uint4 *__restrict__ image, float4 *__restrict__ y,
               int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + OFF_BAR);  // L1 x2, L2 x2, drain
    uint32_t *tmslot = reinterpret_cast<uint32_t *>(smem + OFF_BAR + 48);
    volatile int *abort = reinterpret_cast<volatile int *>(smem + OFF_BAR + 56);
    const int tid = threadIdx.x, warp = tid >> 5;
    const ClGeom &g = G.g;
    const uint32_t s_base = smem_u32(smem);

    // zero the slack cells past the tiles once (rows of halo positions may read them)
    for (int i = tid; i < (XS - XC); i += THREADS)
        *reinterpret_cast<uint4 *>(smem + OFF_X + (XC + i) * 16) = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < 4 * (HS - HC); i += THREADS) {
        const int ch = i / (HS - HC), c = HC + i % (HS - HC);
        *reinterpret_cast<uint4 *>(smem + OFF_H + (ch * HS + c) * 16) = make_uint4(0, 0, 0, 0);
    }
    if (tid == 0) {
        for (int i = 0; i < 5; ++i) mbar_init(&bar[i], 1);
        *abort = 0;
        fence_mbar_init();
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmslot)),
                     "r"(TM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const Ctx cx{smem, s_base + OFF_X, s_base + OFF_H, s_base + OFF_W1, s_base + OFF_W2, *tmslot, bar, abort, err,
                 tid, warp, tid & 31};
    uint32_t ph[4] = {0, 0, 0, 0};
    int loaded = -1;  // face whose weight image is in shared memory

    for (int tile = blockIdx.x; tile < G.toff[6]; tile += gridDim.x) {
        int f = 0;
        while (f < 5 && tile >= G.toff[f + 1]) ++f;
        const int bi = tile - G.toff[f];
        const int t10 = (bi % G.nb1[f]) * B1, t20 = (bi / G.nb1[f]) * B2;
        if (f != loaded) {  // the face's weight image: layer-1 steps, then layer-2 taps
            const uint4 *src = image + (size_t)f * (IMAGE / 8);
            for (int i = tid; i < IMAGE / 8; i += THREADS) reinterpret_cast<uint4 *>(smem)[i] = src[i];
            loaded = f;
        }
        bool go;
        switch (f) {
            case 0: go = tile_pass<0>(g, t10, t20, u, v, w, P, zinv, kap, y, cx, ph); break;
            case 1: go = tile_pass<1>(g, t10, t20, u, v, w, P, zinv, kap, y, cx, ph); break;
            case 2: go = tile_pass<2>(g, t10, t20, u, v, w, P, zinv, kap, y, cx, ph); break;
            case 3: go = tile_pass<3>(g, t10, t20, u, v, w, P, zinv, kap, y, cx, ph); break;
            case 4: go = tile_pass<4>(g, t10, t20, u, v, w, P, zinv, kap, y, cx, ph); break;
            default: go = tile_pass<5>(g, t10, t20, u, v, w, P, zinv, kap, y, cx, ph); break;
        }
        if (!go) break;
    }
    // drain: every MMA this CTA issued has completed before its tensor memory is freed
    if (tid == 0) {
        fence_after();
        commit(&bar[4]);
        mbar_wait(&bar[4], 0, err, KERR_CLOSURE, nullptr);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cx.tm), "r"(TM_COLS));
}

// rim cells: sum over the cell's faces of G_f[depth] . y_f, added to the fields
// (or written to dout)
__global__ void __launch_bounds__(CL_THREADS)
    closure_combine(const ClGeom g, float *__restrict__ u, float *__restrict__ v, float *__restrict__ w,
                    float *__restrict__ P, const float *__restrict__ zinv, const float *__restrict__ Gc,
                    const float4 *__restrict__ y, float *__restrict__ dout, long long dstride) {
    __shared__ float sG[CL_NG];
    for (int i = threadIdx.x; i < CL_NG; i += blockDim.x) sG[i] = Gc[i];
    __syncthreads();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.roff[6];
         n += (long long)gridDim.x * blockDim.x) {
        int c[3];
        rim_cell(g, n, c);
        float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int Ax = 0; Ax < 3; ++Ax) {
            int a;
            const int f = rim_face(g, Ax, c[Ax], a);
            if (f < 0) continue;
            const float4 yv = y[g.hoff[f] + face_lin(g, f, c[0], c[1], c[2])];
            const float *gg = sG + (f * CL_RIM + a - 1) * CL_COUT;
            d[0] = fmaf(gg[0], yv.x, d[0]);
            d[1] = fmaf(gg[1], yv.y, d[1]);
            d[2] = fmaf(gg[2], yv.z, d[2]);
            d[3] = fmaf(gg[3], yv.w, d[3]);
        }
        const long long id = gidx(g, c[0], c[1], c[2]);
        const float dp = d[3] / zinv[id];
        if (dout) {
            dout[id] = d[0];
            dout[dstride + id] = d[1];
            dout[2 * dstride + id] = d[2];
            dout[3 * dstride + id] = dp;
        } else {
            u[id] += d[0];
            v[id] += d[1];
            w[id] += d[2];
            P[id] += dp;
        }
    }
}

}  // namespace tc

static uint16_t bf16_bits(float x) {
    const float r = cl_round_bf16(x);
    uint32_t b;
    std::memcpy(&b, &r, 4);
    return (uint16_t)(b >> 16);
}

size_t cl_tc_image_halves() { return (size_t)6 * tc::IMAGE; }

void cl_pack_tc(const float *canon, uint16_t *img) {
    const float *W1 = canon, *W2 = canon + CL_NW1;
    for (int f = 0; f < 6; ++f) {
        uint16_t *b1 = img + (size_t)f * tc::IMAGE, *b2 = b1 + tc::W1_BYTES / 2;
        const int A = f >> 1, sg = (f & 1) ? 1 : -1;
        for (int s = 0; s < tc::NK1; ++s) {
            const int rho = s >> 1, hh = s & 1, dl1 = rho % 3 - 1, dl2 = rho / 3 - 1;
            for (int c = 0; c < 2; ++c) {
                const bool pad = hh && c == 1;
                const int dl0 = (hh ? 1 : -1) + c;
                int dz, dx, dy;  // block-local tap -> global tap
                if (A == 0) { dz = sg * dl0; dx = dl1; dy = dl2; }
                else if (A == 1) { dz = dl0; dx = sg * dl1; dy = dl2; }
                else { dz = dl0; dy = sg * dl1; dx = dl2; }
                const int tap = ((dy + 1) * 3 + (dx + 1)) * 3 + (dz + 1);
                for (int n = 0; n < CL_CH; ++n)
                    for (int ch = 0; ch < CL_CIN; ++ch)
                        b1[((s * 2 + c) * 32 + n) * 8 + ch] = pad ? 0 : bf16_bits(W1[(n * CL_CIN + ch) * 27 + tap]);
            }
        }
        for (int t = 0; t < 27; ++t)
            for (int q = 0; q < 2; ++q)
                for (int c = 0; c < 2; ++c)
                    for (int n = 0; n < 16; ++n)
                        for (int ch = 0; ch < 8; ++ch)
                            b2[(((t * 2 + q) * 2 + c) * 16 + n) * 8 + ch] =
                                n < CL_COUT ? bf16_bits(W2[((f * CL_COUT + n) * CL_CH + 16 * q + 8 * c + ch) * 27 + t])
                                            : 0;
    }
}

cudaError_t cl_tc_prepare() {
    return cudaFuncSetAttribute(tc::closure_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::SMEM);
}

cudaError_t cl_launch_apply_tc(const ClGeom &g, float *u, float *v, float *w, float *P, const float *zinv,
                               const float *kap, const uint16_t *image, const float *Gc, float4 *y, int *err,
                               float *dout, long long dstride, int nsm, cudaStream_t st) {
    tc::Geo G{};
    G.g = g;
    int t = 0;
    for (int f = 0; f < 6; ++f) {
        G.toff[f] = t;
        G.nb1[f] = (g.T1[f] + tc::B1 - 1) / tc::B1;
        t += G.nb1[f] * ((g.T2[f] + tc::B2 - 1) / tc::B2);
    }
    G.toff[6] = t;
    const int grid = std::max(1, std::min(t, nsm));
    tc::closure_tc<<<grid, tc::THREADS, tc::SMEM, st>>>(G, u, v, w, P, zinv, kap,
                                                        reinterpret_cast<const uint4 *>(image), y, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const long long n = g.roff[6];
    const int cg = (int)std::max(1LL, std::min<long long>((n + CL_THREADS - 1) / CL_THREADS, 152 * 16));
    tc::closure_combine<<<cg, CL_THREADS, 0, st>>>(g, u, v, w, P, zinv, Gc, y, dout, dstride);
    return cudaGetLastError();
}

}  // namespace a3d
