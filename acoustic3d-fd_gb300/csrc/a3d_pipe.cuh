// a3d_pipe.cuh — the y-marching TMA pipeline shared by every stencil kernel.
//
// A CTA owns a contiguous range of the sweep's (tile, plane) units (cta_range; in
// chunk, tile, plane order, or the wave plan's order), split by make_seg into
// segments of consecutive output planes [ya, yb) of one 32 x TX tile.
// For each segment it streams planes q = ya-4 .. yb+3; item q carries the copy of
// plane q of the fields whose y-derivative is taken ("A", kept in an 8-plane
// register window) and, for q >= ya+4, everything else the update at the output
// plane o = q-4 reads ("B").  One producer thread issues the TMA copies; the
// consumer warps wait, compute, release (per warp: the warp converges, then its
// lane 0 arrives on the empty barriers, which count consumer warps).
//
// Every wait is bounded (mbar_wait); a timeout records an error code, raises a
// CTA-wide abort flag so the other role stops, and the producer drains all
// copies it issued before the CTA exits.
#pragma once
#include <type_traits>

#include "a3d_common.cuh"

namespace a3d {

// A segment's planes [ya, yb) are the pipeline's output planes; [oa, ob) are the
// sweep's own output planes, the same range unless the pipeline runs EXT planes
// beyond it on each side (the fused isotropic step computes velocities 4 planes
// past the pressure planes it outputs).
struct Seg {
    int tile, ya, yb, z0, x0, oa, ob;
    int shot;  // shot of a multi-shot sweep (0 otherwise)
};

template <int TX, int EXT = 0>
__device__ __forceinline__ Seg make_seg(const Sweep &sw, long long w, long long w1, long long &wend) {
    Seg s;
    int c = 0;
    if (sw.wave) {  // virtual order of the wave plan (Sweep::wave): this CTA's units
        const long long G = gridDim.x, b = blockIdx.x, NY = sw.NY;
        const long long T = (long long)sw.ntz * sw.ntx * sw.nshot, P = T / G, R = T - P * G;
        const long long i = w - (b * P * NY + (b * R * NY) / G);
        long long tile, y;
        if (i < P * NY) {  // whole columns: tile b + k G
            tile = (i / NY) * G + b;
            y = i % NY;
        } else {           // this CTA's run of the last R tiles' units
            const long long q = (b * R * NY) / G + (i - P * NY);
            tile = P * G + q / NY;
            y = q % NY;
        }
        s.tile = (int)tile;
        s.ya = sw.y_begin + (int)y;
        wend = w + (NY - y);  // the column ends
        if (wend > w1) wend = w1;
    } else {
        const long long full = (long long)sw.ntz * sw.ntx * sw.nshot * sw.Yc;  // units of a full chunk
        c = (int)(w / full);
        const long long r = w - c * full;
        const int len = min(sw.Yc, sw.NY - c * sw.Yc);
        s.tile = (int)(r / len);
        s.ya = sw.y_begin + c * sw.Yc + (int)(r % len);
        wend = c * full + (long long)(s.tile + 1) * len;
        if (wend > w1) wend = w1;
    }
    s.yb = s.ya + (int)(wend - w);
    int gt;  // tile of the grid
    if (sw.nshot <= 1) {
        s.shot = 0;
        gt = s.tile;
    } else {  // blocks of B grid tiles, each visited for every shot (Sweep::sblk)
        const long long T = (long long)sw.ntz * sw.ntx;
        const long long B = sw.sblk > 1 ? (sw.sblk < T ? sw.sblk : T) : 1;
        const long long v = s.tile, span = B * sw.nshot, nfull = T / B;
        if (v < nfull * span) {
            const long long r = v % span;
            s.shot = (int)(r / B);
            gt = (int)((v / span) * B + r % B);
        } else {  // the last, shorter block
            const long long r = v - nfull * span, tl = T - nfull * B;
            s.shot = (int)(r / tl);
            gt = (int)(nfull * B + r % tl);
        }
    }
    int zt = gt % sw.ntz;
    const int xt = gt / sw.ntz;
    if (sw.rot) {
        const long long nch = (sw.NY + sw.Yc - 1) / sw.Yc, col = (long long)c * sw.ntx + xt;
        zt = (int)((zt + col * sw.ntz / (nch * sw.ntx)) % sw.ntz);
    }
    s.z0 = MM + 32 * zt;
    s.x0 = MM + TX * xt;
    s.oa = s.ya;
    s.ob = s.yb;
    s.ya -= EXT;
    s.yb += EXT;
    return s;
}

// ===========================================================================
// Merged-item pipeline with a phase-unrolled consumer.
//
// Item j of a segment (plane q = ya-4+j) carries the A copy of plane q and, from
// q = ya+4 on, the B copies of output plane o = q-4; all of them complete on
// full[j % KA], so a consumer waits once per plane.  A stages are released HOLD
// items after their arrival (HOLD = 4 when the output step reads the in-plane
// neighbours of A at plane o, 0 when only the y-window reads A), B stages right
// after the output step.  An 8-plane register window rotates by renaming: plane
// q sits in slot (item index mod 8), and the window code is dispatched on that
// phase (with_phase), so no register moves shift the window.
namespace detail {
template <int I, int N, class F>
__device__ __forceinline__ void static_for(F &&f) {
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}
}  // namespace detail

// Ring geometry of the merged pipeline.  A stages have a fixed size; B items are
// allocated in order from a circular byte ring of RB bytes, each taking only the
// bytes it needs (items whose tile or plane touches the damped PML carry split
// components, interior items do not), so more planes fit in flight.
//   D = 0: 8 A stages, 4 B slots, RB = 4 largest items
//   D = 1: 16 A stages, 8 B slots, RB = 8 largest items
//   D = 2: 12 A stages, 12 B slots, RB = what is left of half an SM's shared memory
//          (two CTAs per SM), the deepest rings two CTAs per SM can hold
constexpr size_t SMEM_PER_SM = 233472;  // 228 KB per SM (sm_100 family)
constexpr size_t SMEM_RESERVED_PER_CTA = 1024;

template <int KA_, int KB_>
struct PipeBarsM {
    uint64_t full[KA_], emptyA[KA_], emptyB[KB_];
    uint32_t boff[KB_];  // byte offset of the B item in each slot (written by the producer)
    uint32_t bsz[KB_];   // bytes the item occupies, including wrap-around waste
    int abort_flag;
    __device__ void init(int nconsumers) {  // nconsumers: consumer warps
        for (int i = 0; i < KA_; ++i) { mbar_init(&full[i], 1); mbar_init(&emptyA[i], nconsumers); }
        for (int i = 0; i < KB_; ++i) mbar_init(&emptyB[i], nconsumers);
        abort_flag = 0;
        fence_mbar_init();
    }
    __device__ volatile int *abort_ptr() { return &abort_flag; }
};

template <int D, size_t A_STRIDE, size_t B_MAX>
struct Ring {
    static constexpr int KA = D == 0 ? 8 : (D == 1 ? 16 : 12);
    static constexpr int KB = D == 0 ? 4 : (D == 1 ? 8 : 12);
    using Bars = PipeBarsM<KA, KB>;
    static constexpr size_t FIXED = KA * A_STRIDE + (sizeof(Bars) + 127) / 128 * 128;
    static constexpr size_t BUDGET = SMEM_PER_SM / 2 - SMEM_RESERVED_PER_CTA;
    static constexpr size_t RB = D == 0 ? 4 * B_MAX
                               : D == 1 ? 8 * B_MAX
                                        : (BUDGET > FIXED + B_MAX ? (BUDGET - FIXED) / 128 * 128 : B_MAX);
    static constexpr size_t B_OFF = KA * A_STRIDE;  // ring B follows the A stages
    static constexpr size_t BAR_OFF = B_OFF + RB;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(Bars);
    static_assert(B_MAX % 128 == 0 && A_STRIDE % 128 == 0, "stages are 128-byte aligned");
};

// Producer (one thread): for every item, bsize(seg, o) gives the bytes of the B
// part of output plane o (a multiple of 128), the ring allocates them, and
// issue(sa, bdst, bbytes, bar, seg, q) posts the item's expect_tx on bar and
// issues its copies: the A copy of plane q into A stage sa and, when bdst is not
// null, the B copies of plane q-4 into bdst.
template <int TX, int KA, int KB, size_t RB, int EXT = 0, class BSize, class Issue>
__device__ __forceinline__ void pipe_produce_m(const Sweep &sw, long long w0, long long w1,
                                               PipeBarsM<KA, KB> &b, unsigned char *ringB, int *err,
                                               BSize bsize, Issue issue) {
    volatile int *ab = b.abort_ptr();
    uint32_t ja = 0, jb = 0;
    uint32_t head = 0, used = 0, tail = 0;  // B ring: next free byte, bytes held, oldest live item
    bool ok = true;
    for (long long w = w0; w < w1 && ok;) {
        long long wend;
        const Seg s = make_seg<TX, EXT>(sw, w, w1, wend);
        for (int q = s.ya - MM; q < s.yb + MM; ++q) {
            const uint32_t sa = ja % KA;
            if (ja >= KA && !(ok = mbar_wait(&b.emptyA[sa], ((ja / KA) - 1) & 1, err, KERR_EMPTY_TIMEOUT, ab)))
                break;
            unsigned char *bdst = nullptr;
            uint32_t sz = 0;
            if (q - MM >= s.ya) {
                sz = bsize(s, q - MM);
                for (;;) {
                    if (tail == jb) head = used = 0;  // ring empty: start over at byte 0
                    uint32_t off = head, waste = 0;
                    if (off + sz > RB) {
                        waste = (uint32_t)RB - off;
                        off = 0;
                    }
                    if (jb - tail < (uint32_t)KB && used + waste + sz <= (uint32_t)RB) {
                        const uint32_t slot = jb % KB;
                        b.boff[slot] = off;
                        b.bsz[slot] = waste + sz;
                        used += waste + sz;
                        head = off + sz;
                        bdst = ringB + off;
                        break;
                    }
                    // wait for the consumers to release the oldest live item
                    if (!(ok = mbar_wait(&b.emptyB[tail % KB], (tail / KB) & 1, err, KERR_EMPTY_TIMEOUT, ab)))
                        break;
                    used -= b.bsz[tail % KB];
                    ++tail;
                }
                if (!ok) break;
                ++jb;
            }
            issue(sa, bdst, sz, &b.full[sa], s, q);
            ++ja;
        }
        w = wend;
    }
    // drain (also after an abort): every issued copy lands on a full barrier
    for (uint32_t j = (ja > KA ? ja - KA : 0); j < ja; ++j)
        if (!mbar_wait(&b.full[j % KA], (j / KA) & 1, err, KERR_DRAIN_TIMEOUT, nullptr)) break;
}

// Phase dispatch: f(std::integral_constant<int, ph & 7>) through an 8-way switch, so
// only the code that touches a rotating register window is replicated per phase.
template <class F>
__device__ __forceinline__ void with_phase(int ph, F &&f) {
    switch (ph & 7) {
    case 0: f(std::integral_constant<int, 0>{}); break;
    case 1: f(std::integral_constant<int, 1>{}); break;
    case 2: f(std::integral_constant<int, 2>{}); break;
    case 3: f(std::integral_constant<int, 3>{}); break;
    case 4: f(std::integral_constant<int, 4>{}); break;
    case 5: f(std::integral_constant<int, 5>{}); break;
    case 6: f(std::integral_constant<int, 6>{}); break;
    default: f(std::integral_constant<int, 7>{}); break;
    }
}

// Consumers (all consumer threads):
//   onSeg(seg)                         at a segment start
//   fill(ph, sa, seg, q)               planes q = ya-4 .. ya+3 (window fill); ph = item
//                                      index in the segment (= q - ya + 4), a constant
//   step(ph, sa, sh, bp, seg, q)       planes q >= ya+4: A stage sa (plane q), A stage sh
//                                      (plane q-HOLD), the B item of output plane q-4 at bp;
//                                      ph = item index mod 8 (run time: see with_phase)
// Returns false on abort.
template <int TX, int KA, int KB, int HOLD, int EXT = 0, class OnSeg, class Fill, class Step>
__device__ __forceinline__ bool pipe_run(const Sweep &sw, long long w0, long long w1,
                                         PipeBarsM<KA, KB> &b, const unsigned char *ringB, int *err,
                                         OnSeg onSeg, Fill fill, Step step) {
    static_assert(HOLD == 0 || HOLD == MM, "A stages are held 0 or 4 items");
    volatile int *ab = b.abort_ptr();
    const bool lead = (threadIdx.x & 31) == 0;
    uint32_t ja = 0, jb = 0;
    bool ok = true;
    for (long long w = w0; w < w1;) {
        long long wend;
        const Seg s = make_seg<TX, EXT>(sw, w, w1, wend);
        onSeg(s);
        detail::static_for<0, 8>([&](auto ph) {
            if (!ok) return;
            const uint32_t sa = ja % KA;
            if (!(ok = mbar_wait(&b.full[sa], (ja / KA) & 1, err, KERR_FULL_TIMEOUT, ab))) return;
            fill(ph, sa, s, s.ya - MM + decltype(ph)::value);
            __syncwarp();
            if (lead && ja >= HOLD) mbar_arrive(&b.emptyA[(ja - HOLD) % KA]);
            ++ja;
        });
        if (!ok) return false;
        const int qe = s.yb + MM;
        for (int q = s.ya + MM; q < qe; ++q) {
            const uint32_t sa = ja % KA, sh = (ja - HOLD) % KA, sb = jb % KB;
            if (!mbar_wait(&b.full[sa], (ja / KA) & 1, err, KERR_FULL_TIMEOUT, ab)) return false;
            step(q - s.ya + MM, sa, sh, ringB + b.boff[sb], s, q);
            __syncwarp();
            if (lead) {
                mbar_arrive(&b.emptyB[sb]);
                mbar_arrive(&b.emptyA[sh]);
            }
            ++ja;
            ++jb;
        }
        w = wend;
    }
    return true;
}

}  // namespace a3d
