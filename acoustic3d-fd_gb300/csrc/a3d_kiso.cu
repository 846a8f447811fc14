// a3d_kiso.cu — 1st-order isotropic engine (staggered u, v, w, P with density).
//
// One step = two sweeps (the reference's five launches + five device syncs,
// ..iso..:523-565, become two launches):
//   iso_vel:    u,v,w <- c2*u - c1*dt/d * D+P * (1/rho)    (..iso..:99-142)
//               the dipole source is added to the sweep's view of P only
//               (..iso..:52-96 adds it to P, which update_stress then overwrites)
//   iso_stress: P <- P - rho v^2 dt (D-u/dx + D-v/dy + D-w/dz) (..iso..:145-190)
//               with split components kept only on PML-damped axes, the receiver
//               gather at model depth 0 (..iso..:294-304) and the mute fused.
// Each consumer warp owns R consecutive x rows of the 32 x TX tile (lane = z), so
// the per-plane pipeline work is shared by R cells and the x-derivative reads
// R + 7 tile rows instead of 8 R.
#include <climits>

#include "a3d_k1dev.cuh"

namespace a3d {

// ===========================================================================
// iso_vel: maps {P (box H), u, v, w (core), 1/rho (core, float)}
template <int TX, class S, int D>
struct IsoVelL {
    static constexpr int AW = ZHalo<S>::W, AH = TX + 8;  // P tile: [AH][AW], z halo ZH
    static constexpr uint32_t A_BYTES = AW * AH * sizeof(S);
    static constexpr uint32_t C = 32 * TX;  // core elements
    static constexpr uint32_t B_BYTES = 3 * C * sizeof(S) + C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF, TOTAL = RG::TOTAL;
};

// Launch bounds name one CTA per SM as the minimum: without that, ptxas held some
// shapes to 56-64 registers with spills (iso_vel 16x1: 84 bytes); with it none
// spills, and on one GB300 the 256^3 shot ran 1.8 % faster (the 2nd-order and TTI
// kernels, which lost 5 % and 0.6 % that way, keep the default).
template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1), 1)
    iso_vel(const __grid_constant__ Maps<5> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using L = IsoVelL<TX, S, D>;
    using T = typename Arith<S>::T;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R), NC = 32 * NW, AW = L::AW;
    constexpr int ZS = WFieldZShift<S>::v;  // z offset of wavefield maps (2-byte storage)
    constexpr int ZH = ZHalo<S>::ZH;        // first z cell of the tile inside a P row
    static_assert(NW >= 1, "a warp covers 2R tile rows");
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<typename L::Bars *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::B_OFF;
    if (threadIdx.x == 0) bars.init(NW);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == NW) {  // producer warp: one thread issues every copy
        if (lane != 0) return;
        for (int i = 0; i < 5; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce_m<TX, L::KA, L::KB, L::RB>(
            p.sw, w0, w1, bars, ringB, p.err, [](const Seg &, int) { return (uint32_t)L::B_STRIDE; },
            [&](uint32_t sa, unsigned char *dst, uint32_t, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + (dst ? L::B_BYTES : 0u));
                tma_load_3d(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0 - ZH + ZS, s.x0 - MM, q);
                if (!dst) return;
                const int o = q - MM;
                tma_load_3d(dst, &mp.m[1], bar, s.z0 + ZS, s.x0, o);
                tma_load_3d(dst + L::C * sizeof(S), &mp.m[2], bar, s.z0 + ZS, s.x0, o);
                tma_load_3d(dst + 2 * L::C * sizeof(S), &mp.m[3], bar, s.z0 + ZS, s.x0, o);
                tma_load_3d(dst + 3 * L::C * sizeof(S), &mp.m[4], bar, s.z0, s.x0, o);
            });
        return;
    }

    // lane: z cells zl, zl+1 of the tile (zl = 2 (lane mod 16)) in tile rows
    // xw .. xw+R-1, where the two half-warps take consecutive groups of R rows
    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    const int c0 = (xw + MM) * AW + zl + ZH;  // this lane's first cell pair in an A tile
    T2 win[R][8];                             // P at the last 8 planes, slot = item mod 8
    bool act[R], both = true;
    T cx1d[R], cx2[R];
    T2 cz1d{0, 0}, cz2{0, 0};
    uint32_t gb[R];  // in-plane offsets of this lane's first cell per row
    int srcq = INT_MIN;
    // y coefficients of the next output plane, loaded one plane ahead so that their
    // global-load latency overlaps the current plane's work
    float cy1n = 0, cy2n = 0;
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
    // the dipole enters the sweep's view of P (..iso..:94): patch the A tile of the
    // source plane in place (it serves the window push and, 4 planes later, the
    // in-plane neighbours), then make the write visible to every consumer warp
    auto inject = [&](S *A, const Seg &s) {
        const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - (s.z0 - ZH);
        if (threadIdx.x == 0) {
            if (lz >= 0 && lz < AW) A[lx * AW + lz] = to_store<S, T>(ld<T>(A, lx * AW + lz) + (T)p.amp0);
            if (lz + 2 >= 0 && lz + 2 < AW)
                A[lx * AW + lz + 2] = to_store<S, T>(ld<T>(A, lx * AW + lz + 2) + (T)p.amp1);
            fence_proxy_async();  // the stage is refilled by TMA later
        }
        consumer_sync(NC);
    };
    pipe_run<TX, L::KA, L::KB, MM>(
        p.sw, w0, w1, bars, ringB, p.err,
        [&](const Seg &s) {
            const int iz = s.z0 + zl;
            const bool zact = iz < p.nnz - MM;
            both = iz + 1 < p.nnz - MM;
            const int cza = min(iz, p.nnz - 1), czb = min(iz + 1, p.nnz - 1);
            cz1d = T2{scl<S>((T)p.cz1[cza] * (T)p.dtz, p.svp), scl<S>((T)p.cz1[czb] * (T)p.dtz, p.svp)};
            cz2 = T2{(T)p.cz2[cza], (T)p.cz2[czb]};
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                cx1d[r] = scl<S>((T)p.cx1[cxi] * (T)p.dtx, p.svp);
                cx2[r] = (T)p.cx2[cxi];
                gb[r] = (uint32_t)iz + (uint32_t)p.ldz * (uint32_t)cxi;
            }
            const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - (s.z0 - ZH);
            srcq = (p.inj && lx >= 0 && lx < L::AH && lz + 2 >= 0 && lz < AW) ? p.s_y : INT_MIN;
            cy1n = p.cy1[s.ya];
            cy2n = p.cy2[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &s, int q) {
            constexpr int P = decltype(ph)::value;
            S *A = reinterpret_cast<S *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
#pragma unroll
            for (int r = 0; r < R; ++r) win[r][P] = ld2<T>(A, c0 + r * AW);
        },
        [&](int ph, uint32_t sa, uint32_t sh, const unsigned char *sbp, const Seg &s, int q) {
            S *A = reinterpret_cast<S *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
            // window push of P(q) and the y-derivative at o = q - 4 (..iso..:126)
            T2 yy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int P = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    win[r][P] = ld2<T>(A, c0 + r * AW);
                    T a = 0, b = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {  // P(o+1+m) in slot (P+5+m)&7, P(o-m) in (P+4-m)&7
                        const T2 hi = win[r][(P + 5 + im) & 7], lo = win[r][(P + 4 - im) & 7];
                        a = fma_t(k[im], hi.a - lo.a, a);
                        b = fma_t(k[im], hi.b - lo.b, b);
                    }
                    yy[r] = T2{a, b};
                }
            });
            // output plane o = q - 4: its P tile is the A stage held since item q - 4
            const int o = q - MM;
            const S *Ao = reinterpret_cast<const S *>(ringA + sh * L::A_STRIDE);
            const S *Bu = reinterpret_cast<const S *>(sbp);
            const S *Bv = Bu + L::C, *Bw = Bu + 2 * L::C;
            const float *Br = reinterpret_cast<const float *>(sbp + 3 * L::C * sizeof(S));
            // P at tile rows xw+1 .. xw+R+7 of this lane's z pair: xs[j] = P(x = xw - 3 + j)
            T2 xs[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) xs[j] = ld2<T>(Ao, c0 + (j + 1 - MM) * AW);
            const T cy1d = scl<S>((T)cy1n * (T)p.dty, p.svp), cy2 = (T)cy2n;
            cy1n = p.cy1[o + 1];  // o + 1 <= nny - 4: in bounds
            cy2n = p.cy2[o + 1];
            const uint32_t po = pstride * (uint32_t)o;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int bi = (xw + r) * 32 + zl;
                // P along z at halo'd row positions zl .. zl+9 (position zl+4 = cell a)
                T2 zp[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(Ao, c0 + r * AW - MM + 2 * m);
                const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a,
                                  zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
                T xa = 0, xb = 0, za = 0, zb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // ..iso..:125-127
                    xa = fma_t(k[im], xs[r + 4 + im].a - xs[r + 3 - im].a, xa);
                    xb = fma_t(k[im], xs[r + 4 + im].b - xs[r + 3 - im].b, xb);
                    za = fma_t(k[im], zv[5 + im] - zv[4 - im], za);
                    zb = fma_t(k[im], zv[6 + im] - zv[5 - im], zb);
                }
                const float2 ri = *reinterpret_cast<const float2 *>(Br + bi);  // 1/rho
                const T2 uo = ld2<T>(Bu, bi), vo = ld2<T>(Bv, bi), wo = ld2<T>(Bw, bi);
                xa = xa * (T)ri.x;
                xb = xb * (T)ri.y;
                const T ya = yy[r].a * (T)ri.x, yb = yy[r].b * (T)ri.y;
                za = za * (T)ri.x;
                zb = zb * (T)ri.y;
                const T una = fma_t(cx2[r], uo.a, -(cx1d[r] * xa)), unb = fma_t(cx2[r], uo.b, -(cx1d[r] * xb));
                const T vna = fma_t(cy2, vo.a, -(cy1d * ya)), vnb = fma_t(cy2, vo.b, -(cy1d * yb));
                const T wna = fma_t(cz2.a, wo.a, -(cz1d.a * za)), wnb = fma_t(cz2.b, wo.b, -(cz1d.b * zb));
                if (act[r]) {
                    const uint32_t g = gb[r] + po;
                    st2m<S, T>(u, g, una, unb, both);
                    st2m<S, T>(v, g, vna, vnb, both);
                    st2m<S, T>(w, g, wna, wnb, both);
                }
            }
        });
}


// ===========================================================================
// iso_stress: maps {v (core), u (box HX), w (box HZ), P (core), rho, vp (core, float),
//                   px, py, pz (core; loaded only for tiles/planes on a damped axis)}
template <int TX, class S, int D>
struct IsoStrL {
    static constexpr uint32_t C = 32 * TX;
    static constexpr uint32_t UX = 32 * (TX + 8), WZ = ZHalo<S>::W * TX;  // w tile: [TX][W], z halo ZH
    static constexpr uint32_t A_BYTES = C * sizeof(S);
    // fixed part of a B item (u, w, P, rho, vp), then one tile per damped axis
    static constexpr uint32_t B_FIXED = (UX + WZ + C) * sizeof(S) + 2 * C * 4;
    static constexpr uint32_t AUX = C * sizeof(S);
    static constexpr uint32_t B_BYTES = B_FIXED + 3 * AUX;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static_assert(B_FIXED % 128 == 0 && AUX % 128 == 0, "B item parts are 128-byte aligned");
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF, TOTAL = RG::TOTAL;
};

template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1), 1)
    iso_stress(const __grid_constant__ Maps<9> mp, S *__restrict__ P,
               const __grid_constant__ K1Params p) {
    using L = IsoStrL<TX, S, D>;
    using T = typename Arith<S>::T;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R);
    constexpr int ZS = WFieldZShift<S>::v;  // z offset of wavefield maps (2-byte storage)
    static_assert(NW >= 1, "a warp covers 2R tile rows");
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<typename L::Bars *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::B_OFF;
    if (threadIdx.x == 0) bars.init(NW);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t oW = L::UX * sizeof(S), oP = (L::UX + L::WZ) * sizeof(S),
                     oR = (L::UX + L::WZ + L::C) * sizeof(S), oV = oR + L::C * 4,
                     oX = L::B_FIXED;  // px, py, pz tiles follow the fixed part
    constexpr uint32_t AUX = L::AUX;

    if (warp == NW) {  // producer warp: one thread issues every copy
        if (lane != 0) return;
        for (int i = 0; i < 9; ++i) prefetch_tmap(&mp.m[i]);
        // split components only for tiles / planes on a damped axis, packed after the
        // fixed part in x, y, z order
        auto naux = [&](const Seg &s, int o) {
            return (uint32_t)range_damped(s.x0, TX, p.ulo[0], p.uhi[0]) +
                   (uint32_t)range_damped(o, 1, p.ulo[1], p.uhi[1]) +
                   (uint32_t)range_damped(s.z0, 32, p.ulo[2], p.uhi[2]);
        };
        pipe_produce_m<TX, L::KA, L::KB, L::RB>(
            p.sw, w0, w1, bars, ringB, p.err, [&](const Seg &s, int o) { return L::B_FIXED + AUX * naux(s, o); },
            [&](uint32_t sa, unsigned char *dst, uint32_t bbytes, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + bbytes);
                tma_load_3d(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0 + ZS, s.x0, q);
                if (!dst) return;
                const int o = q - MM;
                tma_load_3d(dst, &mp.m[1], bar, s.z0 + ZS, s.x0 - MM, o);
                tma_load_3d(dst + oW, &mp.m[2], bar, s.z0 - ZHalo<S>::ZH + ZS, s.x0, o);
                tma_load_3d(dst + oP, &mp.m[3], bar, s.z0 + ZS, s.x0, o);
                tma_load_3d(dst + oR, &mp.m[4], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oV, &mp.m[5], bar, s.z0, s.x0, o);
                unsigned char *ax = dst + oX;
                const int zs = s.z0 + ZS;
                if (range_damped(s.x0, TX, p.ulo[0], p.uhi[0])) { tma_load_3d(ax, &mp.m[6], bar, zs, s.x0, o); ax += AUX; }
                if (range_damped(o, 1, p.ulo[1], p.uhi[1])) { tma_load_3d(ax, &mp.m[7], bar, zs, s.x0, o); ax += AUX; }
                if (range_damped(s.z0, 32, p.ulo[2], p.uhi[2])) tma_load_3d(ax, &mp.m[8], bar, zs, s.x0, o);
            });
        return;
    }

    // lane: z cells zl, zl+1 of the tile (zl = 2 (lane mod 16)) in tile rows
    // xw .. xw+R-1, where the two half-warps take consecutive groups of R rows
    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    T2 win[R][8];  // v at the last 8 planes, slot = item mod 8
    bool act[R], dxm[R], reca[R], recb[R], both = true, dza = false, dzb = false;
    float ax1[R], ax2[R];
    float2 az1{1, 1}, az2{1, 1};
    uint32_t gb[R];
    int trb[R];          // receiver trace index of this lane's row, ix - npml
    bool fast = false;   // tile undamped in x and z, every cell active, no receivers
    bool tdx = false, tdz = false;  // the tile touches the damped x / z range (split tiles loaded)
    float ay1n = 1, ay2n = 1;        // y coefficients of the next output plane (loaded one ahead)
    S *px = reinterpret_cast<S *>(p.px), *py = reinterpret_cast<S *>(p.py),
      *pz = reinterpret_cast<S *>(p.pz);
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
    const T dtx = scl<S>((T)p.dtx, p.spv), dty = scl<S>((T)p.dty, p.spv), dtz = scl<S>((T)p.dtz, p.spv);
    pipe_run<TX, L::KA, L::KB, 0>(
        p.sw, w0, w1, bars, ringB, p.err,
        [&](const Seg &s) {
            const int iz = s.z0 + zl;
            const bool zact = iz < p.nnz - MM;
            both = iz + 1 < p.nnz - MM;
            const int cza = min(iz, p.nnz - 1), czb = min(iz + 1, p.nnz - 1);
            az1 = float2{p.az1[cza], p.az1[czb]};
            az2 = float2{p.az2[cza], p.az2[czb]};
            dza = damped(az1.x, az2.x);
            dzb = damped(az1.y, az2.y);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                ax1[r] = p.ax1[cxi];
                ax2[r] = p.ax2[cxi];
                dxm[r] = damped(ax1[r], ax2[r]);
                const bool rx = act[r] && ix >= p.npml && ix < p.npml + p.nx;
                reca[r] = rx && iz == p.npml;
                recb[r] = rx && both && iz + 1 == p.npml;
                trb[r] = ix - p.npml;
                gb[r] = (uint32_t)iz + (uint32_t)p.ldz * (uint32_t)cxi;
            }
            tdx = range_damped(s.x0, TX, p.ulo[0], p.uhi[0]);
            tdz = range_damped(s.z0, 32, p.ulo[2], p.uhi[2]);
            fast = !tdx && !tdz && !(p.npml >= s.z0 && p.npml < s.z0 + 32);
            ay1n = p.ay1[s.ya];
            ay2n = p.ay2[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &, int) {
            constexpr int Q = decltype(ph)::value;
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
#pragma unroll
            for (int r = 0; r < R; ++r) win[r][Q] = ld2<T>(A, (xw + r) * 32 + zl);
        },
        [&](int ph, uint32_t sa, uint32_t, const unsigned char *sbp, const Seg &, int q) {
            const int o = q - MM;
            // y-derivative at o from the window v(o-4 .. o+3) (plane o+m in slot
            // (ph+4+m)&7; ..iso..:179), then v(q) replaces v(q-8), which it last served
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
            T2 yy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int Q = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    T ya = 0, yb = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {
                        const T2 hi = win[r][(Q + 4 + im) & 7], lo = win[r][(Q + 3 - im) & 7];
                        ya = fma_t(k[im], hi.a - lo.a, ya);
                        yb = fma_t(k[im], hi.b - lo.b, yb);
                    }
                    yy[r] = T2{ya, yb};
                    win[r][Q] = ld2<T>(A, (xw + r) * 32 + zl);
                }
            });
            const S *Bu = reinterpret_cast<const S *>(sbp);
            const S *Bw = reinterpret_cast<const S *>(sbp + oW);
            const S *Bp = reinterpret_cast<const S *>(sbp + oP);
            const float *Br = reinterpret_cast<const float *>(sbp + oR);
            const float *Bvp = reinterpret_cast<const float *>(sbp + oV);
            // split tiles as packed by the producer: x, then y, then z, present ones only
            const S *Bx = reinterpret_cast<const S *>(sbp + oX);
            const S *By = Bx + (tdx ? L::C : 0u);
            const S *Bz = By + ((o < p.ulo[1] || o >= p.uhi[1]) ? L::C : 0u);
            // u at tile rows xw .. xw+R+6 of this lane's z pair: us[j] = u(x = xw - 4 + j)
            T2 us[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) us[j] = ld2<T>(Bu, (xw + j) * 32 + zl);
            const bool dym = o < p.ulo[1] || o >= p.uhi[1];  // == damped(ay1[o], ay2[o])
            const uint32_t po = pstride * (uint32_t)o;
            const float ay1 = ay1n, ay2 = ay2n;
            ay1n = p.ay1[o + 1];  // o + 1 <= nny - 4: in bounds
            ay2n = p.ay2[o + 1];
            // derivatives of row r: x from the u rows, z from the halo'd w row
            // (positions zl .. zl+9, position zl+4 = cell a), ..iso..:178-180
            auto deriv = [&](int r, T2 &xx, T2 &zz) {
                T2 zp[5];
#pragma unroll
                for (int m = 0; m < 5; ++m)
                    zp[m] = ld2<T>(Bw, (xw + r) * ZHalo<S>::W + (ZHalo<S>::ZH - MM) + zl + 2 * m);
                const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a,
                                  zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
                T xa = 0, xb = 0, za = 0, zb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {
                    xa = fma_t(k[im], us[r + 4 + im].a - us[r + 3 - im].a, xa);
                    xb = fma_t(k[im], us[r + 4 + im].b - us[r + 3 - im].b, xb);
                    za = fma_t(k[im], zv[4 + im] - zv[3 - im], za);
                    zb = fma_t(k[im], zv[5 + im] - zv[4 - im], zb);
                }
                xx = T2{xa, xb};
                zz = T2{za, zb};
            };
            if (fast && !dym) {  // undamped interior tile and plane: P - gx - gy - gz, a1 == 1
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int bi = (xw + r) * 32 + zl;
                    T2 xx, zz;
                    deriv(r, xx, zz);
                    const float2 rv = *reinterpret_cast<const float2 *>(Br + bi);
                    const float2 vv = *reinterpret_cast<const float2 *>(Bvp + bi);
                    const T2 Po = ld2<T>(Bp, bi);
                    // (((1 * rho) * vp) * vp) == (rho * vp) * vp  (..iso..:182-184)
                    const T ta = ((T)rv.x * (T)vv.x) * (T)vv.x, tb = ((T)rv.y * (T)vv.y) * (T)vv.y;
                    const T pa = ((Po.a - (ta * dtx) * xx.a) - (ta * dty) * yy[r].a) - (ta * dtz) * zz.a;
                    const T pb = ((Po.b - (tb * dtx) * xx.b) - (tb * dty) * yy[r].b) - (tb * dtz) * zz.b;
                    st2<S, T>(P, gb[r] + po, pa, pb);
                }
                return;
            }
            const bool yrec = o >= p.npml && o < p.npml + p.ny;
            // General update (tiles or planes on a damped axis), the oracle's engine form
            // (engine_pupdate) for both cells of the lane without branches: a damped axis
            // keeps its split component, an undamped one subtracts its term directly; the
            // selects keep the operation order, so undamped cells get ((P - gx) - gy) - gz.
            // a1 == 1 off the PML, so one product chain serves every cell (..iso..:182-184).
            auto upd = [&](T Po, T xx, T yy_, T zz, float rv, float vv, bool dx, bool dz, float ax1_, float ax2_,
                           float az1_, float az2_, T cx, T cy, T cz, T &nx, T &ny, T &nz) -> T {
                const T gx = (((((T)ax1_ * (T)rv) * (T)vv) * (T)vv) * dtx) * xx;
                const T gy = (((((T)ay1 * (T)rv) * (T)vv) * (T)vv) * dty) * yy_;
                const T gz = (((((T)az1_ * (T)rv) * (T)vv) * (T)vv) * dtz) * zz;
                T q = Po;
                q = dx ? q - cx : q;
                q = dym ? q - cy : q;
                q = dz ? q - cz : q;
                q = dx ? q : q - gx;
                q = dym ? q : q - gy;
                q = dz ? q : q - gz;
                nx = fma_t((T)ax2_, cx, -gx);
                ny = fma_t((T)ay2, cy, -gy);
                nz = fma_t((T)az2_, cz, -gz);
                q = dx ? q + nx : q;
                q = dym ? q + ny : q;
                q = dz ? q + nz : q;
                return q;
            };
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int bi = (xw + r) * 32 + zl;
                T2 xx, zz;
                deriv(r, xx, zz);
                const float2 rv = *reinterpret_cast<const float2 *>(Br + bi);
                const float2 vv = *reinterpret_cast<const float2 *>(Bvp + bi);
                const T2 Po = ld2<T>(Bp, bi);
                // split components present in this item (tile- and plane-level flags)
                const T2 cx = tdx ? ld2<T>(Bx, bi) : T2{0, 0};
                const T2 cy = dym ? ld2<T>(By, bi) : T2{0, 0};
                const T2 cz = tdz ? ld2<T>(Bz, bi) : T2{0, 0};
                const uint32_t g = gb[r] + po;
                T nxa, nya, nza, nxb, nyb, nzb;
                const T pa = upd(Po.a, xx.a, yy[r].a, zz.a, rv.x, vv.x, dxm[r], dza, ax1[r], ax2[r], az1.x, az2.x,
                                 cx.a, cy.a, cz.a, nxa, nya, nza);
                const T pb = upd(Po.b, xx.b, yy[r].b, zz.b, rv.y, vv.y, dxm[r], dzb, ax1[r], ax2[r], az1.y, az2.y,
                                 cx.b, cy.b, cz.b, nxb, nyb, nzb);
                if (act[r]) {
                    st2m<S, T>(P, g, pa, pb, both);
                    if (dxm[r]) st2m<S, T>(px, g, nxa, nxb, both);
                    if (dym) st2m<S, T>(py, g, nya, nyb, both);
                    if (dza && dzb && both) {
                        st2<S, T>(pz, g, nza, nzb);
                    } else {
                        if (dza) pz[g] = to_store<S, T>(nza);
                        if (dzb && both) pz[g + 1] = to_store<S, T>(nzb);
                    }
                }
                if (yrec && (reca[r] | recb[r])) {  // ..iso..:294-304
                    const size_t tr = (size_t)trb[r] + (size_t)p.nx * (o - p.npml);
                    T rr = scl<S>(reca[r] ? pa : pb, p.rec_scale);
                    if (p.mute_nt && p.it < p.mute_nt[tr]) rr = T(0);
                    p.rec[tr * p.nt + p.it] = (float)rr;
                }
            }
        });
}

// ===========================================================================
template <int TX, class S, int D, int R>
static cudaError_t launch_iso_t(const K1Launch &L, cudaStream_t st) {
    K1Params p = L.p;
    constexpr int NT = 32 * (TX / (2 * R) + 1);
    if (L.kind == K1_ISO_VEL) {
        static SmemAttr attr;
        Maps<5> mp;
        for (int i = 0; i < 5; ++i) mp.m[i] = L.maps[i];
        auto kern = iso_vel<TX, S, D, R>;
        const int grid = k1_sweep<TX>(p, kern, NT, IsoVelL<TX, S, D>::TOTAL, L.grid, L.mode, L.rot);
        return k1_launch(kern, NT, IsoVelL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr, mp,
                         (S *)L.out0, (S *)L.out1, (S *)L.out2, p);
    }
    static SmemAttr attr;
    Maps<9> mp;
    for (int i = 0; i < 9; ++i) mp.m[i] = L.maps[i];
    auto kern = iso_stress<TX, S, D, R>;
    const int grid = k1_sweep<TX>(p, kern, NT, IsoStrL<TX, S, D>::TOTAL, L.grid, L.mode, L.rot);
    return k1_launch(kern, NT, IsoStrL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr, mp, (S *)L.out0, p);
}

// configurations: (tile width, rows per warp) in {8, 16} x {1, 2} and (16, 4), two ring depths
// 2-byte storage: tile shapes (8, 1), (16, 1), (16, 2) at ring depths 0 and 2
template <class S>
static cudaError_t launch_iso_half(const K1Launch &L, cudaStream_t st) {
    if (L.depth == 1 || L.rows == 4 || (L.tx == 8 && L.rows != 1)) return cudaErrorInvalidConfiguration;
    if (L.tx == 8) return L.depth ? launch_iso_t<8, S, 2, 1>(L, st) : launch_iso_t<8, S, 0, 1>(L, st);
    if (L.rows == 1) return L.depth ? launch_iso_t<16, S, 2, 1>(L, st) : launch_iso_t<16, S, 0, 1>(L, st);
    return L.depth ? launch_iso_t<16, S, 2, 2>(L, st) : launch_iso_t<16, S, 0, 2>(L, st);
}

cudaError_t launch_iso(const K1Launch &L, cudaStream_t st) {
    if (L.fp64) return launch_iso_t<8, double, 0, 2>(L, st);
    if (L.half == 1) return launch_iso_half<__nv_bfloat16>(L, st);
    if (L.half == 2) return launch_iso_half<__half>(L, st);
    // one of three ring depths for each (tile width, rows per lane) shape
#define A3D_BY_DEPTH(TX_, R_)                                                   \
    return L.depth == 2 ? launch_iso_t<TX_, float, 2, R_>(L, st)                \
         : L.depth == 1 ? launch_iso_t<TX_, float, 1, R_>(L, st)                \
                        : launch_iso_t<TX_, float, 0, R_>(L, st)
    if (L.tx == 16) {
        if (L.rows == 4) A3D_BY_DEPTH(16, 4);
        if (L.rows == 1) A3D_BY_DEPTH(16, 1);
        A3D_BY_DEPTH(16, 2);
    }
    if (L.rows == 1) A3D_BY_DEPTH(8, 1);
    A3D_BY_DEPTH(8, 2);
#undef A3D_BY_DEPTH
}

}  // namespace a3d
