// a3d_kvti.cuh — 1st-order pseudo-acoustic VTI engine (u, v, w, P, Q; rho, eps, delta):
// the kernel templates, instantiated by a3d_kvti.cu (one shot per launch),
// a3d_kvti_ms.cu (multi-shot sweeps) and a3d_kvti_pf.cu (float16 u, v, w with float
// P, Q: PF = true), which compile in parallel.
//
//   vti_vel:    u,v <- D+P (x, y);  w <- D+_z Q;  / rho          (..vti..:91-128)
//               the Ricker monopole enters the sweep's views of P and Q only
//   vti_stress: P <- P - rho v^2 [(1+2e')(D-u/dx + D-v/dy) + sqrt(1+2d') D-w/dz]
//               Q <- Q - rho v^2 [sqrt(1+2d')(D-u/dx + D-v/dy) + D-w/dz]
//               e', d' tapered inside the SV ball round the source (..vti..:131-203),
//               split components only on damped PML axes, record + mute fused.
#pragma once
#include <climits>
#include <type_traits>

#include "a3d_k1dev.cuh"

namespace a3d {

// ===========================================================================
// vti_vel: maps {P (HX), Q (HZ), u, v, w (core), 1/rho (core float)}; S stores u, v,
// w and SP stores P, Q (the same type, or float with 2-byte velocities)
template <int TX, class S, int D, class SP = S>
struct VtiVelL {
    static constexpr int QW = ZHalo<SP>::W;  // Q tile rows: z halo ZH
    static constexpr uint32_t C = 32 * TX, PX = 32 * (TX + 8), QZ = QW * TX;
    static constexpr uint32_t A_BYTES = PX * sizeof(SP);
    static constexpr uint32_t B_BYTES = QZ * sizeof(SP) + 3 * C * sizeof(S) + C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF, TOTAL = RG::TOTAL;
};

// Launch bounds of the one-shot kernels name one CTA per SM as the minimum, so that
// ptxas does not hold shapes to fewer registers with spills (measured on one GB300:
// the 384x384x256 shot 1.8 % faster).  The multi-shot kernels keep ptxas's default
// (0: no minimum): with the minimum their float16 sweep of 64 shots took 27.2 ms per
// stress launch against 25.0 ms.
template <int TX, class S, int D, int R, bool MS, bool PF>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1), MS ? 0 : 1)
    vti_vel(const __grid_constant__ Maps<6> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using SP = std::conditional_t<PF, float, S>;  // P, Q storage
    using L = VtiVelL<TX, S, D, SP>;
    using T = typename Arith<S>::T;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R), NC = 32 * NW, QW = L::QW;
    constexpr int ZS = WFieldZShift<S>::v;                          // u, v, w maps
    constexpr int ZSP = WFieldZShift<SP>::v, ZH = ZHalo<SP>::ZH;    // P, Q maps
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
    constexpr size_t oU = L::QZ * sizeof(SP), oV = oU + L::C * sizeof(S), oW = oV + L::C * sizeof(S),
                     oR = oW + L::C * sizeof(S);

    if (warp == NW) {  // producer warp: one thread issues every copy
        if (lane != 0) return;
        for (int i = 0; i < 6; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce_m<TX, L::KA, L::KB, L::RB>(
            p.sw, w0, w1, bars, ringB, p.err, [](const Seg &, int) { return (uint32_t)L::B_STRIDE; },
            [&](uint32_t sa, unsigned char *dst, uint32_t, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + (dst ? L::B_BYTES : 0u));
                tma_field<MS>(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0 + ZSP, s.x0 - MM, q, s.shot);
                if (!dst) return;
                const int o = q - MM;
                tma_field<MS>(dst, &mp.m[1], bar, s.z0 - ZH + ZSP, s.x0, o, s.shot);
                tma_field<MS>(dst + oU, &mp.m[2], bar, s.z0 + ZS, s.x0, o, s.shot);
                tma_field<MS>(dst + oV, &mp.m[3], bar, s.z0 + ZS, s.x0, o, s.shot);
                tma_field<MS>(dst + oW, &mp.m[4], bar, s.z0 + ZS, s.x0, o, s.shot);
                tma_load_3d(dst + oR, &mp.m[5], bar, s.z0, s.x0, o);  // 1/rho: one copy for every shot
            });
        return;
    }

    // lane: z cells zl, zl+1 of the tile in tile rows xw .. xw+R-1 (two half-warps)
    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    const int c0 = (xw + MM) * 32 + zl;  // this lane's first cell pair in the P tile
    T2 win[R][8];                        // P at the last 8 planes, slot = item mod 8
    bool act[R], both = true;
    T cx1d[R], cx2[R];
    T2 cz1d{0, 0}, cz2{0, 0};
    uint32_t gb[R];
    int srcP = INT_MIN, srcQ = INT_MIN;  // plane of the monopole in this tile's P / Q tiles
    float cy1n = 0, cy2n = 0;            // y coefficients of the next output plane
    int3 sc = make_int3(0, 0, 0);        // source cell of the segment's shot
    S *uk = u, *vk = v, *wk = w;         // the segment's shot's fields
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
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
            sc = shot_cell<MS>(p, s.shot);
            if constexpr (MS) {
                const size_t fo = (size_t)s.shot * p.fstride;
                uk = u + fo; vk = v + fo; wk = w + fo;
            }
            // the monopole enters the sweep's views of P and Q (..vti..:85-86)
            const int lxp = sc.x - (s.x0 - MM), lzp = sc.z - s.z0;
            srcP = (p.inj && lxp >= 0 && lxp < TX + 8 && lzp >= 0 && lzp < 32) ? sc.y : INT_MIN;
            const int lxq = sc.x - s.x0, lzq = sc.z - (s.z0 - ZH);
            srcQ = (p.inj && lxq >= 0 && lxq < TX && lzq >= 0 && lzq < QW) ? sc.y : INT_MIN;
            cy1n = p.cy1[s.ya];
            cy2n = p.cy2[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &s, int q) {
            constexpr int P_ = decltype(ph)::value;
            SP *A = reinterpret_cast<SP *>(ringA + sa * L::A_STRIDE);
            if (q == srcP) {
                if (threadIdx.x == 0) {
                    const int at = (sc.x - (s.x0 - MM)) * 32 + (sc.z - s.z0);
                    A[at] = to_store<SP, T>(ld<T>(A, at) + (T)p.amp0);
                    fence_proxy_async();
                }
                consumer_sync(NC);
            }
#pragma unroll
            for (int r = 0; r < R; ++r) win[r][P_] = ld2<T>(A, c0 + r * 32);
        },
        [&](int ph, uint32_t sa, uint32_t sh, const unsigned char *sbc, const Seg &s, int q) {
            SP *A = reinterpret_cast<SP *>(ringA + sa * L::A_STRIDE);
            unsigned char *sbp = const_cast<unsigned char *>(sbc);
            const int o = q - MM;
            if (q == srcP || o == srcQ) {  // one plane per shot and tile: patch, then publish
                if (threadIdx.x == 0) {
                    if (q == srcP) {
                        const int at = (sc.x - (s.x0 - MM)) * 32 + (sc.z - s.z0);
                        A[at] = to_store<SP, T>(ld<T>(A, at) + (T)p.amp0);
                    }
                    if (o == srcQ) {
                        SP *Bq = reinterpret_cast<SP *>(sbp);
                        const int at = (sc.x - s.x0) * QW + (sc.z - (s.z0 - ZH));
                        Bq[at] = to_store<SP, T>(ld<T>(Bq, at) + (T)p.amp1);
                    }
                    fence_proxy_async();
                }
                consumer_sync(NC);
            }
            T2 yy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int P_ = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    win[r][P_] = ld2<T>(A, c0 + r * 32);
                    T a = 0, b = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {  // P(o+1+m) in slot (P+5+m)&7, P(o-m) in (P+4-m)&7
                        const T2 hi = win[r][(P_ + 5 + im) & 7], lo = win[r][(P_ + 4 - im) & 7];
                        a = fma_t(k[im], hi.a - lo.a, a);
                        b = fma_t(k[im], hi.b - lo.b, b);
                    }
                    yy[r] = T2{a, b};
                }
            });
            const SP *Ao = reinterpret_cast<const SP *>(ringA + sh * L::A_STRIDE);
            const SP *Bq = reinterpret_cast<const SP *>(sbp);
            const S *Bu = reinterpret_cast<const S *>(sbp + oU);
            const S *Bv = reinterpret_cast<const S *>(sbp + oV);
            const S *Bw = reinterpret_cast<const S *>(sbp + oW);
            const float *Br = reinterpret_cast<const float *>(sbp + oR);
            // P at tile rows xw+1 .. xw+R+7 of this lane's z pair: xs[j] = P(x = xw - 3 + j)
            T2 xs[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) xs[j] = ld2<T>(Ao, c0 + (j + 1 - MM) * 32);
            const T cy1d = scl<S>((T)cy1n * (T)p.dty, p.svp), cy2 = (T)cy2n;
            cy1n = p.cy1[o + 1];  // o + 1 <= nny - 4: in bounds
            cy2n = p.cy2[o + 1];
            const uint32_t po = pstride * (uint32_t)o;
#pragma unroll
            for (int r = 0; r < R; ++r) {  // ..vti..:113-125
                const int bi = (xw + r) * 32 + zl;
                // Q along z at halo'd row positions ZH-4+zl .. ZH+5+zl (ZH+zl = cell a)
                T2 zp[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(Bq, (xw + r) * QW + (ZH - MM) + zl + 2 * m);
                const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a,
                                  zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
                T xa = 0, xb = 0, za = 0, zb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {
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
                    st2m<S, T>(uk, g, una, unb, both);
                    st2m<S, T>(vk, g, vna, vnb, both);
                    st2m<S, T>(wk, g, wna, wnb, both);
                }
            }
        });
}

// ===========================================================================
// vti_stress: maps {v (core), u (HX), w (HZ), P, Q (core), rho, vp, eps, del (core float),
//                   px, py, pz, qx, qy, qz (core; only for tiles/planes on a damped axis)}
template <int TX, class S, int D, class SP = S>
struct VtiStrL {
    static constexpr uint32_t C = 32 * TX, UX = 32 * (TX + 8), WZ = ZHalo<S>::W * TX;
    static constexpr uint32_t A_BYTES = C * sizeof(S);
    // fixed part of a B item (u, w, P, Q, rho, vp, eps, del), then the (p, q) split
    // pair of each damped axis, in x, y, z order; S stores u, v, w, SP P, Q and splits
    static constexpr uint32_t B_FIXED = (UX + WZ) * sizeof(S) + 2 * C * sizeof(SP) + 4 * C * 4;
    static constexpr uint32_t AUX = C * sizeof(SP);
    static constexpr uint32_t B_BYTES = B_FIXED + 6 * AUX;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static_assert(B_FIXED % 128 == 0 && AUX % 128 == 0, "B item parts are 128-byte aligned");
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF, TOTAL = RG::TOTAL;
};

// epsilon/delta after the SV-ball taper (..vti..:154-175): hi/lo table per r^2
__device__ __forceinline__ void sv_eedd(const K1Params &p, int3 sc, int ix, int iy, int iz, float eps,
                                        float del, float &ee, float &dd) {
    const int rx = ix - sc.x, ry = iy - sc.y, rz = iz - sc.z;
    const int d2 = rx * rx + ry * ry + rz * rz;
    if (d2 > 225) { ee = eps; dd = del; return; }
    const float2 t = p.taper[d2];
    ee = mul_df(eps, t.x, t.y);
    dd = mul_df(del, t.x, t.y);
}

// the VTI pressure pair of one cell, ..vti..:176-200: returns P and Q, the new
// split components of damped axes in np3 / nq3 (the select-based engine form of
// the oracle's engine_pupdate, operation order kept)
template <class T>
__device__ __forceinline__ void vti_cell(T Po, T Qo, T xx, T yy, T zz, float rv, float vv, float ee,
                                         float dd, bool dx, bool dy, bool dz, float ax1, float ay1,
                                         float az1, float ax2, float ay2, float az2, const T cp[3],
                                         const T cq[3], T dtx, T dty, T dtz, T &Pn, T &Qn, T np3[3],
                                         T nq3[3]) {
    T e1, sd;
    if constexpr (sizeof(T) == 4) {
        e1 = 1.0f + 2.0f * ee;
        sd = sqrtf(1.0f + 2.0f * dd);
    } else {
        e1 = T(1) + T(2) * (T)ee;
        sd = sqrt(T(1) + T(2) * (T)dd);
    }
    const T kx = (((T)ax1 * (T)rv) * (T)vv) * (T)vv, ky = (((T)ay1 * (T)rv) * (T)vv) * (T)vv,
            kz = (((T)az1 * (T)rv) * (T)vv) * (T)vv;
    const T gP[3] = {((kx * e1) * dtx) * xx, ((ky * e1) * dty) * yy, ((kz * sd) * dtz) * zz};
    const T gQ[3] = {((kx * sd) * dtx) * xx, ((ky * sd) * dty) * yy, (kz * dtz) * zz};
    const bool d3[3] = {dx, dy, dz};
    const float a2[3] = {ax2, ay2, az2};
    T qp = Po, qq = Qo;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        qp = d3[a] ? qp - cp[a] : qp;
        qq = d3[a] ? qq - cq[a] : qq;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        qp = d3[a] ? qp : qp - gP[a];
        qq = d3[a] ? qq : qq - gQ[a];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        np3[a] = fma_t((T)a2[a], cp[a], -gP[a]);
        nq3[a] = fma_t((T)a2[a], cq[a], -gQ[a]);
        qp = d3[a] ? qp + np3[a] : qp;
        qq = d3[a] ? qq + nq3[a] : qq;
    }
    Pn = qp;
    Qn = qq;
}

template <int TX, class S, int D, int R, bool MS, bool PF>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1), MS ? 0 : 1)
    vti_stress(const __grid_constant__ Maps<15> mp, std::conditional_t<PF, float, S> *__restrict__ P,
               std::conditional_t<PF, float, S> *__restrict__ Q, const __grid_constant__ K1Params p) {
    using SP = std::conditional_t<PF, float, S>;  // P, Q and split-component storage
    using L = VtiStrL<TX, S, D, SP>;
    using T = typename Arith<S>::T;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R);
    constexpr int ZS = WFieldZShift<S>::v, ZH = ZHalo<S>::ZH, WW = ZHalo<S>::W;  // u, v, w maps
    constexpr int ZSP = WFieldZShift<SP>::v;                                      // P, Q, split maps
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
    constexpr size_t oW = L::UX * sizeof(S), oP = oW + L::WZ * sizeof(S), oQ = oP + L::C * sizeof(SP),
                     oF = oQ + L::C * sizeof(SP),  // then rho, vp, eps, del floats
                     oX = L::B_FIXED;             // split pairs of the damped axes follow
    constexpr uint32_t AUX = L::AUX;
    SP *px = (SP *)p.px, *py = (SP *)p.py, *pz = (SP *)p.pz, *qx = (SP *)p.qx, *qy = (SP *)p.qy, *qz = (SP *)p.qz;

    if (warp == NW) {  // producer warp: one thread issues every copy
        if (lane != 0) return;
        for (int i = 0; i < 15; ++i) prefetch_tmap(&mp.m[i]);
        auto naux = [&](const Seg &s, int o) {
            return (uint32_t)range_damped(s.x0, TX, p.ulo[0], p.uhi[0]) +
                   (uint32_t)range_damped(o, 1, p.ulo[1], p.uhi[1]) +
                   (uint32_t)range_damped(s.z0, 32, p.ulo[2], p.uhi[2]);
        };
        pipe_produce_m<TX, L::KA, L::KB, L::RB>(
            p.sw, w0, w1, bars, ringB, p.err,
            [&](const Seg &s, int o) { return L::B_FIXED + 2 * AUX * naux(s, o); },
            [&](uint32_t sa, unsigned char *dst, uint32_t bbytes, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + bbytes);
                tma_field<MS>(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0 + ZS, s.x0, q, s.shot);
                if (!dst) return;
                const int o = q - MM;
                tma_field<MS>(dst, &mp.m[1], bar, s.z0 + ZS, s.x0 - MM, o, s.shot);
                tma_field<MS>(dst + oW, &mp.m[2], bar, s.z0 - ZH + ZS, s.x0, o, s.shot);
                tma_field<MS>(dst + oP, &mp.m[3], bar, s.z0 + ZSP, s.x0, o, s.shot);
                tma_field<MS>(dst + oQ, &mp.m[4], bar, s.z0 + ZSP, s.x0, o, s.shot);
                // rho, vp, eps, del: one copy for every shot
                for (int k = 0; k < 4; ++k) tma_load_3d(dst + oF + k * L::C * 4, &mp.m[5 + k], bar, s.z0, s.x0, o);
                unsigned char *ax = dst + oX;
                const bool dm[3] = {range_damped(s.x0, TX, p.ulo[0], p.uhi[0]), range_damped(o, 1, p.ulo[1], p.uhi[1]),
                                    range_damped(s.z0, 32, p.ulo[2], p.uhi[2])};
                for (int a = 0; a < 3; ++a)
                    if (dm[a]) {
                        tma_field<MS>(ax, &mp.m[9 + a], bar, s.z0 + ZSP, s.x0, o, s.shot);
                        tma_field<MS>(ax + AUX, &mp.m[12 + a], bar, s.z0 + ZSP, s.x0, o, s.shot);
                        ax += 2 * AUX;
                    }
            });
        return;
    }

    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    T2 win[R][8];  // v at the last 8 planes, slot = item mod 8
    bool act[R], dxm[R], reca[R], recb[R], both = true, dza = false, dzb = false;
    float ax1[R], ax2[R];
    float2 az1{1, 1}, az2{1, 1};
    uint32_t gb[R];
    int trb[R];
    bool fast = false, tdx = false, tdz = false;
    int zmin = 0;  // tile's first z (SV-ball distance test)
    int x0s = 0;
    int3 sc = make_int3(0, 0, 0);  // source cell of the segment's shot
    SP *Pk = P, *Qk = Q;           // the segment's shot's fields
    float *reck = p.rec;
    const int *mutek = p.mute_nt;
    float ay1n = 1, ay2n = 1;
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
            zmin = s.z0;
            x0s = s.x0;
            sc = shot_cell<MS>(p, s.shot);
            if constexpr (MS) {
                const size_t fo = (size_t)s.shot * p.fstride_p;
                Pk = P + fo; Qk = Q + fo;
                px = (SP *)p.px + fo; py = (SP *)p.py + fo; pz = (SP *)p.pz + fo;
                qx = (SP *)p.qx + fo; qy = (SP *)p.qy + fo; qz = (SP *)p.qz + fo;
                reck = p.rec + (size_t)s.shot * p.rstride;
                mutek = p.mute_nt ? p.mute_nt + (size_t)s.shot * p.nx * p.ny : nullptr;
            }
            ay1n = p.ay1[s.ya];
            ay2n = p.ay2[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &, int) {
            constexpr int Q_ = decltype(ph)::value;
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
#pragma unroll
            for (int r = 0; r < R; ++r) win[r][Q_] = ld2<T>(A, (xw + r) * 32 + zl);
        },
        [&](int ph, uint32_t sa, uint32_t, const unsigned char *sbp, const Seg &, int q) {
            const int o = q - MM;
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
            T2 yy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int Q_ = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    T ya = 0, yb = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {  // v(o+m) in slot (Q+4+m)&7
                        const T2 hi = win[r][(Q_ + 4 + im) & 7], lo = win[r][(Q_ + 3 - im) & 7];
                        ya = fma_t(k[im], hi.a - lo.a, ya);
                        yb = fma_t(k[im], hi.b - lo.b, yb);
                    }
                    yy[r] = T2{ya, yb};
                    win[r][Q_] = ld2<T>(A, (xw + r) * 32 + zl);
                }
            });
            const S *Bu = reinterpret_cast<const S *>(sbp);
            const S *Bw = reinterpret_cast<const S *>(sbp + oW);
            const SP *Bp = reinterpret_cast<const SP *>(sbp + oP);
            const SP *Bq = reinterpret_cast<const SP *>(sbp + oQ);
            const float *F = reinterpret_cast<const float *>(sbp + oF);
            T2 us[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) us[j] = ld2<T>(Bu, (xw + j) * 32 + zl);
            const bool dym = o < p.ulo[1] || o >= p.uhi[1];
            const uint32_t po = pstride * (uint32_t)o;
            const float ay1 = ay1n, ay2 = ay2n;
            ay1n = p.ay1[o + 1];  // o + 1 <= nny - 4: in bounds
            ay2n = p.ay2[o + 1];
            // does the SV ball (r^2 <= 225 round the source) reach this tile plane?
            const int dy = o - sc.y;
            const int ddx = max(0, max(x0s - sc.x, sc.x - (x0s + TX - 1)));
            const int ddz = max(0, max(zmin - sc.z, sc.z - (zmin + 31)));
            const bool ball = dy * dy + ddx * ddx + ddz * ddz <= 225;
            // split pairs as packed by the producer: x, then y, then z, present ones only
            const SP *Xp = reinterpret_cast<const SP *>(sbp + oX);
            const SP *Yp = Xp + (tdx ? 2 * L::C : 0u);
            const SP *Zp = Yp + (dym ? 2 * L::C : 0u);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int bi = (xw + r) * 32 + zl, cw = (xw + r) * WW + (ZH - MM) + zl;
                T2 zp[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(Bw, cw + 2 * m);
                const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a,
                                  zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
                T xa = 0, xb = 0, za = 0, zb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // ..vti..:183-185
                    xa = fma_t(k[im], us[r + 4 + im].a - us[r + 3 - im].a, xa);
                    xb = fma_t(k[im], us[r + 4 + im].b - us[r + 3 - im].b, xb);
                    za = fma_t(k[im], zv[4 + im] - zv[3 - im], za);
                    zb = fma_t(k[im], zv[5 + im] - zv[4 - im], zb);
                }
                const float2 rv = *reinterpret_cast<const float2 *>(F + bi);
                const float2 vv = *reinterpret_cast<const float2 *>(F + L::C + bi);
                const float2 ep = *reinterpret_cast<const float2 *>(F + 2 * L::C + bi);
                const float2 de = *reinterpret_cast<const float2 *>(F + 3 * L::C + bi);
                float eea = ep.x, dda = de.x, eeb = ep.y, ddb = de.y;
                if (ball) {
                    const int ix = x0s + xw + r, iz = zmin + zl;
                    sv_eedd(p, sc, ix, o, iz, ep.x, de.x, eea, dda);
                    sv_eedd(p, sc, ix, o, iz + 1, ep.y, de.y, eeb, ddb);
                }
                const T2 Po = ld2<T>(Bp, bi), Qo = ld2<T>(Bq, bi);
                const uint32_t g = gb[r] + po;
                T pa, qa, pb, qb;
                if (fast && !dym) {  // no damped axis: ((P - gx) - gy) - gz, a1 == 1
                    const T c0[3] = {0, 0, 0};
                    T n0[3], n1[3];
                    vti_cell<T>(Po.a, Qo.a, xa, yy[r].a, za, rv.x, vv.x, eea, dda, false, false, false, 1.f, 1.f,
                                1.f, 1.f, 1.f, 1.f, c0, c0, dtx, dty, dtz, pa, qa, n0, n1);
                    vti_cell<T>(Po.b, Qo.b, xb, yy[r].b, zb, rv.y, vv.y, eeb, ddb, false, false, false, 1.f, 1.f,
                                1.f, 1.f, 1.f, 1.f, c0, c0, dtx, dty, dtz, pb, qb, n0, n1);
                    st2<SP, T>(Pk, g, pa, pb);
                    st2<SP, T>(Qk, g, qa, qb);
                    continue;
                }
                const T2 cpx = tdx ? ld2<T>(Xp, bi) : T2{0, 0}, cqx = tdx ? ld2<T>(Xp + L::C, bi) : T2{0, 0};
                const T2 cpy = dym ? ld2<T>(Yp, bi) : T2{0, 0}, cqy = dym ? ld2<T>(Yp + L::C, bi) : T2{0, 0};
                const T2 cpz = tdz ? ld2<T>(Zp, bi) : T2{0, 0}, cqz = tdz ? ld2<T>(Zp + L::C, bi) : T2{0, 0};
                const T cpa[3] = {cpx.a, cpy.a, cpz.a}, cqa[3] = {cqx.a, cqy.a, cqz.a};
                const T cpb[3] = {cpx.b, cpy.b, cpz.b}, cqb[3] = {cqx.b, cqy.b, cqz.b};
                T npa[3], nqa[3], npb[3], nqb[3];
                vti_cell<T>(Po.a, Qo.a, xa, yy[r].a, za, rv.x, vv.x, eea, dda, dxm[r], dym, dza, ax1[r], ay1,
                            az1.x, ax2[r], ay2, az2.x, cpa, cqa, dtx, dty, dtz, pa, qa, npa, nqa);
                vti_cell<T>(Po.b, Qo.b, xb, yy[r].b, zb, rv.y, vv.y, eeb, ddb, dxm[r], dym, dzb, ax1[r], ay1,
                            az1.y, ax2[r], ay2, az2.y, cpb, cqb, dtx, dty, dtz, pb, qb, npb, nqb);
                if (act[r]) {
                    st2m<SP, T>(Pk, g, pa, pb, both);
                    st2m<SP, T>(Qk, g, qa, qb, both);
                    if (dxm[r]) { st2m<SP, T>(px, g, npa[0], npb[0], both); st2m<SP, T>(qx, g, nqa[0], nqb[0], both); }
                    if (dym) { st2m<SP, T>(py, g, npa[1], npb[1], both); st2m<SP, T>(qy, g, nqa[1], nqb[1], both); }
                    if (dza && dzb && both) {
                        st2<SP, T>(pz, g, npa[2], npb[2]);
                        st2<SP, T>(qz, g, nqa[2], nqb[2]);
                    } else {
                        if (dza) { pz[g] = to_store<SP, T>(npa[2]); qz[g] = to_store<SP, T>(nqa[2]); }
                        if (dzb && both) { pz[g + 1] = to_store<SP, T>(npb[2]); qz[g + 1] = to_store<SP, T>(nqb[2]); }
                    }
                }
                if (o >= p.npml && o < p.npml + p.ny && (reca[r] | recb[r])) {  // ..vti..:313-323
                    const size_t tr = (size_t)trb[r] + (size_t)p.nx * (o - p.npml);
                    T rr = scl<S>(reca[r] ? pa : pb, p.rec_scale);
                    if (mutek && p.it < mutek[tr]) rr = T(0);
                    reck[tr * p.nt + p.it] = (float)rr;
                }
            }
        });
}

template <int TX, class S, int D, int R, bool MS, bool PF = false>
static inline cudaError_t launch_vti_s(const K1Launch &L, cudaStream_t st) {
    using SP = std::conditional_t<PF, float, S>;
    K1Params p = L.p;
    p.sw.nshot = MS ? (L.nshot > 1 ? L.nshot : 1) : 1;
    p.sw.sblk = MS ? L.sblk : 1;
    constexpr int NT = 32 * (TX / (2 * R) + 1);
    if (L.kind == K1_VTI_VEL) {
        static SmemAttr attr;
        Maps<6> mp;
        for (int i = 0; i < 6; ++i) mp.m[i] = L.maps[i];
        auto kern = vti_vel<TX, S, D, R, MS, PF>;
        const int grid = k1_sweep<TX>(p, kern, NT, VtiVelL<TX, S, D, SP>::TOTAL, L.grid, L.mode, L.rot);
        return k1_launch(kern, NT, VtiVelL<TX, S, D, SP>::TOTAL, p.sw.W, grid, st, attr, mp, (S *)L.out0,
                         (S *)L.out1, (S *)L.out2, p);
    }
    static SmemAttr attr;
    Maps<15> mp;
    for (int i = 0; i < 15; ++i) mp.m[i] = L.maps[i];
    auto kern = vti_stress<TX, S, D, R, MS, PF>;
    const int grid = k1_sweep<TX>(p, kern, NT, VtiStrL<TX, S, D, SP>::TOTAL, L.grid, L.mode, L.rot);
    return k1_launch(kern, NT, VtiStrL<TX, S, D, SP>::TOTAL, p.sw.W, grid, st, attr, mp, (SP *)L.out0,
                     (SP *)L.out1, p);
}

}  // namespace a3d
