// a3d_ktti.cuh — 1st-order pseudo-acoustic TTI engine (tilt theta, azimuth phi; no
// density): the kernel templates, instantiated by a3d_ktti.cu (FP32, FP64, 2-byte
// storage) and a3d_ktti_pf.cu (float16 u, v, w with float P, Q), which compile in
// parallel.
//
//   tti_vel:    xx = ct cp DxP - ct sp DyP - st DzP;  yy = sp DxP + cp DyP;
//               zz = st cp DxQ - st sp DyQ + ct DzQ;  u,v,w <- c2 u - c1 dt/d * (xx,yy,zz)
//               (..tti..:68-112; all six D+ derivatives, P and Q with z/x halo)
//   tti_stress: the same rotation of D-u, D-v, D-w, then the VTI coefficients
//               without density (..tti..:115-201), record + mute fused.
// cos/sin of theta and phi are evaluated once at setup (float), not per step.
// Wavefields may be stored in 2 bytes (bfloat16, or float16 with power-of-two
// scales folded into the coefficients); the arithmetic stays float.  With PF the
// pressures P, Q and their split components are float while u, v, w keep S.
#pragma once
#include <climits>
#include <type_traits>

#include "a3d_k1dev.cuh"

namespace a3d {

// ===========================================================================
// tti_vel: maps {P (H), Q (H), u, v, w (core), ct, st, cp, sp (core float)};
// SP: element type of P and Q
template <int TX, class S, int D, class SP = S>
struct TtiVelL {
    static constexpr int AW = ZHalo<SP>::W, AH = TX + 8;  // P / Q tile [AH][AW], z halo ZH
    static constexpr uint32_t C = 32 * TX, H = AW * AH;
    static constexpr uint32_t A_BYTES = 2 * H * sizeof(SP);  // P tile, then Q tile
    static constexpr uint32_t B_BYTES = 3 * C * sizeof(S) + 4 * C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static_assert((H * sizeof(SP)) % 128 == 0, "the Q tile starts 128-byte aligned");
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF, TOTAL = RG::TOTAL;
};

// the rotations of ..tti..:101-103 / 184-186 with the contractions nvcc applies
template <class T>
__device__ __forceinline__ void tti_rot(T ct, T st, T cp, T sp, T ax, T ay, T az, T bx, T by, T cx_,
                                        T cy_, T cz_, T &xx, T &yy, T &zz) {
    xx = fma_t(-st, az, fma_t(ct * cp, ax, -((ct * sp) * ay)));
    yy = fma_t(sp, bx, cp * by);
    zz = fma_t(ct, cz_, fma_t(st * cp, cx_, -((st * sp) * cy_)));
}

// the eight-point first derivatives of a cell pair along z from a halo'd row:
// zv[i] = row position zl + i (zl + 4 = cell a); forward (fwd) or backward
template <class T, class S>
__device__ __forceinline__ void dz2(const S *row, const T k[4], bool fwd, T &da, T &db) {
    Two<T> zp[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(row, 2 * m);
    const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a, zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
    T a = 0, b = 0;
#pragma unroll
    for (int im = 0; im < 4; ++im) {
        if (fwd) {
            a = fma_t(k[im], zv[5 + im] - zv[4 - im], a);
            b = fma_t(k[im], zv[6 + im] - zv[5 - im], b);
        } else {
            a = fma_t(k[im], zv[4 + im] - zv[3 - im], a);
            b = fma_t(k[im], zv[5 + im] - zv[4 - im], b);
        }
    }
    da = a;
    db = b;
}

template <int TX, class S, int D, int R, bool PF>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1))
    tti_vel(const __grid_constant__ Maps<9> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using SP = std::conditional_t<PF, float, S>;  // P, Q storage
    using L = TtiVelL<TX, S, D, SP>;
    using T = typename Arith<S>::T;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R), NC = 32 * NW, AW = L::AW;
    constexpr int ZS = WFieldZShift<S>::v;    // z offset of the u, v, w maps (2-byte storage)
    constexpr int ZSP = WFieldZShift<SP>::v;  // the same for the P, Q maps
    constexpr int ZH = ZHalo<SP>::ZH;         // first z cell of the tile inside a P / Q row
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
    constexpr size_t oF = 3 * L::C * sizeof(S);

    if (warp == NW) {  // producer warp: one thread issues every copy
        if (lane != 0) return;
        for (int i = 0; i < 9; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce_m<TX, L::KA, L::KB, L::RB>(
            p.sw, w0, w1, bars, ringB, p.err, [](const Seg &, int) { return (uint32_t)L::B_STRIDE; },
            [&](uint32_t sa, unsigned char *dst, uint32_t, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + (dst ? L::B_BYTES : 0u));
                unsigned char *a = ringA + sa * L::A_STRIDE;
                tma_load_3d(a, &mp.m[0], bar, s.z0 - ZH + ZSP, s.x0 - MM, q);
                tma_load_3d(a + L::H * sizeof(SP), &mp.m[1], bar, s.z0 - ZH + ZSP, s.x0 - MM, q);
                if (!dst) return;
                const int o = q - MM;
                for (int k = 0; k < 3; ++k)
                    tma_load_3d(dst + k * L::C * sizeof(S), &mp.m[2 + k], bar, s.z0 + ZS, s.x0, o);
                for (int k = 0; k < 4; ++k) tma_load_3d(dst + oF + k * L::C * 4, &mp.m[5 + k], bar, s.z0, s.x0, o);
            });
        return;
    }

    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    const int c0 = (xw + MM) * AW + zl + ZH;  // this lane's first cell pair in a P / Q tile
    T2 wp[R][8], wq[R][8];                    // P and Q at the last 8 planes, slot = item mod 8
    bool act[R], both = true;
    T cx1d[R], cx2[R];
    T2 cz1d{0, 0}, cz2{0, 0};
    uint32_t gb[R];
    int srcq = INT_MIN;
    float cy1n = 0, cy2n = 0;
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
    // the monopole enters the sweep's views of P and Q (..tti..:62-63)
    auto inject = [&](SP *A, const Seg &s) {
        if (threadIdx.x == 0) {
            const int at = (p.s_x - (s.x0 - MM)) * AW + (p.s_z - (s.z0 - ZH));
            A[at] = to_store<SP, T>(ld<T>(A, at) + (T)p.amp0);
            A[L::H + at] = to_store<SP, T>(ld<T>(A, L::H + at) + (T)p.amp1);
            fence_proxy_async();
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
            srcq = (p.inj && lx >= 0 && lx < L::AH && lz >= 0 && lz < AW) ? p.s_y : INT_MIN;
            cy1n = p.cy1[s.ya];
            cy2n = p.cy2[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &s, int q) {
            constexpr int P_ = decltype(ph)::value;
            SP *A = reinterpret_cast<SP *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                wp[r][P_] = ld2<T>(A, c0 + r * AW);
                wq[r][P_] = ld2<T>(A, L::H + c0 + r * AW);
            }
        },
        [&](int ph, uint32_t sa, uint32_t sh, const unsigned char *sbp, const Seg &s, int q) {
            SP *A = reinterpret_cast<SP *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
            T2 Py[R], Qy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int P_ = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    wp[r][P_] = ld2<T>(A, c0 + r * AW);
                    wq[r][P_] = ld2<T>(A, L::H + c0 + r * AW);
                    T pa = 0, pb = 0, qa = 0, qb = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {  // ..tti..:94-99, forward in y
                        const int hi = (P_ + 5 + im) & 7, lo = (P_ + 4 - im) & 7;
                        pa = fma_t(k[im], wp[r][hi].a - wp[r][lo].a, pa);
                        pb = fma_t(k[im], wp[r][hi].b - wp[r][lo].b, pb);
                        qa = fma_t(k[im], wq[r][hi].a - wq[r][lo].a, qa);
                        qb = fma_t(k[im], wq[r][hi].b - wq[r][lo].b, qb);
                    }
                    Py[r] = T2{pa, pb};
                    Qy[r] = T2{qa, qb};
                }
            });
            const int o = q - MM;
            const SP *Ao = reinterpret_cast<const SP *>(ringA + sh * L::A_STRIDE), *Bo = Ao + L::H;
            const S *Bu = reinterpret_cast<const S *>(sbp);
            const float *F = reinterpret_cast<const float *>(sbp + oF);
            const T cy1d = scl<S>((T)cy1n * (T)p.dty, p.svp), cy2 = (T)cy2n;
            cy1n = p.cy1[o + 1];  // o + 1 <= nny - 4: in bounds
            cy2n = p.cy2[o + 1];
            const uint32_t po = pstride * (uint32_t)o;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int bi = (xw + r) * 32 + zl, cr = c0 + r * AW;
                T pxa = 0, pxb = 0, qxa = 0, qxb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // forward in x: rows r+1+m and r-m
                    const T2 ph_ = ld2<T>(Ao, cr + (im + 1) * AW), pl = ld2<T>(Ao, cr - im * AW);
                    const T2 qh = ld2<T>(Bo, cr + (im + 1) * AW), ql = ld2<T>(Bo, cr - im * AW);
                    pxa = fma_t(k[im], ph_.a - pl.a, pxa);
                    pxb = fma_t(k[im], ph_.b - pl.b, pxb);
                    qxa = fma_t(k[im], qh.a - ql.a, qxa);
                    qxb = fma_t(k[im], qh.b - ql.b, qxb);
                }
                T pza, pzb, qza, qzb;
                dz2<T, SP>(Ao + cr - MM, k, true, pza, pzb);
                dz2<T, SP>(Bo + cr - MM, k, true, qza, qzb);
                const float2 ct = *reinterpret_cast<const float2 *>(F + bi);
                const float2 st_ = *reinterpret_cast<const float2 *>(F + L::C + bi);
                const float2 cp = *reinterpret_cast<const float2 *>(F + 2 * L::C + bi);
                const float2 sp = *reinterpret_cast<const float2 *>(F + 3 * L::C + bi);
                T xa, ya, za, xb, yb, zb;
                tti_rot<T>((T)ct.x, (T)st_.x, (T)cp.x, (T)sp.x, pxa, Py[r].a, pza, pxa, Py[r].a, qxa, Qy[r].a, qza,
                           xa, ya, za);
                tti_rot<T>((T)ct.y, (T)st_.y, (T)cp.y, (T)sp.y, pxb, Py[r].b, pzb, pxb, Py[r].b, qxb, Qy[r].b, qzb,
                           xb, yb, zb);
                const T2 uo = ld2<T>(Bu, bi), vo = ld2<T>(Bu, L::C + bi), wo = ld2<T>(Bu, 2 * L::C + bi);
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
// tti_stress: maps {u, v, w (H), P, Q (core), vp, eps, del, ct, st, cp, sp (core float),
//                   px, py, pz, qx, qy, qz (core; only for tiles/planes on a damped axis)}
// (SP: element type of P, Q and the split components)
template <int TX, class S, int D, class SP = S>
struct TtiStrL {
    static constexpr int AW = ZHalo<S>::W, AH = TX + 8;  // u / v / w tile [AH][AW], z halo ZH
    static constexpr uint32_t C = 32 * TX, H = AW * AH;
    static constexpr uint32_t A_BYTES = 3 * H * sizeof(S);  // u, v, w tiles
    static constexpr uint32_t B_FIXED = 2 * C * sizeof(SP) + 7 * C * 4;
    static constexpr uint32_t AUX = C * sizeof(SP);
    static constexpr uint32_t B_BYTES = B_FIXED + 6 * AUX;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static_assert((H * sizeof(S)) % 128 == 0 && B_FIXED % 128 == 0 && AUX % 128 == 0, "128-byte aligned parts");
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF, TOTAL = RG::TOTAL;
};

__device__ __forceinline__ void sv_eedd_t(const K1Params &p, int ix, int iy, int iz, float eps,
                                          float del, float &ee, float &dd) {
    const int rx = ix - p.s_x, ry = iy - p.s_y, rz = iz - p.s_z;
    const int d2 = rx * rx + ry * ry + rz * rz;
    if (d2 > 225) { ee = eps; dd = del; return; }
    const float2 t = p.taper[d2];
    ee = mul_df(eps, t.x, t.y);
    dd = mul_df(del, t.x, t.y);
}

// the TTI pressure pair of one cell (..tti..:187-200, VTI coefficients without
// density): returns P and Q, the new split components of damped axes in np3 / nq3
// (select-based engine form of the oracle's engine_pupdate, operation order kept)
template <class T>
__device__ __forceinline__ void tti_cell(T Po, T Qo, T xx, T yy, T zz, float vv, float ee, float dd,
                                         const bool d3[3], const float a1[3], const float a2[3],
                                         const T cp[3], const T cq[3], T dtx, T dty, T dtz, T &Pn,
                                         T &Qn, T np3[3], T nq3[3]) {
    T e1, sd;
    if constexpr (sizeof(T) == 4) {
        e1 = 1.0f + 2.0f * ee;
        sd = sqrtf(1.0f + 2.0f * dd);
    } else {
        e1 = T(1) + T(2) * (T)ee;
        sd = sqrt(T(1) + T(2) * (T)dd);
    }
    const T kx = ((T)a1[0] * (T)vv) * (T)vv, ky = ((T)a1[1] * (T)vv) * (T)vv, kz = ((T)a1[2] * (T)vv) * (T)vv;
    const T gP[3] = {((kx * e1) * dtx) * xx, ((ky * e1) * dty) * yy, ((kz * sd) * dtz) * zz};
    const T gQ[3] = {((kx * sd) * dtx) * xx, ((ky * sd) * dty) * yy, (kz * dtz) * zz};
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

template <int TX, class S, int D, int R, bool PF>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1))
    tti_stress(const __grid_constant__ Maps<18> mp, std::conditional_t<PF, float, S> *__restrict__ P,
               std::conditional_t<PF, float, S> *__restrict__ Q, const __grid_constant__ K1Params p) {
    using SP = std::conditional_t<PF, float, S>;  // P, Q and split-component storage
    using L = TtiStrL<TX, S, D, SP>;
    using T = typename Arith<S>::T;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R), AW = L::AW;
    constexpr int ZS = WFieldZShift<S>::v;  // z offset of wavefield maps (2-byte storage)
    constexpr int ZH = ZHalo<S>::ZH;        // first z cell of the tile inside a u / v / w row
    constexpr int ZSP = WFieldZShift<SP>::v;  // z offset of the P, Q and split maps
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
    constexpr size_t oF = 2 * L::C * sizeof(SP);  // vp eps del ct st cp sp
    constexpr size_t oX = L::B_FIXED;             // split pairs of the damped axes follow
    constexpr uint32_t AUX = L::AUX;
    SP *px = (SP *)p.px, *py = (SP *)p.py, *pz = (SP *)p.pz, *qx = (SP *)p.qx, *qy = (SP *)p.qy, *qz = (SP *)p.qz;

    if (warp == NW) {  // producer warp: one thread issues every copy
        if (lane != 0) return;
        for (int i = 0; i < 18; ++i) prefetch_tmap(&mp.m[i]);
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
                unsigned char *a = ringA + sa * L::A_STRIDE;
                for (int k = 0; k < 3; ++k)
                    tma_load_3d(a + k * L::H * sizeof(S), &mp.m[k], bar, s.z0 - ZH + ZS, s.x0 - MM, q);
                if (!dst) return;
                const int o = q - MM;
                tma_load_3d(dst, &mp.m[3], bar, s.z0 + ZSP, s.x0, o);
                tma_load_3d(dst + L::C * sizeof(SP), &mp.m[4], bar, s.z0 + ZSP, s.x0, o);
                for (int k = 0; k < 7; ++k) tma_load_3d(dst + oF + k * L::C * 4, &mp.m[5 + k], bar, s.z0, s.x0, o);
                unsigned char *ax = dst + oX;
                const bool dm[3] = {range_damped(s.x0, TX, p.ulo[0], p.uhi[0]), range_damped(o, 1, p.ulo[1], p.uhi[1]),
                                    range_damped(s.z0, 32, p.ulo[2], p.uhi[2])};
                for (int d = 0; d < 3; ++d)
                    if (dm[d]) {
                        tma_load_3d(ax, &mp.m[12 + d], bar, s.z0 + ZSP, s.x0, o);
                        tma_load_3d(ax + AUX, &mp.m[15 + d], bar, s.z0 + ZSP, s.x0, o);
                        ax += 2 * AUX;
                    }
            });
        return;
    }

    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    const int c0 = (xw + MM) * AW + zl + ZH;  // this lane's first cell pair in a u / v / w tile
    T2 wu[R][8], wv[R][8], ww[R][8];          // u, v, w at the last 8 planes, slot = item mod 8
    bool act[R], dxm[R], reca[R], recb[R], both = true, dza = false, dzb = false;
    float ax1[R], ax2[R];
    float2 az1{1, 1}, az2{1, 1};
    uint32_t gb[R];
    int trb[R];
    bool tdx = false, tdz = false;
    int zmin = 0, x0s = 0;
    float ay1n = 1, ay2n = 1;
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
    // 2-byte storage: P, Q hold sigma_P values, u, v, w sigma_v values
    const T dtx = scl<S>((T)p.dtx, p.spv), dty = scl<S>((T)p.dty, p.spv), dtz = scl<S>((T)p.dtz, p.spv);
    pipe_run<TX, L::KA, L::KB, MM>(
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
            zmin = s.z0;
            x0s = s.x0;
            ay1n = p.ay1[s.ya];
            ay2n = p.ay2[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &, int) {
            constexpr int Q_ = decltype(ph)::value;
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                wu[r][Q_] = ld2<T>(A, c0 + r * AW);
                wv[r][Q_] = ld2<T>(A, L::H + c0 + r * AW);
                ww[r][Q_] = ld2<T>(A, 2 * L::H + c0 + r * AW);
            }
        },
        [&](int ph, uint32_t sa, uint32_t sh, const unsigned char *sbp, const Seg &, int q) {
            const int o = q - MM;
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
            // backward y-derivatives at o from the windows (plane o+m in slot (ph+4+m)&7),
            // then the planes q replace q-8 (..tti..:174-182)
            T2 uy[R], vy[R], wy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int Q_ = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    T ua = 0, ub = 0, va = 0, vb = 0, wa = 0, wb = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {
                        const int hi = (Q_ + 4 + im) & 7, lo = (Q_ + 3 - im) & 7;
                        ua = fma_t(k[im], wu[r][hi].a - wu[r][lo].a, ua);
                        ub = fma_t(k[im], wu[r][hi].b - wu[r][lo].b, ub);
                        va = fma_t(k[im], wv[r][hi].a - wv[r][lo].a, va);
                        vb = fma_t(k[im], wv[r][hi].b - wv[r][lo].b, vb);
                        wa = fma_t(k[im], ww[r][hi].a - ww[r][lo].a, wa);
                        wb = fma_t(k[im], ww[r][hi].b - ww[r][lo].b, wb);
                    }
                    uy[r] = T2{ua, ub};
                    vy[r] = T2{va, vb};
                    wy[r] = T2{wa, wb};
                    wu[r][Q_] = ld2<T>(A, c0 + r * AW);
                    wv[r][Q_] = ld2<T>(A, L::H + c0 + r * AW);
                    ww[r][Q_] = ld2<T>(A, 2 * L::H + c0 + r * AW);
                }
            });
            const S *U = reinterpret_cast<const S *>(ringA + sh * L::A_STRIDE), *V = U + L::H, *W = U + 2 * L::H;
            const SP *Bp = reinterpret_cast<const SP *>(sbp), *Bq = Bp + L::C;
            const float *F = reinterpret_cast<const float *>(sbp + oF);
            const bool dym = o < p.ulo[1] || o >= p.uhi[1];
            const uint32_t po = pstride * (uint32_t)o;
            const float ay1 = ay1n, ay2 = ay2n;
            ay1n = p.ay1[o + 1];  // o + 1 <= nny - 4: in bounds
            ay2n = p.ay2[o + 1];
            const int dy = o - p.s_y;
            const int ddx = max(0, max(x0s - p.s_x, p.s_x - (x0s + TX - 1)));
            const int ddz = max(0, max(zmin - p.s_z, p.s_z - (zmin + 31)));
            const bool ball = dy * dy + ddx * ddx + ddz * ddz <= 225;
            const SP *Xp = reinterpret_cast<const SP *>(sbp + oX);
            const SP *Yp = Xp + (tdx ? 2 * L::C : 0u);
            const SP *Zp = Yp + (dym ? 2 * L::C : 0u);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int bi = (xw + r) * 32 + zl, cr = c0 + r * AW;
                T uxa = 0, uxb = 0, vxa = 0, vxb = 0, wxa = 0, wxb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // backward in x: rows r+m and r-1-m
                    const T2 uh = ld2<T>(U, cr + im * AW), ul = ld2<T>(U, cr - (im + 1) * AW);
                    const T2 vh = ld2<T>(V, cr + im * AW), vl = ld2<T>(V, cr - (im + 1) * AW);
                    const T2 wh = ld2<T>(W, cr + im * AW), wl = ld2<T>(W, cr - (im + 1) * AW);
                    uxa = fma_t(k[im], uh.a - ul.a, uxa);
                    uxb = fma_t(k[im], uh.b - ul.b, uxb);
                    vxa = fma_t(k[im], vh.a - vl.a, vxa);
                    vxb = fma_t(k[im], vh.b - vl.b, vxb);
                    wxa = fma_t(k[im], wh.a - wl.a, wxa);
                    wxb = fma_t(k[im], wh.b - wl.b, wxb);
                }
                T uza, uzb, wza, wzb;  // the z-derivative of v is not used (..tti..:174-182)
                dz2<T, S>(U + cr - MM, k, false, uza, uzb);
                dz2<T, S>(W + cr - MM, k, false, wza, wzb);
                const float2 vv = *reinterpret_cast<const float2 *>(F + bi);
                const float2 ep = *reinterpret_cast<const float2 *>(F + L::C + bi);
                const float2 de = *reinterpret_cast<const float2 *>(F + 2 * L::C + bi);
                const float2 ct = *reinterpret_cast<const float2 *>(F + 3 * L::C + bi);
                const float2 st_ = *reinterpret_cast<const float2 *>(F + 4 * L::C + bi);
                const float2 cp = *reinterpret_cast<const float2 *>(F + 5 * L::C + bi);
                const float2 sp = *reinterpret_cast<const float2 *>(F + 6 * L::C + bi);
                T xa, ya, za, xb, yb, zb;
                tti_rot<T>((T)ct.x, (T)st_.x, (T)cp.x, (T)sp.x, uxa, uy[r].a, uza, vxa, vy[r].a, wxa, wy[r].a, wza,
                           xa, ya, za);
                tti_rot<T>((T)ct.y, (T)st_.y, (T)cp.y, (T)sp.y, uxb, uy[r].b, uzb, vxb, vy[r].b, wxb, wy[r].b, wzb,
                           xb, yb, zb);
                float eea = ep.x, dda = de.x, eeb = ep.y, ddb = de.y;
                if (ball) {
                    const int ix = x0s + xw + r, iz = zmin + zl;
                    sv_eedd_t(p, ix, o, iz, ep.x, de.x, eea, dda);
                    sv_eedd_t(p, ix, o, iz + 1, ep.y, de.y, eeb, ddb);
                }
                const T2 Po = ld2<T>(Bp, bi), Qo = ld2<T>(Bq, bi);
                const T2 cpx = tdx ? ld2<T>(Xp, bi) : T2{0, 0}, cqx = tdx ? ld2<T>(Xp + L::C, bi) : T2{0, 0};
                const T2 cpy = dym ? ld2<T>(Yp, bi) : T2{0, 0}, cqy = dym ? ld2<T>(Yp + L::C, bi) : T2{0, 0};
                const T2 cpz = tdz ? ld2<T>(Zp, bi) : T2{0, 0}, cqz = tdz ? ld2<T>(Zp + L::C, bi) : T2{0, 0};
                const T cpa[3] = {cpx.a, cpy.a, cpz.a}, cqa[3] = {cqx.a, cqy.a, cqz.a};
                const T cpb[3] = {cpx.b, cpy.b, cpz.b}, cqb[3] = {cqx.b, cqy.b, cqz.b};
                const bool d3a[3] = {dxm[r], dym, dza}, d3b[3] = {dxm[r], dym, dzb};
                const float a1a[3] = {ax1[r], ay1, az1.x}, a2a[3] = {ax2[r], ay2, az2.x};
                const float a1b[3] = {ax1[r], ay1, az1.y}, a2b[3] = {ax2[r], ay2, az2.y};
                T pa, qa, pb, qb, npa[3], nqa[3], npb[3], nqb[3];
                tti_cell<T>(Po.a, Qo.a, xa, ya, za, vv.x, eea, dda, d3a, a1a, a2a, cpa, cqa, dtx, dty, dtz, pa, qa,
                            npa, nqa);
                tti_cell<T>(Po.b, Qo.b, xb, yb, zb, vv.y, eeb, ddb, d3b, a1b, a2b, cpb, cqb, dtx, dty, dtz, pb, qb,
                            npb, nqb);
                const uint32_t g = gb[r] + po;
                if (act[r]) {
                    st2m<SP, T>(P, g, pa, pb, both);
                    st2m<SP, T>(Q, g, qa, qb, both);
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
                if (o >= p.npml && o < p.npml + p.ny && (reca[r] | recb[r])) {  // ..tti..:313-323
                    const size_t tr = (size_t)trb[r] + (size_t)p.nx * (o - p.npml);
                    T rr = scl<S>(reca[r] ? pa : pb, p.rec_scale);
                    if (p.mute_nt && p.it < p.mute_nt[tr]) rr = T(0);
                    p.rec[tr * p.nt + p.it] = (float)rr;
                }
            }
        });
}

template <int TX, class S, int D, int R, bool PF = false>
static inline cudaError_t launch_tti_t(const K1Launch &L, cudaStream_t st) {
    using SP = std::conditional_t<PF, float, S>;
    K1Params p = L.p;
    constexpr int NT = 32 * (TX / (2 * R) + 1);
    if (L.kind == K1_TTI_VEL) {
        static SmemAttr attr;
        Maps<9> mp;
        for (int i = 0; i < 9; ++i) mp.m[i] = L.maps[i];
        auto kern = tti_vel<TX, S, D, R, PF>;
        const int grid = k1_sweep<TX>(p, kern, NT, TtiVelL<TX, S, D, SP>::TOTAL, L.grid, L.mode, L.rot);
        return k1_launch(kern, NT, TtiVelL<TX, S, D, SP>::TOTAL, p.sw.W, grid, st, attr, mp, (S *)L.out0,
                         (S *)L.out1, (S *)L.out2, p);
    }
    static SmemAttr attr;
    Maps<18> mp;
    for (int i = 0; i < 18; ++i) mp.m[i] = L.maps[i];
    auto kern = tti_stress<TX, S, D, R, PF>;
    const int grid = k1_sweep<TX>(p, kern, NT, TtiStrL<TX, S, D, SP>::TOTAL, L.grid, L.mode, L.rot);
    return k1_launch(kern, NT, TtiStrL<TX, S, D, SP>::TOTAL, p.sw.W, grid, st, attr, mp, (SP *)L.out0,
                     (SP *)L.out1, p);
}

}  // namespace a3d
