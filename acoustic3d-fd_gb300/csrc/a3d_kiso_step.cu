// a3d_kiso_step.cu — 1st-order isotropic engine, one fused sweep per time step (FP32).
//
// The two-sweep form (a3d_kiso.cu) moves 60 B per cell and step: the velocity sweep
// reads P, u, v, w, 1/rho and writes u, v, w; the stress sweep reads them back with
// P, rho, vp.  Here one y-march does both.  At item q (P plane q arrives) the
// consumer warps
//   1. update P at o2 = q - 8 (..iso..:145-190) from the new v of planes o2-4 .. o2+3
//      (a register window), the new u and w of plane o2 with their x / z halos (a
//      shared-memory ring of the last 6 velocity steps) and P, rho, vp of plane o2;
//   2. update u, v, w at o1 = q - 4 (..iso..:99-142) from P planes o1-3 .. o1+4 (a
//      register window) and the P tile of plane o1 with 8-cell x and z halos,
//      including the 4 halo rows of u and halo columns of w that step 1 of this
//      tile will need; the neighbouring tiles compute the same halo values.
// The warps share the ring through per-slot mbarriers (written by all / read by all),
// so a warp waits for the others only when it needs their rows, up to 4 steps later.
// Velocities and P are read from one buffer set and written to the other (the
// engine swaps the sets every step; un, vn, wn, Pn are the set written), so halo
// reads never see a neighbour's new
// values.  A segment of pressure planes [oa, ob) runs velocities over
// [oa - 4, ob + 4).  Arithmetic and operation order are iso_vel's and iso_stress's
// (the oracle's engine form), so records are bit-identical to the two-sweep form.
// Compulsory traffic: u, v, w, P, 1/rho, rho, vp read, u, v, w, P written: 44 B.
#include <climits>

#include "a3d_k1dev.cuh"

namespace a3d {

template <int TX, int D>
struct IsoStepL {
    static_assert(D == 0 || D == 1, "fused step: ring depths 0 and 1");
    static constexpr int AW = 48, AH = TX + 16;  // P tile [AH][AW] from (x0 - 8, z0 - 8)
    static constexpr uint32_t A_BYTES = AW * AH * 4;
    static constexpr uint32_t C = 32 * TX, UX = 32 * (TX + 8), WZ = 40 * TX, RH = 40 * (TX + 8);
    // velocity part of a B item (plane o1): u (x halo), v, w (z halo), 1/rho (both halos)
    static constexpr uint32_t OU = 0, OV = UX * 4, OW = OV + C * 4, ORI = OW + WZ * 4, BV = ORI + RH * 4;
    // pressure part (plane o2, present while o2 is an output plane): P, rho, vp, then
    // one split tile per damped axis
    static constexpr uint32_t OP = BV, ORHO = OP + C * 4, OVP = ORHO + C * 4, OX = OVP + C * 4, AUX = C * 4;
    static constexpr uint32_t B_BYTES = OX + 3 * AUX;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static_assert(BV % 128 == 0 && OX % 128 == 0 && AUX % 128 == 0, "B item parts are 128-byte aligned");
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF;
    // rings of the new u ([TX+8][32], x halo) and w ([TX][40], z halo) of the last NR
    // velocity steps, with per-slot barriers: velDone (every consumer warp wrote its part)
    // and strDone (every consumer warp finished reading it for the pressure update)
    static constexpr int NR = 6;
    static constexpr size_t RU_OFF = (RG::TOTAL + 127) / 128 * 128, RW_OFF = RU_OFF + NR * UX * 4;
    static constexpr size_t RBAR_OFF = RW_OFF + NR * WZ * 4;
    static constexpr size_t TOTAL = RBAR_OFF + 2 * NR * sizeof(uint64_t);
};

template <int TX, int D, int R>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1))
    iso_step(const __grid_constant__ Maps<11> mp, float *__restrict__ un, float *__restrict__ vn,
             float *__restrict__ wn, float *__restrict__ Pn, const __grid_constant__ K1Params p) {
    using L = IsoStepL<TX, D>;
    using T = float;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R), NC = 32 * NW, AW = L::AW;
    static_assert(NW >= 1 && 8 * R <= 32, "warp / halo task shape");
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<typename L::Bars *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::B_OFF;
    float *ringU = reinterpret_cast<float *>(smem + L::RU_OFF);
    float *ringW = reinterpret_cast<float *>(smem + L::RW_OFF);
    uint64_t *velDone = reinterpret_cast<uint64_t *>(smem + L::RBAR_OFF), *strDone = velDone + L::NR;
    if (threadIdx.x == 0) {
        for (int i = 0; i < L::NR; ++i) {
            mbar_init(&velDone[i], NW);
            mbar_init(&strDone[i], NW);
        }
        bars.init(NW);  // fences the barrier initialisations
    }
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == NW) {  // producer warp: one thread issues every copy
        if (lane != 0) return;
        for (int i = 0; i < 11; ++i) prefetch_tmap(&mp.m[i]);
        auto naux = [&](const Seg &s, int o) {
            return (uint32_t)range_damped(s.x0, TX, p.ulo[0], p.uhi[0]) +
                   (uint32_t)range_damped(o, 1, p.ulo[1], p.uhi[1]) +
                   (uint32_t)range_damped(s.z0, 32, p.ulo[2], p.uhi[2]);
        };
        auto str = [](const Seg &s, int o1) { return o1 - MM >= s.oa && o1 - MM < s.ob; };
        pipe_produce_m<TX, L::KA, L::KB, L::RB, MM>(
            p.sw, w0, w1, bars, ringB, p.err,
            [&](const Seg &s, int o1) {
                return L::BV + (str(s, o1) ? (L::OX - L::BV) + L::AUX * naux(s, o1 - MM) : 0u);
            },
            [&](uint32_t sa, unsigned char *dst, uint32_t bbytes, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + bbytes);
                tma_load_3d(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0 - 8, s.x0 - 8, q);
                if (!dst) return;
                const int o1 = q - MM;
                tma_load_3d(dst + L::OU, &mp.m[1], bar, s.z0, s.x0 - MM, o1);
                tma_load_3d(dst + L::OV, &mp.m[2], bar, s.z0, s.x0, o1);
                tma_load_3d(dst + L::OW, &mp.m[3], bar, s.z0 - MM, s.x0, o1);
                tma_load_3d(dst + L::ORI, &mp.m[4], bar, s.z0 - MM, s.x0 - MM, o1);
                if (!str(s, o1)) return;
                const int o2 = o1 - MM;
                tma_load_3d(dst + L::OP, &mp.m[5], bar, s.z0, s.x0, o2);
                tma_load_3d(dst + L::ORHO, &mp.m[6], bar, s.z0, s.x0, o2);
                tma_load_3d(dst + L::OVP, &mp.m[7], bar, s.z0, s.x0, o2);
                unsigned char *ax = dst + L::OX;
                if (range_damped(s.x0, TX, p.ulo[0], p.uhi[0])) { tma_load_3d(ax, &mp.m[8], bar, s.z0, s.x0, o2); ax += L::AUX; }
                if (range_damped(o2, 1, p.ulo[1], p.uhi[1])) { tma_load_3d(ax, &mp.m[9], bar, s.z0, s.x0, o2); ax += L::AUX; }
                if (range_damped(s.z0, 32, p.ulo[2], p.uhi[2])) tma_load_3d(ax, &mp.m[10], bar, s.z0, s.x0, o2);
            });
        return;
    }

    // lane: z cells zl, zl+1 of the tile (zl = 2 (lane mod 16)) in tile rows
    // xw .. xw+R-1, where the two half-warps take consecutive groups of R rows
    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    const int c0 = (xw + 8) * AW + zl + 8;  // this lane's first cell pair in a P tile
    // halo work of this lane: u at halo rows hr[k] (tile rows -4..-1, TX..TX+3; half-warp
    // hw takes rows hw, hw + 2 NW, ...), w at one (z pair, row) of the 4 x TX halo
    // columns (task t = warp + NW lane for lane < 8 R)
    constexpr int NHU = (8 + 2 * NW - 1) / (2 * NW);
    const int hw = warp * 2 + (lane >> 4);
    T2 winP[R][8];  // P at the last 8 planes, slot = item mod 8
    T2 winV[R][8];  // new v at the last 8 velocity planes, slot = item mod 8
    bool act[R], both = true;
    T cx1d[R], cx2[R];
    T2 cz1d{0, 0}, cz2{0, 0};
    uint32_t gb[R];
    // halo u rows
    int hr[NHU];
    bool hact[NHU];
    T hcx1d[NHU], hcx2[NHU];
    // halo w task
    const int wt = warp + NW * lane;
    const bool wtask = lane < 8 * R && wt < 4 * TX;
    const int wrow = wt >> 2, wzo = (wt & 3) < 2 ? 2 * (wt & 3) : 32 + 2 * (wt & 3);  // z offset in the w row (40)
    bool wacta = false, wactb = false;
    T2 wcz1d{0, 0}, wcz2{0, 0};
    // pressure update coefficients
    bool dxm[R], reca[R], recb[R], dza = false, dzb = false;
    float ax1[R], ax2[R];
    float2 az1{1, 1}, az2{1, 1};
    int trb[R];
    bool fast = false, tdx = false, tdz = false;
    int srcq = INT_MIN;
    float cy1n = 0, cy2n = 0;
    // step counter of this CTA: step J writes ring slot J mod NR, and its pressure
    // update reads the slot step J - 4 wrote (both within one segment when it runs)
    uint32_t J = 0;
    volatile int *ab = bars.abort_ptr();
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
    const T dtx = (T)p.dtx, dty = (T)p.dty, dtz = (T)p.dtz;
    auto inject = [&](float *A, const Seg &s) {
        const int lx = p.s_x - (s.x0 - 8), lz = p.s_z - (s.z0 - 8);
        if (threadIdx.x == 0) {
            if (lz >= 0 && lz < AW) A[lx * AW + lz] = A[lx * AW + lz] + (T)p.amp0;
            if (lz + 2 >= 0 && lz + 2 < AW) A[lx * AW + lz + 2] = A[lx * AW + lz + 2] + (T)p.amp1;
            fence_proxy_async();  // the stage is refilled by TMA later
        }
        consumer_sync(NC);
    };
    pipe_run<TX, L::KA, L::KB, MM, MM>(
        p.sw, w0, w1, bars, ringB, p.err,
        [&](const Seg &s) {
            const int iz = s.z0 + zl;
            const bool zact = iz < p.nnz - MM;
            both = iz + 1 < p.nnz - MM;
            const int cza = min(iz, p.nnz - 1), czb = min(iz + 1, p.nnz - 1);
            cz1d = T2{(T)p.cz1[cza] * dtz, (T)p.cz1[czb] * dtz};
            cz2 = T2{(T)p.cz2[cza], (T)p.cz2[czb]};
            az1 = float2{p.az1[cza], p.az1[czb]};
            az2 = float2{p.az2[cza], p.az2[czb]};
            dza = damped(az1.x, az2.x);
            dzb = damped(az1.y, az2.y);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                cx1d[r] = (T)p.cx1[cxi] * dtx;
                cx2[r] = (T)p.cx2[cxi];
                ax1[r] = p.ax1[cxi];
                ax2[r] = p.ax2[cxi];
                dxm[r] = damped(ax1[r], ax2[r]);
                const bool rx = act[r] && ix >= p.npml && ix < p.npml + p.nx;
                reca[r] = rx && iz == p.npml;
                recb[r] = rx && both && iz + 1 == p.npml;
                trb[r] = ix - p.npml;
                gb[r] = (uint32_t)iz + (uint32_t)p.ldz * (uint32_t)cxi;
            }
#pragma unroll
            for (int j = 0; j < NHU; ++j) {
                const int hk = hw + 2 * NW * j;  // 0..7 -> rows -4..-1, TX..TX+3
                hr[j] = hk < 4 ? hk - 4 : TX + hk - 4;
                const int ix = s.x0 + hr[j];
                hact[j] = hk < 8 && zact && ix >= MM && ix < p.nnx - MM;
                const int cxi = min(max(ix, 0), p.nnx - 1);
                hcx1d[j] = (T)p.cx1[cxi] * dtx;
                hcx2[j] = (T)p.cx2[cxi];
            }
            {
                const int iza = s.z0 - MM + wzo, ixw = s.x0 + wrow;
                const bool xa = wtask && ixw < p.nnx - MM;
                wacta = xa && iza >= MM && iza < p.nnz - MM;
                wactb = xa && iza + 1 >= MM && iza + 1 < p.nnz - MM;
                const int ca = min(max(iza, 0), p.nnz - 1), cb = min(max(iza + 1, 0), p.nnz - 1);
                wcz1d = T2{(T)p.cz1[ca] * dtz, (T)p.cz1[cb] * dtz};
                wcz2 = T2{(T)p.cz2[ca], (T)p.cz2[cb]};
            }
            tdx = range_damped(s.x0, TX, p.ulo[0], p.uhi[0]);
            tdz = range_damped(s.z0, 32, p.ulo[2], p.uhi[2]);
            fast = !tdx && !tdz && !(p.npml >= s.z0 && p.npml < s.z0 + 32);
            const int lx = p.s_x - (s.x0 - 8), lz = p.s_z - (s.z0 - 8);
            srcq = (p.inj && lx >= 0 && lx < L::AH && lz + 2 >= 0 && lz < AW) ? p.s_y : INT_MIN;
            cy1n = p.cy1[s.ya];
            cy2n = p.cy2[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &s, int q) {
            constexpr int Q = decltype(ph)::value;
            float *A = reinterpret_cast<float *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
#pragma unroll
            for (int r = 0; r < R; ++r) winP[r][Q] = ld2<T>(A, c0 + r * AW);
        },
        [&](int ph, uint32_t sa, uint32_t sh, const unsigned char *sbp, const Seg &s, int q) {
            float *A = reinterpret_cast<float *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
            const int o1 = q - MM, o2 = o1 - MM;
            // window push of P(q) and the y-derivative of P at o1 (..iso..:126)
            T2 yyP[R];
            with_phase(ph, [&](auto pc) {
                constexpr int Q = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    winP[r][Q] = ld2<T>(A, c0 + r * AW);
                    T a = 0, b = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {  // P(o1+1+m) in slot (Q+5+m)&7, P(o1-m) in (Q+4-m)&7
                        const T2 hi = winP[r][(Q + 5 + im) & 7], lo = winP[r][(Q + 4 - im) & 7];
                        a = fma_t(k[im], hi.a - lo.a, a);
                        b = fma_t(k[im], hi.b - lo.b, b);
                    }
                    yyP[r] = T2{a, b};
                }
            });

            // ---- 1. pressure at o2 (..iso..:145-190)
            const bool pres = o2 >= s.oa && o2 < s.ob;
            if (pres)  // every warp has written step J - 4's ring slot
                mbar_wait(&velDone[(J - 4) % L::NR], ((J - 4) / L::NR) & 1, p.err, KERR_FULL_TIMEOUT, ab);
            if (pres) {
                T2 yy[R];  // D-y v at o2 from v(o2-4 .. o2+3): plane o2+m in slot (ph+4+m)&7
                with_phase(ph, [&](auto pc) {
                    constexpr int Q = decltype(pc)::value;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        T ya = 0, yb = 0;
#pragma unroll
                        for (int im = 0; im < 4; ++im) {
                            const T2 hi = winV[r][(Q + 4 + im) & 7], lo = winV[r][(Q + 3 - im) & 7];
                            ya = fma_t(k[im], hi.a - lo.a, ya);
                            yb = fma_t(k[im], hi.b - lo.b, yb);
                        }
                        yy[r] = T2{ya, yb};
                    }
                });
                const float *Bu = ringU + ((J - 4) % L::NR) * L::UX;
                const float *Bw = ringW + ((J - 4) % L::NR) * L::WZ;
                const float *Bp = reinterpret_cast<const float *>(sbp + L::OP);
                const float *Br = reinterpret_cast<const float *>(sbp + L::ORHO);
                const float *Bvp = reinterpret_cast<const float *>(sbp + L::OVP);
                const float *Bx = reinterpret_cast<const float *>(sbp + L::OX);
                const bool dym = o2 < p.ulo[1] || o2 >= p.uhi[1];
                const float *By = Bx + (tdx ? L::C : 0u);
                const float *Bz = By + (dym ? L::C : 0u);
                T2 us[R + 7];  // us[j] = u(x = xw - 4 + j)
#pragma unroll
                for (int j = 0; j < R + 7; ++j) us[j] = ld2<T>(Bu, (xw + j) * 32 + zl);
                const uint32_t po = pstride * (uint32_t)o2;
                const float ay1 = p.ay1[o2], ay2 = p.ay2[o2];
                auto deriv = [&](int r, T2 &xx, T2 &zz) {
                    T2 zp[5];
#pragma unroll
                    for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(Bw, (xw + r) * 40 + zl + 2 * m);
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
                        const T ta = (rv.x * vv.x) * vv.x, tb = (rv.y * vv.y) * vv.y;
                        const T pa = ((Po.a - (ta * dtx) * xx.a) - (ta * dty) * yy[r].a) - (ta * dtz) * zz.a;
                        const T pb = ((Po.b - (tb * dtx) * xx.b) - (tb * dty) * yy[r].b) - (tb * dtz) * zz.b;
                        st2<float, T>(Pn, gb[r] + po, pa, pb);
                    }
                } else {
                    const bool yrec = o2 >= p.npml && o2 < p.npml + p.ny;
                    auto upd = [&](T Po, T xx, T yy_, T zz, float rv, float vv, bool dx, bool dz, float ax1_,
                                   float ax2_, float az1_, float az2_, T cx, T cy, T cz, T &nx, T &ny, T &nz) -> T {
                        const T gx = ((((ax1_ * rv) * vv) * vv) * dtx) * xx;
                        const T gy = ((((ay1 * rv) * vv) * vv) * dty) * yy_;
                        const T gz = ((((az1_ * rv) * vv) * vv) * dtz) * zz;
                        T qv = Po;
                        qv = dx ? qv - cx : qv;
                        qv = dym ? qv - cy : qv;
                        qv = dz ? qv - cz : qv;
                        qv = dx ? qv : qv - gx;
                        qv = dym ? qv : qv - gy;
                        qv = dz ? qv : qv - gz;
                        nx = fma_t(ax2_, cx, -gx);
                        ny = fma_t(ay2, cy, -gy);
                        nz = fma_t(az2_, cz, -gz);
                        qv = dx ? qv + nx : qv;
                        qv = dym ? qv + ny : qv;
                        qv = dz ? qv + nz : qv;
                        return qv;
                    };
                    float *px = reinterpret_cast<float *>(p.px), *py = reinterpret_cast<float *>(p.py),
                          *pz = reinterpret_cast<float *>(p.pz);
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const int bi = (xw + r) * 32 + zl;
                        T2 xx, zz;
                        deriv(r, xx, zz);
                        const float2 rv = *reinterpret_cast<const float2 *>(Br + bi);
                        const float2 vv = *reinterpret_cast<const float2 *>(Bvp + bi);
                        const T2 Po = ld2<T>(Bp, bi);
                        const T2 cx = tdx ? ld2<T>(Bx, bi) : T2{0, 0};
                        const T2 cy = dym ? ld2<T>(By, bi) : T2{0, 0};
                        const T2 cz = tdz ? ld2<T>(Bz, bi) : T2{0, 0};
                        const uint32_t g = gb[r] + po;
                        T nxa, nya, nza, nxb, nyb, nzb;
                        const T pa = upd(Po.a, xx.a, yy[r].a, zz.a, rv.x, vv.x, dxm[r], dza, ax1[r], ax2[r], az1.x,
                                         az2.x, cx.a, cy.a, cz.a, nxa, nya, nza);
                        const T pb = upd(Po.b, xx.b, yy[r].b, zz.b, rv.y, vv.y, dxm[r], dzb, ax1[r], ax2[r], az1.y,
                                         az2.y, cx.b, cy.b, cz.b, nxb, nyb, nzb);
                        if (act[r]) {
                            st2m<float, T>(Pn, g, pa, pb, both);
                            if (dxm[r]) st2m<float, T>(px, g, nxa, nxb, both);
                            if (dym) st2m<float, T>(py, g, nya, nyb, both);
                            if (dza && dzb && both) {
                                st2<float, T>(pz, g, nza, nzb);
                            } else {
                                if (dza) pz[g] = nza;
                                if (dzb && both) pz[g + 1] = nzb;
                            }
                        }
                        if (yrec && (reca[r] | recb[r])) {  // ..iso..:294-304
                            const size_t tr = (size_t)trb[r] + (size_t)p.nx * (o2 - p.npml);
                            T rr = reca[r] ? pa : pb;
                            if (p.mute_nt && p.it < p.mute_nt[tr]) rr = T(0);
                            p.rec[tr * p.nt + p.it] = (float)rr;
                        }
                    }
                }
            }
            __syncwarp();
            if (lane == 0 && J >= 4) mbar_arrive(&strDone[(J - 4) % L::NR]);
            // the slot about to be written was read by the pressure update of step
            // J - NR + 4: wait until every warp is past it
            if (J >= (uint32_t)L::NR)
                mbar_wait(&strDone[J % L::NR], ((J / L::NR) - 1) & 1, p.err, KERR_FULL_TIMEOUT, ab);

            // ---- 2. velocities at o1 (..iso..:99-142), core cells and the halos
            float *Ru = ringU + (J % L::NR) * L::UX;
            float *Rw = ringW + (J % L::NR) * L::WZ;
            const T cy1d = (T)cy1n * dty, cy2 = (T)cy2n;
            cy1n = p.cy1[min(o1 + 1, p.nny - 1)];
            cy2n = p.cy2[min(o1 + 1, p.nny - 1)];
            const bool vel = o1 >= MM && o1 < p.nny - MM;  // ghost planes keep zero velocities
            const float *Ao = reinterpret_cast<const float *>(ringA + sh * L::A_STRIDE);
            const float *Bu = reinterpret_cast<const float *>(sbp + L::OU);
            const float *Bv = reinterpret_cast<const float *>(sbp + L::OV);
            const float *Bw = reinterpret_cast<const float *>(sbp + L::OW);
            const float *Bri = reinterpret_cast<const float *>(sbp + L::ORI);
            const uint32_t po = pstride * (uint32_t)o1;
            T2 vnew[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                // P at tile rows: xs[j] = P(x = xw - 3 + j)
                T2 xs[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) xs[j] = ld2<T>(Ao, c0 + (r + j - 3) * AW);
                T2 zp[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(Ao, c0 + r * AW - MM + 2 * m);
                const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a,
                                  zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
                T xa = 0, xb = 0, za = 0, zb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // ..iso..:125-127
                    xa = fma_t(k[im], xs[4 + im].a - xs[3 - im].a, xa);
                    xb = fma_t(k[im], xs[4 + im].b - xs[3 - im].b, xb);
                    za = fma_t(k[im], zv[5 + im] - zv[4 - im], za);
                    zb = fma_t(k[im], zv[6 + im] - zv[5 - im], zb);
                }
                const int row = xw + r;
                const float2 ri = *reinterpret_cast<const float2 *>(Bri + (row + 4) * 40 + 4 + zl);
                const T2 uo = ld2<T>(Bu, (row + 4) * 32 + zl), vo = ld2<T>(Bv, row * 32 + zl),
                         wo = ld2<T>(Bw, row * 40 + 4 + zl);
                xa = xa * ri.x;
                xb = xb * ri.y;
                const T ya = yyP[r].a * ri.x, yb = yyP[r].b * ri.y;
                za = za * ri.x;
                zb = zb * ri.y;
                const T una = fma_t(cx2[r], uo.a, -(cx1d[r] * xa)), unb = fma_t(cx2[r], uo.b, -(cx1d[r] * xb));
                const T vna = fma_t(cy2, vo.a, -(cy1d * ya)), vnb = fma_t(cy2, vo.b, -(cy1d * yb));
                const T wna = fma_t(cz2.a, wo.a, -(cz1d.a * za)), wnb = fma_t(cz2.b, wo.b, -(cz1d.b * zb));
                const bool on = vel && act[r];
                // the second cell of a pair past the sweep stays zero, as a never-updated cell
                const T ub = on && both ? unb : T(0), vb = on && both ? vnb : T(0), wb = on && both ? wnb : T(0);
                *reinterpret_cast<float2 *>(Ru + (row + 4) * 32 + zl) = make_float2(on ? una : T(0), ub);
                *reinterpret_cast<float2 *>(Rw + row * 40 + 4 + zl) = make_float2(on ? wna : T(0), wb);
                vnew[r] = T2{on ? vna : T(0), vb};
                if (on) {
                    const uint32_t g = gb[r] + po;
                    st2m<float, T>(un, g, una, unb, both);
                    st2m<float, T>(vn, g, vna, vnb, both);
                    st2m<float, T>(wn, g, wna, wnb, both);
                }
            }
            with_phase(ph, [&](auto pc) {
                constexpr int Q = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) winV[r][Q] = vnew[r];
            });
            // u at the halo rows (x derivative only)
#pragma unroll
            for (int j = 0; j < NHU; ++j) {
                if (hw + 2 * NW * j >= 8) break;
                const int hx = hr[j];
                const int cp = (hx + 8) * AW + zl + 8;  // P(x = x0 + hx) at this lane's z pair
                T2 xs[8];
#pragma unroll
                for (int m = 0; m < 8; ++m) xs[m] = ld2<T>(Ao, cp + (m - 3) * AW);
                T xa = 0, xb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {
                    xa = fma_t(k[im], xs[4 + im].a - xs[3 - im].a, xa);
                    xb = fma_t(k[im], xs[4 + im].b - xs[3 - im].b, xb);
                }
                const float2 ri = *reinterpret_cast<const float2 *>(Bri + (hx + 4) * 40 + 4 + zl);
                const T2 uo = ld2<T>(Bu, (hx + 4) * 32 + zl);
                xa = xa * ri.x;
                xb = xb * ri.y;
                const T una = fma_t(hcx2[j], uo.a, -(hcx1d[j] * xa)), unb = fma_t(hcx2[j], uo.b, -(hcx1d[j] * xb));
                const bool on = vel && hact[j];
                *reinterpret_cast<float2 *>(Ru + (hx + 4) * 32 + zl) =
                    make_float2(on ? una : T(0), on && both ? unb : T(0));
            }
            // w at the halo columns (z derivative only)
            if (wtask) {
                const int cp = (wrow + 8) * AW + (wzo + 4);  // P(z = z0 - 4 + wzo), row wrow
                T2 zp[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(Ao, cp - MM + 2 * m);
                const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a,
                                  zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
                T za = 0, zb = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {
                    za = fma_t(k[im], zv[5 + im] - zv[4 - im], za);
                    zb = fma_t(k[im], zv[6 + im] - zv[5 - im], zb);
                }
                const float2 ri = *reinterpret_cast<const float2 *>(Bri + (wrow + 4) * 40 + wzo);
                const T2 wo = ld2<T>(Bw, wrow * 40 + wzo);
                za = za * ri.x;
                zb = zb * ri.y;
                const T wna = fma_t(wcz2.a, wo.a, -(wcz1d.a * za)), wnb = fma_t(wcz2.b, wo.b, -(wcz1d.b * zb));
                *reinterpret_cast<float2 *>(Rw + wrow * 40 + wzo) =
                    make_float2(vel && wacta ? wna : T(0), vel && wactb ? wnb : T(0));
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&velDone[J % L::NR]);
            ++J;
        });
}

// ===========================================================================
template <int TX, int D, int R>
static cudaError_t launch_step_t(const K1Launch &L, cudaStream_t st) {
    K1Params p = L.p;
    constexpr int NT = 32 * (TX / (2 * R) + 1);
    static SmemAttr attr;
    Maps<11> mp;
    for (int i = 0; i < 11; ++i) mp.m[i] = L.maps[i];
    auto kern = iso_step<TX, D, R>;
    const int grid = k1_sweep<TX>(p, kern, NT, IsoStepL<TX, D>::TOTAL, L.grid, L.mode, L.rot);
    return k1_launch(kern, NT, IsoStepL<TX, D>::TOTAL, p.sw.W, grid, st, attr, mp, (float *)L.out0,
                     (float *)L.out1, (float *)L.out2, (float *)L.out3, p);
}

// shapes (tile width, rows per lane) in {8, 16} x {1, 2}, ring depths 0 and 1
cudaError_t launch_iso_step(const K1Launch &L, cudaStream_t st) {
    if (L.fp64 || L.half || L.depth > 1 || L.rows == 4) return cudaErrorInvalidConfiguration;
    if (L.tx == 16) {
        if (L.rows == 1) return L.depth ? launch_step_t<16, 1, 1>(L, st) : launch_step_t<16, 0, 1>(L, st);
        return L.depth ? launch_step_t<16, 1, 2>(L, st) : launch_step_t<16, 0, 2>(L, st);
    }
    if (L.rows == 1) return L.depth ? launch_step_t<8, 1, 1>(L, st) : launch_step_t<8, 0, 1>(L, st);
    return L.depth ? launch_step_t<8, 1, 2>(L, st) : launch_step_t<8, 0, 2>(L, st);
}

}  // namespace a3d
