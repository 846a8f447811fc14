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
    static constexpr int KA = Depth<D>::KA, KB = Depth<D>::KB;
    static constexpr int AW = 40, AH = TX + 8;
    static constexpr uint32_t A_BYTES = AW * AH * sizeof(S);
    static constexpr uint32_t C = 32 * TX;  // core elements
    static constexpr uint32_t B_BYTES = 3 * C * sizeof(S) + C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBarsM<KA, KB>);
};

template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / R) + 32)
    iso_vel(const __grid_constant__ Maps<5> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using L = IsoVelL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NW = TX / R, NC = 32 * NW, AW = L::AW;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBarsM<L::KA, L::KB> *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::KA * L::A_STRIDE;
    if (threadIdx.x == 0) bars.init(NW);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == NW) {
        if (lane != 0) return;
        for (int i = 0; i < 5; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce_m<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, p.err, [&](uint32_t sa, int sb, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + (sb >= 0 ? L::B_BYTES : 0u));
                tma_load_3d(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0 - MM, s.x0 - MM, q);
                if (sb < 0) return;
                unsigned char *dst = ringB + sb * L::B_STRIDE;
                const int o = q - MM;
                tma_load_3d(dst, &mp.m[1], bar, s.z0, s.x0, o);
                tma_load_3d(dst + L::C * sizeof(S), &mp.m[2], bar, s.z0, s.x0, o);
                tma_load_3d(dst + 2 * L::C * sizeof(S), &mp.m[3], bar, s.z0, s.x0, o);
                tma_load_3d(dst + 3 * L::C * sizeof(S), &mp.m[4], bar, s.z0, s.x0, o);
            });
        return;
    }

    const int tz = lane, xw = warp * R;  // this warp's first tile row
    const int c0 = (xw + MM) * AW + tz + MM;  // this thread's first cell in an A tile
    T win[R][8];                              // P at the last 8 planes, slot = item mod 8
    bool act[R];
    T cx1d[R], cx2[R], cz1d = 0, cz2 = 0;
    uint32_t gb[R];  // in-plane offsets of this thread's cells
    int srcq = INT_MIN;
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
    // the dipole enters the sweep's view of P (..iso..:94): patch the A tile of the
    // source plane in place (it serves the window push and, 4 planes later, the
    // in-plane neighbours), then make the write visible to every consumer warp
    auto inject = [&](S *A, const Seg &s) {
        const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - (s.z0 - MM);
        if (threadIdx.x == 0) {
            if (lz >= 0 && lz < AW) A[lx * AW + lz] = to_store<S, T>(ld<T>(A, lx * AW + lz) + (T)p.amp0);
            if (lz + 2 >= 0 && lz + 2 < AW)
                A[lx * AW + lz + 2] = to_store<S, T>(ld<T>(A, lx * AW + lz + 2) + (T)p.amp1);
            fence_proxy_async();  // the stage is refilled by TMA later
        }
        consumer_sync(NC);
    };
    pipe_run<TX, L::KA, L::KB, MM>(
        p.sw, w0, w1, bars, p.err,
        [&](const Seg &s) {
            const int iz = s.z0 + tz;
            const bool zact = iz < p.nnz - MM;
            const int cz = min(iz, p.nnz - 1);
            cz1d = (T)p.cz1[cz] * (T)p.dtz;
            cz2 = (T)p.cz2[cz];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                cx1d[r] = (T)p.cx1[cxi] * (T)p.dtx;
                cx2[r] = (T)p.cx2[cxi];
                gb[r] = (uint32_t)iz + (uint32_t)p.ldz * (uint32_t)cxi;
            }
            const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - (s.z0 - MM);
            srcq = (p.inj && lx >= 0 && lx < L::AH && lz + 2 >= 0 && lz < AW) ? p.s_y : INT_MIN;
        },
        [&](auto ph, uint32_t sa, const Seg &s, int q) {
            constexpr int P = decltype(ph)::value;
            S *A = reinterpret_cast<S *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
#pragma unroll
            for (int r = 0; r < R; ++r) win[r][P] = ld<T>(A, c0 + r * AW);
        },
        [&](int ph, uint32_t sa, uint32_t sh, uint32_t sb, const Seg &s, int q) {
            S *A = reinterpret_cast<S *>(ringA + sa * L::A_STRIDE);
            if (q == srcq) inject(A, s);
            // window push of P(q) and the y-derivative at o = q - 4 (..iso..:126)
            T yy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int P = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    win[r][P] = ld<T>(A, c0 + r * AW);
                    T a = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im)  // P(o+1+m) in slot (P+5+m)&7, P(o-m) in (P+4-m)&7
                        a = fma_t(k[im], win[r][(P + 5 + im) & 7] - win[r][(P + 4 - im) & 7], a);
                    yy[r] = a;
                }
            });
            // output plane o = q - 4: its P tile is the A stage held since item q - 4
            const int o = q - MM;
            const S *Ao = reinterpret_cast<const S *>(ringA + sh * L::A_STRIDE);
            const unsigned char *sbp = ringB + sb * L::B_STRIDE;
            const S *Bu = reinterpret_cast<const S *>(sbp);
            const S *Bv = Bu + L::C, *Bw = Bu + 2 * L::C;
            const float *Br = reinterpret_cast<const float *>(sbp + 3 * L::C * sizeof(S));
            // P at tile rows xw+1 .. xw+R+7 of this z column: xs[j] = P(x = xw - 3 + j)
            T xs[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) xs[j] = ld<T>(Ao, c0 + (j + 1 - MM) * AW);
            const T cy1d = (T)p.cy1[o] * (T)p.dty, cy2 = (T)p.cy2[o];
            const uint32_t po = pstride * (uint32_t)o;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int c = c0 + r * AW, bi = (xw + r) * 32 + tz;
                T xx = 0, zz = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // ..iso..:125-127
                    xx = fma_t(k[im], xs[r + 4 + im] - xs[r + 3 - im], xx);
                    zz = fma_t(k[im], ld<T>(Ao, c + im + 1) - ld<T>(Ao, c - im), zz);
                }
                const T ri = (T)Br[bi];  // 1/rho
                xx = xx * ri;
                const T yr = yy[r] * ri;
                zz = zz * ri;
                const T un = fma_t(cx2[r], ld<T>(Bu, bi), -(cx1d[r] * xx));
                const T vn = fma_t(cy2, ld<T>(Bv, bi), -(cy1d * yr));
                const T wn = fma_t(cz2, ld<T>(Bw, bi), -(cz1d * zz));
                if (act[r]) {
                    const uint32_t g = gb[r] + po;
                    u[g] = to_store<S, T>(un);
                    v[g] = to_store<S, T>(vn);
                    w[g] = to_store<S, T>(wn);
                }
            }
        });
}

// ===========================================================================
// iso_stress: maps {v (core), u (box HX), w (box HZ), P (core), rho, vp (core, float),
//                   px, py, pz (core; loaded only for tiles/planes on a damped axis)}
template <int TX, class S, int D>
struct IsoStrL {
    static constexpr int KA = Depth<D>::KA, KB = Depth<D>::KB;
    static constexpr uint32_t C = 32 * TX;
    static constexpr uint32_t UX = 32 * (TX + 8), WZ = 40 * TX;
    static constexpr uint32_t A_BYTES = C * sizeof(S);
    static constexpr uint32_t B_FIXED = (UX + WZ + C) * sizeof(S) + 2 * C * 4;
    static constexpr uint32_t B_BYTES = B_FIXED + 3 * C * sizeof(S);
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBarsM<KA, KB>);
};

template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / R) + 32)
    iso_stress(const __grid_constant__ Maps<9> mp, S *__restrict__ P,
               const __grid_constant__ K1Params p) {
    using L = IsoStrL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NW = TX / R;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBarsM<L::KA, L::KB> *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::KA * L::A_STRIDE;
    if (threadIdx.x == 0) bars.init(NW);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t oW = L::UX * sizeof(S), oP = (L::UX + L::WZ) * sizeof(S),
                     oR = (L::UX + L::WZ + L::C) * sizeof(S), oV = oR + L::C * 4,
                     oX = L::B_FIXED;  // px, py, pz tiles follow the fixed part
    constexpr uint32_t AUX = L::C * sizeof(S);

    if (warp == NW) {
        if (lane != 0) return;
        for (int i = 0; i < 9; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce_m<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, p.err, [&](uint32_t sa, int sb, uint64_t *bar, const Seg &s, int q) {
                if (sb < 0) {
                    mbar_arrive_expect_tx(bar, L::A_BYTES);
                    tma_load_3d(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0, s.x0, q);
                    return;
                }
                const int o = q - MM;
                const bool nx_ = range_damped(s.x0, TX, p.ulo[0], p.uhi[0]);
                const bool ny_ = range_damped(o, 1, p.ulo[1], p.uhi[1]);
                const bool nz_ = range_damped(s.z0, 32, p.ulo[2], p.uhi[2]);
                mbar_arrive_expect_tx(bar, L::A_BYTES + L::B_FIXED + AUX * ((int)nx_ + (int)ny_ + (int)nz_));
                tma_load_3d(ringA + sa * L::A_STRIDE, &mp.m[0], bar, s.z0, s.x0, q);
                unsigned char *dst = ringB + sb * L::B_STRIDE;
                tma_load_3d(dst, &mp.m[1], bar, s.z0, s.x0 - MM, o);
                tma_load_3d(dst + oW, &mp.m[2], bar, s.z0 - MM, s.x0, o);
                tma_load_3d(dst + oP, &mp.m[3], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oR, &mp.m[4], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oV, &mp.m[5], bar, s.z0, s.x0, o);
                if (nx_) tma_load_3d(dst + oX, &mp.m[6], bar, s.z0, s.x0, o);
                if (ny_) tma_load_3d(dst + oX + AUX, &mp.m[7], bar, s.z0, s.x0, o);
                if (nz_) tma_load_3d(dst + oX + 2 * AUX, &mp.m[8], bar, s.z0, s.x0, o);
            });
        return;
    }

    const int tz = lane, xw = warp * R;
    T win[R][8];  // v at the last 8 planes, slot = item mod 8
    bool dzm = false, act[R], dxm[R], rec[R];
    float ax1[R], ax2[R], az1 = 1, az2 = 1;
    uint32_t gb[R];
    int trb[R];  // receiver trace index of this cell at y = npml, or -1
    bool fast = false;  // tile undamped in x and z, every cell active, no receivers
    uint32_t g0 = 0;    // in-plane offset of this thread's first cell
    S *px = reinterpret_cast<S *>(p.px), *py = reinterpret_cast<S *>(p.py),
      *pz = reinterpret_cast<S *>(p.pz);
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
    const T dtx = (T)p.dtx, dty = (T)p.dty, dtz = (T)p.dtz;
    pipe_run<TX, L::KA, L::KB, 0>(
        p.sw, w0, w1, bars, p.err,
        [&](const Seg &s) {
            const int iz = s.z0 + tz;
            const bool zact = iz < p.nnz - MM;
            const int cz = min(iz, p.nnz - 1);
            az1 = p.az1[cz];
            az2 = p.az2[cz];
            dzm = damped(az1, az2);
            const bool rec_z = iz == p.npml;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                ax1[r] = p.ax1[cxi];
                ax2[r] = p.ax2[cxi];
                dxm[r] = damped(ax1[r], ax2[r]);
                rec[r] = act[r] && rec_z && ix >= p.npml && ix < p.npml + p.nx;
                trb[r] = ix - p.npml;
                gb[r] = (uint32_t)iz + (uint32_t)p.ldz * (uint32_t)cxi;
            }
            g0 = gb[0];
            fast = !range_damped(s.x0, TX, p.ulo[0], p.uhi[0]) && !range_damped(s.z0, 32, p.ulo[2], p.uhi[2]) &&
                   !(p.npml >= s.z0 && p.npml < s.z0 + 32);
        },
        [&](auto ph, uint32_t sa, const Seg &, int) {
            constexpr int Q = decltype(ph)::value;
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
#pragma unroll
            for (int r = 0; r < R; ++r) win[r][Q] = ld<T>(A, (xw + r) * 32 + tz);
        },
        [&](int ph, uint32_t sa, uint32_t, uint32_t sb, const Seg &, int q) {
            const int o = q - MM;
            // y-derivative at o from the window v(o-4 .. o+3) (plane o+m in slot
            // (ph+4+m)&7; ..iso..:179), then v(q) replaces v(q-8), which it last served
            const S *A = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
            T yy[R];
            with_phase(ph, [&](auto pc) {
                constexpr int Q = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    T a = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im)
                        a = fma_t(k[im], win[r][(Q + 4 + im) & 7] - win[r][(Q + 3 - im) & 7], a);
                    yy[r] = a;
                    win[r][Q] = ld<T>(A, (xw + r) * 32 + tz);
                }
            });
            const unsigned char *sbp = ringB + sb * L::B_STRIDE;
            const S *Bu = reinterpret_cast<const S *>(sbp);
            const S *Bw = reinterpret_cast<const S *>(sbp + oW);
            const S *Bp = reinterpret_cast<const S *>(sbp + oP);
            const float *Br = reinterpret_cast<const float *>(sbp + oR);
            const float *Bvp = reinterpret_cast<const float *>(sbp + oV);
            const S *Bx = reinterpret_cast<const S *>(sbp + oX);
            const S *By = Bx + L::C, *Bz = Bx + 2 * L::C;
            // u at tile rows xw .. xw+R+6 of this z column: us[j] = u(x = xw - 4 + j)
            T us[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) us[j] = ld<T>(Bu, (xw + j) * 32 + tz);
            const bool dym = o < p.ulo[1] || o >= p.uhi[1];  // == damped(ay1[o], ay2[o])
            const uint32_t po = pstride * (uint32_t)o;
            if (fast && !dym) {  // undamped interior tile and plane: P - gx - gy - gz, a1 == 1
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int bi = (xw + r) * 32 + tz, cw = (xw + r) * 40 + tz + MM;
                    T xx = 0, zz = 0;
#pragma unroll
                    for (int im = 0; im < 4; ++im) {  // ..iso..:178-180
                        xx = fma_t(k[im], us[r + 4 + im] - us[r + 3 - im], xx);
                        zz = fma_t(k[im], ld<T>(Bw, cw + im) - ld<T>(Bw, cw - im - 1), zz);
                    }
                    // (((1 * rho) * vp) * vp) == (rho * vp) * vp  (..iso..:182-184)
                    const T t = ((T)Br[bi] * (T)Bvp[bi]) * (T)Bvp[bi];
                    const T gx = (t * dtx) * xx, gy = (t * dty) * yy[r], gz = (t * dtz) * zz;
                    P[g0 + (uint32_t)(r * p.ldz) + po] = to_store<S, T>(((ld<T>(Bp, bi) - gx) - gy) - gz);
                }
                return;
            }
            const float ay1 = p.ay1[o], ay2 = p.ay2[o];
            const bool yrec = o >= p.npml && o < p.npml + p.ny;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int bi = (xw + r) * 32 + tz, cw = (xw + r) * 40 + tz + MM;
                T xx = 0, zz = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // ..iso..:178-180
                    xx = fma_t(k[im], us[r + 4 + im] - us[r + 3 - im], xx);
                    zz = fma_t(k[im], ld<T>(Bw, cw + im) - ld<T>(Bw, cw - im - 1), zz);
                }
                const T yr = yy[r];
                const T rv = (T)Br[bi], vv = (T)Bvp[bi];
                T gx, gy, gz;
                const bool dmp = dxm[r] | dym | dzm;
                if (!dmp) {  // a1 == 1 on every axis: (((1 * rho) * vp) * vp) == (rho * vp) * vp
                    const T t = (rv * vv) * vv;
                    gx = (t * dtx) * xx;
                    gy = (t * dty) * yr;
                    gz = (t * dtz) * zz;
                } else {  // ..iso..:182-184
                    gx = (((((T)ax1[r] * rv) * vv) * vv) * dtx) * xx;
                    gy = (((((T)ay1 * rv) * vv) * vv) * dty) * yr;
                    gz = (((((T)az1 * rv) * vv) * vv) * dtz) * zz;
                }
                const T Po = ld<T>(Bp, bi);
                const uint32_t g = gb[r] + po;
                T Pn;
                if (!dmp) {
                    Pn = ((Po - gx) - gy) - gz;
                } else {
                    T cx = dxm[r] ? ld<T>(Bx, bi) : T(0), cy = dym ? ld<T>(By, bi) : T(0),
                      cz = dzm ? ld<T>(Bz, bi) : T(0);
                    Pn = pupdate_r<T>(Po, gx, gy, gz, dxm[r], dym, dzm, ax2[r], ay2, az2, cx, cy, cz);
                    if (act[r]) {
                        if (dxm[r]) px[g] = to_store<S, T>(cx);
                        if (dym) py[g] = to_store<S, T>(cy);
                        if (dzm) pz[g] = to_store<S, T>(cz);
                    }
                }
                if (act[r]) P[g] = to_store<S, T>(Pn);
                if (rec[r] && yrec) {  // ..iso..:294-304
                    const size_t tr = (size_t)trb[r] + (size_t)p.nx * (o - p.npml);
                    T rr = Pn;
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
    constexpr int NT = 32 * (TX / R) + 32;
    if (L.kind == K1_ISO_VEL) {
        static bool attr = false;
        Maps<5> mp;
        for (int i = 0; i < 5; ++i) mp.m[i] = L.maps[i];
        auto kern = iso_vel<TX, S, D, R>;
        const int grid = k1_sweep<TX>(p, kern, NT, IsoVelL<TX, S, D>::TOTAL, L.grid, L.mode);
        return k1_launch(kern, NT, IsoVelL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr, mp,
                         (S *)L.out0, (S *)L.out1, (S *)L.out2, p);
    }
    static bool attr = false;
    Maps<9> mp;
    for (int i = 0; i < 9; ++i) mp.m[i] = L.maps[i];
    auto kern = iso_stress<TX, S, D, R>;
    const int grid = k1_sweep<TX>(p, kern, NT, IsoStrL<TX, S, D>::TOTAL, L.grid, L.mode);
    return k1_launch(kern, NT, IsoStrL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr, mp, (S *)L.out0, p);
}

// configurations: (tile width, rows per warp) in {8, 16} x {1, 2} and (16, 4), two ring depths
cudaError_t launch_iso(const K1Launch &L, cudaStream_t st) {
    if (L.fp64) return launch_iso_t<8, double, 0, 2>(L, st);
    if (L.tx == 16) {
        if (L.rows == 4) return L.deep ? launch_iso_t<16, float, 1, 4>(L, st) : launch_iso_t<16, float, 0, 4>(L, st);
        if (L.rows == 1) return L.deep ? launch_iso_t<16, float, 1, 1>(L, st) : launch_iso_t<16, float, 0, 1>(L, st);
        return L.deep ? launch_iso_t<16, float, 1, 2>(L, st) : launch_iso_t<16, float, 0, 2>(L, st);
    }
    if (L.rows == 1) return L.deep ? launch_iso_t<8, float, 1, 1>(L, st) : launch_iso_t<8, float, 0, 1>(L, st);
    return L.deep ? launch_iso_t<8, float, 1, 2>(L, st) : launch_iso_t<8, float, 0, 2>(L, st);
}

}  // namespace a3d
