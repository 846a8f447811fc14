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
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
};

template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / R) + 32)
    iso_vel(const __grid_constant__ Maps<5> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using L = IsoVelL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NW = TX / R, NC = 32 * NW;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBars<L::KA, L::KB> *>(smem + L::BAR_OFF);
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
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE, L::B_BYTES,
            p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                tma_load_3d(dst, &mp.m[0], bar, s.z0 - MM, s.x0 - MM, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                tma_load_3d(dst, &mp.m[1], bar, s.z0, s.x0, o);
                tma_load_3d(dst + L::C * sizeof(S), &mp.m[2], bar, s.z0, s.x0, o);
                tma_load_3d(dst + 2 * L::C * sizeof(S), &mp.m[3], bar, s.z0, s.x0, o);
                tma_load_3d(dst + 3 * L::C * sizeof(S), &mp.m[4], bar, s.z0, s.x0, o);
            });
        return;
    }

    const int tz = lane, xw = warp * R;  // this warp's first tile row
    T win[R][9];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int i = 0; i < 9; ++i) win[r][i] = T(0);
    int iz = 0;
    bool zact = false, act[R];
    T cx1[R], cx2[R], cz1 = 0, cz2 = 0;
    size_t gb[R];  // this column's row offsets in the fields
    const size_t pstride = (size_t)p.ldz * p.nnx;
    pipe_consume<TX, L::KA, L::KB>(
        p.sw, w0, w1, bars, ringA, L::A_STRIDE, ringB, L::B_STRIDE, p.err,
        [&](const Seg &s) {
            iz = s.z0 + tz;
            zact = iz < p.nnz - MM;
            const int cz = min(iz, p.nnz - 1);
            cz1 = (T)p.cz1[cz];
            cz2 = (T)p.cz2[cz];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                cx1[r] = (T)p.cx1[cxi];
                cx2[r] = (T)p.cx2[cxi];
                gb[r] = (size_t)iz + (size_t)p.ldz * cxi;
            }
        },
        [&](unsigned char *st, const Seg &s, int q) {
            S *A = reinterpret_cast<S *>(st);
            if (p.inj && q == p.s_y) {  // the dipole enters the view of P, ..iso..:94
                const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - (s.z0 - MM);
                if (threadIdx.x == 0 && lx >= 0 && lx < L::AH) {
                    if (lz >= 0 && lz < L::AW)
                        A[lx * L::AW + lz] = to_store<S, T>(ld<T>(A, lx * L::AW + lz) + (T)p.amp0);
                    if (lz + 2 >= 0 && lz + 2 < L::AW)
                        A[lx * L::AW + lz + 2] = to_store<S, T>(ld<T>(A, lx * L::AW + lz + 2) + (T)p.amp1);
                }
                consumer_sync(NC);
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {
#pragma unroll
                for (int i = 0; i < 8; ++i) win[r][i] = win[r][i + 1];
                win[r][8] = ld<T>(A, (xw + r + MM) * L::AW + tz + MM);
            }
        },
        [&](unsigned char *sa, unsigned char *sb, const Seg &, int o) {
            if (!zact) return;
            const S *A = reinterpret_cast<const S *>(sa);
            const S *Bu = reinterpret_cast<const S *>(sb);
            const S *Bv = Bu + L::C, *Bw = Bu + 2 * L::C;
            const float *Br = reinterpret_cast<const float *>(sb + 3 * L::C * sizeof(S));
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            // P at tile rows xw+1 .. xw+R+7 of this z column: xs[j] = P(x = xw - 3 + j)
            T xs[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) xs[j] = ld<T>(A, (xw + 1 + j) * L::AW + tz + MM);
            const T cy1 = (T)p.cy1[o], cy2 = (T)p.cy2[o];
            const size_t po = pstride * o;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (!act[r]) continue;
                const int c = (xw + r + MM) * L::AW + tz + MM, bi = (xw + r) * 32 + tz;
                T xx = 0, yy = 0, zz = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // ..iso..:125-127
                    yy = fma_t(k[im], win[r][5 + im] - win[r][4 - im], yy);
                    xx = fma_t(k[im], xs[r + 4 + im] - xs[r + 3 - im], xx);
                    zz = fma_t(k[im], ld<T>(A, c + im + 1) - ld<T>(A, c - im), zz);
                }
                const T ri = (T)Br[bi];  // 1/rho
                xx = xx * ri;
                yy = yy * ri;
                zz = zz * ri;
                const size_t g = gb[r] + po;
                u[g] = to_store<S, T>(fma_t(cx2[r], ld<T>(Bu, bi), -((cx1[r] * (T)p.dtx) * xx)));
                v[g] = to_store<S, T>(fma_t(cy2, ld<T>(Bv, bi), -((cy1 * (T)p.dty) * yy)));
                w[g] = to_store<S, T>(fma_t(cz2, ld<T>(Bw, bi), -((cz1 * (T)p.dtz) * zz)));
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
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
};

template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / R) + 32)
    iso_stress(const __grid_constant__ Maps<9> mp, S *__restrict__ P,
               const __grid_constant__ K1Params p) {
    using L = IsoStrL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NW = TX / R;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBars<L::KA, L::KB> *>(smem + L::BAR_OFF);
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
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE, 0, p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                tma_load_3d(dst, &mp.m[0], bar, s.z0, s.x0, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                const bool nx_ = range_damped(s.x0, TX, p.ulo[0], p.uhi[0]);
                const bool ny_ = range_damped(o, 1, p.ulo[1], p.uhi[1]);
                const bool nz_ = range_damped(s.z0, 32, p.ulo[2], p.uhi[2]);
                mbar_arrive_expect_tx(bar, L::B_FIXED + AUX * ((int)nx_ + (int)ny_ + (int)nz_));
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
    T win[R][9];
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int i = 0; i < 9; ++i) win[r][i] = T(0);
    int iz = 0;
    bool zact = false, dzm = false, act[R], dxm[R], rec[R];
    float ax1[R], ax2[R], az1 = 1, az2 = 1;
    int ixr[R];
    S *px = reinterpret_cast<S *>(p.px), *py = reinterpret_cast<S *>(p.py),
      *pz = reinterpret_cast<S *>(p.pz);
    const size_t pstride = (size_t)p.ldz * p.nnx;
    pipe_consume<TX, L::KA, L::KB>(
        p.sw, w0, w1, bars, ringA, L::A_STRIDE, ringB, L::B_STRIDE, p.err,
        [&](const Seg &s) {
            iz = s.z0 + tz;
            zact = iz < p.nnz - MM;
            const int cz = min(iz, p.nnz - 1);
            az1 = p.az1[cz];
            az2 = p.az2[cz];
            dzm = damped(az1, az2);
            const bool rec_z = iz == p.npml;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                ixr[r] = ix;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                ax1[r] = p.ax1[cxi];
                ax2[r] = p.ax2[cxi];
                dxm[r] = damped(ax1[r], ax2[r]);
                rec[r] = rec_z && ix >= p.npml && ix < p.npml + p.nx;
            }
        },
        [&](unsigned char *st, const Seg &, int) {
            const S *A = reinterpret_cast<const S *>(st);
#pragma unroll
            for (int r = 0; r < R; ++r) {
#pragma unroll
                for (int i = 0; i < 8; ++i) win[r][i] = win[r][i + 1];
                win[r][8] = ld<T>(A, (xw + r) * 32 + tz);
            }
        },
        [&](unsigned char *, unsigned char *sb, const Seg &, int o) {
            if (!zact) return;
            const S *Bu = reinterpret_cast<const S *>(sb);
            const S *Bw = reinterpret_cast<const S *>(sb + oW);
            const S *Bp = reinterpret_cast<const S *>(sb + oP);
            const float *Br = reinterpret_cast<const float *>(sb + oR);
            const float *Bvp = reinterpret_cast<const float *>(sb + oV);
            const S *Bx = reinterpret_cast<const S *>(sb + oX);
            const S *By = Bx + L::C, *Bz = Bx + 2 * L::C;
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            // u at tile rows xw .. xw+R+6 of this z column: us[j] = u(x = xw - 4 + j)
            T us[R + 7];
#pragma unroll
            for (int j = 0; j < R + 7; ++j) us[j] = ld<T>(Bu, (xw + j) * 32 + tz);
            const float ay1 = p.ay1[o], ay2 = p.ay2[o];
            const bool dym = damped(ay1, ay2);
            const size_t po = pstride * o;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (!act[r]) continue;
                const int bi = (xw + r) * 32 + tz, cw = (xw + r) * 40 + tz + MM;
                T xx = 0, yy = 0, zz = 0;
#pragma unroll
                for (int im = 0; im < 4; ++im) {  // ..iso..:178-180
                    yy = fma_t(k[im], win[r][4 + im] - win[r][3 - im], yy);
                    xx = fma_t(k[im], us[r + 4 + im] - us[r + 3 - im], xx);
                    zz = fma_t(k[im], ld<T>(Bw, cw + im) - ld<T>(Bw, cw - im - 1), zz);
                }
                const T rv = (T)Br[bi], vv = (T)Bvp[bi];
                const T gx = (((((T)ax1[r] * rv) * vv) * vv) * (T)p.dtx) * xx;  // ..iso..:182-184
                const T gy = (((((T)ay1 * rv) * vv) * vv) * (T)p.dty) * yy;
                const T gz = (((((T)az1 * rv) * vv) * vv) * (T)p.dtz) * zz;
                const size_t g = (size_t)iz + (size_t)p.ldz * ixr[r] + po;
                T cx = dxm[r] ? ld<T>(Bx, bi) : T(0), cy = dym ? ld<T>(By, bi) : T(0),
                  cz = dzm ? ld<T>(Bz, bi) : T(0);
                const T Pn = pupdate_r<T>(ld<T>(Bp, bi), gx, gy, gz, dxm[r], dym, dzm, ax2[r], ay2, az2,
                                          cx, cy, cz);
                P[g] = to_store<S, T>(Pn);
                if (dxm[r]) px[g] = to_store<S, T>(cx);
                if (dym) py[g] = to_store<S, T>(cy);
                if (dzm) pz[g] = to_store<S, T>(cz);
                if (rec[r] && o >= p.npml && o < p.npml + p.ny) {  // ..iso..:294-304
                    const size_t tr = (size_t)(ixr[r] - p.npml) + (size_t)p.nx * (o - p.npml);
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
