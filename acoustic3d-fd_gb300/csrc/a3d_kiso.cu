// a3d_kiso.cu — 1st-order isotropic engine (staggered u, v, w, P with density).
//
// One step = two sweeps (the reference's five launches + five device syncs,
// ..iso..:523-565, become two launches):
//   iso_vel:    u,v,w <- c2*u - c1*dt/d * D+P / rho        (..iso..:99-142)
//               the dipole source is added to the sweep's view of P only
//               (..iso..:52-96 adds it to P, which update_stress then overwrites)
//   iso_stress: P <- P - rho v^2 dt (D-u/dx + D-v/dy + D-w/dz) (..iso..:145-190)
//               with split components kept only on PML-damped axes, the receiver
//               gather at model depth 0 (..iso..:294-304) and the mute fused.
#include "a3d_k1dev.cuh"

namespace a3d {

// ===========================================================================
// iso_vel: maps {P (box H), u, v, w (core), rho (core, float)}
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

template <int TX, class S, int D>
__global__ void __launch_bounds__(32 * TX + 32)
    iso_vel(const __grid_constant__ Maps<5> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using L = IsoVelL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NC = 32 * TX;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBars<L::KA, L::KB> *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::KA * L::A_STRIDE;
    if (threadIdx.x == 0) bars.init(NC);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == TX) {
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

    const int tx = warp, tz = lane;
    T win[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) win[i] = T(0);
    int iz = 0, ix = 0;
    bool active = false;
    T cx1 = 0, cx2 = 0, cz1 = 0, cz2 = 0;
    pipe_consume<TX, L::KA, L::KB>(
        p.sw, w0, w1, bars, ringA, L::A_STRIDE, ringB, L::B_STRIDE, p.err,
        [&](const Seg &s) {
            iz = s.z0 + tz;
            ix = s.x0 + tx;
            active = iz < p.nnz - MM && ix < p.nnx - MM;
            const int cz = min(iz, p.nnz - 1), cxi = min(ix, p.nnx - 1);
            cx1 = (T)p.cx1[cxi]; cx2 = (T)p.cx2[cxi];
            cz1 = (T)p.cz1[cz]; cz2 = (T)p.cz2[cz];
        },
        [&](unsigned char *st, const Seg &s, int q) {
            S *A = reinterpret_cast<S *>(st);
            if (p.inj && q == p.s_y) {  // the dipole enters the view of P, ..iso..:94
                const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - (s.z0 - MM);
                if (lx >= 0 && lx < L::AH) {
                    if (threadIdx.x == 0 && lz >= 0 && lz < L::AW)
                        A[lx * L::AW + lz] = to_store<S, T>((T)from_store<T, S>(A[lx * L::AW + lz]) + (T)p.amp0);
                    if (threadIdx.x == 0 && lz + 2 >= 0 && lz + 2 < L::AW)
                        A[lx * L::AW + lz + 2] =
                            to_store<S, T>((T)from_store<T, S>(A[lx * L::AW + lz + 2]) + (T)p.amp1);
                }
                consumer_sync(NC);
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) win[i] = win[i + 1];
            win[8] = from_store<T, S>(A[(tx + MM) * L::AW + tz + MM]);
        },
        [&](unsigned char *sa, unsigned char *sb, const Seg &s, int o) {
            if (!active) return;
            const S *A = reinterpret_cast<const S *>(sa);
            const S *Bu = reinterpret_cast<const S *>(sb);
            const S *Bv = Bu + L::C, *Bw = Bu + 2 * L::C;
            const float *Br = reinterpret_cast<const float *>(sb + 3 * L::C * sizeof(S));
            const int c = (tx + MM) * L::AW + tz + MM, bi = tx * 32 + tz;
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            T xx = 0, yy = 0, zz = 0;
#pragma unroll
            for (int im = 0; im < 4; ++im) {  // ..iso..:125-127
                yy = fma_t(k[im], win[5 + im] - win[4 - im], yy);
                xx = fma_t(k[im], from_store<T, S>(A[c + (im + 1) * L::AW]) - from_store<T, S>(A[c - im * L::AW]), xx);
                zz = fma_t(k[im], from_store<T, S>(A[c + im + 1]) - from_store<T, S>(A[c - im]), zz);
            }
            const T r = (T)Br[bi];
            xx = xx / r;
            yy = yy / r;
            zz = zz / r;
            const T cy1 = (T)p.cy1[o], cy2 = (T)p.cy2[o];
            const size_t g = gidx<S>(p, iz, ix, o);
            u[g] = to_store<S, T>(fma_t(cx2, from_store<T, S>(Bu[bi]), -((cx1 * (T)p.dtx) * xx)));
            v[g] = to_store<S, T>(fma_t(cy2, from_store<T, S>(Bv[bi]), -((cy1 * (T)p.dty) * yy)));
            w[g] = to_store<S, T>(fma_t(cz2, from_store<T, S>(Bw[bi]), -((cz1 * (T)p.dtz) * zz)));
        });
}

// ===========================================================================
// iso_stress: maps {v (core), u (box HX), w (box HZ), P (core), rho, vp (core, float)}
template <int TX, class S, int D>
struct IsoStrL {
    static constexpr int KA = Depth<D>::KA, KB = Depth<D>::KB;
    static constexpr uint32_t C = 32 * TX;
    static constexpr uint32_t UX = 32 * (TX + 8), WZ = 40 * TX;
    static constexpr uint32_t A_BYTES = C * sizeof(S);
    static constexpr uint32_t B_BYTES = (UX + WZ + C) * sizeof(S) + 2 * C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
};

template <int TX, class S, int D>
__global__ void __launch_bounds__(32 * TX + 32)
    iso_stress(const __grid_constant__ Maps<6> mp, S *__restrict__ P,
               const __grid_constant__ K1Params p) {
    using L = IsoStrL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NC = 32 * TX;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBars<L::KA, L::KB> *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::KA * L::A_STRIDE;
    if (threadIdx.x == 0) bars.init(NC);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t oW = L::UX * sizeof(S), oP = (L::UX + L::WZ) * sizeof(S),
                     oR = (L::UX + L::WZ + L::C) * sizeof(S), oV = oR + L::C * 4;

    if (warp == TX) {
        if (lane != 0) return;
        for (int i = 0; i < 6; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE, L::B_BYTES,
            p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                tma_load_3d(dst, &mp.m[0], bar, s.z0, s.x0, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                tma_load_3d(dst, &mp.m[1], bar, s.z0, s.x0 - MM, o);
                tma_load_3d(dst + oW, &mp.m[2], bar, s.z0 - MM, s.x0, o);
                tma_load_3d(dst + oP, &mp.m[3], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oR, &mp.m[4], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oV, &mp.m[5], bar, s.z0, s.x0, o);
            });
        return;
    }

    const int tx = warp, tz = lane;
    T win[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) win[i] = T(0);
    int iz = 0, ix = 0;
    bool active = false, dxm = false, dzm = false, rec_col = false;
    float ax1 = 1, ax2 = 1, az1 = 1, az2 = 1;
    S *px = reinterpret_cast<S *>(p.px), *py = reinterpret_cast<S *>(p.py),
      *pz = reinterpret_cast<S *>(p.pz);
    pipe_consume<TX, L::KA, L::KB>(
        p.sw, w0, w1, bars, ringA, L::A_STRIDE, ringB, L::B_STRIDE, p.err,
        [&](const Seg &s) {
            iz = s.z0 + tz;
            ix = s.x0 + tx;
            active = iz < p.nnz - MM && ix < p.nnx - MM;
            const int cz = min(iz, p.nnz - 1), cxi = min(ix, p.nnx - 1);
            ax1 = p.ax1[cxi]; ax2 = p.ax2[cxi]; az1 = p.az1[cz]; az2 = p.az2[cz];
            dxm = damped(ax1, ax2);
            dzm = damped(az1, az2);
            rec_col = iz == p.npml && ix >= p.npml && ix < p.npml + p.nx;
        },
        [&](unsigned char *st, const Seg &, int) {
            const S *A = reinterpret_cast<const S *>(st);
#pragma unroll
            for (int i = 0; i < 8; ++i) win[i] = win[i + 1];
            win[8] = from_store<T, S>(A[tx * 32 + tz]);
        },
        [&](unsigned char *, unsigned char *sb, const Seg &s, int o) {
            if (!active) return;
            const S *Bu = reinterpret_cast<const S *>(sb);
            const S *Bw = reinterpret_cast<const S *>(sb + oW);
            const S *Bp = reinterpret_cast<const S *>(sb + oP);
            const float *Br = reinterpret_cast<const float *>(sb + oR);
            const float *Bvp = reinterpret_cast<const float *>(sb + oV);
            const int bi = tx * 32 + tz;
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            T xx = 0, yy = 0, zz = 0;
#pragma unroll
            for (int im = 0; im < 4; ++im) {  // ..iso..:178-180
                yy = fma_t(k[im], win[4 + im] - win[3 - im], yy);
                xx = fma_t(k[im], from_store<T, S>(Bu[(tx + MM + im) * 32 + tz]) -
                                      from_store<T, S>(Bu[(tx + MM - im - 1) * 32 + tz]), xx);
                zz = fma_t(k[im], from_store<T, S>(Bw[tx * 40 + tz + MM + im]) -
                                      from_store<T, S>(Bw[tx * 40 + tz + MM - im - 1]), zz);
            }
            const float ay1 = p.ay1[o], ay2 = p.ay2[o];
            const T rv = (T)Br[bi], vv = (T)Bvp[bi];
            const T gx = (((((T)ax1 * rv) * vv) * vv) * (T)p.dtx) * xx;  // ..iso..:182-184
            const T gy = (((((T)ay1 * rv) * vv) * vv) * (T)p.dty) * yy;
            const T gz = (((((T)az1 * rv) * vv) * vv) * (T)p.dtz) * zz;
            const size_t g = gidx<S>(p, iz, ix, o);
            const T Pn = pupdate<T, S>(from_store<T, S>(Bp[bi]), gx, gy, gz, dxm,
                                       damped(ay1, ay2), dzm, ax2, ay2, az2, px, py, pz, g);
            P[g] = to_store<S, T>(Pn);
            if (rec_col && o >= p.npml && o < p.npml + p.ny) {  // ..iso..:294-304
                const size_t tr = (size_t)(ix - p.npml) + (size_t)p.nx * (o - p.npml);
                T r = Pn;
                if (p.mute_nt && p.it < p.mute_nt[tr]) r = T(0);
                p.rec[tr * p.nt + p.it] = (float)r;
            }
        });
}

// ===========================================================================
template <int TX, class S, int D>
static cudaError_t launch_iso_t(const K1Launch &L, cudaStream_t st) {
    K1Params p = L.p;
    if (L.kind == K1_ISO_VEL) {
        static bool attr = false;
        Maps<5> mp;
        for (int i = 0; i < 5; ++i) mp.m[i] = L.maps[i];
        auto kern = iso_vel<TX, S, D>;
        const int grid = k1_sweep<TX>(p, kern, 32 * TX + 32, IsoVelL<TX, S, D>::TOTAL, L.grid, L.mode);
        return k1_launch(kern, 32 * TX + 32, IsoVelL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr, mp,
                         (S *)L.out0, (S *)L.out1, (S *)L.out2, p);
    }
    static bool attr = false;
    Maps<6> mp;
    for (int i = 0; i < 6; ++i) mp.m[i] = L.maps[i];
    auto kern = iso_stress<TX, S, D>;
    const int grid = k1_sweep<TX>(p, kern, 32 * TX + 32, IsoStrL<TX, S, D>::TOTAL, L.grid, L.mode);
    return k1_launch(kern, 32 * TX + 32, IsoStrL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr, mp, (S *)L.out0, p);
}

cudaError_t launch_iso(const K1Launch &L, cudaStream_t st) {
    if (L.fp64) return launch_iso_t<8, double, 0>(L, st);
    if (L.tx == 16) return L.deep ? launch_iso_t<16, float, 1>(L, st) : launch_iso_t<16, float, 0>(L, st);
    return L.deep ? launch_iso_t<8, float, 1>(L, st) : launch_iso_t<8, float, 0>(L, st);
}

}  // namespace a3d
