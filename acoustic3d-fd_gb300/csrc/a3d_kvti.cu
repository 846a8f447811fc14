// a3d_kvti.cu — 1st-order pseudo-acoustic VTI engine (u, v, w, P, Q; rho, eps, delta).
//
//   vti_vel:    u,v <- D+P (x, y);  w <- D+_z Q;  / rho          (..vti..:91-128)
//               the Ricker monopole enters the sweep's views of P and Q only
//   vti_stress: P <- P - rho v^2 [(1+2e')(D-u/dx + D-v/dy) + sqrt(1+2d') D-w/dz]
//               Q <- Q - rho v^2 [sqrt(1+2d')(D-u/dx + D-v/dy) + D-w/dz]
//               e', d' tapered inside the SV ball round the source (..vti..:131-203),
//               split components only on damped PML axes, record + mute fused.
#include "a3d_k1dev.cuh"

namespace a3d {

// ===========================================================================
// vti_vel: maps {P (HX), Q (HZ), u, v, w (core), 1/rho (core float)}
template <int TX, class S, int D>
struct VtiVelL {
    static constexpr int KA = Depth<D>::KA, KB = Depth<D>::KB;
    static constexpr uint32_t C = 32 * TX, PX = 32 * (TX + 8), QZ = 40 * TX;
    static constexpr uint32_t A_BYTES = PX * sizeof(S);
    static constexpr uint32_t B_BYTES = (QZ + 3 * C) * sizeof(S) + C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
};

template <int TX, class S, int D>
__global__ void __launch_bounds__(32 * TX + 32)
    vti_vel(const __grid_constant__ Maps<6> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using L = VtiVelL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NC = 32 * TX;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBars<L::KA, L::KB> *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::KA * L::A_STRIDE;
    if (threadIdx.x == 0) bars.init(NC / 32);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t oU = L::QZ * sizeof(S), oV = oU + L::C * sizeof(S), oW = oV + L::C * sizeof(S),
                     oR = oW + L::C * sizeof(S);
    if (warp == TX) {
        if (lane != 0) return;
        for (int i = 0; i < 6; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE, L::B_BYTES, p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                tma_load_3d(dst, &mp.m[0], bar, s.z0, s.x0 - MM, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                tma_load_3d(dst, &mp.m[1], bar, s.z0 - MM, s.x0, o);
                tma_load_3d(dst + oU, &mp.m[2], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oV, &mp.m[3], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oW, &mp.m[4], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oR, &mp.m[5], bar, s.z0, s.x0, o);
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
            if (p.inj && q == p.s_y) {  // monopole into P (..vti..:85)
                const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - s.z0;
                if (threadIdx.x == 0 && lx >= 0 && lx < TX + 8 && lz >= 0 && lz < 32)
                    A[lx * 32 + lz] = to_store<S, T>(ld<T>(A, lx * 32 + lz) + (T)p.amp0);
                consumer_sync(NC);
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) win[i] = win[i + 1];
            win[8] = ld<T>(A, (tx + MM) * 32 + tz);
        },
        [&](unsigned char *sa, unsigned char *sb, const Seg &s, int o) {
            S *Bq = reinterpret_cast<S *>(sb);
            if (p.inj && o == p.s_y) {  // monopole into Q (..vti..:86)
                const int lx = p.s_x - s.x0, lz = p.s_z - (s.z0 - MM);
                if (threadIdx.x == 0 && lx >= 0 && lx < TX && lz >= 0 && lz < 40)
                    Bq[lx * 40 + lz] = to_store<S, T>(ld<T>(Bq, lx * 40 + lz) + (T)p.amp1);
                consumer_sync(NC);
            }
            if (!active) return;
            const S *A = reinterpret_cast<const S *>(sa);
            const S *Bu = reinterpret_cast<const S *>(sb + oU);
            const S *Bv = reinterpret_cast<const S *>(sb + oV);
            const S *Bw = reinterpret_cast<const S *>(sb + oW);
            const float *Br = reinterpret_cast<const float *>(sb + oR);
            const int bi = tx * 32 + tz, ca = (tx + MM) * 32 + tz, cq = tx * 40 + tz + MM;
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            T xx = 0, yy = 0, zz = 0;
#pragma unroll
            for (int im = 0; im < 4; ++im) {  // ..vti..:113-115
                yy = fma_t(k[im], win[5 + im] - win[4 - im], yy);
                xx = fma_t(k[im], ld<T>(A, ca + (im + 1) * 32) - ld<T>(A, ca - im * 32), xx);
                zz = fma_t(k[im], ld<T>(Bq, cq + im + 1) - ld<T>(Bq, cq - im), zz);
            }
            const T ri = (T)Br[bi];  // 1/rho
            xx = xx * ri;
            yy = yy * ri;
            zz = zz * ri;
            const T cy1 = (T)p.cy1[o], cy2 = (T)p.cy2[o];
            const size_t g = gidx<S>(p, iz, ix, o);
            u[g] = to_store<S, T>(fma_t(cx2, ld<T>(Bu, bi), -((cx1 * (T)p.dtx) * xx)));
            v[g] = to_store<S, T>(fma_t(cy2, ld<T>(Bv, bi), -((cy1 * (T)p.dty) * yy)));
            w[g] = to_store<S, T>(fma_t(cz2, ld<T>(Bw, bi), -((cz1 * (T)p.dtz) * zz)));
        });
}

// ===========================================================================
// vti_stress: maps {v (core), u (HX), w (HZ), P, Q (core), rho, vp, eps, del (core float)}
template <int TX, class S, int D>
struct VtiStrL {
    static constexpr int KA = Depth<D>::KA, KB = Depth<D>::KB;
    static constexpr uint32_t C = 32 * TX, UX = 32 * (TX + 8), WZ = 40 * TX;
    static constexpr uint32_t A_BYTES = C * sizeof(S);
    static constexpr uint32_t B_BYTES = (UX + WZ + 2 * C) * sizeof(S) + 4 * C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
};

// epsilon/delta after the SV-ball taper (..vti..:154-175): hi/lo table per r^2
__device__ __forceinline__ void sv_eedd(const K1Params &p, int ix, int iy, int iz, float eps,
                                        float del, float &ee, float &dd) {
    const int rx = ix - p.s_x, ry = iy - p.s_y, rz = iz - p.s_z;
    const int d2 = rx * rx + ry * ry + rz * rz;
    if (d2 > 225) { ee = eps; dd = del; return; }
    const float2 t = p.taper[d2];
    ee = mul_df(eps, t.x, t.y);
    dd = mul_df(del, t.x, t.y);
}

template <int TX, class S, int D>
__global__ void __launch_bounds__(32 * TX + 32)
    vti_stress(const __grid_constant__ Maps<9> mp, S *__restrict__ P, S *__restrict__ Q,
               const __grid_constant__ K1Params p) {
    using L = VtiStrL<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NC = 32 * TX;
    extern __shared__ __align__(128) unsigned char smem[];
    auto &bars = *reinterpret_cast<PipeBars<L::KA, L::KB> *>(smem + L::BAR_OFF);
    unsigned char *ringA = smem, *ringB = smem + L::KA * L::A_STRIDE;
    if (threadIdx.x == 0) bars.init(NC / 32);
    __syncthreads();
    long long w0, w1;
    cta_range(p.sw, w0, w1);
    if (w0 >= w1) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr size_t oW = L::UX * sizeof(S), oP = oW + L::WZ * sizeof(S), oQ = oP + L::C * sizeof(S),
                     oF = oQ + L::C * sizeof(S);  // then rho, vp, eps, del floats
    if (warp == TX) {
        if (lane != 0) return;
        for (int i = 0; i < 9; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE, L::B_BYTES, p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                tma_load_3d(dst, &mp.m[0], bar, s.z0, s.x0, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                tma_load_3d(dst, &mp.m[1], bar, s.z0, s.x0 - MM, o);
                tma_load_3d(dst + oW, &mp.m[2], bar, s.z0 - MM, s.x0, o);
                tma_load_3d(dst + oP, &mp.m[3], bar, s.z0, s.x0, o);
                tma_load_3d(dst + oQ, &mp.m[4], bar, s.z0, s.x0, o);
                for (int k = 0; k < 4; ++k)
                    tma_load_3d(dst + oF + k * L::C * 4, &mp.m[5 + k], bar, s.z0, s.x0, o);
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
    S *px = (S *)p.px, *py = (S *)p.py, *pz = (S *)p.pz, *qx = (S *)p.qx, *qy = (S *)p.qy, *qz = (S *)p.qz;
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
            win[8] = ld<T>(A, tx * 32 + tz);
        },
        [&](unsigned char *, unsigned char *sb, const Seg &, int o) {
            if (!active) return;
            const S *Bu = reinterpret_cast<const S *>(sb);
            const S *Bw = reinterpret_cast<const S *>(sb + oW);
            const S *Bp = reinterpret_cast<const S *>(sb + oP);
            const S *Bq = reinterpret_cast<const S *>(sb + oQ);
            const float *F = reinterpret_cast<const float *>(sb + oF);
            const int bi = tx * 32 + tz;
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            T xx = 0, yy = 0, zz = 0;
#pragma unroll
            for (int im = 0; im < 4; ++im) {  // ..vti..:183-185
                yy = fma_t(k[im], win[4 + im] - win[3 - im], yy);
                xx = fma_t(k[im], ld<T>(Bu, (tx + MM + im) * 32 + tz) - ld<T>(Bu, (tx + MM - im - 1) * 32 + tz), xx);
                zz = fma_t(k[im], ld<T>(Bw, tx * 40 + tz + MM + im) - ld<T>(Bw, tx * 40 + tz + MM - im - 1), zz);
            }
            float ee, dd;
            sv_eedd(p, ix, o, iz, F[2 * L::C + bi], F[3 * L::C + bi], ee, dd);
            const float ay1 = p.ay1[o], ay2 = p.ay2[o];
            const T rv = (T)F[bi], vv = (T)F[L::C + bi];
            T e1, sd;
            if constexpr (sizeof(T) == 4) {
                e1 = 1.0f + 2.0f * ee;
                sd = sqrtf(1.0f + 2.0f * dd);
            } else {
                e1 = T(1) + T(2) * (T)ee;
                sd = sqrt(T(1) + T(2) * (T)dd);
            }
            const T kx = (((T)ax1 * rv) * vv) * vv, ky = (((T)ay1 * rv) * vv) * vv,
                    kz = (((T)az1 * rv) * vv) * vv;
            const T gPx = ((kx * e1) * (T)p.dtx) * xx, gPy = ((ky * e1) * (T)p.dty) * yy,
                    gPz = ((kz * sd) * (T)p.dtz) * zz;
            const T gQx = ((kx * sd) * (T)p.dtx) * xx, gQy = ((ky * sd) * (T)p.dty) * yy,
                    gQz = (kz * (T)p.dtz) * zz;
            const bool dym = damped(ay1, ay2);
            const size_t g = gidx<S>(p, iz, ix, o);
            const T Pn = pupdate<T, S>(ld<T>(Bp, bi), gPx, gPy, gPz, dxm, dym, dzm, ax2, ay2, az2, px, py, pz, g);
            const T Qn = pupdate<T, S>(ld<T>(Bq, bi), gQx, gQy, gQz, dxm, dym, dzm, ax2, ay2, az2, qx, qy, qz, g);
            P[g] = to_store<S, T>(Pn);
            Q[g] = to_store<S, T>(Qn);
            if (rec_col && o >= p.npml && o < p.npml + p.ny) {
                const size_t tr = (size_t)(ix - p.npml) + (size_t)p.nx * (o - p.npml);
                T r = Pn;
                if (p.mute_nt && p.it < p.mute_nt[tr]) r = T(0);
                p.rec[tr * p.nt + p.it] = (float)r;
            }
        });
}

template <int TX, class S, int D>
static cudaError_t launch_vti_t(const K1Launch &L, cudaStream_t st) {
    K1Params p = L.p;
    if (L.kind == K1_VTI_VEL) {
        static bool attr = false;
        Maps<6> mp;
        for (int i = 0; i < 6; ++i) mp.m[i] = L.maps[i];
        const int grid = k1_sweep<TX>(p, vti_vel<TX, S, D>, 32 * TX + 32, VtiVelL<TX, S, D>::TOTAL, L.grid, L.mode);
        return k1_launch(vti_vel<TX, S, D>, 32 * TX + 32, VtiVelL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr,
                         mp, (S *)L.out0, (S *)L.out1, (S *)L.out2, p);
    }
    static bool attr = false;
    Maps<9> mp;
    for (int i = 0; i < 9; ++i) mp.m[i] = L.maps[i];
    const int grid = k1_sweep<TX>(p, vti_stress<TX, S, D>, 32 * TX + 32, VtiStrL<TX, S, D>::TOTAL, L.grid, L.mode);
    return k1_launch(vti_stress<TX, S, D>, 32 * TX + 32, VtiStrL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr,
                     mp, (S *)L.out0, (S *)L.out1, p);
}

cudaError_t launch_vti(const K1Launch &L, cudaStream_t st) {
    if (L.fp64) return launch_vti_t<8, double, 0>(L, st);
    if (L.tx == 16) return L.depth ? launch_vti_t<16, float, 1>(L, st) : launch_vti_t<16, float, 0>(L, st);
    return L.depth ? launch_vti_t<8, float, 1>(L, st) : launch_vti_t<8, float, 0>(L, st);
}

}  // namespace a3d
