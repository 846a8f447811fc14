// a3d_ktti.cu — 1st-order pseudo-acoustic TTI engine (tilt theta, azimuth phi; no density).
//
//   tti_vel:    xx = ct cp DxP - ct sp DyP - st DzP;  yy = sp DxP + cp DyP;
//               zz = st cp DxQ - st sp DyQ + ct DzQ;  u,v,w <- c2 u - c1 dt/d * (xx,yy,zz)
//               (..tti..:68-112; all six D+ derivatives, P and Q with z/x halo)
//   tti_stress: the same rotation of D-u, D-v, D-w, then the VTI coefficients
//               without density (..tti..:115-201), record + mute fused.
// cos/sin of theta and phi are evaluated once at setup (float), not per step.
#include "a3d_k1dev.cuh"

namespace a3d {

// ===========================================================================
// tti_vel: maps {P (H), Q (H), u, v, w (core), ct, st, cp, sp (core float)}
template <int TX, class S, int D>
struct TtiVelL {
    static constexpr int KA = Depth<D>::KA, KB = Depth<D>::KB;
    static constexpr int AW = 40, AH = TX + 8;
    static constexpr uint32_t C = 32 * TX, H = AW * AH;
    static constexpr uint32_t A_BYTES = 2 * H * sizeof(S);
    static constexpr uint32_t B_BYTES = 3 * C * sizeof(S) + 4 * C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
};

// the rotations of ..tti..:101-103 / 184-186 with the contractions nvcc applies
template <class T>
__device__ __forceinline__ void tti_rot(T ct, T st, T cp, T sp, T ax, T ay, T az, T bx, T by, T cx_,
                                        T cy_, T cz_, T &xx, T &yy, T &zz) {
    xx = fma_t(-st, az, fma_t(ct * cp, ax, -((ct * sp) * ay)));
    yy = fma_t(sp, bx, cp * by);
    zz = fma_t(ct, cz_, fma_t(st * cp, cx_, -((st * sp) * cy_)));
}

template <int TX, class S, int D>
__global__ void __launch_bounds__(32 * TX + 32)
    tti_vel(const __grid_constant__ Maps<9> mp, S *__restrict__ u, S *__restrict__ v,
            S *__restrict__ w, const __grid_constant__ K1Params p) {
    using L = TtiVelL<TX, S, D>;
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
    constexpr size_t oF = 3 * L::C * sizeof(S);
    if (warp == TX) {
        if (lane != 0) return;
        for (int i = 0; i < 9; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE, L::B_BYTES, p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                tma_load_3d(dst, &mp.m[0], bar, s.z0 - MM, s.x0 - MM, q);
                tma_load_3d(dst + L::H * sizeof(S), &mp.m[1], bar, s.z0 - MM, s.x0 - MM, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                for (int k = 0; k < 3; ++k)
                    tma_load_3d(dst + k * L::C * sizeof(S), &mp.m[2 + k], bar, s.z0, s.x0, o);
                for (int k = 0; k < 4; ++k)
                    tma_load_3d(dst + oF + k * L::C * 4, &mp.m[5 + k], bar, s.z0, s.x0, o);
            });
        return;
    }
    const int tx = warp, tz = lane;
    T wp[9], wq[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) wp[i] = wq[i] = T(0);
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
            S *A = reinterpret_cast<S *>(st), *B = A + L::H;
            if (p.inj && q == p.s_y) {  // monopole into P and Q (..tti..:62-63)
                const int lx = p.s_x - (s.x0 - MM), lz = p.s_z - (s.z0 - MM);
                if (threadIdx.x == 0 && lx >= 0 && lx < L::AH && lz >= 0 && lz < L::AW) {
                    A[lx * L::AW + lz] = to_store<S, T>(ld<T>(A, lx * L::AW + lz) + (T)p.amp0);
                    B[lx * L::AW + lz] = to_store<S, T>(ld<T>(B, lx * L::AW + lz) + (T)p.amp1);
                }
                consumer_sync(NC);
            }
            const int c = (tx + MM) * L::AW + tz + MM;
#pragma unroll
            for (int i = 0; i < 8; ++i) { wp[i] = wp[i + 1]; wq[i] = wq[i + 1]; }
            wp[8] = ld<T>(A, c);
            wq[8] = ld<T>(B, c);
        },
        [&](unsigned char *sa, unsigned char *sb, const Seg &, int o) {
            if (!active) return;
            const S *A = reinterpret_cast<const S *>(sa), *B = A + L::H;
            const S *Bu = reinterpret_cast<const S *>(sb);
            const float *F = reinterpret_cast<const float *>(sb + oF);
            const int c = (tx + MM) * L::AW + tz + MM, bi = tx * 32 + tz;
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            T Px = 0, Py = 0, Pz = 0, Qx = 0, Qy = 0, Qz = 0;
#pragma unroll
            for (int im = 0; im < 4; ++im) {  // ..tti..:94-99
                Py = fma_t(k[im], wp[5 + im] - wp[4 - im], Py);
                Px = fma_t(k[im], ld<T>(A, c + (im + 1) * L::AW) - ld<T>(A, c - im * L::AW), Px);
                Pz = fma_t(k[im], ld<T>(A, c + im + 1) - ld<T>(A, c - im), Pz);
                Qy = fma_t(k[im], wq[5 + im] - wq[4 - im], Qy);
                Qx = fma_t(k[im], ld<T>(B, c + (im + 1) * L::AW) - ld<T>(B, c - im * L::AW), Qx);
                Qz = fma_t(k[im], ld<T>(B, c + im + 1) - ld<T>(B, c - im), Qz);
            }
            T xx, yy, zz;
            tti_rot<T>((T)F[bi], (T)F[L::C + bi], (T)F[2 * L::C + bi], (T)F[3 * L::C + bi], Px, Py, Pz,
                       Px, Py, Qx, Qy, Qz, xx, yy, zz);
            const T cy1 = (T)p.cy1[o], cy2 = (T)p.cy2[o];
            const size_t g = gidx<S>(p, iz, ix, o);
            u[g] = to_store<S, T>(fma_t(cx2, ld<T>(Bu, bi), -((cx1 * (T)p.dtx) * xx)));
            v[g] = to_store<S, T>(fma_t(cy2, ld<T>(Bu, L::C + bi), -((cy1 * (T)p.dty) * yy)));
            w[g] = to_store<S, T>(fma_t(cz2, ld<T>(Bu, 2 * L::C + bi), -((cz1 * (T)p.dtz) * zz)));
        });
}

// ===========================================================================
// tti_stress: maps {u, v, w (H), P, Q (core), vp, eps, del, ct, st, cp, sp (core float)}
template <int TX, class S, int D>
struct TtiStrL {
    static constexpr int KA = Depth<D>::KA, KB = Depth<D>::KB;
    static constexpr int AW = 40, AH = TX + 8;
    static constexpr uint32_t C = 32 * TX, H = AW * AH;
    static constexpr uint32_t A_BYTES = 3 * H * sizeof(S);
    static constexpr uint32_t B_BYTES = 2 * C * sizeof(S) + 7 * C * 4;
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
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

template <int TX, class S, int D>
__global__ void __launch_bounds__(32 * TX + 32)
    tti_stress(const __grid_constant__ Maps<12> mp, S *__restrict__ P, S *__restrict__ Q,
               const __grid_constant__ K1Params p) {
    using L = TtiStrL<TX, S, D>;
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
    constexpr size_t oF = 2 * L::C * sizeof(S);  // vp eps del ct st cp sp
    if (warp == TX) {
        if (lane != 0) return;
        for (int i = 0; i < 12; ++i) prefetch_tmap(&mp.m[i]);
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE, L::B_BYTES, p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                for (int k = 0; k < 3; ++k)
                    tma_load_3d(dst + k * L::H * sizeof(S), &mp.m[k], bar, s.z0 - MM, s.x0 - MM, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                tma_load_3d(dst, &mp.m[3], bar, s.z0, s.x0, o);
                tma_load_3d(dst + L::C * sizeof(S), &mp.m[4], bar, s.z0, s.x0, o);
                for (int k = 0; k < 7; ++k)
                    tma_load_3d(dst + oF + k * L::C * 4, &mp.m[5 + k], bar, s.z0, s.x0, o);
            });
        return;
    }
    const int tx = warp, tz = lane;
    T wu[9], wv[9], ww[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) wu[i] = wv[i] = ww[i] = T(0);
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
            const int c = (tx + MM) * L::AW + tz + MM;
#pragma unroll
            for (int i = 0; i < 8; ++i) { wu[i] = wu[i + 1]; wv[i] = wv[i + 1]; ww[i] = ww[i + 1]; }
            wu[8] = ld<T>(A, c);
            wv[8] = ld<T>(A, L::H + c);
            ww[8] = ld<T>(A, 2 * L::H + c);
        },
        [&](unsigned char *sa, unsigned char *sb, const Seg &, int o) {
            if (!active) return;
            const S *U = reinterpret_cast<const S *>(sa), *V = U + L::H, *W = U + 2 * L::H;
            const S *Bp = reinterpret_cast<const S *>(sb), *Bq = Bp + L::C;
            const float *F = reinterpret_cast<const float *>(sb + oF);
            const int c = (tx + MM) * L::AW + tz + MM, bi = tx * 32 + tz;
            const T k[4] = {(T)C8_0, (T)C8_1, (T)C8_2, (T)C8_3};
            T ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, wx = 0, wy = 0, wz = 0;
#pragma unroll
            for (int im = 0; im < 4; ++im) {  // ..tti..:174-182 (vz is unused there)
                uy = fma_t(k[im], wu[4 + im] - wu[3 - im], uy);
                ux = fma_t(k[im], ld<T>(U, c + im * L::AW) - ld<T>(U, c - (im + 1) * L::AW), ux);
                uz = fma_t(k[im], ld<T>(U, c + im) - ld<T>(U, c - im - 1), uz);
                vy = fma_t(k[im], wv[4 + im] - wv[3 - im], vy);
                vx = fma_t(k[im], ld<T>(V, c + im * L::AW) - ld<T>(V, c - (im + 1) * L::AW), vx);
                wy = fma_t(k[im], ww[4 + im] - ww[3 - im], wy);
                wx = fma_t(k[im], ld<T>(W, c + im * L::AW) - ld<T>(W, c - (im + 1) * L::AW), wx);
                wz = fma_t(k[im], ld<T>(W, c + im) - ld<T>(W, c - im - 1), wz);
            }
            T xx, yy, zz;
            tti_rot<T>((T)F[3 * L::C + bi], (T)F[4 * L::C + bi], (T)F[5 * L::C + bi], (T)F[6 * L::C + bi],
                       ux, uy, uz, vx, vy, wx, wy, wz, xx, yy, zz);
            float ee, dd;
            sv_eedd_t(p, ix, o, iz, F[L::C + bi], F[2 * L::C + bi], ee, dd);
            const float ay1 = p.ay1[o], ay2 = p.ay2[o];
            const T vv = (T)F[bi];
            T e1, sd;
            if constexpr (sizeof(T) == 4) {
                e1 = 1.0f + 2.0f * ee;
                sd = sqrtf(1.0f + 2.0f * dd);
            } else {
                e1 = T(1) + T(2) * (T)ee;
                sd = sqrt(T(1) + T(2) * (T)dd);
            }
            const T kx = ((T)ax1 * vv) * vv, ky = ((T)ay1 * vv) * vv, kz = ((T)az1 * vv) * vv;
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
static cudaError_t launch_tti_t(const K1Launch &L, cudaStream_t st) {
    K1Params p = L.p;
    if (L.kind == K1_TTI_VEL) {
        static bool attr = false;
        Maps<9> mp;
        for (int i = 0; i < 9; ++i) mp.m[i] = L.maps[i];
        const int grid = k1_sweep<TX>(p, tti_vel<TX, S, D>, 32 * TX + 32, TtiVelL<TX, S, D>::TOTAL, L.grid, L.mode);
        return k1_launch(tti_vel<TX, S, D>, 32 * TX + 32, TtiVelL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr,
                         mp, (S *)L.out0, (S *)L.out1, (S *)L.out2, p);
    }
    static bool attr = false;
    Maps<12> mp;
    for (int i = 0; i < 12; ++i) mp.m[i] = L.maps[i];
    const int grid = k1_sweep<TX>(p, tti_stress<TX, S, D>, 32 * TX + 32, TtiStrL<TX, S, D>::TOTAL, L.grid, L.mode);
    return k1_launch(tti_stress<TX, S, D>, 32 * TX + 32, TtiStrL<TX, S, D>::TOTAL, p.sw.W, grid, st, attr,
                     mp, (S *)L.out0, (S *)L.out1, p);
}

cudaError_t launch_tti(const K1Launch &L, cudaStream_t st) {
    if (L.fp64) return launch_tti_t<8, double, 0>(L, st);
    if (L.tx == 16) return L.depth ? launch_tti_t<16, float, 1>(L, st) : launch_tti_t<16, float, 0>(L, st);
    return L.depth ? launch_tti_t<8, float, 1>(L, st) : launch_tti_t<8, float, 0>(L, st);
}

}  // namespace a3d
