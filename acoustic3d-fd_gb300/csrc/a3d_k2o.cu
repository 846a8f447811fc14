// a3d_k2o.cu — 2nd-order engine: one fused kernel per time step.
//
// Replaces, per step, the reference's six launches (Toa_3dfd_cuda.cu:443-453:
// dipole, cuda_step_fd3d, two cuda_absorb_bndr, cuda_record, cuda_trans_xy2txy)
// with one persistent, warp-specialised y-marching sweep:
//
//   * A producer warp streams, plane by plane, the current level with a 4-cell
//     z/x halo (TMA box {32+8, TX+8, 1}) into a ring of KA stages, and the raw
//     previous level and vv = (v dt)^2 at the output plane (boxes {32, TX, 1})
//     into a ring of KB stages.
//   * Consumer warps (R tile rows each, lane = z) keep an 8-plane register
//     window for the y-derivative (the 9th plane is read from its fresh tile)
//     and read the z/x neighbours from the halo'd tile.
//
// State kept in two buffers X (current) and Y (previous, raw):
//   prev   = sponge(Y)                          reference: absorb of p0 after swap
//   next   = 2 cur - prev + vv * lap(cur)       2O:295, double steps done in float
//   Y     <- sponge(next) +/- w[it+1]           absorb of p1, then next step's dipole
//   record = sponge(X) at the receivers          cuda_record on p0 after absorb
// so the only HBM traffic is X and Y read, vv read, Y written: 16 B per cell.
#include "a3d_k1dev.cuh"

namespace a3d {

template <int TX, class S, int D>
struct K2OSmem {
    static constexpr int AW = 40, AH = TX + 8;  // A tile: [AH][AW]
    static constexpr int A_ELEMS = AW * AH;
    static constexpr int B_ELEMS = 32 * TX;
    static constexpr uint32_t A_BYTES = (uint32_t)(A_ELEMS * sizeof(S));
    static constexpr uint32_t B_BYTES = (uint32_t)(B_ELEMS * sizeof(S));
    static constexpr uint32_t VV_BYTES = (uint32_t)(B_ELEMS * sizeof(float));
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + VV_BYTES + 127) / 128 * 128;
    // A: halo'd current-level stages (4 held for the in-plane neighbours); B: prev/vv
    using RG = Ring<D, A_STRIDE, B_STRIDE>;
    using Bars = typename RG::Bars;
    static constexpr int KA = RG::KA, KB = RG::KB;
    static constexpr size_t RB = RG::RB, B_OFF = RG::B_OFF, BAR_OFF = RG::BAR_OFF, TOTAL = RG::TOTAL;
};

template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / (2 * R) + 1))
    k2o_step(const __grid_constant__ CUtensorMap tm_cur, const __grid_constant__ CUtensorMap tm_prev,
             const __grid_constant__ CUtensorMap tm_vv, S *__restrict__ ybuf,
             const __grid_constant__ K2OParams p) {
    using L = K2OSmem<TX, S, D>;
    using T = typename Arith<S>::T;
    using T2 = Two<T>;
    constexpr int NW = TX / (2 * R), AW = L::AW;  // consumer warps, 2R tile rows each
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
        prefetch_tmap(&tm_cur);
        prefetch_tmap(&tm_prev);
        prefetch_tmap(&tm_vv);
        pipe_produce_m<TX, L::KA, L::KB, L::RB>(
            p.sw, w0, w1, bars, ringB, p.err, [](const Seg &, int) { return (uint32_t)L::B_STRIDE; },
            [&](uint32_t sa, unsigned char *dst, uint32_t, uint64_t *bar, const Seg &s, int q) {
                mbar_arrive_expect_tx(bar, L::A_BYTES + (dst ? L::B_BYTES + L::VV_BYTES : 0u));
                tma_load_3d(ringA + sa * L::A_STRIDE, &tm_cur, bar, s.z0 - MM, s.x0 - MM, q);
                if (!dst) return;
                tma_load_3d(dst, &tm_prev, bar, s.z0, s.x0, q - MM);
                tma_load_3d(dst + L::B_BYTES, &tm_vv, bar, s.z0, s.x0, q - MM);
            });
        return;
    }

    // lane: z cells zl, zl+1 of the tile (zl = 2 (lane mod 16)) in tile rows
    // xw .. xw+R-1, where the two half-warps take consecutive groups of R rows
    const int zl = 2 * (lane & 15), xw = warp * 2 * R + (lane >> 4) * R;
    const int c0 = (xw + MM) * AW + zl + MM;  // this lane's first cell pair in an A tile
    // current level at the last 8 planes, slot = item mod 8; the 9th plane of the
    // y-stencil (the newest, q) is read from its A tile before it enters the window
    T2 win[R][8];
    int iz = 0;
    bool act[R], both = true, reca[R], recb[R], srow[R];
    int trb[R];
    uint32_t gb[R];
    float2 fza{0.f, 0.f}, fzb{0.f, 0.f}, fx[R];
    float2 fyn{0.f, 0.f};  // y sponge factor of the next output plane (loaded one plane ahead)
    const T k1 = (T)S8_1, k2 = (T)S8_2, k3 = (T)S8_3, k4 = (T)S8_4;
    const T dz2 = (T)p.dz2, dx2 = (T)p.dx2, dy2 = (T)p.dy2;
    const uint32_t pstride = (uint32_t)p.ldz * (uint32_t)p.nnx;
    pipe_run<TX, L::KA, L::KB, MM>(
        p.sw, w0, w1, bars, ringB, p.err,
        [&](const Seg &s) {
            iz = s.z0 + zl;
            const bool zact = iz < p.nnz - MM;
            both = iz + 1 < p.nnz - MM;
            // sponge factors of this lane's cells (hi == 0: no sponge on that face)
            fza = p.fz[min(iz, p.nnz - 1)];
            fzb = p.fz[min(iz + 1, p.nnz - 1)];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                act[r] = zact && ix < p.nnx - MM;
                const int cxi = min(ix, p.nnx - 1);
                fx[r] = p.fx[cxi];
                const bool rx = act[r] && ix >= p.rx0 && ix < p.rx0 + p.nx;
                reca[r] = rx && iz == p.gz;
                recb[r] = rx && both && iz + 1 == p.gz;
                trb[r] = ix - p.rx0;
                srow[r] = act[r] && ix == p.s_x;
                gb[r] = (uint32_t)iz + (uint32_t)p.ldz * (uint32_t)cxi;
            }
            fyn = p.fy[s.ya];
        },
        [&](auto ph, uint32_t sa, const Seg &, int) {
            constexpr int Q = decltype(ph)::value;
            const S *At = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
#pragma unroll
            for (int r = 0; r < R; ++r) win[r][Q] = ld2<T>(At, c0 + r * AW);
        },
        [&](int ph, uint32_t sa, uint32_t sh, const unsigned char *sbp, const Seg &, int q) {
            const int o = q - MM;
            const S *At = reinterpret_cast<const S *>(ringA + sa * L::A_STRIDE);
            // y part of the Laplacian from the window cur(o-4 .. o+3) (plane o+m in slot
            // (ph+4+m)&7) and the fresh plane cur(o+4) = cur(q) (2O:288), which then
            // replaces cur(q-8) in the window
            T2 cur[R], c3[R];
            with_phase(ph, [&](auto pc) {
                constexpr int Q = decltype(pc)::value;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const T2 *wr = win[r];
                    const T2 nw = ld2<T>(At, c0 + r * AW);
                    const T2 cc = wr[(Q + 4) & 7];
                    T a = (T)S8_0 * cc.a, b = (T)S8_0 * cc.b;
                    a = fma_t(k1, wr[(Q + 5) & 7].a + wr[(Q + 3) & 7].a, a);
                    b = fma_t(k1, wr[(Q + 5) & 7].b + wr[(Q + 3) & 7].b, b);
                    a = fma_t(k2, wr[(Q + 6) & 7].a + wr[(Q + 2) & 7].a, a);
                    b = fma_t(k2, wr[(Q + 6) & 7].b + wr[(Q + 2) & 7].b, b);
                    a = fma_t(k3, wr[(Q + 7) & 7].a + wr[(Q + 1) & 7].a, a);
                    b = fma_t(k3, wr[(Q + 7) & 7].b + wr[(Q + 1) & 7].b, b);
                    a = fma_t(k4, nw.a + wr[Q].a, a);
                    b = fma_t(k4, nw.b + wr[Q].b, b);
                    cur[r] = cc;
                    c3[r] = T2{a, b};
                    win[r][Q] = nw;
                }
            });
            const S *Ao = reinterpret_cast<const S *>(ringA + sh * L::A_STRIDE);
            const S *Bp = reinterpret_cast<const S *>(sbp);
            const float *Bv = reinterpret_cast<const float *>(sbp + L::B_BYTES);
            const float2 fy = fyn;
            fyn = p.fy[o + 1];  // o + 1 <= nny - 4: in bounds
            // current level at tile rows xw .. xw+R+7 of this lane's z pair: xs[j] = cur(x = xw - 4 + j)
            T2 xs[R + 8];
#pragma unroll
            for (int j = 0; j < R + 8; ++j) xs[j] = ld2<T>(Ao, c0 + (j - MM) * AW);
            const uint32_t po = pstride * (uint32_t)o;
            const bool yrec = o >= p.ry0 && o < p.ry0 + p.ny;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int bi = (xw + r) * 32 + zl;
                // current level along z at halo'd row positions zl .. zl+9 (zl+4 = cell a)
                T2 zp[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) zp[m] = ld2<T>(Ao, c0 + r * AW - MM + 2 * m);
                const T zv[10] = {zp[0].a, zp[0].b, zp[1].a, zp[1].b, zp[2].a,
                                  zp[2].b, zp[3].a, zp[3].b, zp[4].a, zp[4].b};
                const T2 pv = ld2<T>(Bp, bi);
                const float2 vv = *reinterpret_cast<const float2 *>(Bv + bi);
                T out[2];
#pragma unroll
                for (int e = 0; e < 2; ++e) {  // the lane's two cells
                    const T cc = e ? cur[r].b : cur[r].a;
                    const float2 fz = e ? fzb : fza;
                    T c1 = (T)S8_0 * cc, c2 = c1;
                    // z from the tile, x from the shared rows (2O:284-289)
                    c1 = fma_t(k1, zv[3 + e] + zv[5 + e], c1);
                    c2 = fma_t(k1, (e ? xs[r + 3].b : xs[r + 3].a) + (e ? xs[r + 5].b : xs[r + 5].a), c2);
                    c1 = fma_t(k2, zv[2 + e] + zv[6 + e], c1);
                    c2 = fma_t(k2, (e ? xs[r + 2].b : xs[r + 2].a) + (e ? xs[r + 6].b : xs[r + 6].a), c2);
                    c1 = fma_t(k3, zv[1 + e] + zv[7 + e], c1);
                    c2 = fma_t(k3, (e ? xs[r + 1].b : xs[r + 1].a) + (e ? xs[r + 7].b : xs[r + 7].a), c2);
                    c1 = fma_t(k4, zv[0 + e] + zv[8 + e], c1);
                    c2 = fma_t(k4, (e ? xs[r].b : xs[r].a) + (e ? xs[r + 8].b : xs[r + 8].a), c2);
                    c1 *= dz2;
                    c2 *= dx2;
                    const T m = (T)(e ? vv.y : vv.x) * ((c1 + c2) + (e ? c3[r].b : c3[r].a) * dy2);
                    const T prev = sponge3<T>(e ? pv.b : pv.a, fy, fx[r], fz);
                    T nxt;
                    if constexpr (sizeof(T) == 4)
                        nxt = upd2o(cc, prev, m);
                    else
                        nxt = (T(2) * cc - prev) + m;
                    nxt = sponge3<T>(nxt, fy, fx[r], fz);
                    if (srow[r] && o == p.s_y) {  // next step's dipole (2O:184-185)
                        if (iz + e == p.s_z) nxt = nxt + (T)p.w_next;
                        if (iz + e == p.s_z + 2) nxt = nxt - (T)p.w_next;
                    }
                    out[e] = nxt;
                }
                if (act[r]) st2m<S, T>(ybuf, gb[r] + po, out[0], out[1], both);
                if (yrec && (reca[r] | recb[r])) {  // cuda_record after absorb (2O:452)
                    const size_t tr = (size_t)trb[r] + (size_t)p.nx * (o - p.ry0);
                    T rr = reca[r] ? sponge3<T>(cur[r].a, fy, fx[r], fza) : sponge3<T>(cur[r].b, fy, fx[r], fzb);
                    if (p.mute_nt && p.it < p.mute_nt[tr]) rr = T(0);
                    p.rec[tr * p.nt + p.it] = (float)rr;
                }
            }
        });
}

// ---------------------------------------------------------------------------
// host launcher

template <int TX, class S, int D, int R>
static cudaError_t launch_k2o_t(const K2OLaunch &L, cudaStream_t st) {
    using SM = K2OSmem<TX, S, D>;
    auto kern = k2o_step<TX, S, D, R>;
    constexpr int NT = 32 * (TX / (2 * R) + 1);
    static SmemAttr attr;
    if (!smem_fits(SM::TOTAL)) return cudaErrorInvalidConfiguration;
    if (cudaError_t e = ensure_smem_attr(kern, SM::TOTAL, attr); e != cudaSuccess) return e;
    K2OParams p = L.p;
    p.sw.ntz = (p.nnz - 2 * MM + 31) / 32;
    p.sw.nshot = 1;
    p.sw.ntx = (p.nnx - 2 * MM + TX - 1) / TX;
    p.sw.y_begin = MM;
    p.sw.NY = p.nny - 2 * MM;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NT, SM::TOTAL);
    int grid = plan_sweep(p.sw, occ, L.mode);
    if (L.grid > 0) grid = L.grid;
    kern<<<grid, NT, SM::TOTAL, st>>>(L.tm_cur, L.tm_prev, L.tm_vv,
                                                reinterpret_cast<S *>(L.ybuf), p);
    return cudaGetLastError();
}

// configurations: (tile width, rows per warp) in {8, 16} x {1, 2} and (16, 4), two ring depths
cudaError_t launch_k2o(const K2OLaunch &L, cudaStream_t st) {
    if (L.fp64) return launch_k2o_t<8, double, 0, 2>(L, st);
    // one of three ring depths for each (tile width, rows per lane) shape
#define A3D_BY_DEPTH(TX_, R_)                                                   \
    return L.depth == 2 ? launch_k2o_t<TX_, float, 2, R_>(L, st)                \
         : L.depth == 1 ? launch_k2o_t<TX_, float, 1, R_>(L, st)                \
                        : launch_k2o_t<TX_, float, 0, R_>(L, st)
    if (L.tx == 16) {
        if (L.rows == 4) A3D_BY_DEPTH(16, 4);
        if (L.rows == 1) A3D_BY_DEPTH(16, 1);
        A3D_BY_DEPTH(16, 2);
    }
    if (L.rows == 1) A3D_BY_DEPTH(8, 1);
    A3D_BY_DEPTH(8, 2);
#undef A3D_BY_DEPTH
}

size_t k2o_smem_bytes(int tx, bool fp64) {
    if (fp64) return K2OSmem<8, double, 0>::TOTAL;
    return tx == 16 ? K2OSmem<16, float, 0>::TOTAL : K2OSmem<8, float, 0>::TOTAL;
}

}  // namespace a3d
