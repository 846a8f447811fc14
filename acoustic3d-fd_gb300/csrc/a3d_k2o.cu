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
//   * Consumer warps (one 32-cell z row each) keep a 9-plane register window
//     for the y-derivative and read the z/x neighbours from the halo'd tile.
//
// State kept in two buffers X (current) and Y (previous, raw):
//   prev   = sponge(Y)                          reference: absorb of p0 after swap
//   next   = 2 cur - prev + vv * lap(cur)       2O:295, double steps done in float
//   Y     <- sponge(next) +/- w[it+1]           absorb of p1, then next step's dipole
//   record = sponge(X) at the receivers          cuda_record on p0 after absorb
// so the only HBM traffic is X and Y read, vv read, Y written: 16 B per cell.
#include "a3d_kernels.cuh"
#include "a3d_pipe.cuh"

namespace a3d {

template <int TX, class S, int D>
struct K2OSmem {
    static constexpr int KA = Depth<D>::KA;  // halo'd current-level stages (4 live + rest in flight)
    static constexpr int KB = Depth<D>::KB;  // prev/vv stages
    static constexpr int AW = 40, AH = TX + 8;  // A tile: [AH][AW]
    static constexpr int A_ELEMS = AW * AH;
    static constexpr int B_ELEMS = 32 * TX;
    static constexpr uint32_t A_BYTES = (uint32_t)(A_ELEMS * sizeof(S));
    static constexpr uint32_t B_BYTES = (uint32_t)(B_ELEMS * sizeof(S));
    static constexpr uint32_t VV_BYTES = (uint32_t)(B_ELEMS * sizeof(float));
    static constexpr size_t A_STRIDE = (A_BYTES + 127) / 128 * 128;
    static constexpr size_t B_STRIDE = (B_BYTES + VV_BYTES + 127) / 128 * 128;
    static constexpr size_t BAR_OFF = KA * A_STRIDE + KB * B_STRIDE;
    static constexpr size_t TOTAL = BAR_OFF + sizeof(PipeBars<KA, KB>);
};

template <int TX, class S, int D, int R>
__global__ void __launch_bounds__(32 * (TX / R) + 32)
    k2o_step(const __grid_constant__ CUtensorMap tm_cur, const __grid_constant__ CUtensorMap tm_prev,
             const __grid_constant__ CUtensorMap tm_vv, S *__restrict__ ybuf,
             const __grid_constant__ K2OParams p) {
    using L = K2OSmem<TX, S, D>;
    using T = typename Arith<S>::T;
    constexpr int NW = TX / R;  // consumer warps, R tile rows each
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
        prefetch_tmap(&tm_cur);
        prefetch_tmap(&tm_prev);
        prefetch_tmap(&tm_vv);
        pipe_produce<TX, L::KA, L::KB>(
            p.sw, w0, w1, bars, ringA, L::A_STRIDE, L::A_BYTES, ringB, L::B_STRIDE,
            L::B_BYTES + L::VV_BYTES, p.err,
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int q) {
                tma_load_3d(dst, &tm_cur, bar, s.z0 - MM, s.x0 - MM, q);
            },
            [&](unsigned char *dst, uint64_t *bar, const Seg &s, int o) {
                tma_load_3d(dst, &tm_prev, bar, s.z0, s.x0, o);
                tma_load_3d(dst + L::B_BYTES, &tm_vv, bar, s.z0, s.x0, o);
            });
        return;
    }

    const int tz = lane, xw = warp * R;
    T win[R][9];  // current level at planes q-8 .. q, per row
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int i = 0; i < 9; ++i) win[r][i] = T(0);
    int iz = 0;
    bool zact = false, act[R], rec[R];
    int ixr[R];
    float2 fz{0.f, 0.f}, fx[R];
    const T k1 = (T)S8_1, k2 = (T)S8_2, k3 = (T)S8_3, k4 = (T)S8_4;
    const size_t pstride = (size_t)p.ldz * p.nnx;
    pipe_consume<TX, L::KA, L::KB>(
        p.sw, w0, w1, bars, ringA, L::A_STRIDE, ringB, L::B_STRIDE, p.err,
        [&](const Seg &s) {
            iz = s.z0 + tz;
            zact = iz < p.nnz - MM;
            // sponge factors of this column (hi == 0: no sponge on that face)
            fz = p.fz[min(iz, p.nnz - 1)];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ix = s.x0 + xw + r;
                ixr[r] = ix;
                act[r] = zact && ix < p.nnx - MM;
                fx[r] = p.fx[min(ix, p.nnx - 1)];
                rec[r] = iz == p.gz && ix >= p.rx0 && ix < p.rx0 + p.nx;
            }
        },
        [&](unsigned char *st, const Seg &, int) {
            const S *At = reinterpret_cast<const S *>(st);
#pragma unroll
            for (int r = 0; r < R; ++r) {
#pragma unroll
                for (int i = 0; i < 8; ++i) win[r][i] = win[r][i + 1];
                win[r][8] = (T)At[(xw + r + MM) * L::AW + tz + MM];
            }
        },
        [&](unsigned char *sa, unsigned char *sb, const Seg &, int o) {
            if (!zact) return;
            const S *Ao = reinterpret_cast<const S *>(sa);
            const S *Bp = reinterpret_cast<const S *>(sb);
            const float *Bv = reinterpret_cast<const float *>(sb + L::B_BYTES);
            const float2 fy = p.fy[o];
            // current level at tile rows xw .. xw+R+7 of this z column: xs[j] = cur(x = xw - 4 + j)
            T xs[R + 8];
#pragma unroll
            for (int j = 0; j < R + 8; ++j) xs[j] = (T)Ao[(xw + j) * L::AW + tz + MM];
            const size_t po = pstride * o;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (!act[r]) continue;
                const int c = (xw + r + MM) * L::AW + tz + MM, bi = (xw + r) * 32 + tz;
                const T cur = win[r][4];
                T c1 = (T)S8_0 * cur, c2 = c1, c3 = c1;
                // z from the tile, x from the shared rows, y from the window (2O:284-289)
                c1 = fma_t(k1, (T)Ao[c - 1] + (T)Ao[c + 1], c1);
                c2 = fma_t(k1, xs[r + 3] + xs[r + 5], c2);
                c3 = fma_t(k1, win[r][5] + win[r][3], c3);
                c1 = fma_t(k2, (T)Ao[c - 2] + (T)Ao[c + 2], c1);
                c2 = fma_t(k2, xs[r + 2] + xs[r + 6], c2);
                c3 = fma_t(k2, win[r][6] + win[r][2], c3);
                c1 = fma_t(k3, (T)Ao[c - 3] + (T)Ao[c + 3], c1);
                c2 = fma_t(k3, xs[r + 1] + xs[r + 7], c2);
                c3 = fma_t(k3, win[r][7] + win[r][1], c3);
                c1 = fma_t(k4, (T)Ao[c - 4] + (T)Ao[c + 4], c1);
                c2 = fma_t(k4, xs[r] + xs[r + 8], c2);
                c3 = fma_t(k4, win[r][8] + win[r][0], c3);
                c1 *= (T)p.dz2;
                c2 *= (T)p.dx2;
                c3 *= (T)p.dy2;
                const T m = (T)Bv[bi] * ((c1 + c2) + c3);
                const T prev = sponge3<T>((T)Bp[bi], fy, fx[r], fz);
                T nxt;
                if constexpr (sizeof(T) == 4)
                    nxt = upd2o(cur, prev, m);
                else
                    nxt = (T(2) * cur - prev) + m;
                nxt = sponge3<T>(nxt, fy, fx[r], fz);
                if (ixr[r] == p.s_x && o == p.s_y) {  // next step's dipole (2O:184-185)
                    if (iz == p.s_z) nxt = nxt + (T)p.w_next;
                    if (iz == p.s_z + 2) nxt = nxt - (T)p.w_next;
                }
                ybuf[(size_t)iz + (size_t)p.ldz * ixr[r] + po] = to_store<S, T>(nxt);
                if (rec[r] && o >= p.ry0 && o < p.ry0 + p.ny) {  // cuda_record after absorb (2O:452)
                    const size_t tr = (size_t)(ixr[r] - p.rx0) + (size_t)p.nx * (o - p.ry0);
                    T rr = sponge3<T>(cur, fy, fx[r], fz);
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
    constexpr int NT = 32 * (TX / R) + 32;
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)SM::TOTAL);
        if (e != cudaSuccess) return e;
        attr_done = true;
    }
    K2OParams p = L.p;
    p.sw.ntz = (p.nnz - 2 * MM + 31) / 32;
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
    if (L.tx == 16) {
        if (L.rows == 4) return L.deep ? launch_k2o_t<16, float, 1, 4>(L, st) : launch_k2o_t<16, float, 0, 4>(L, st);
        if (L.rows == 1) return L.deep ? launch_k2o_t<16, float, 1, 1>(L, st) : launch_k2o_t<16, float, 0, 1>(L, st);
        return L.deep ? launch_k2o_t<16, float, 1, 2>(L, st) : launch_k2o_t<16, float, 0, 2>(L, st);
    }
    if (L.rows == 1) return L.deep ? launch_k2o_t<8, float, 1, 1>(L, st) : launch_k2o_t<8, float, 0, 1>(L, st);
    return L.deep ? launch_k2o_t<8, float, 1, 2>(L, st) : launch_k2o_t<8, float, 0, 2>(L, st);
}

size_t k2o_smem_bytes(int tx, bool fp64) {
    if (fp64) return K2OSmem<8, double, 0>::TOTAL;
    return tx == 16 ? K2OSmem<16, float, 0>::TOTAL : K2OSmem<8, float, 0>::TOTAL;
}

}  // namespace a3d
