// a3d_closure.cu — the learned absorbing rim: inference kernels (hidden layer on
// the face boxes, correction of the rim cells), the training kernels (teacher
// states from a wide-PML run, loss, gradients, Adam), the training object behind
// the a3d_closure_* C API, and the tap that copies an engine's state out.
//
// Kernels are plain CUDA-core code: one thread per cell, weights in shared memory
// as float values of bfloat16 numbers, hidden activations stored as bfloat16,
// float accumulation with explicit fmaf (the library builds with --fmad=false).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/acoustic3d.h"
#include "a3d_closure_dev.cuh"

namespace a3d {

int fail(int code, const char *fmt, ...);

#define CL_TRY(x)                                                                      \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess)                                                         \
            return fail(A3D_E_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));      \
    } while (0)

// ---------------------------------------------------------------------------
// geometry and parameter layout (host)

ClGeom cl_geom(int nnz, int nnx, int nny, long long ldz) {
    ClGeom g{};
    g.nn[0] = nnz; g.nn[1] = nnx; g.nn[2] = nny;
    g.ldz = ldz;
    long long off = 0;
    for (int f = 0; f < 6; ++f) {
        const int A = f >> 1, a1 = A == 0 ? 1 : 0, a2 = A == 2 ? 1 : 2;
        g.T1[f] = g.nn[a1] - 8;
        g.T2[f] = g.nn[a2] - 8;
        g.hoff[f] = off;
        off += 7LL * g.T1[f] * g.T2[f];
    }
    g.hoff[6] = off;
    // x rims (whole y, z extent), then y rims inside the x interior, then z rims
    // inside both: six disjoint boxes covering every rim cell once
    const int nz8 = nnz - 8, ny8 = nny - 8, nxi = nnx - 2 * CL_PAD, nyi = nny - 2 * CL_PAD;
    const int lo[6][3] = {{4, 4, 4}, {4, nnx - CL_PAD, 4}, {4, CL_PAD, 4}, {4, CL_PAD, nny - CL_PAD},
                          {4, CL_PAD, CL_PAD}, {nnz - CL_PAD, CL_PAD, CL_PAD}};
    const int ex[6][3] = {{nz8, CL_RIM, ny8}, {nz8, CL_RIM, ny8}, {nz8, nxi, CL_RIM}, {nz8, nxi, CL_RIM},
                          {CL_RIM, nxi, nyi}, {CL_RIM, nxi, nyi}};
    off = 0;
    for (int b = 0; b < 6; ++b) {
        for (int k = 0; k < 3; ++k) { g.blo[b][k] = lo[b][k]; g.bext[b][k] = ex[b][k]; }
        g.roff[b] = off;
        off += (long long)ex[b][0] * ex[b][1] * ex[b][2];
    }
    g.roff[6] = off;
    return g;
}

// round to the nearest bfloat16, ties to even (inputs are finite)
float cl_round_bf16(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

void cl_pack_params(const float *canon, float *packed) {
    const float *W1 = canon, *W2 = canon + CL_NW1, *G = canon + CL_NW1 + CL_NW2;
    float *P1 = packed, *P2 = packed + CL_NW1, *PG = packed + CL_NW1 + CL_NW2;
    for (int j = 0; j < CL_CH; ++j)
        for (int i = 0; i < CL_CIN; ++i)
            for (int t = 0; t < 27; ++t)
                P1[(t * CL_CIN + i) * CL_CH + j] = cl_round_bf16(W1[(j * CL_CIN + i) * 27 + t]);
    for (int f = 0; f < 6; ++f)
        for (int o = 0; o < CL_COUT; ++o)
            for (int j = 0; j < CL_CH; ++j)
                for (int t = 0; t < 27; ++t)
                    P2[((f * 27 + t) * CL_CH + j) * CL_COUT + o] =
                        cl_round_bf16(W2[((f * CL_COUT + o) * CL_CH + j) * 27 + t]);
    for (int k = 0; k < CL_NG; ++k) PG[k] = cl_round_bf16(G[k]);
}

// ---------------------------------------------------------------------------
// hidden layer: h_f = relu(W1 * x) on every face-box cell (bfloat16 out)

__global__ void __launch_bounds__(CL_THREADS)
    cl_hidden(const ClGeom g, const float *__restrict__ u, const float *__restrict__ v,
              const float *__restrict__ w, const float *__restrict__ P, const float *__restrict__ zinv,
              const float *__restrict__ kap, const float *__restrict__ W1c, __nv_bfloat16 *__restrict__ h) {
    __shared__ __align__(16) float sW[CL_NW1];
    for (int i = threadIdx.x; i < CL_NW1; i += blockDim.x) sW[i] = W1c[i];
    __syncthreads();
    const long long total = g.hoff[6];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < total;
         n += (long long)gridDim.x * blockDim.x) {
        int f = 0;
        while (f < 5 && n >= g.hoff[f + 1]) ++f;
        int c[3], a;
        face_cell(g, f, n - g.hoff[f], c, a);
        float acc[CL_CH];
#pragma unroll
        for (int j = 0; j < CL_CH; ++j) acc[j] = 0.0f;
#pragma unroll 1
        for (int t = 0; t < 27; ++t) {
            const int dz = t % 3 - 1, dx = (t / 3) % 3 - 1, dy = t / 9 - 1;
            float x[8];
            load_x(u, v, w, P, zinv, kap, gidx(g, c[0] + dz, c[1] + dx, c[2] + dy), x);
            const float4 *ws = reinterpret_cast<const float4 *>(sW + t * CL_CIN * CL_CH);
#pragma unroll
            for (int i = 0; i < CL_CIN; ++i)
#pragma unroll
                for (int q = 0; q < CL_CH / 4; ++q) {
                    const float4 wv = ws[i * (CL_CH / 4) + q];
                    acc[4 * q] = fmaf(wv.x, x[i], acc[4 * q]);
                    acc[4 * q + 1] = fmaf(wv.y, x[i], acc[4 * q + 1]);
                    acc[4 * q + 2] = fmaf(wv.z, x[i], acc[4 * q + 2]);
                    acc[4 * q + 3] = fmaf(wv.w, x[i], acc[4 * q + 3]);
                }
        }
        uint4 *hp = reinterpret_cast<uint4 *>(h + n * CL_CH);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint32_t r[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const __nv_bfloat162 b2 =
                    __floats2bfloat162_rn(fmaxf(acc[8 * q + 2 * k], 0.0f), fmaxf(acc[8 * q + 2 * k + 1], 0.0f));
                r[k] = *reinterpret_cast<const uint32_t *>(&b2);
            }
            hp[q] = make_uint4(r[0], r[1], r[2], r[3]);
        }
    }
}

constexpr size_t CL_APPLY_SMEM = (size_t)(CL_NW2 + CL_NG) * 4;

// correction of every rim cell: added to the fields in place, or (dout set) written
// to dout as four fields of the grid's layout (u, v, w, P corrections; stride dstride)
__global__ void __launch_bounds__(CL_THREADS)
    cl_apply(const ClGeom g, float *__restrict__ u, float *__restrict__ v, float *__restrict__ w,
             float *__restrict__ P, const float *__restrict__ zinv, const float *__restrict__ W2c,
             const float *__restrict__ Gc, const __nv_bfloat16 *__restrict__ h, float *__restrict__ dout,
             long long dstride) {
    extern __shared__ __align__(16) float smem_cl[];
    float *sG = smem_cl + CL_NW2;
    for (int i = threadIdx.x; i < CL_NW2; i += blockDim.x) smem_cl[i] = W2c[i];
    for (int i = threadIdx.x; i < CL_NG; i += blockDim.x) sG[i] = Gc[i];
    __syncthreads();
    const float4 *sW2 = reinterpret_cast<const float4 *>(smem_cl);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.roff[6];
         n += (long long)gridDim.x * blockDim.x) {
        int c[3];
        rim_cell(g, n, c);
        float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 1
        for (int A = 0; A < 3; ++A) {
            int a;
            const int f = rim_face(g, A, c[A], a);
            if (f < 0) continue;
            float y[4];
            face_out(g, f, c, sW2, h, y);
            const float *gg = sG + (f * CL_RIM + a - 1) * CL_COUT;
#pragma unroll
            for (int o = 0; o < 4; ++o) d[o] = fmaf(gg[o], y[o], d[o]);
        }
        const long long id = gidx(g, c[0], c[1], c[2]);
        const float dp = d[3] / zinv[id];
        if (dout) {
            dout[id] = d[0];
            dout[dstride + id] = d[1];
            dout[2 * dstride + id] = d[2];
            dout[3 * dstride + id] = dp;
        } else {
            u[id] += d[0];
            v[id] += d[1];
            w[id] += d[2];
            P[id] += dp;
        }
    }
}

__global__ void cl_scales(const float *__restrict__ rho, const float *__restrict__ vp, float courant,
                          float *__restrict__ zinv, float *__restrict__ kap, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float z = rho[i] * vp[i];
        zinv[i] = z > 0.0f ? 1.0f / z : 0.0f;
        kap[i] = vp[i] * courant;
    }
}

__global__ void cl_tap(int nnz, int nnx, int nny, long long ldz, int off, const float *__restrict__ u,
                       const float *__restrict__ v, const float *__restrict__ w, const float *__restrict__ P,
                       float *__restrict__ out) {
    const int bz = nnz - 2 * off, bx = nnx - 2 * off, by = nny - 2 * off;
    const long long nb = (long long)bz * bx * by;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nb;
         n += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(n % bz), x = (int)((n / bz) % bx), y = (int)(n / ((long long)bz * bx));
        const long long id = (long long)(z + off) + ldz * ((long long)(x + off) + (long long)nnx * (y + off));
        out[n] = u[id];
        out[nb + n] = v[id];
        out[2 * nb + n] = w[id];
        out[3 * nb + n] = P[id];
    }
}

static int grid_for(long long n, int per = CL_THREADS, int cap = 152 * 16) {
    const long long b = (n + per - 1) / per;
    return (int)std::max(1LL, std::min<long long>(b, cap));
}

cudaError_t cl_launch_scales(const float *rho, const float *vp, float courant, float *zinv, float *kap, size_t n,
                             cudaStream_t st) {
    cl_scales<<<grid_for((long long)n), CL_THREADS, 0, st>>>(rho, vp, courant, zinv, kap, n);
    return cudaGetLastError();
}

cudaError_t cl_prepare() {
    return cudaFuncSetAttribute(cl_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CL_APPLY_SMEM);
}

cudaError_t cl_launch_hidden(const ClGeom &g, const float *u, const float *v, const float *w, const float *P,
                             const float *zinv, const float *kap, const float *packed, __nv_bfloat16 *h,
                             cudaStream_t st) {
    cl_hidden<<<grid_for(g.hoff[6]), CL_THREADS, 0, st>>>(g, u, v, w, P, zinv, kap, packed, h);
    return cudaGetLastError();
}

cudaError_t cl_launch_correct(const ClGeom &g, float *u, float *v, float *w, float *P, const float *zinv,
                              const float *packed, const __nv_bfloat16 *h, float *dout, long long dstride,
                              cudaStream_t st) {
    cl_apply<<<grid_for(g.roff[6]), CL_THREADS, CL_APPLY_SMEM, st>>>(g, u, v, w, P, zinv, packed + CL_NW1,
                                                                     packed + CL_NW1 + CL_NW2, h, dout, dstride);
    return cudaGetLastError();
}

cudaError_t cl_launch_apply(const ClGeom &g, float *u, float *v, float *w, float *P, const float *zinv,
                            const float *kap, const float *packed, __nv_bfloat16 *h, cudaStream_t st) {
    cudaError_t e = cl_launch_hidden(g, u, v, w, P, zinv, kap, packed, h, st);
    if (e != cudaSuccess) return e;
    return cl_launch_correct(g, u, v, w, P, zinv, packed, h, nullptr, 0, st);
}

cudaError_t cl_launch_tap(int nnz, int nnx, int nny, long long ldz, int off, const float *u, const float *v,
                          const float *w, const float *P, float *out, cudaStream_t st) {
    const long long nb = (long long)(nnz - 2 * off) * (nnx - 2 * off) * (nny - 2 * off);
    cl_tap<<<grid_for(nb), CL_THREADS, 0, st>>>(nnz, nnx, nny, ldz, off, u, v, w, P, out);
    return cudaGetLastError();
}

}  // namespace a3d
