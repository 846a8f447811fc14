// a3d_closure_train.cu — training of the learned rim on teacher states.
//
// A teacher state pair (S_t, S_t+1) is the wavefield of a wide-PML run cropped to
// the rim grid (model + 10 cells per face) at two consecutive steps.  The student
// step from S_t is the engine's undamped update on the rim grid, whose outer 4
// cells hold zeros: X = step(S_t).  The closure is trained so that its correction
// of X in the rim reproduces the teacher, with the loss
//
//   L = sum over rim cells, channels o of (delta_o - (S_t+1 - X)_o)^2 / E,
//   E = sum over rim cells of |(u, v, w, P / (rho vp)) of X|^2,
//
// channel 3 (pressure) divided by rho vp like the closure's input.  Gradients are
// exact for the network as evaluated (bfloat16 weights and hidden activations,
// float accumulation); Adam updates float master weights, and each update is
// rounded to bfloat16 again for the next forward pass.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/acoustic3d.h"
#include "a3d_closure_dev.cuh"
#include "a3d_kernels.cuh"

namespace a3d {

int fail(int code, const char *fmt, ...);

#define CL_TRY(x)                                                                      \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess)                                                         \
            return fail(A3D_E_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));      \
    } while (0)

constexpr int CL_CHUNK = 1024;          // face-box cells per block of the weight-gradient kernels
constexpr int CL_GT = 27 * CL_CH;       // their threads: one per (tap, hidden channel)

struct ClChunks {
    long long cstart[7];  // first block of face f
};

// ---------------------------------------------------------------------------
// student step: the engine's undamped update on the dense rim grid (ldz = nnz)

__device__ __forceinline__ bool updated(const ClGeom &g, long long n, int &z, int &x, int &y) {
    z = (int)(n % g.nn[0]);
    x = (int)((n / g.nn[0]) % g.nn[1]);
    y = (int)(n / ((long long)g.nn[0] * g.nn[1]));
    return z >= MM && z < g.nn[0] - MM && x >= MM && x < g.nn[1] - MM && y >= MM && y < g.nn[2] - MM;
}

// u, v, w <- u, v, w - dt/d * (D+ P) / rho   (..iso..:99-142, undamped)
__global__ void cl_std_vel(const ClGeom g, const float *__restrict__ S0, long long fs, const float *__restrict__ rho,
                           float dtx, float dty, float dtz, float *__restrict__ X) {
    const float k[4] = {C8_0, C8_1, C8_2, C8_3};
    const float *P = S0 + 3 * fs;
    const long long sx = g.ldz, sy = g.ldz * g.nn[1];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < fs; n += (long long)gridDim.x * blockDim.x) {
        int z, x, y;
        if (!updated(g, n, z, x, y)) {
            X[n] = X[fs + n] = X[2 * fs + n] = 0.0f;
            continue;
        }
        float ax = 0.0f, ay = 0.0f, az = 0.0f;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            ax = fmaf(k[m], P[n + (m + 1) * sx] - P[n - m * sx], ax);
            ay = fmaf(k[m], P[n + (m + 1) * sy] - P[n - m * sy], ay);
            az = fmaf(k[m], P[n + (m + 1)] - P[n - m], az);
        }
        const float ri = 1.0f / rho[n];
        X[n] = S0[n] - dtx * (ax * ri);
        X[fs + n] = S0[fs + n] - dty * (ay * ri);
        X[2 * fs + n] = S0[2 * fs + n] - dtz * (az * ri);
    }
}

// P <- P - rho vp^2 dt (D-u/dx + D-v/dy + D-w/dz)   (..iso..:145-190, undamped)
__global__ void cl_std_str(const ClGeom g, const float *__restrict__ S0, long long fs, const float *__restrict__ rho,
                           const float *__restrict__ vp, float dtx, float dty, float dtz, float *__restrict__ X) {
    const float k[4] = {C8_0, C8_1, C8_2, C8_3};
    const float *U = X, *V = X + fs, *W = X + 2 * fs, *P0 = S0 + 3 * fs;
    const long long sx = g.ldz, sy = g.ldz * g.nn[1];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < fs; n += (long long)gridDim.x * blockDim.x) {
        int z, x, y;
        if (!updated(g, n, z, x, y)) {
            X[3 * fs + n] = 0.0f;
            continue;
        }
        float ax = 0.0f, ay = 0.0f, az = 0.0f;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            ax = fmaf(k[m], U[n + m * sx] - U[n - (m + 1) * sx], ax);
            ay = fmaf(k[m], V[n + m * sy] - V[n - (m + 1) * sy], ay);
            az = fmaf(k[m], W[n + m] - W[n - (m + 1)], az);
        }
        const float t = (rho[n] * vp[n]) * vp[n];
        X[3 * fs + n] = ((P0[n] - (t * dtx) * ax) - (t * dty) * ay) - (t * dtz) * az;
    }
}

// ---------------------------------------------------------------------------
// loss normalisation: E = sum over rim cells of the balanced channels of X squared

__global__ void __launch_bounds__(CL_THREADS)
    cl_energy(const ClGeom g, const float *__restrict__ X, long long fs, const float *__restrict__ zinv,
              float *__restrict__ E) {
    float s = 0.0f;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.roff[6];
         n += (long long)gridDim.x * blockDim.x) {
        int c[3];
        rim_cell(g, n, c);
        const long long id = gidx(g, c[0], c[1], c[2]);
        const float p = X[3 * fs + id] * zinv[id];
        s = fmaf(X[id], X[id], s);
        s = fmaf(X[fs + id], X[fs + id], s);
        s = fmaf(X[2 * fs + id], X[2 * fs + id], s);
        s = fmaf(p, p, s);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(E, s);
}

__global__ void cl_inv(const float *__restrict__ E, float scale, float *__restrict__ inv) {
    inv[0] = E[0] > 0.0f ? scale / E[0] : 0.0f;
}

// ---------------------------------------------------------------------------
// output layer, loss, its gradient at the outputs (e_f = dL/dy_f) and dL/dG

constexpr size_t CL_OUT_SMEM = (size_t)(CL_NW2 + 2 * CL_NG + 1) * 4;

__global__ void __launch_bounds__(CL_THREADS)
    cl_train_out(const ClGeom g, const float *__restrict__ X, const float *__restrict__ T, long long fs,
                 const float *__restrict__ zinv, const float *__restrict__ W2c, const float *__restrict__ Gc,
                 const __nv_bfloat16 *__restrict__ h, const float *__restrict__ inv_norm, float4 *__restrict__ e,
                 float *__restrict__ gG, float *__restrict__ loss) {
    extern __shared__ __align__(16) float smem_cl[];
    float *sG = smem_cl + CL_NW2, *sdG = sG + CL_NG, *sloss = sdG + CL_NG;
    for (int i = threadIdx.x; i < CL_NW2; i += blockDim.x) smem_cl[i] = W2c[i];
    for (int i = threadIdx.x; i < CL_NG; i += blockDim.x) { sG[i] = Gc[i]; sdG[i] = 0.0f; }
    if (threadIdx.x == 0) *sloss = 0.0f;
    __syncthreads();
    const float4 *sW2 = reinterpret_cast<const float4 *>(smem_cl);
    const float inv = *inv_norm;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.roff[6];
         n += (long long)gridDim.x * blockDim.x) {
        int c[3];
        rim_cell(g, n, c);
        float y[3][4];
        int ff[3], aa[3], nf = 0;
        float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 1
        for (int A = 0; A < 3; ++A) {
            int a;
            const int f = rim_face(g, A, c[A], a);
            if (f < 0) continue;
            face_out(g, f, c, sW2, h, y[nf]);
            const float *gg = sG + (f * CL_RIM + a - 1) * CL_COUT;
#pragma unroll
            for (int o = 0; o < 4; ++o) d[o] = fmaf(gg[o], y[nf][o], d[o]);
            ff[nf] = f;
            aa[nf] = a;
            ++nf;
        }
        const long long id = gidx(g, c[0], c[1], c[2]);
        const float zi = zinv[id];
        const float tg[4] = {T[id] - X[id], T[fs + id] - X[fs + id], T[2 * fs + id] - X[2 * fs + id],
                             (T[3 * fs + id] - X[3 * fs + id]) * zi};
        float gd[4], l = 0.0f;
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            const float r = d[o] - tg[o];
            l = fmaf(r, r, l);
            gd[o] = 2.0f * r * inv;
        }
        atomicAdd(sloss, l * inv);
        for (int k = 0; k < nf; ++k) {
            const int f = ff[k];
            const float *gg = sG + (f * CL_RIM + aa[k] - 1) * CL_COUT;
            const long long lin = face_lin(g, f, c[0], c[1], c[2]);
            e[g.hoff[f] + lin] = make_float4(gd[0] * gg[0], gd[1] * gg[1], gd[2] * gg[2], gd[3] * gg[3]);
            float *dg = sdG + (f * CL_RIM + aa[k] - 1) * CL_COUT;
#pragma unroll
            for (int o = 0; o < 4; ++o) atomicAdd(dg + o, gd[o] * y[k][o]);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < CL_NG; i += blockDim.x) atomicAdd(gG + i, sdG[i]);
    if (threadIdx.x == 0) atomicAdd(loss, *sloss);
}

// dL/dz of the hidden layer on every face-box cell: (W2_f^T * e_f) masked by relu
__global__ void __launch_bounds__(CL_THREADS)
    cl_train_dh(const ClGeom g, const float *__restrict__ W2c, const float4 *__restrict__ e,
                const __nv_bfloat16 *__restrict__ h, float *__restrict__ dz) {
    extern __shared__ __align__(16) float smem_cl[];
    for (int i = threadIdx.x; i < CL_NW2; i += blockDim.x) smem_cl[i] = W2c[i];
    __syncthreads();
    const float4 *sW2 = reinterpret_cast<const float4 *>(smem_cl);
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.hoff[6];
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
            const int dzz = t % 3 - 1, dx = (t / 3) % 3 - 1, dy = t / 9 - 1;
            const long long lin = face_lin(g, f, c[0] - dzz, c[1] - dx, c[2] - dy);
            if (lin < 0) continue;
            const float4 ev = e[g.hoff[f] + lin];
            const float4 *ws = sW2 + (f * 27 + t) * CL_CH;
#pragma unroll
            for (int j = 0; j < CL_CH; ++j) {
                const float4 wv = ws[j];
                acc[j] = fmaf(wv.x, ev.x, acc[j]);
                acc[j] = fmaf(wv.y, ev.y, acc[j]);
                acc[j] = fmaf(wv.z, ev.z, acc[j]);
                acc[j] = fmaf(wv.w, ev.w, acc[j]);
            }
        }
        const uint4 *hp = reinterpret_cast<const uint4 *>(h + n * CL_CH);
        float4 *dp = reinterpret_cast<float4 *>(dz + n * CL_CH);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float hv[8];
            unpack8(hp[q], hv);
            dp[2 * q] = make_float4(hv[0] > 0.0f ? acc[8 * q] : 0.0f, hv[1] > 0.0f ? acc[8 * q + 1] : 0.0f,
                                    hv[2] > 0.0f ? acc[8 * q + 2] : 0.0f, hv[3] > 0.0f ? acc[8 * q + 3] : 0.0f);
            dp[2 * q + 1] = make_float4(hv[4] > 0.0f ? acc[8 * q + 4] : 0.0f, hv[5] > 0.0f ? acc[8 * q + 5] : 0.0f,
                                        hv[6] > 0.0f ? acc[8 * q + 6] : 0.0f, hv[7] > 0.0f ? acc[8 * q + 7] : 0.0f);
        }
    }
}

__device__ __forceinline__ void chunk_range(const ClGeom &g, const ClChunks &ch, int &f, long long &n0,
                                            long long &n1) {
    const long long b = blockIdx.x;
    f = 0;
    while (f < 5 && b >= ch.cstart[f + 1]) ++f;
    n0 = g.hoff[f] + (b - ch.cstart[f]) * CL_CHUNK;
    n1 = n0 + CL_CHUNK < g.hoff[f + 1] ? n0 + CL_CHUNK : g.hoff[f + 1];
}

// dL/dW2_f[o][j][tap] = sum over rim cells c of face f of e_f(c)[o] h_f(c + tap)[j]
__global__ void __launch_bounds__(CL_GT)
    cl_train_dw2(const ClGeom g, const ClChunks ch, const float4 *__restrict__ e,
                 const __nv_bfloat16 *__restrict__ h, float *__restrict__ gW2) {
    const int j = threadIdx.x & 31, t = threadIdx.x >> 5;
    const int dzz = t % 3 - 1, dx = (t / 3) % 3 - 1, dy = t / 9 - 1;
    int f;
    long long n0, n1;
    chunk_range(g, ch, f, n0, n1);
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (long long n = n0; n < n1; ++n) {
        int c[3], a;
        face_cell(g, f, n - g.hoff[f], c, a);
        if (a == 0) continue;
        const long long lin = face_lin(g, f, c[0] + dzz, c[1] + dx, c[2] + dy);
        if (lin < 0) continue;
        const float4 ev = e[n];
        const float hv = __bfloat162float(h[(g.hoff[f] + lin) * CL_CH + j]);
        acc[0] = fmaf(ev.x, hv, acc[0]);
        acc[1] = fmaf(ev.y, hv, acc[1]);
        acc[2] = fmaf(ev.z, hv, acc[2]);
        acc[3] = fmaf(ev.w, hv, acc[3]);
    }
#pragma unroll
    for (int o = 0; o < 4; ++o) atomicAdd(gW2 + ((f * CL_COUT + o) * CL_CH + j) * 27 + t, acc[o]);
}

// dL/dW1[j][i][tap] = sum over faces f and face-box cells c of dz_f(c)[j] x_i(c + tap)
__global__ void __launch_bounds__(CL_GT)
    cl_train_dw1(const ClGeom g, const ClChunks ch, const float *__restrict__ X, long long fs,
                 const float *__restrict__ zinv, const float *__restrict__ kap, const float *__restrict__ dz,
                 float *__restrict__ gW1) {
    const int j = threadIdx.x & 31, t = threadIdx.x >> 5;
    const int dzz = t % 3 - 1, dx = (t / 3) % 3 - 1, dy = t / 9 - 1;
    int f;
    long long n0, n1;
    chunk_range(g, ch, f, n0, n1);
    float acc[CL_CIN];
#pragma unroll
    for (int i = 0; i < CL_CIN; ++i) acc[i] = 0.0f;
    for (long long n = n0; n < n1; ++n) {
        int c[3], a;
        face_cell(g, f, n - g.hoff[f], c, a);
        const float d = dz[n * CL_CH + j];
        float x[8];
        load_x(X, X + fs, X + 2 * fs, X + 3 * fs, zinv, kap, gidx(g, c[0] + dzz, c[1] + dx, c[2] + dy), x);
#pragma unroll
        for (int i = 0; i < CL_CIN; ++i) acc[i] = fmaf(d, x[i], acc[i]);
    }
#pragma unroll
    for (int i = 0; i < CL_CIN; ++i) atomicAdd(gW1 + (j * CL_CIN + i) * 27 + t, acc[i]);
}

// ---------------------------------------------------------------------------
// Adam on the float master weights; each updated weight is packed, rounded to
// bfloat16, into the kernels' layout

__device__ __forceinline__ int packed_index(int i) {
    if (i < CL_NW1) {
        const int j = i / (CL_CIN * 27), r = i % (CL_CIN * 27), ii = r / 27, t = r % 27;
        return (t * CL_CIN + ii) * CL_CH + j;
    }
    if (i < CL_NW1 + CL_NW2) {
        const int k = i - CL_NW1, f = k / (CL_COUT * CL_CH * 27), r = k % (CL_COUT * CL_CH * 27);
        const int o = r / (CL_CH * 27), r2 = r % (CL_CH * 27), j = r2 / 27, t = r2 % 27;
        return CL_NW1 + ((f * 27 + t) * CL_CH + j) * CL_COUT + o;
    }
    return i;
}

__global__ void cl_adam(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                        float *__restrict__ v, float *__restrict__ packed, float lr, float b1, float b2, float c1,
                        float c2, float eps, float decay) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= CL_NPARAM) return;
    if (i < CL_NW1 + CL_NW2) p[i] -= lr * decay * p[i];  // decoupled weight decay of the conv kernels
    const float gi = gr[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    packed[packed_index(i)] = __bfloat162float(__float2bfloat16_rn(pi));
}

static int grid_for(long long n) {
    const long long b = (n + CL_THREADS - 1) / CL_THREADS;
    return (int)std::max(1LL, std::min<long long>(b, 152 * 16));
}

}  // namespace a3d

using namespace a3d;

// ---------------------------------------------------------------------------
// training object

struct a3d_closure {
    int device = 0;
    int nx = 0, ny = 0, nz = 0;
    ClGeom g{};
    ClChunks ch{};
    long long nblk = 0;          // blocks of the weight-gradient kernels
    long long cells = 0;         // cells of the dense rim grid
    cudaStream_t st = nullptr;
    std::vector<void *> allocs;
    float *params = nullptr, *packed = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    float *scal = nullptr;       // [0] E, [1] 1/E scaled, [2] loss
    __nv_bfloat16 *h = nullptr;
    float4 *e = nullptr;
    float *dz = nullptr, *dout = nullptr;
    uint16_t *image = nullptr;   // tensor-core weight images (eval_tc)
    float4 *ybuf = nullptr;
    int *errw = nullptr;
    float *stage = nullptr;      // staging buffer for teacher taps
    long long stage_states = 0;
    long long step = 0;
    float decay = 0.0f;          // decoupled weight decay of W1, W2 per unit learning rate
    struct Model { float *rho, *vp, *zinv, *kap; float dtx, dty, dtz; };
    std::vector<Model> models;
    struct Sample { int model; float *X, *T; };
    std::vector<Sample> samples;

    void *dalloc(size_t bytes) {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, bytes) != cudaSuccess) { cudaFree(p); return nullptr; }
        allocs.push_back(p);
        return p;
    }
    ~a3d_closure() {
        if (device >= 0) cudaSetDevice(device);
        for (void *p : allocs) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
    int run_sample(const Sample &s, float scale);
};

int a3d_closure::run_sample(const Sample &s, float scale) {
    const Model &md = models[s.model];
    const long long fs = cells;
    CL_TRY(cudaMemsetAsync(scal, 0, sizeof(float), st));
    cl_energy<<<grid_for(g.roff[6]), CL_THREADS, 0, st>>>(g, s.X, fs, md.zinv, scal);
    cl_inv<<<1, 1, 0, st>>>(scal, scale, scal + 1);
    CL_TRY(cl_launch_hidden(g, s.X, s.X + fs, s.X + 2 * fs, s.X + 3 * fs, md.zinv, md.kap, packed, h, st));
    CL_TRY(cudaMemsetAsync(e, 0, (size_t)g.hoff[6] * sizeof(float4), st));
    cl_train_out<<<grid_for(g.roff[6]), CL_THREADS, CL_OUT_SMEM, st>>>(
        g, s.X, s.T, fs, md.zinv, packed + CL_NW1, packed + CL_NW1 + CL_NW2, h, scal + 1, e,
        grad + CL_NW1 + CL_NW2, scal + 2);
    cl_train_dh<<<grid_for(g.hoff[6]), CL_THREADS, (size_t)CL_NW2 * 4, st>>>(g, packed + CL_NW1, e, h, dz);
    cl_train_dw2<<<(unsigned)nblk, CL_GT, 0, st>>>(g, ch, e, h, grad + CL_NW1);
    cl_train_dw1<<<(unsigned)nblk, CL_GT, 0, st>>>(g, ch, s.X, fs, md.zinv, md.kap, dz, grad);
    CL_TRY(cudaGetLastError());
    return A3D_OK;
}

extern "C" {

int a3d_closure_create(a3d_closure **out, int nx, int ny, int nz, int device) {
    if (!out) return fail(A3D_E_ARG, "null output pointer");
    *out = nullptr;
    if (nx < 1 || ny < 1 || nz < 1) return fail(A3D_E_ARG, "grid %dx%dx%d must be positive", nx, ny, nz);
    CL_TRY(cudaSetDevice(device));
    a3d_closure *c = new a3d_closure();
    c->device = device;
    c->nx = nx; c->ny = ny; c->nz = nz;
    const int nnz = nz + 2 * CL_PAD, nnx = nx + 2 * CL_PAD, nny = ny + 2 * CL_PAD;
    c->g = cl_geom(nnz, nnx, nny, nnz);
    c->cells = (long long)nnz * nnx * nny;
    long long b = 0;
    for (int f = 0; f < 6; ++f) {
        c->ch.cstart[f] = b;
        b += (c->g.hoff[f + 1] - c->g.hoff[f] + CL_CHUNK - 1) / CL_CHUNK;
    }
    c->ch.cstart[6] = b;
    c->nblk = b;
    cudaError_t ce = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cl_prepare();
    if (ce == cudaSuccess)
        ce = cudaFuncSetAttribute(cl_train_out, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)CL_OUT_SMEM);
    if (ce == cudaSuccess)
        ce = cudaFuncSetAttribute(cl_train_dh, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(CL_NW2 * 4));
    if (ce != cudaSuccess) {
        delete c;
        return fail(A3D_E_CUDA, "closure set-up failed: %s", cudaGetErrorString(ce));
    }
    const size_t np = CL_NPARAM * sizeof(float);
    if (!(c->params = (float *)c->dalloc(np)) || !(c->packed = (float *)c->dalloc(np)) ||
        !(c->grad = (float *)c->dalloc(np)) || !(c->m = (float *)c->dalloc(np)) || !(c->v = (float *)c->dalloc(np)) ||
        !(c->scal = (float *)c->dalloc(4 * sizeof(float))) ||
        !(c->h = (__nv_bfloat16 *)c->dalloc((size_t)c->g.hoff[6] * CL_CH * 2)) ||
        !(c->e = (float4 *)c->dalloc((size_t)c->g.hoff[6] * sizeof(float4))) ||
        !(c->dz = (float *)c->dalloc((size_t)c->g.hoff[6] * CL_CH * 4))) {
        delete c;
        return fail(A3D_E_NOMEM, "device allocation failed");
    }
    *out = c;
    return A3D_OK;
}

int a3d_closure_destroy(a3d_closure *c) {
    delete c;
    return A3D_OK;
}

int a3d_closure_set_params(a3d_closure *c, const float *params, size_t n) {
    if (!c || !params) return fail(A3D_E_ARG, "null closure or parameters");
    if (n != (size_t)CL_NPARAM) return fail(A3D_E_ARG, "closure takes %d parameters, got %zu", CL_NPARAM, n);
    CL_TRY(cudaSetDevice(c->device));
    std::vector<float> pk(CL_NPARAM);
    cl_pack_params(params, pk.data());
    CL_TRY(cudaMemcpy(c->params, params, n * 4, cudaMemcpyHostToDevice));
    CL_TRY(cudaMemcpy(c->packed, pk.data(), n * 4, cudaMemcpyHostToDevice));
    CL_TRY(cudaMemset(c->m, 0, n * 4));
    CL_TRY(cudaMemset(c->v, 0, n * 4));
    c->step = 0;
    return A3D_OK;
}

int a3d_closure_get_params(const a3d_closure *c, float *params, size_t n) {
    if (!c || !params) return fail(A3D_E_ARG, "null closure or parameters");
    if (n != (size_t)CL_NPARAM) return fail(A3D_E_ARG, "closure takes %d parameters, got %zu", CL_NPARAM, n);
    CL_TRY(cudaSetDevice(c->device));
    CL_TRY(cudaMemcpy(params, c->params, n * 4, cudaMemcpyDeviceToHost));
    return A3D_OK;
}

int a3d_closure_add_model(a3d_closure *c, const float *vel, const float *rho, float dx, float dy, float dz,
                          float dt, int *model) {
    if (!c || !vel || !rho) return fail(A3D_E_ARG, "null closure or model array");
    if (!(dx > 0) || !(dy > 0) || !(dz > 0) || !(dt > 0)) return fail(A3D_E_ARG, "dx, dy, dz and dt must be positive");
    CL_TRY(cudaSetDevice(c->device));
    const int nnz = c->g.nn[0], nnx = c->g.nn[1], nny = c->g.nn[2];
    std::vector<float> pr((size_t)c->cells), pv((size_t)c->cells);
    for (int y = 0; y < nny; ++y)
        for (int x = 0; x < nnx; ++x)
            for (int z = 0; z < nnz; ++z) {  // edge replication, as the engines pad their models
                const int mz = std::min(std::max(z - CL_PAD, 0), c->nz - 1);
                const int mx = std::min(std::max(x - CL_PAD, 0), c->nx - 1);
                const int my = std::min(std::max(y - CL_PAD, 0), c->ny - 1);
                const size_t src = mz + (size_t)c->nz * (mx + (size_t)c->nx * my);
                const size_t dst = z + (size_t)nnz * (x + (size_t)nnx * y);
                pr[dst] = rho[src];
                pv[dst] = vel[src];
            }
    a3d_closure::Model md{};
    const size_t b = (size_t)c->cells * 4;
    if (!(md.rho = (float *)c->dalloc(b)) || !(md.vp = (float *)c->dalloc(b)) || !(md.zinv = (float *)c->dalloc(b)) ||
        !(md.kap = (float *)c->dalloc(b)))
        return fail(A3D_E_NOMEM, "device allocation failed");
    CL_TRY(cudaMemcpy(md.rho, pr.data(), b, cudaMemcpyHostToDevice));
    CL_TRY(cudaMemcpy(md.vp, pv.data(), b, cudaMemcpyHostToDevice));
    CL_TRY(cl_launch_scales(md.rho, md.vp, dt / std::min(dx, std::min(dy, dz)), md.zinv, md.kap, (size_t)c->cells,
                            c->st));
    CL_TRY(cudaStreamSynchronize(c->st));
    md.dtx = dt / dx;
    md.dty = dt / dy;
    md.dtz = dt / dz;
    c->models.push_back(md);
    if (model) *model = (int)c->models.size() - 1;
    return A3D_OK;
}

int a3d_closure_add_sample(a3d_closure *c, int model, const float *state0_dev, const float *state1_dev) {
    if (!c || !state0_dev || !state1_dev) return fail(A3D_E_ARG, "null closure or state");
    if (model < 0 || model >= (int)c->models.size()) return fail(A3D_E_ARG, "no model %d", model);
    CL_TRY(cudaSetDevice(c->device));
    a3d_closure::Sample s{model, nullptr, nullptr};
    const size_t b = (size_t)c->cells * 4 * 4;
    if (!(s.X = (float *)c->dalloc(b)) || !(s.T = (float *)c->dalloc(b))) return fail(A3D_E_NOMEM, "device allocation failed");
    const a3d_closure::Model &md = c->models[model];
    cl_std_vel<<<grid_for(c->cells), CL_THREADS, 0, c->st>>>(c->g, state0_dev, c->cells, md.rho, md.dtx, md.dty,
                                                             md.dtz, s.X);
    cl_std_str<<<grid_for(c->cells), CL_THREADS, 0, c->st>>>(c->g, state0_dev, c->cells, md.rho, md.vp, md.dtx,
                                                             md.dty, md.dtz, s.X);
    CL_TRY(cudaGetLastError());
    CL_TRY(cudaMemcpyAsync(s.T, state1_dev, b, cudaMemcpyDeviceToDevice, c->st));
    // a state that has run away (closed-loop states of an unstable closure) is refused
    CL_TRY(cudaMemsetAsync(c->scal, 0, sizeof(float), c->st));
    cl_energy<<<grid_for(c->g.roff[6]), CL_THREADS, 0, c->st>>>(c->g, s.X, c->cells, md.zinv, c->scal);
    cl_energy<<<grid_for(c->g.roff[6]), CL_THREADS, 0, c->st>>>(c->g, s.T, c->cells, md.zinv, c->scal);
    float E = 0.0f;
    CL_TRY(cudaMemcpyAsync(&E, c->scal, sizeof(float), cudaMemcpyDeviceToHost, c->st));
    CL_TRY(cudaStreamSynchronize(c->st));
    if (!std::isfinite(E)) {
        for (float *q : {s.X, s.T}) {
            cudaFree(q);
            c->allocs.erase(std::find(c->allocs.begin(), c->allocs.end(), (void *)q));
        }
        return fail(A3D_E_ARG, "teacher pair with a non-finite rim energy refused");
    }
    c->samples.push_back(s);
    return A3D_OK;
}

int a3d_closure_num_samples(const a3d_closure *c) { return c ? (int)c->samples.size() : 0; }

int a3d_closure_set_decay(a3d_closure *c, float decay) {
    if (!c || !(decay >= 0.0f)) return fail(A3D_E_ARG, "weight decay must be >= 0");
    c->decay = decay;
    return A3D_OK;
}

float *a3d_closure_staging(a3d_closure *c, int nstates) {
    if (!c || nstates < 1) {
        fail(A3D_E_ARG, "staging needs a closure and at least one state");
        return nullptr;
    }
    if (cudaSetDevice(c->device) != cudaSuccess) {
        fail(A3D_E_CUDA, "cudaSetDevice failed");
        return nullptr;
    }
    if (nstates > c->stage_states) {
        if (c->stage) {
            cudaFree(c->stage);
            c->allocs.erase(std::find(c->allocs.begin(), c->allocs.end(), (void *)c->stage));
            c->stage = nullptr;
            c->stage_states = 0;
        }
        c->stage = (float *)c->dalloc((size_t)nstates * 4 * (size_t)c->cells * sizeof(float));
        if (!c->stage) {
            fail(A3D_E_NOMEM, "device allocation failed");
            return nullptr;
        }
        c->stage_states = nstates;
    }
    return c->stage;
}

int a3d_closure_train(a3d_closure *c, int epochs, int batch, float lr, unsigned long long seed,
                      float *loss_per_epoch) {
    if (!c) return fail(A3D_E_ARG, "null closure");
    const int ns = (int)c->samples.size();
    if (ns < 1 || epochs < 1 || batch < 1 || !(lr > 0)) return fail(A3D_E_ARG, "training needs samples, epochs, batch and lr > 0");
    CL_TRY(cudaSetDevice(c->device));
    std::mt19937_64 rng(seed);
    std::vector<int> order(ns);
    for (int i = 0; i < ns; ++i) order[i] = i;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        CL_TRY(cudaMemsetAsync(c->scal + 2, 0, sizeof(float), c->st));
        int nb = 0;
        for (int b0 = 0; b0 < ns; b0 += batch, ++nb) {
            const int bn = std::min(batch, ns - b0);
            CL_TRY(cudaMemsetAsync(c->grad, 0, CL_NPARAM * sizeof(float), c->st));
            for (int k = 0; k < bn; ++k) {
                const int r = c->run_sample(c->samples[order[b0 + k]], 1.0f / (float)bn);
                if (r) return r;
            }
            ++c->step;
            const float c1 = 1.0f - (float)std::pow((double)b1, (double)c->step);
            const float c2 = 1.0f - (float)std::pow((double)b2, (double)c->step);
            cl_adam<<<(CL_NPARAM + 255) / 256, 256, 0, c->st>>>(c->params, c->grad, c->m, c->v, c->packed, lr, b1,
                                                                 b2, c1, c2, eps, c->decay);
            CL_TRY(cudaGetLastError());
        }
        float lsum = 0.0f;
        CL_TRY(cudaMemcpyAsync(&lsum, c->scal + 2, sizeof(float), cudaMemcpyDeviceToHost, c->st));
        CL_TRY(cudaStreamSynchronize(c->st));
        if (loss_per_epoch) loss_per_epoch[ep] = lsum / (float)nb;
    }
    return A3D_OK;
}

int a3d_closure_eval(a3d_closure *c, int sample, float *delta_host, float *grad_host, float *loss) {
    if (!c) return fail(A3D_E_ARG, "null closure");
    if (sample < 0 || sample >= (int)c->samples.size()) return fail(A3D_E_ARG, "no sample %d", sample);
    CL_TRY(cudaSetDevice(c->device));
    const a3d_closure::Sample &s = c->samples[sample];
    const a3d_closure::Model &md = c->models[s.model];
    const long long fs = c->cells;
    if (delta_host) {
        if (!c->dout && !(c->dout = (float *)c->dalloc((size_t)fs * 4 * 4))) return fail(A3D_E_NOMEM, "device allocation failed");
        CL_TRY(cudaMemsetAsync(c->dout, 0, (size_t)fs * 4 * 4, c->st));
        CL_TRY(cl_launch_hidden(c->g, s.X, s.X + fs, s.X + 2 * fs, s.X + 3 * fs, md.zinv, md.kap, c->packed, c->h, c->st));
        CL_TRY(cl_launch_correct(c->g, s.X, s.X + fs, s.X + 2 * fs, s.X + 3 * fs, md.zinv, c->packed, c->h, c->dout, fs,
                                 c->st));
        CL_TRY(cudaMemcpyAsync(delta_host, c->dout, (size_t)fs * 4 * 4, cudaMemcpyDeviceToHost, c->st));
    }
    if (grad_host || loss) {
        CL_TRY(cudaMemsetAsync(c->grad, 0, CL_NPARAM * sizeof(float), c->st));
        CL_TRY(cudaMemsetAsync(c->scal + 2, 0, sizeof(float), c->st));
        const int r = c->run_sample(s, 1.0f);
        if (r) return r;
        if (grad_host) CL_TRY(cudaMemcpyAsync(grad_host, c->grad, CL_NPARAM * 4, cudaMemcpyDeviceToHost, c->st));
        if (loss) CL_TRY(cudaMemcpyAsync(loss, c->scal + 2, sizeof(float), cudaMemcpyDeviceToHost, c->st));
    }
    CL_TRY(cudaStreamSynchronize(c->st));
    return A3D_OK;
}

int a3d_closure_eval_tc(a3d_closure *c, int sample, float *delta_host) {
    if (!c || !delta_host) return fail(A3D_E_ARG, "null closure or output");
    if (sample < 0 || sample >= (int)c->samples.size()) return fail(A3D_E_ARG, "no sample %d", sample);
    CL_TRY(cudaSetDevice(c->device));
    const a3d_closure::Sample &s = c->samples[sample];
    const a3d_closure::Model &md = c->models[s.model];
    const long long fs = c->cells;
    if (!c->image) {
        c->image = (uint16_t *)c->dalloc(cl_tc_image_halves() * sizeof(uint16_t));
        c->ybuf = (float4 *)c->dalloc((size_t)c->g.hoff[6] * sizeof(float4));
        c->errw = (int *)c->dalloc(sizeof(int));
        if (!c->image || !c->ybuf || !c->errw) return fail(A3D_E_NOMEM, "device allocation failed");
        CL_TRY(cl_tc_prepare());
    }
    if (!c->dout && !(c->dout = (float *)c->dalloc((size_t)fs * 4 * 4))) return fail(A3D_E_NOMEM, "device allocation failed");
    std::vector<float> p(CL_NPARAM);
    std::vector<uint16_t> img(cl_tc_image_halves());
    CL_TRY(cudaMemcpy(p.data(), c->params, CL_NPARAM * 4, cudaMemcpyDeviceToHost));
    cl_pack_tc(p.data(), img.data());
    CL_TRY(cudaMemcpyAsync(c->image, img.data(), img.size() * 2, cudaMemcpyHostToDevice, c->st));
    CL_TRY(cudaMemsetAsync(c->dout, 0, (size_t)fs * 4 * 4, c->st));
    CL_TRY(cudaMemsetAsync(c->errw, 0, sizeof(int), c->st));
    int nsm = 0;
    CL_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    CL_TRY(cl_launch_apply_tc(c->g, s.X, s.X + fs, s.X + 2 * fs, s.X + 3 * fs, md.zinv, md.kap, c->image,
                              c->packed + CL_NW1 + CL_NW2, c->ybuf, c->errw, c->dout, fs, nsm, c->st));
    int herr = 0;
    CL_TRY(cudaMemcpyAsync(&herr, c->errw, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CL_TRY(cudaMemcpyAsync(delta_host, c->dout, (size_t)fs * 4 * 4, cudaMemcpyDeviceToHost, c->st));
    CL_TRY(cudaStreamSynchronize(c->st));
    if (herr) return fail(A3D_E_KERNEL, "the tensor-core closure gave up a bounded wait (code %d)", herr);
    return A3D_OK;
}

int a3d_closure_teacher(const a3d_closure *c, int sample, float *x_host, float *t_host) {
    if (!c) return fail(A3D_E_ARG, "null closure");
    if (sample < 0 || sample >= (int)c->samples.size()) return fail(A3D_E_ARG, "no sample %d", sample);
    CL_TRY(cudaSetDevice(c->device));
    const a3d_closure::Sample &s = c->samples[sample];
    const size_t b = (size_t)c->cells * 4 * 4;
    if (x_host) CL_TRY(cudaMemcpy(x_host, s.X, b, cudaMemcpyDeviceToHost));
    if (t_host) CL_TRY(cudaMemcpy(t_host, s.T, b, cudaMemcpyDeviceToHost));
    return A3D_OK;
}

}  // extern "C"
