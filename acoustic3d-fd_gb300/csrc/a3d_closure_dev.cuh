// a3d_closure_dev.cuh — device helpers of the learned rim: face-box and rim-cell
// indexing, the input channels, bfloat16 unpacking, and one face's output layer.
#pragma once
#include <stdint.h>

#include "a3d_closure.h"

namespace a3d {

constexpr int CL_THREADS = 256;

__device__ __forceinline__ void face_axes(int f, int &A, int &t1a, int &t2a) {
    A = f >> 1;
    t1a = A == 0 ? 1 : 0;
    t2a = A == 2 ? 1 : 2;
}

// cell lin of face f's box -> global cell c and normal coordinate a (depth + 1).
// z faces run a fastest (a follows z), x and y faces run their z coordinate fastest.
__device__ __forceinline__ void face_cell(const ClGeom &g, int f, long long lin, int c[3], int &a) {
    int A, t1a, t2a;
    face_axes(f, A, t1a, t2a);
    const int T1 = g.T1[f];
    int t1, t2;
    if (A == 0) {
        a = (int)(lin % 7);
        const long long r = lin / 7;
        t1 = (int)(r % T1);
        t2 = (int)(r / T1);
    } else {
        t1 = (int)(lin % T1);
        const long long r = lin / T1;
        a = (int)(r % 7);
        t2 = (int)(r / 7);
    }
    c[A] = (f & 1) ? g.nn[A] - CL_PAD - 1 + a : CL_PAD - a;
    c[t1a] = 4 + t1;
    c[t2a] = 4 + t2;
}

// position of global cell c in face f's box, or -1 outside it
__device__ __forceinline__ long long face_lin(const ClGeom &g, int f, int c0, int c1, int c2) {
    const int c[3] = {c0, c1, c2};
    int A, t1a, t2a;
    face_axes(f, A, t1a, t2a);
    const int a = (f & 1) ? c[A] - (g.nn[A] - CL_PAD - 1) : CL_PAD - c[A];
    const int t1 = c[t1a] - 4, t2 = c[t2a] - 4;
    if (a < 0 || a >= 7 || t1 < 0 || t1 >= g.T1[f] || t2 < 0 || t2 >= g.T2[f]) return -1;
    return A == 0 ? a + 7LL * (t1 + (long long)g.T1[f] * t2) : t1 + (long long)g.T1[f] * (a + 7LL * t2);
}

// rim cell n (0 <= n < roff[6]) -> global cell
__device__ __forceinline__ void rim_cell(const ClGeom &g, long long n, int c[3]) {
    int b = 0;
    while (b < 5 && n >= g.roff[b + 1]) ++b;
    long long r = n - g.roff[b];
    c[0] = g.blo[b][0] + (int)(r % g.bext[b][0]);
    r /= g.bext[b][0];
    c[1] = g.blo[b][1] + (int)(r % g.bext[b][1]);
    c[2] = g.blo[b][2] + (int)(r / g.bext[b][1]);
}

// face of axis A holding cell coordinate x in its rim (-1 if none), with a = depth + 1
__device__ __forceinline__ int rim_face(const ClGeom &g, int A, int x, int &a) {
    if (x >= 4 && x < CL_PAD) { a = CL_PAD - x; return 2 * A; }
    if (x >= g.nn[A] - CL_PAD && x < g.nn[A] - 4) { a = x - (g.nn[A] - CL_PAD - 1); return 2 * A + 1; }
    return -1;
}

__device__ __forceinline__ long long gidx(const ClGeom &g, int z, int x, int y) {
    return (long long)z + g.ldz * ((long long)x + (long long)g.nn[1] * y);
}

// the eight input channels at one cell, rounded to bfloat16 (the network's input type)
__device__ __forceinline__ void load_x(const float *__restrict__ u, const float *__restrict__ v,
                                       const float *__restrict__ w, const float *__restrict__ P,
                                       const float *__restrict__ zinv, const float *__restrict__ kap,
                                       long long id, float x[8]) {
    x[0] = u[id];
    x[1] = v[id];
    x[2] = w[id];
    x[3] = P[id] * zinv[id];
    const float k = kap[id];
    x[4] = k * x[0];
    x[5] = k * x[1];
    x[6] = k * x[2];
    x[7] = k * x[3];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = __bfloat162float(__float2bfloat16_rn(x[i]));  // bfloat16 inputs
}

__device__ __forceinline__ void unpack8(const uint4 &q, float f[8]) {
    const uint32_t r[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        f[2 * k] = __uint_as_float(r[k] << 16);
        f[2 * k + 1] = __uint_as_float(r[k] & 0xFFFF0000u);
    }
}

// y_f = W2_f * h_f at rim cell c of face f (a = depth + 1)
__device__ __forceinline__ void face_out(const ClGeom &g, int f, const int c[3], const float4 *__restrict__ sW2,
                                         const __nv_bfloat16 *__restrict__ h, float y[4]) {
    y[0] = y[1] = y[2] = y[3] = 0.0f;
#pragma unroll 1
    for (int t = 0; t < 27; ++t) {
        const int dz = t % 3 - 1, dx = (t / 3) % 3 - 1, dy = t / 9 - 1;
        const long long lin = face_lin(g, f, c[0] + dz, c[1] + dx, c[2] + dy);
        if (lin < 0) continue;
        const uint4 *hp = reinterpret_cast<const uint4 *>(h + (g.hoff[f] + lin) * CL_CH);
        const float4 *ws = sW2 + (f * 27 + t) * CL_CH;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float hv[8];
            unpack8(hp[q], hv);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float4 wv = ws[8 * q + k];
                y[0] = fmaf(wv.x, hv[k], y[0]);
                y[1] = fmaf(wv.y, hv[k], y[1]);
                y[2] = fmaf(wv.z, hv[k], y[2]);
                y[3] = fmaf(wv.w, hv[k], y[3]);
            }
        }
    }
}

}  // namespace a3d
