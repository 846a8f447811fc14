/*
 * a3d_oracle.c — CPU restatement of the reference forward-modelling engines.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle the CUDA engines are tested against (tests,
 * smoke check, CPU-baseline leg of the benchmark).  The product path never uses it.
 *
 * Setup pieces (padding, wavelets, PML profiles, direct-wave mute) live here and
 * are shared by both precisions; the time loops are in a3d_oracle_loops.inc,
 * which this file includes twice (REAL = float, REAL = double).
 *
 * Every function cites the reference code it restates (paths relative to the
 * reference project):
 *   2O  = src/Toa_3dfd_cuda.cu
 *   ISO = src/Toa_gpu_3diso_fd_1orderfunciton.cu
 *   VTI = src/Toa_gpu_3dvti_fd_1orderfunciton.cu
 *   TTI = src/Toa_gpu_3dtti_fd_1orderfunciton.cu
 *
 * Build with -ffp-contract=off: every fused multiply-add is written out with
 * fmaf()/fma() where the reference's nvcc build contracts one, so the results
 * do not depend on the host compiler's contraction choices.
 */
#include "a3d_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MM 4                       /* stencil half-width (2O:18, ISO:33)        */
#define PI_REF 3.141592653         /* the reference's pi/PI macro (2O:14, ISO:28) */

/* 8th-order staggered first-derivative coefficients, ISO:37 / VTI:40 / TTI:17. */
static const float C8[MM] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};
/* 8th-order second-derivative coefficients, 2O:32. */
static const float S8[MM + 1] = {(float)(-205.0 / 72.0), (float)(8.0 / 5.0), (float)(-1.0 / 5.0),
                                 (float)(8.0 / 315.0), (float)(-1.0 / 560.0)};

/* ------------------------------------------------------------------------- */
/* float helpers used by the engine form (and by the CUDA kernels, bit for bit) */

/* Knuth two-sum: s + e == a + b exactly. */
static inline void two_sum(float a, float b, float *s, float *e) {
    float x = a + b;
    float bv = x - a;
    float av = x - bv;
    *e = (a - av) + (b - bv);
    *s = x;
}

/* (float)((2.0*cur - prev) + (double)m) evaluated with float operations only
 * (2O:295 computes it in double). */
static inline float upd2o_f(float cur, float prev, float m) {
    float s, e, t, f;
    two_sum(2.0f * cur, -prev, &s, &e);
    two_sum(s, m, &t, &f);
    return t + (f + e);
}

/* (float)(F * (double)v) for a double factor F = fhi + flo, float operations only
 * (the sponge multiply of 2O:139-151 and the SV-ball taper of VTI:163-166). */
static inline float mul_df(float v, float fhi, float flo) {
    float p = fhi * v;
    float err = fmaf(fhi, v, -p);
    return p + fmaf(flo, v, err);
}

/* x rounded to the nearest float16 value (ties to even, float16 subnormals,
 * overflow to infinity), returned as float: IEEE 754 binary16 rounding restated
 * on the float's bits, the conversion the CUDA engine's float16 stores make. */
static inline float round_f16(float x) {
    uint32_t b;
    memcpy(&b, &x, 4);
    const uint32_t sign = b & 0x80000000u, a = b & 0x7fffffffu;
    if (a > 0x7f800000u) return x;                       /* NaN */
    if (a >= 0x477ff000u) {                              /* |x| >= 65520: infinity */
        const uint32_t r = sign | 0x7f800000u;
        float f;
        memcpy(&f, &r, 4);
        return f;
    }
    if (a >= 0x38800000u) {                              /* normal float16: 10 fraction bits */
        const uint32_t r = ((a + 0xfffu + ((a >> 13) & 1u)) & ~0x1fffu) | sign;
        float f;
        memcpy(&f, &r, 4);
        return f;
    }
    const float q = nearbyintf(fabsf(x) * 16777216.0f) / 16777216.0f;  /* multiples of 2^-24 */
    return sign ? -q : q;
}

float a3d_oracle_round_f16(float x) { return round_f16(x); }

/* x rounded to the nearest bfloat16 value (ties to even; overflow to infinity),
 * returned as float: the conversion the CUDA engine's bfloat16 stores make. */
static inline float round_bf16(float x) {
    uint32_t b;
    memcpy(&b, &x, 4);
    if ((b & 0x7fffffffu) > 0x7f800000u) return x;      /* NaN */
    b = (b + 0x7fffu + ((b >> 16) & 1u)) & 0xffff0000u;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

float a3d_oracle_round_bf16(float x) { return round_bf16(x); }

/* x rounded to a 24-bit float: float's sign and exponent, 15 fraction bits (the low
 * 8 rounded off, ties to even; overflow to infinity) */
static inline float round_f24(float x) {
    uint32_t b;
    memcpy(&b, &x, 4);
    if ((b & 0x7fffffffu) > 0x7f800000u) return x;      /* NaN */
    b = (b + 0x7fu + ((b >> 8) & 1u)) & ~0xffu;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

float a3d_oracle_round_f24(float x) { return round_f24(x); }

/* a velocity as the FP16V engine stores it: float16 of scale * v, divided back
 * (scale and 1/scale are powers of two, so both products are exact) */
static inline float store_f16s(float v, float scale, float inv) { return round_f16(v * scale) * inv; }

/* ------------------------------------------------------------------------- */
/* setup pieces                                                               */

/* Ricker wavelet of the 2nd-order engine, 2O:34-43. */
float a3d_oracle_ricker2o(int it, float dt, float fm) {
    float a = (float)it * dt;
    double d = (double)a - 1.0 / (double)fm;
    float fa = fabsf((float)d);
    float tmp = (float)(PI_REF * (double)fm * (double)fa);
    tmp = tmp * tmp;
    return (float)((1.0 - 2.0 * (double)tmp) * (double)expf(-tmp));
}

/* Source wavelets of the 1st-order engines, ISO:60-87 (VTI:62-79 and TTI:39-56
 * carry the same expressions for wtype 1..3).  t is the float-accumulated time. */
float a3d_oracle_wavelet(int wtype, float t, float favg) {
    float tdelay = (float)(1.0 / (double)favg);
    float ts = t - tdelay;
    float x_, xx_, source = 0.0f;
    const double pi = PI_REF;
    if (wtype == 1) {
        x_ = favg * ts;
        xx_ = x_ * x_;
        source = (float)((1.0 - 2.0 * pi * pi * (double)xx_) * exp(-(pi * pi * (double)xx_)));
    } else if (wtype == 2) {
        x_ = (float)((double)((-4.0f) * favg * favg) * pi * pi / log(0.1));
        source = (float)((-2.0) * pi * pi * (double)ts * (double)expf(-x_ * ts * ts));
    } else if (wtype == 3) {
        x_ = (float)((double)((-1.0f) * favg * favg) * pi * pi / log(0.1));
        source = expf(-x_ * ts * ts);
    } else if (wtype == 4) {
        x_ = (float)(exp((double)(-favg * favg) * pi * pi * (double)ts * (double)ts) * (double)ts);
        source = -x_;
    } else if (wtype == 5) {
        x_ = (float)(-1.0 / (2.0 * (double)favg * (double)favg * pi * pi));
        x_ = (float)((double)x_ * exp((double)(-favg * favg) * pi * pi * (double)ts * (double)ts));
        source = x_;
    } else if (wtype == 6) {
        double den = (double)(4.0f * favg * favg * favg) * pi * pi * (double)sqrtf((float)pi);
        x_ = (float)(-erf((double)favg * pi * (double)ts) / den);
        source = x_;
    }
    return source;
}

/* PML strength d0, ISO:193-195 (VTI:206-208, TTI:204-206). */
float a3d_oracle_d0(const float *vp, int nnx, int nny, int nnz, int npml, float dx, float dy,
                    float dz) {
    float s = dx + dy;
    s = s + dz;
    double v = (double)vp[((long)nny * nnx * nnz) / 2];
    return (float)(10.0 * v * log(100000.0) / (2.0 * (double)npml * ((double)s / 3.0)));
}

/* PML profiles along one axis of n model cells, ISO:263-291 (VTI/TTI:282-310).
 * c1,c2 — velocity (half-cell) coefficients; a1,a2 — pressure (integer-cell). */
void a3d_oracle_pml(float dt, float d0, int n, int npml, float *c1, float *c2, float *a1,
                    float *a2) {
    const float dtd0 = dt * d0;
    for (int id = 0; id < n + 2 * npml; ++id) {
        if (id < npml) {
            double r = ((double)npml - 0.5 - (double)id) / (double)npml;
            double e = (double)dtd0 * (r * r);
            c1[id] = (float)(1.0 / (1.0 + e / 2.0));
            c2[id] = (float)((double)c1[id] * (1.0 - e / 2.0));
            double ra = ((double)(npml - id) * 1.0) / (double)npml;
            double ea = (double)dtd0 * (ra * ra);
            a1[id] = (float)(1.0 / (1.0 + ea / 2.0));
            a2[id] = (float)((double)a1[id] * (1.0 - ea / 2.0));
        } else if (id < npml + n) {
            c1[id] = c2[id] = a1[id] = a2[id] = 1.0f;
        } else {
            double r = (0.5 + (double)id - (double)n - (double)npml) / (double)npml;
            double e = (double)dtd0 * (r * r);
            c1[id] = (float)(1.0 / (1.0 + e / 2.0));
            c2[id] = (float)((double)c1[id] * (1.0 - e / 2.0));
            double ra = ((double)(id - n - npml) * 1.0) / (double)npml;
            double ea = (double)dtd0 * (ra * ra);
            a1[id] = (float)(1.0 / (1.0 + ea / 2.0));
            a2[id] = (float)((double)a1[id] * (1.0 - ea / 2.0));
        }
    }
}

/* First muted sample count of trace (ix,iy): samples it < mute_nt are zeroed.
 * ISO:337-345 (VTI/TTI:354-362, 2O:88-96).  v0 is the mute velocity. */
int a3d_oracle_mute_nt(int ix, int iy, int sx, int sy, int sz, float dx, float dy, float dz,
                       float dt, float fm, float v0) {
    float mx = dx * (float)abs(ix - sx);
    float my = dy * (float)abs(iy - sy);
    float mz = dz * (float)sz;
    float sum = mx * mx + my * my;
    sum = sum + mz * mz;
    float t0 = sqrtf(sum) / v0;
    int mu_t = (int)(2.0 / (double)(dt * fm));
    return (int)(t0 / dt) + mu_t + 60;
}

/* Edge-replicate padding of a model (z fastest, then x, then y) into a grid with
 * `pad` extra cells on every face.  The three sequential one-axis copies of
 * ISO:198-238 (and velocity_transform, 2O:300-347) compose to a clamp. */
static float *pad_model(const float *m, int nx, int ny, int nz, int pad) {
    const int nnx = nx + 2 * pad, nny = ny + 2 * pad, nnz = nz + 2 * pad;
    float *p = (float *)malloc(sizeof(float) * (size_t)nnx * nny * nnz);
    if (!p) return NULL;
    for (int iy = 0; iy < nny; ++iy) {
        int cy = iy - pad < 0 ? 0 : (iy - pad >= ny ? ny - 1 : iy - pad);
        for (int ix = 0; ix < nnx; ++ix) {
            int cx = ix - pad < 0 ? 0 : (ix - pad >= nx ? nx - 1 : ix - pad);
            const float *src = m + ((size_t)cy * nx + cx) * nz;
            float *dst = p + ((size_t)iy * nnx + ix) * nnz;
            for (int iz = 0; iz < nnz; ++iz) {
                int cz = iz - pad < 0 ? 0 : (iz - pad >= nz ? nz - 1 : iz - pad);
                dst[iz] = src[cz];
            }
        }
    }
    return p;
}

static int check_cfg(const a3d_oracle_cfg *c) {
    if (!c || c->nx < 1 || c->ny < 1 || c->nz < 1 || c->nt < 1 || c->npml < 1) return -1;
    if (c->sx < 0 || c->sx >= c->nx || c->sy < 0 || c->sy >= c->ny || c->sz < 0 ||
        c->sz >= c->nz)
        return -1;
    return 0;
}

static void set_threads(const a3d_oracle_cfg *c) {
#ifdef _OPENMP
    if (c->threads > 0) omp_set_num_threads(c->threads);
#else
    (void)c;
#endif
}

static int take_snap(const a3d_oracle_cfg *c, int it) {
    if (c->snap_every <= 0) return 0;
    if (c->snap_skip0 && it == 0) return 0;
    return it % c->snap_every == 0;
}

/* SV-suppression taper inside the source ball, VTI:154-175 (TTI:139-160):
 * returns the double factor that multiplies epsilon/delta, or -1.0 outside. */
static double sv_taper(int rx, int ry, int rz) {
    const int R = 15, r = 4;
    int d2 = rx * rx + ry * ry + rz * rz;
    if (d2 > R * R) return -1.0;
    if (d2 <= r * r) return 0.0;
    return 0.5 * (1 - cos(PI_REF * ((double)(sqrtf((float)d2) - (float)r) * 4.0 / (R * 3.0 - 1))));
}

/* ------------------------------------------------------------------------- */
/* time loops, float and double                                               */

#define REAL float
#define RFMA fmaf
#define SUF(name) name##_f32
#define IS_F32 1
#include "a3d_oracle_loops.inc"
#undef REAL
#undef RFMA
#undef SUF
#undef IS_F32

#define REAL double
#define RFMA fma
#define SUF(name) name##_f64
#define IS_F32 0
#include "a3d_oracle_loops.inc"
#undef REAL
#undef RFMA
#undef SUF
#undef IS_F32
