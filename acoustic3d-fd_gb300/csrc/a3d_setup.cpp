// a3d_setup.cpp — host-side shot setup (see a3d_setup.h).
// Compiled with -ffp-contract=off so the double expressions round exactly as
// written, on x86 and aarch64 alike.
#include "a3d_setup.h"

#include <cmath>
#include <cstdlib>

namespace a3d {

static const double PI_REF = 3.141592653;  // the reference's pi / PI macro (2O:14, ISO:28)

float ricker2o(int it, float dt, float fm) {
    const float a = (float)it * dt;                    // it*dt in float
    const double d = (double)a - 1.0 / (double)fm;     // - 1.0/fm in double
    const float fa = fabsf((float)d);                  // fabsf takes a float
    float tmp = (float)(PI_REF * (double)fm * (double)fa);
    tmp = tmp * tmp;
    return (float)((1.0 - 2.0 * (double)tmp) * (double)expf(-tmp));
}

float wavelet1(int wtype, float t, float favg) {
    const float tdelay = (float)(1.0 / (double)favg);
    const float ts = t - tdelay;
    const double pi = PI_REF;
    float x_, xx_, source = 0.0f;
    switch (wtype) {
        case 1:  // Ricker
            x_ = favg * ts;
            xx_ = x_ * x_;
            source = (float)((1.0 - 2.0 * pi * pi * (double)xx_) * exp(-(pi * pi * (double)xx_)));
            break;
        case 2:  // derivative of Gaussian; exp of a float argument is expf on the device
            x_ = (float)((double)((-4.0f) * favg * favg) * pi * pi / log(0.1));
            source = (float)((-2.0) * pi * pi * (double)ts * (double)expf(-x_ * ts * ts));
            break;
        case 3:  // Gaussian
            x_ = (float)((double)((-1.0f) * favg * favg) * pi * pi / log(0.1));
            source = expf(-x_ * ts * ts);
            break;
        case 4:  // integral of Ricker
            x_ = (float)(exp((double)(-favg * favg) * pi * pi * (double)ts * (double)ts) * (double)ts);
            source = -x_;
            break;
        case 5:  // double integral of Ricker
            x_ = (float)(-1.0 / (2.0 * (double)favg * (double)favg * pi * pi));
            x_ = (float)((double)x_ * exp((double)(-favg * favg) * pi * pi * (double)ts * (double)ts));
            source = x_;
            break;
        case 6: {  // triple integral of Ricker
            const double den = (double)(4.0f * favg * favg * favg) * pi * pi * (double)sqrtf((float)pi);
            source = (float)(-erf((double)favg * pi * (double)ts) / den);
            break;
        }
        default:
            source = 0.0f;
    }
    return source;
}

float pml_d0(float vmid, int npml, float dx, float dy, float dz) {
    float s = dx + dy;
    s = s + dz;
    return (float)(10.0 * (double)vmid * log(100000.0) / (2.0 * (double)npml * ((double)s / 3.0)));
}

void pml_profile(float dt, float d0, int n, int npml, float *c1, float *c2, float *a1, float *a2) {
    const float dtd0 = dt * d0;
    for (int id = 0; id < n + 2 * npml; ++id) {
        if (id >= npml && id < npml + n) {
            c1[id] = c2[id] = a1[id] = a2[id] = 1.0f;
            continue;
        }
        double r, ra;
        if (id < npml) {
            r = ((double)npml - 0.5 - (double)id) / (double)npml;
            ra = ((double)(npml - id) * 1.0) / (double)npml;
        } else {
            r = (0.5 + (double)id - (double)n - (double)npml) / (double)npml;
            ra = ((double)(id - n - npml) * 1.0) / (double)npml;
        }
        const double e = (double)dtd0 * (r * r), ea = (double)dtd0 * (ra * ra);
        c1[id] = (float)(1.0 / (1.0 + e / 2.0));
        c2[id] = (float)((double)c1[id] * (1.0 - e / 2.0));
        a1[id] = (float)(1.0 / (1.0 + ea / 2.0));
        a2[id] = (float)((double)a1[id] * (1.0 - ea / 2.0));
    }
}

int mute_nt(int ix, int iy, int sx, int sy, int sz, float dx, float dy, float dz, float dt,
            float fm, float v0) {
    const float mx = dx * (float)std::abs(ix - sx);
    const float my = dy * (float)std::abs(iy - sy);
    const float mz = dz * (float)sz;
    float sum = mx * mx + my * my;
    sum = sum + mz * mz;
    const float t0 = sqrtf(sum) / v0;
    const int mu_t = (int)(2.0 / (double)(dt * fm));
    return (int)(t0 / dt) + mu_t + 60;
}

void sponge_factors(int n, int npd, float *hl) {
    const int mm = 4, nn = n + 2 * mm + 2 * npd;
    const float qp = -0.25f;
    for (int i = 0; i < nn; ++i) {
        double F = 0.0;
        if (i < npd) {
            const double r = (double)(npd - i) / (1.0 * npd);
            F = (double)qp * (r * r) + 1;
        } else if (i >= 2 * mm + npd + n) {
            const double r = (double)(i - 2 * mm - npd - n) / (1.0 * npd);
            F = (double)qp * (r * r) + 1;
        }
        const float hi = (float)F;
        hl[2 * i] = hi;
        hl[2 * i + 1] = (float)(F - (double)hi);
    }
}

void sv_taper_table(float *hl) {
    const int R = 15, r = 4;
    for (int d2 = 0; d2 <= R * R; ++d2) {
        double f = 0.0;
        if (d2 > r * r)
            f = 0.5 * (1 - cos(PI_REF * ((double)(sqrtf((float)d2) - (float)r) * 4.0 / (R * 3.0 - 1))));
        const float hi = (float)f;
        hl[2 * d2] = hi;
        hl[2 * d2 + 1] = (float)(f - (double)hi);
    }
}

}  // namespace a3d
