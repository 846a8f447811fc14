// a3d_engine.cu — engine object: model upload, tensor maps, the time loops of
// the four physics, and the in-memory C API (a3d_*).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <array>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "a3d_engine.h"

namespace a3d {

static thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    fprintf(stderr, "acoustic3d: %s\n", buf);
    return code;
}
void clear_error() { g_err.clear(); }

#define CUDA_TRY(x)                                                                    \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess)                                                         \
            return fail(A3D_E_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));      \
    } while (0)

static int g_sms = 0;
int plan_sweep(Sweep &sw, int occ, int mode) {
    const long long slots = (long long)(g_sms > 0 ? g_sms : 148) * (occ > 0 ? occ : 1);
    if (sw.nshot < 1) sw.nshot = 1;
    const long long ntiles = (long long)sw.ntz * sw.ntx * sw.nshot;
    sw.W = ntiles * sw.NY;
    sw.wave = 0;
    if (mode == 2) {  // wave: whole tile columns in waves of one CTA per slot (Sweep::wave)
        sw.Yc = sw.NY;
        sw.wave = 1;
        const long long g = sw.W / 16 > 1 ? sw.W / 16 : 1;
        return (int)(slots < g ? slots : g);
    }
    if (mode == 1) {  // fill: one full wave, chunk length from the nearest chunk count
        long long C = (slots + ntiles / 2) / ntiles;
        const long long cmax = sw.NY / 16 > 1 ? sw.NY / 16 : 1;
        C = C < 1 ? 1 : (C > cmax ? cmax : C);
        sw.Yc = (int)((sw.NY + C - 1) / C);
        return (int)(slots < sw.W / 16 ? slots : (sw.W / 16 > 0 ? sw.W / 16 : 1));
    }
    if (ntiles <= slots) {
        long long C = slots / ntiles;
        const long long cmax = sw.NY / 16 > 1 ? sw.NY / 16 : 1;
        if (C > cmax) C = cmax;
        sw.Yc = (int)((sw.NY + C - 1) / C);
        C = (sw.NY + sw.Yc - 1) / sw.Yc;
        return (int)(ntiles * C);
    }
    sw.Yc = sw.NY;
    return (int)slots;
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// 3-D map over a padded field: dims (nnz, nnx, nny), row stride ldz elements.
// dtype: 0 float, 1 bfloat16, 2 float16, 3 double.  A 2-byte field's base (the
// allocation + zoff elements) is only 8-byte aligned, so its map starts 4 elements
// earlier (16-byte aligned) and kernels add 4 to its z coordinates.
// With nshot > 1 the map is 4-D: nshot copies of the field, shot_bytes apart (the
// 4th coordinate selects the shot of a multi-shot sweep).
static int make_map(CUtensorMap *m, const void *base, int dtype, const Grid &g, int box0, int box1,
                    int nshot = 1, size_t shot_bytes = 0) {
    auto enc = encode_fn();
    if (!enc) return fail(A3D_E_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const size_t es = dtype == 3 ? 8 : (dtype == 0 ? 4 : 2);
    const int zs = es == 2 ? 4 : 0;
    const char *b = static_cast<const char *>(base) - zs * es;
    cuuint64_t dims[4] = {(cuuint64_t)(g.nnz + zs), (cuuint64_t)g.nnx, (cuuint64_t)g.nny, (cuuint64_t)nshot};
    cuuint64_t strides[3] = {(cuuint64_t)(g.ldz * es), (cuuint64_t)((size_t)g.ldz * g.nnx * es),
                             (cuuint64_t)shot_bytes};
    cuuint32_t box[4] = {(cuuint32_t)box0, (cuuint32_t)box1, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    const CUtensorMapDataType dt = dtype == 3   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                   : dtype == 1 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                   : dtype == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    CUresult r = enc(m, dt, nshot > 1 ? 4 : 3, const_cast<char *>(b), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(A3D_E_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return A3D_OK;
}

int make_field_map(CUtensorMap *m, const void *base, int dtype, const Grid &g, int box0, int box1) {
    return make_map(m, base, dtype, g, box0, box1);
}

// zhalo: width of z-halo'd boxes (40, or 48 for 2-byte storage: see ZHalo)
static int box_dims(int box, int tx, int &b0, int &b1, int zhalo = 40) {
    b0 = box == BOX_H2 ? 48 : ((box == BOX_HZ || box == BOX_H) ? zhalo : 32);
    b1 = box == BOX_H2 ? tx + 16 : ((box == BOX_HX || box == BOX_H) ? tx + 8 : tx);
    return 0;
}

// crop of the model window of a padded field into dense float [ny][nx][nz]
template <class S>
__global__ void crop_window(const S *f, float *out, int nx, int ny, int nz, int pad, int ldz,
                            int nnx, float scale) {
    const size_t n = (size_t)nx * ny * nz;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int iz = (int)(i % nz);
        const size_t r = i / nz;
        const int ix = (int)(r % nx), iy = (int)(r / nx);
        out[i] = (float)f[(size_t)(iz + pad) + (size_t)ldz * ((size_t)(ix + pad) + (size_t)nnx * (iy + pad))] * scale;
    }
}

}  // namespace a3d

using namespace a3d;

a3d_engine::~a3d_engine() {
    if (st) cudaStreamSynchronize(st);
    if (snap_st) cudaStreamSynchronize(snap_st);
    for (int k = 0; k < NSNAP; ++k) {
        if (snap_ring_host[k]) cudaFreeHost(snap_ring_host[k]);
        if (snap_cropped[k]) cudaEventDestroy(snap_cropped[k]);
        if (snap_copied[k]) cudaEventDestroy(snap_copied[k]);
    }
    if (snap_st) cudaStreamDestroy(snap_st);
    for (cudaEvent_t ev : kev) cudaEventDestroy(ev);
    for (void *p : allocs) cudaFree(p);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (st) cudaStreamDestroy(st);
}

void *a3d_engine::dalloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, bytes) != cudaSuccess) { cudaFree(p); return nullptr; }
    allocs.push_back(p);
    dev_bytes += bytes;
    return p;
}

void *a3d_engine::dfield(size_t es) {
    char *p = (char *)dalloc(g.elems() * es);
    return p ? p + Grid::zoff * es : nullptr;
}

void *a3d_engine::dfield_batch(bool pressure) {
    const size_t es = fsize(pressure);
    char *p = (char *)dalloc((pressure ? fstride_p : fstride) * es * nbatch);
    return p ? p + Grid::zoff * es : nullptr;
}

// edge-replicated padding of a model on the device: the reference's three one-axis
// copies (..iso..:198-260 pad_vv) compose to a clamp of each index into the model
// (zeros outside the field's cells); mode 1 stores 1 / value (0 where the value is 0),
// mode 2 (value * s)^2
__global__ void pad_field(const float *__restrict__ m, float *__restrict__ out, int nx, int ny, int nz, int pad,
                          int nnx, int nny, int nnz, int ldz, size_t elems, int mode, float sc) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < elems; i += (size_t)gridDim.x * blockDim.x) {
        float v = 0.0f;
        if (i >= (size_t)Grid::zoff) {
            const size_t f = i - Grid::zoff;
            const int iz = (int)(f % ldz);
            const size_t r = f / ldz;
            const int ix = (int)(r % nnx), iy = (int)(r / nnx);
            if (iz < nnz && iy < nny) {
                const int cz = min(max(iz - pad, 0), nz - 1), cx = min(max(ix - pad, 0), nx - 1),
                          cy = min(max(iy - pad, 0), ny - 1);
                v = m[(size_t)cz + (size_t)nz * ((size_t)cx + (size_t)nx * cy)];
                if (mode == 1) v = v != 0.0f ? 1.0f / v : 0.0f;
                else if (mode == 2) { const float t = v * sc; v = t * t; }
            }
        }
        out[i] = v;
    }
}

// upload a model (nx*ny*nz host floats) into a new padded field; raw: a device
// scratch buffer of the model's size; m == nullptr pads what raw already holds
static int upload_model(a3d_engine *e, const float *m, float **dst, float *raw, int mode = 0, float sc = 0.0f) {
    const Grid &g = e->g;
    *dst = (float *)e->dfield(4);
    if (!*dst) return fail(A3D_E_NOMEM, "device allocation of %zu bytes failed", e->field_bytes(4));
    if (m) {
        const int r = stage_to_device(raw, m, (size_t)g.nx * g.ny * g.nz * 4, e->st);
        if (r) return r;
    }
    pad_field<<<1024, 256>>>(raw, (float *)e->field_alloc(*dst, 4), g.nx, g.ny, g.nz, g.pad, g.nnx, g.nny, g.nnz,
                             g.ldz, g.elems(), mode, sc);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaDeviceSynchronize());
    return A3D_OK;
}

// out[i] = cosf(a[i]) (sine: sinf) for n values, split over the host's threads
static void host_trig(const float *a, float *out, size_t n, bool sine) {
    auto part = [=](size_t lo, size_t hi) {
        for (size_t i = lo; i < hi; ++i) out[i] = sine ? sinf(a[i]) : cosf(a[i]);
    };
    size_t nth = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), 32);
    nth = std::min(nth, n / 65536 + 1);
    std::vector<std::thread> ts;
    const size_t chunk = (n + nth - 1) / nth;
    size_t next = std::min(n, chunk);  // this thread takes [0, chunk); threads take the rest
    try {
        while (next < n) {
            const size_t hi = std::min(n, next + chunk);
            ts.emplace_back(part, next, hi);
            next = hi;
        }
    } catch (...) {  // a thread could not be started: this thread computes what is left
    }
    part(0, std::min(n, chunk));
    if (next < n) part(next, n);
    for (auto &t : ts) t.join();
}

static int engine_setup(a3d_engine *e, const float *vel, const float *rho, const float *eps,
                        const float *del, const float *theta, const float *phi) {
    const a3d_config &c = e->cfg;
    const Grid &g = e->g;
    std::vector<float> tmp;
    float *raw = nullptr;  // device scratch for one model array
    CUDA_TRY(cudaMalloc(&raw, (size_t)c.nx * c.ny * c.nz * 4));
    struct FreeRaw { float *p; ~FreeRaw() { cudaFree(p); } } free_raw{raw};
    // u, v, w (pressure = false) and P, Q, split components (pressure = true)
    auto field = [&](void **p, bool pressure = false) -> int {
        *p = e->nbatch > 1 ? e->dfield_batch(pressure) : e->dfield(e->fsize(pressure));
        return *p ? A3D_OK : fail(A3D_E_NOMEM, "device allocation of a %dx%dx%d field failed", g.nnz, g.nnx, g.nny);
    };
    int rc;
    e->rec = (float *)e->dalloc((size_t)c.nt * c.nx * c.ny * 4 * e->nbatch);
    e->d_mute = (int *)e->dalloc((size_t)c.nx * c.ny * 4 * e->nbatch);
    if (e->nbatch > 1) {  // shot cells far outside the grid until a run sets them
        std::vector<int4> far(e->nbatch, make_int4(-100, -100, -100, 0));
        e->d_shots = (int4 *)e->dalloc(far.size() * sizeof(int4));
        if (!e->d_shots) return fail(A3D_E_NOMEM, "device allocation failed");
        CUDA_TRY(cudaMemcpy(e->d_shots, far.data(), far.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    e->snap_dev = (float *)e->dalloc((size_t)c.nx * c.ny * c.nz * 4);
    if (!e->rec || !e->d_mute || !e->snap_dev) return fail(A3D_E_NOMEM, "record allocation failed");

    if (c.physics == A3D_2ORDER) {
        // vv = (v dt)^2 on the padded grid (Toa_3dfd_cuda.cu:300-347)
        if ((rc = upload_model(e, vel, &e->vv, raw, 2, c.dt))) return rc;
        e->v_mute = (size_t)c.nx * c.ny * c.nz > 1 ? vel[1] : vel[0];  // 2O:403
        if ((rc = field(&e->X)) || (rc = field(&e->Y))) return rc;
        // sponge factors per axis
        std::vector<float> hl;
        float2 **dst[3] = {&e->fz, &e->fx, &e->fy};
        const int n3[3] = {c.nz, c.nx, c.ny}, nn3[3] = {g.nnz, g.nnx, g.nny};
        for (int a = 0; a < 3; ++a) {
            hl.assign(2 * (size_t)nn3[a], 0.0f);
            sponge_factors(n3[a], e->npml, hl.data());
            *dst[a] = (float2 *)e->dalloc(hl.size() * 4);
            if (!*dst[a]) return fail(A3D_E_NOMEM, "device allocation failed");
            CUDA_TRY(cudaMemcpy(*dst[a], hl.data(), hl.size() * 4, cudaMemcpyHostToDevice));
        }
        e->w2o.resize(c.nt);
        for (int it = 0; it < c.nt; ++it) e->w2o[it] = ricker2o(it, c.dt, c.fm);
        const bool f64 = e->fp64;
        void *buf[2] = {e->X, e->Y};
        for (int t = 0; t < 2; ++t) {
            const int tx = t ? 16 : 8;
            for (int b = 0; b < 2; ++b) {
                if ((rc = make_map(&e->m2o_cur[t][b], buf[b], f64 ? 3 : 0, g, 40, tx + 8))) return rc;
                if ((rc = make_map(&e->m2o_prev[t][b], buf[b], f64 ? 3 : 0, g, 32, tx))) return rc;
            }
            if ((rc = make_map(&e->m2o_vv[t], e->vv, 0, g, 32, tx))) return rc;
        }
        return A3D_OK;
    }

    // 1st-order engines
    if ((rc = upload_model(e, vel, &e->vp, raw))) return rc;
    if (c.physics != A3D_TTI) {
        if ((rc = upload_model(e, rho, &e->rho, raw))) return rc;
        // the velocity sweeps multiply by 1/rho (float reciprocal) of the rho just uploaded
        if ((rc = upload_model(e, nullptr, &e->rinv, raw, 1))) return rc;
    }
    if (c.physics != A3D_ISO) {
        if ((rc = upload_model(e, eps, &e->eps, raw))) return rc;
        if ((rc = upload_model(e, del, &e->del, raw))) return rc;
    }
    if (c.physics == A3D_TTI) {
        // cos/sin of tilt and azimuth in float on the host (libm, as the oracle and
        // ..tti..:101-103 evaluate them), on the model cells over host threads, then
        // padded on the device like every model array: edge replication commutes
        // with a pointwise function, so every grid cell gets the value of cos / sin
        // of its padded angle
        tmp.resize((size_t)c.nx * c.ny * c.nz);
        float **dst[4] = {&e->tct, &e->tst, &e->tcp, &e->tsp};
        for (int k = 0; k < 4; ++k) {
            host_trig(k < 2 ? theta : phi, tmp.data(), tmp.size(), k % 2 == 1);
            if ((rc = upload_model(e, tmp.data(), dst[k], raw))) return rc;
        }
    }
    // mute velocity: the padded model's element 1, i.e. model cell (0,0,0) (..iso..:340)
    e->v_mute = vel[0];
    if (c.physics != A3D_ISO) e->v_mute = vel[0] * sqrtf(1.0f + 2.0f * eps[0]);  // ..vti..:357
    if ((rc = field(&e->u)) || (rc = field(&e->v)) || (rc = field(&e->w)) || (rc = field(&e->P, true)) ||
        (rc = field(&e->px, true)) || (rc = field(&e->py, true)) || (rc = field(&e->pz, true)))
        return rc;
    if (e->fused_ok && ((rc = field(&e->u2)) || (rc = field(&e->v2)) || (rc = field(&e->w2)) || (rc = field(&e->P2))))
        return rc;
    if (c.physics != A3D_ISO) {
        if ((rc = field(&e->Q, true)) || (rc = field(&e->qx, true)) || (rc = field(&e->qy, true)) ||
            (rc = field(&e->qz, true)))
            return rc;
    }
    // PML profiles (..iso..:193-195 and 263-291): d0 from the padded model's middle element
    const size_t mid = ((size_t)g.nny * g.nnx * g.nnz) / 2;  // flat index in the reference's dense layout
    const int miz = (int)(mid % g.nnz), mix = (int)((mid / g.nnz) % g.nnx), miy = (int)(mid / ((size_t)g.nnz * g.nnx));
    float vmid;
    {
        int cz = std::min(std::max(miz - g.pad, 0), c.nz - 1), cx = std::min(std::max(mix - g.pad, 0), c.nx - 1),
            cy = std::min(std::max(miy - g.pad, 0), c.ny - 1);
        vmid = vel[cz + (size_t)c.nz * (cx + (size_t)c.nx * cy)];
    }
    const float d0 = pml_d0(vmid, e->npml, c.dx, c.dy, c.dz);
    std::vector<float> pm(4 * (size_t)(g.nnx + g.nny + g.nnz));
    float *q = pm.data();
    const int n3[3] = {c.nx, c.ny, c.nz}, nn3[3] = {g.nnx, g.nny, g.nnz};
    for (int a = 0; a < 3; ++a) {
        if (e->learned)  // undamped rim: every coefficient 1, the closure absorbs
            std::fill(q, q + 4 * nn3[a], 1.0f);
        else
            pml_profile(c.dt, d0, n3[a], e->npml, q, q + nn3[a], q + 2 * nn3[a], q + 3 * nn3[a]);
        q += 4 * nn3[a];
    }
    {   // pressure-undamped interval of each axis (x, y, z)
        const float *qa = pm.data();
        for (int a = 0; a < 3; ++a) {
            const float *a1 = qa + 2 * nn3[a], *a2 = qa + 3 * nn3[a];
            int lo = nn3[a], hi = 0;
            for (int i = 0; i < nn3[a]; ++i)
                if (a1[i] == 1.0f && a2[i] == 1.0f) { lo = std::min(lo, i); hi = std::max(hi, i + 1); }
            for (int i = lo; i < hi; ++i)  // the interval must be contiguous
                if (!(a1[i] == 1.0f && a2[i] == 1.0f)) return fail(A3D_E_ARG, "PML profile not contiguous");
            e->ulo[a] = lo;
            e->uhi[a] = hi;
            qa += 4 * nn3[a];
        }
    }
    e->pml = (float *)e->dalloc(pm.size() * 4);
    if (!e->pml) return fail(A3D_E_NOMEM, "device allocation failed");
    CUDA_TRY(cudaMemcpy(e->pml, pm.data(), pm.size() * 4, cudaMemcpyHostToDevice));
    {
        float tb[2 * 226];
        sv_taper_table(tb);
        e->taper = (float2 *)e->dalloc(sizeof tb);
        if (!e->taper) return fail(A3D_E_NOMEM, "device allocation failed");
        CUDA_TRY(cudaMemcpy(e->taper, tb, sizeof tb, cudaMemcpyHostToDevice));
    }
    // injected amplitudes per step; t accumulates in float (..iso..:521)
    e->amp0.resize(c.nt);
    e->amp1.resize(c.nt);
    e->inj.resize(c.nt);
    const float tdelay = (float)(1.0 / (double)c.fm);
    float t = c.dt;
    for (int it = 0; it < c.nt; ++it, t += c.dt) {
        const float src = wavelet1(c.physics == A3D_ISO ? c.wtype : 1, t, c.fm);
        e->inj[it] = t <= 2.0f * tdelay;
        if (c.physics == A3D_ISO) {
            const float pfac = 10000.0f;  // ..iso..:407
            e->amp0[it] = -pfac * src;
            e->amp1[it] = pfac * src;
        } else {
            const float pfac = 10.0f;     // ..vti..:431, ..tti..:437
            e->amp0[it] = pfac * src;
            e->amp1[it] = pfac * src;
        }
    }
    // float16 storage scales (powers of two, so every rescaling is exact): P so that
    // the largest injected amplitude maps to 2^11 (headroom to the float16 maximum
    // 65504); u, v, w by the velocity-to-pressure ratio dx rho / dt on top of that
    // (rho = 1 for TTI, which has no density), so that both kinds of field sit in the
    // same part of the float16 range.  bfloat16 keeps float's exponent range and
    // needs no scaling.
    if (e->half == 2) {
        float amax = 0.0f;
        for (int it = 0; it < c.nt; ++it)
            if (e->inj[it]) amax = std::max(amax, std::max(std::fabs(e->amp0[it]), std::fabs(e->amp1[it])));
        double rsum = 0.0;
        const size_t n = (size_t)c.nx * c.ny * c.nz;
        for (size_t i = 0; i < n; ++i) rsum += rho ? rho[i] : 1.0f;
        const double rmean = rsum / (double)n;
        const double dmin = std::min(c.dx, std::min(c.dy, c.dz));
        if (amax > 0.0f) e->sig_p = std::ldexp(1.0f, (int)std::floor(std::log2(2048.0 / amax)));
        e->sig_v = e->sig_p * std::ldexp(1.0f, (int)std::lround(std::log2(dmin * rmean / c.dt)));
        if (e->pfloat) e->sig_p = 1.0f;  // float pressures: unscaled; u, v, w keep their range
    }
    // tensor maps for both tile widths
    const bool f64 = e->fp64;
    for (int t = 0; t < 2; ++t) {
    const int tx = t ? 16 : 8;
    CUtensorMap *mvel = e->mvel[t], *mstr = e->mstr[t];
    int b0, b1;
    // pressure fields (P, Q, split components) are float under A3D_FP16V
    auto mk = [&](CUtensorMap *m, const void *p, bool isfield, int box) {
        const bool pf = isfield && e->pfloat && (p == e->P || p == e->Q || p == e->px || p == e->py ||
                                                 p == e->pz || p == e->qx || p == e->qy || p == e->qz);
        const int dt = isfield ? (f64 ? 3 : (pf ? 0 : e->half)) : 0;
        box_dims(box, tx, b0, b1, dt == 1 || dt == 2 ? 48 : 40);
        if (isfield && e->nbatch > 1)  // every shot's copy of a wavefield: 4-D map
            return make_map(m, p, dt, g, b0, b1, e->nbatch,
                            pf ? e->fstride_p * e->esz_p : e->fstride * e->esz);
        return make_map(m, p, dt, g, b0, b1);
    };
    if (c.physics == A3D_ISO) {
        e->nvel = 5;
        if ((rc = mk(&mvel[0], e->P, true, BOX_H)) || (rc = mk(&mvel[1], e->u, true, BOX_CORE)) ||
            (rc = mk(&mvel[2], e->v, true, BOX_CORE)) || (rc = mk(&mvel[3], e->w, true, BOX_CORE)) ||
            (rc = mk(&mvel[4], e->rinv, false, BOX_CORE)))
            return rc;
        e->nstr = 9;
        if ((rc = mk(&mstr[0], e->v, true, BOX_CORE)) || (rc = mk(&mstr[1], e->u, true, BOX_HX)) ||
            (rc = mk(&mstr[2], e->w, true, BOX_HZ)) || (rc = mk(&mstr[3], e->P, true, BOX_CORE)) ||
            (rc = mk(&mstr[4], e->rho, false, BOX_CORE)) || (rc = mk(&mstr[5], e->vp, false, BOX_CORE)) ||
            (rc = mk(&mstr[6], e->px, true, BOX_CORE)) || (rc = mk(&mstr[7], e->py, true, BOX_CORE)) ||
            (rc = mk(&mstr[8], e->pz, true, BOX_CORE)))
            return rc;
        for (int b = 0; b < 2 && e->fused_ok; ++b) {  // fused step reading set b
            CUtensorMap *ms = e->mstep[t][b];
            void *su = b ? e->u2 : e->u, *sv = b ? e->v2 : e->v, *sw = b ? e->w2 : e->w, *sp = b ? e->P2 : e->P;
            if ((rc = mk(&ms[0], sp, true, BOX_H2)) || (rc = mk(&ms[1], su, true, BOX_HX)) ||
                (rc = mk(&ms[2], sv, true, BOX_CORE)) || (rc = mk(&ms[3], sw, true, BOX_HZ)) ||
                (rc = mk(&ms[4], e->rinv, false, BOX_H)) || (rc = mk(&ms[5], sp, true, BOX_CORE)) ||
                (rc = mk(&ms[6], e->rho, false, BOX_CORE)) || (rc = mk(&ms[7], e->vp, false, BOX_CORE)) ||
                (rc = mk(&ms[8], e->px, true, BOX_CORE)) || (rc = mk(&ms[9], e->py, true, BOX_CORE)) ||
                (rc = mk(&ms[10], e->pz, true, BOX_CORE)))
                return rc;
        }
    } else if (c.physics == A3D_VTI) {
        e->nvel = 6;
        if ((rc = mk(&mvel[0], e->P, true, BOX_HX)) || (rc = mk(&mvel[1], e->Q, true, BOX_HZ)) ||
            (rc = mk(&mvel[2], e->u, true, BOX_CORE)) || (rc = mk(&mvel[3], e->v, true, BOX_CORE)) ||
            (rc = mk(&mvel[4], e->w, true, BOX_CORE)) || (rc = mk(&mvel[5], e->rinv, false, BOX_CORE)))
            return rc;
        e->nstr = 15;
        if ((rc = mk(&mstr[0], e->v, true, BOX_CORE)) || (rc = mk(&mstr[1], e->u, true, BOX_HX)) ||
            (rc = mk(&mstr[2], e->w, true, BOX_HZ)) || (rc = mk(&mstr[3], e->P, true, BOX_CORE)) ||
            (rc = mk(&mstr[4], e->Q, true, BOX_CORE)) || (rc = mk(&mstr[5], e->rho, false, BOX_CORE)) ||
            (rc = mk(&mstr[6], e->vp, false, BOX_CORE)) || (rc = mk(&mstr[7], e->eps, false, BOX_CORE)) ||
            (rc = mk(&mstr[8], e->del, false, BOX_CORE)) || (rc = mk(&mstr[9], e->px, true, BOX_CORE)) ||
            (rc = mk(&mstr[10], e->py, true, BOX_CORE)) || (rc = mk(&mstr[11], e->pz, true, BOX_CORE)) ||
            (rc = mk(&mstr[12], e->qx, true, BOX_CORE)) || (rc = mk(&mstr[13], e->qy, true, BOX_CORE)) ||
            (rc = mk(&mstr[14], e->qz, true, BOX_CORE)))
            return rc;
    } else {
        e->nvel = 9;
        if ((rc = mk(&mvel[0], e->P, true, BOX_H)) || (rc = mk(&mvel[1], e->Q, true, BOX_H)) ||
            (rc = mk(&mvel[2], e->u, true, BOX_CORE)) || (rc = mk(&mvel[3], e->v, true, BOX_CORE)) ||
            (rc = mk(&mvel[4], e->w, true, BOX_CORE)) || (rc = mk(&mvel[5], e->tct, false, BOX_CORE)) ||
            (rc = mk(&mvel[6], e->tst, false, BOX_CORE)) || (rc = mk(&mvel[7], e->tcp, false, BOX_CORE)) ||
            (rc = mk(&mvel[8], e->tsp, false, BOX_CORE)))
            return rc;
        e->nstr = 18;
        if ((rc = mk(&mstr[0], e->u, true, BOX_H)) || (rc = mk(&mstr[1], e->v, true, BOX_H)) ||
            (rc = mk(&mstr[2], e->w, true, BOX_H)) || (rc = mk(&mstr[3], e->P, true, BOX_CORE)) ||
            (rc = mk(&mstr[4], e->Q, true, BOX_CORE)) || (rc = mk(&mstr[5], e->vp, false, BOX_CORE)) ||
            (rc = mk(&mstr[6], e->eps, false, BOX_CORE)) || (rc = mk(&mstr[7], e->del, false, BOX_CORE)) ||
            (rc = mk(&mstr[8], e->tct, false, BOX_CORE)) || (rc = mk(&mstr[9], e->tst, false, BOX_CORE)) ||
            (rc = mk(&mstr[10], e->tcp, false, BOX_CORE)) || (rc = mk(&mstr[11], e->tsp, false, BOX_CORE)) ||
            (rc = mk(&mstr[12], e->px, true, BOX_CORE)) || (rc = mk(&mstr[13], e->py, true, BOX_CORE)) ||
            (rc = mk(&mstr[14], e->pz, true, BOX_CORE)) || (rc = mk(&mstr[15], e->qx, true, BOX_CORE)) ||
            (rc = mk(&mstr[16], e->qy, true, BOX_CORE)) || (rc = mk(&mstr[17], e->qz, true, BOX_CORE)))
            return rc;
    }
    }
    return A3D_OK;
}

static int prepare_profiling(a3d_engine *e, int per_step) {
    if (!e->profiling) return A3D_OK;
    const size_t need = (size_t)per_step * e->cfg.nt;
    while (e->kev.size() < need) {
        cudaEvent_t ev;
        CUDA_TRY(cudaEventCreate(&ev));
        e->kev.push_back(ev);
    }
    return A3D_OK;
}

static int check_kernel_error(a3d_engine *e) {
    int herr = 0;
    CUDA_TRY(cudaMemcpyAsync(&herr, e->d_err, sizeof(int), cudaMemcpyDeviceToHost, e->st));
    CUDA_TRY(cudaStreamSynchronize(e->st));
    if (herr)
        return fail(A3D_E_KERNEL, "a kernel gave up a bounded wait (code %d); results are invalid", herr);
    return A3D_OK;
}

// Autotuner: times every candidate launch configuration (tile width, ring depth,
// sweep plan) of each kernel kind on this engine's own grid — 1 untimed and 3
// timed launches each, CUDA events on the engine stream — and keeps the fastest.
// Candidates that do not fit (shared memory) are skipped.  The wavefields hold
// garbage afterwards; run() clears them before every shot.
// The isotropic FP32 engine has two forms of its step: the two sweeps (velocity,
// stress) and the fused sweep.  Unless A3D_FUSED or a pinned A3D_TUNE decides, both
// are tuned and the faster one (summed launch times of the two sweeps against the
// fused step's) runs.
// Tuned launch shapes are remembered per process for each (device, physics,
// storage, padded grid, absorber, step forms, tile request), so engines made again
// for the same grid — a3d_forward_host calls, shots on equal windows — skip the tuner.
static std::mutex g_tune_mu;
static std::map<std::string, std::pair<std::array<a3d_engine::Tune, 2>, bool>> g_tune_cache;

int a3d_engine::autotune() {
    const char *fz = getenv("A3D_FUSED"), *pin = getenv("A3D_TUNE");
    const bool forced = fz && (fz[0] == '0' || fz[0] == '1');
    if (forced || (pin && *pin && !fp64)) {
        fused = fused_ok && fz && fz[0] == '1';
        return autotune_form();
    }
    char key[256];
    snprintf(key, sizeof key, "%d/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d", device, cfg.physics, cfg.storage, g.nnz, g.nnx,
             g.nny, npml, (int)learned, (int)fused_ok, cfg.tile_x, nbatch);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            tune[0] = it->second.first[0];
            tune[1] = it->second.first[1];
            tuned = true;
            if (it->second.second && fused_ok) {
                fused = true;
                return A3D_OK;
            }
            return drop_fused();
        }
    }
    fused = false;
    int rc = autotune_form();
    if (rc) return rc;
    if (!fused_ok) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = {{tune[0], tune[1]}, false};
        return A3D_OK;
    }
    const Tune two[2] = {tune[0], tune[1]};
    fused = true;
    if ((rc = autotune_form())) return rc;
    if (tune[0].ms >= two[0].ms + two[1].ms) {
        tune[0] = two[0];
        tune[1] = two[1];
        rc = drop_fused();
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = {{tune[0], tune[1]}, fused};
    return rc;
}

// run the two-sweep form from now on; the second buffer set only serves the fused
// step, so it is given back
int a3d_engine::drop_fused() {
    fused = false;
    for (void **f : {&u2, &v2, &w2, &P2}) {
        if (!*f) continue;
        void *a = field_alloc(*f, esz);
        auto it = std::find(allocs.begin(), allocs.end(), a);
        if (it != allocs.end()) {
            CUDA_TRY(cudaFree(a));
            allocs.erase(it);
            dev_bytes -= field_bytes(esz);
        }
        *f = nullptr;
    }
    fused_ok = false;
    return A3D_OK;
}

int a3d_engine::autotune_form() {
    const a3d_config &c = cfg;
    std::vector<Tune> cand;
    const int fixed_tx = c.tile_x == 8 || c.tile_x == 16 ? c.tile_x : 0;
    // (tile width, rows per warp): the 2nd-order and isotropic kernels share tile
    // rows among a warp's lanes; the VTI/TTI kernels use one row per warp
    const bool multirow = c.physics != A3D_TTI;  // TTI kernels: one row per warp
    std::vector<std::pair<int, int>> shapes;
    if (multirow) shapes = {{8, 1}, {16, 1}, {8, 2}, {16, 2}, {16, 4}};  // VTI skips (16, 4)
    else shapes = {{8, 1}, {16, 1}};
    if (fused) shapes = {{8, 1}, {16, 1}, {8, 2}, {16, 2}};  // the fused step: ring depths 0 and 1
    const int maxdepth = fused ? 1 : 2;
    // A3D_TUNE="tx,rows,depth,plan[,rot][;tx,rows,depth,plan[,rot]]" pins the launch
    // configuration of each kernel kind (velocity; stress) instead of timing candidates
    if (const char *env = getenv("A3D_TUNE"); env && *env && !fp64) {
        const char *q = env;
        for (int k = 0; k < 2; ++k) {
            int tx = 0, rows = 0, depth = 0, mode = 0, n = 0, rot = 0, n2 = 0;
            if (sscanf(q, "%d,%d,%d,%d%n", &tx, &rows, &depth, &mode, &n) != 4 || (tx != 8 && tx != 16) ||
                depth < 0 || depth > maxdepth || (fused && rows == 4) ||
                (rows != 1 && rows != 2 && rows != 4) || (rows == 4 && tx != 16) || mode < 0 || mode > 2)
                return fail(A3D_E_ARG, "A3D_TUNE: expected tx,rows,depth,plan[,rot][;...], got \"%s\"", env);
            int sblk = 1, n3 = 0;
            if (q[n] == ',') {
                if (sscanf(q + n + 1, "%d%n", &rot, &n2) != 1 || rot < 0 || rot > 1)
                    return fail(A3D_E_ARG, "A3D_TUNE: expected tx,rows,depth,plan[,rot[,sblk]][;...], got \"%s\"", env);
                n += 1 + n2;
                if (q[n] == ',') {  // tile block of a multi-shot sweep
                    if (sscanf(q + n + 1, "%d%n", &sblk, &n3) != 1 || sblk < 1)
                        return fail(A3D_E_ARG, "A3D_TUNE: expected tx,rows,depth,plan[,rot[,sblk]][;...], got \"%s\"", env);
                    n += 1 + n3;
                }
            }
            if (!multirow && rows != 1) return fail(A3D_E_ARG, "A3D_TUNE: this physics runs one row per warp");
            tune[k] = Tune{tx, depth, mode, rows};
            tune[k].ms = 0;
            tune[k].rot = c.physics == A3D_2ORDER ? 0 : rot;
            tune[k].sblk = sblk;
            q += n;
            if (*q == ';') ++q;
            else if (k == 0) { tune[1] = tune[0]; break; }
        }
        tuned = true;
        return A3D_OK;
    }
    if (c.tile_x < 0 || fp64) {  // fixed defaults (and the FP64 run): 32x8, shallow rings, lockstep and fill plans
        for (int m = 0; m < 2; ++m) cand.push_back(Tune{8, 0, m, multirow ? 2 : 1});
    } else {
        for (auto sh : shapes)
            for (int d = 0; d <= maxdepth; ++d)
                for (int m = 0; m < 3; ++m)
                    if (!fixed_tx || sh.first == fixed_tx) cand.push_back(Tune{sh.first, d, m, sh.second});
    }
    const int kinds = c.physics == A3D_2ORDER || fused ? 1 : 2;
    cudaEvent_t t0, t1;
    CUDA_TRY(cudaEventCreate(&t0));
    CUDA_TRY(cudaEventCreate(&t1));
    // one launch of kernel kind kk with shape tc on the engine's fields (no source)
    auto launch_kind = [&](int kk, const Tune &tc) -> cudaError_t {
        const int ti = tc.tx == 16 ? 1 : 0;
        if (c.physics == A3D_2ORDER) {
            K2OLaunch L{};
            L.tx = tc.tx; L.depth = tc.depth; L.mode = tc.mode; L.rows = tc.rows; L.fp64 = fp64;
            L.tm_cur = m2o_cur[ti][0]; L.tm_prev = m2o_prev[ti][1]; L.tm_vv = m2o_vv[ti];
            L.ybuf = Y;
            K2OParams &p = L.p;
            p.nnz = g.nnz; p.nnx = g.nnx; p.nny = g.nny; p.ldz = g.ldz;
            p.nx = c.nx; p.ny = c.ny; p.gz = -1;
            p.fz = fz; p.fx = fx; p.fy = fy;
            p.dz2 = p.dx2 = p.dy2 = 1.0f;
            p.s_x = p.s_y = p.s_z = -100;
            p.rec = rec; p.nt = c.nt; p.err = d_err;
            return launch_k2o(L, st);
        }
        K1Launch L{};
        K1Params &p = L.p;
        p.nnz = g.nnz; p.nnx = g.nnx; p.nny = g.nny; p.ldz = g.ldz;
        p.nx = c.nx; p.ny = c.ny; p.npml = npml;
        p.dtx = p.dty = p.dtz = 0.0f;
        const float *q = pml;
        p.cx1 = q; p.cx2 = q + g.nnx; p.ax1 = q + 2 * g.nnx; p.ax2 = q + 3 * g.nnx; q += 4 * g.nnx;
        p.cy1 = q; p.cy2 = q + g.nny; p.ay1 = q + 2 * g.nny; p.ay2 = q + 3 * g.nny; q += 4 * g.nny;
        p.cz1 = q; p.cz2 = q + g.nnz; p.az1 = q + 2 * g.nnz; p.az2 = q + 3 * g.nnz;
        p.s_x = p.s_y = p.s_z = -100;
        p.taper = taper;
        p.px = px; p.py = py; p.pz = pz; p.qx = qx; p.qy = qy; p.qz = qz;
        for (int a = 0; a < 3; ++a) { p.ulo[a] = ulo[a]; p.uhi[a] = uhi[a]; }
        p.rec = rec; p.nt = c.nt; p.err = d_err;
        const int kv = c.physics == A3D_ISO ? K1_ISO_VEL : (c.physics == A3D_VTI ? K1_VTI_VEL : K1_TTI_VEL);
        L.kind = kv + kk;
        L.maps = kk == 0 ? mvel[ti] : mstr[ti];
        L.nmaps = kk == 0 ? nvel : nstr;
        L.out0 = kk == 0 ? u : P; L.out1 = kk == 0 ? v : Q; L.out2 = w;
        L.tx = tc.tx; L.depth = tc.depth; L.mode = tc.mode; L.rows = tc.rows; L.fp64 = fp64;
        L.half = half;
        L.pf = pfloat;
        L.rot = tc.rot;
        if (nbatch > 1) {  // multi-shot kernels over every copy (no source: d_shots lie outside)
            L.ms = 1;
            L.nshot = nbatch;
            L.sblk = tc.sblk;
            p.shots = d_shots;
            p.fstride = fstride;
            p.fstride_p = fstride_p;
            p.rstride = (size_t)c.nt * c.nx * c.ny;
        }
        p.svp = p.spv = p.rec_scale = 1.0f;
        if (fused) {  // set 0 read, set 1 written
            L.kind = K1_ISO_STEP;
            L.maps = mstep[ti][0];
            L.nmaps = 11;
            L.out0 = u2; L.out1 = v2; L.out2 = w2; L.out3 = P2;
            return launch_iso_step(L, st);
        }
        auto launch = c.physics == A3D_ISO ? launch_iso : (c.physics == A3D_VTI ? launch_vti : launch_tti);
        return launch(L, st);
    };
    // ms per launch of candidate tc of kind k: a warm-up launch, then reps timed ones,
    // each after a launch of the other sweep with shape *other when given, so that
    // the timed launch meets the L2 contents of the time loop; f < 0: it does not run
    auto time_cand = [&](int k, const Tune &tc, float &f, int reps, const Tune *other) -> int {
        f = -1.0f;
        if (launch_kind(k, tc) != cudaSuccess) { cudaGetLastError(); return A3D_OK; }
        float sum = 0;
        for (int r = 0; r < reps; ++r) {
            if (other && launch_kind(1 - k, *other) != cudaSuccess) { cudaGetLastError(); return A3D_OK; }
            CUDA_TRY(cudaEventRecord(t0, st));
            const cudaError_t le = launch_kind(k, tc);
            CUDA_TRY(cudaEventRecord(t1, st));
            CUDA_TRY(cudaEventSynchronize(t1));
            if (le != cudaSuccess) { cudaGetLastError(); return A3D_OK; }
            float e = 0;
            CUDA_TRY(cudaEventElapsedTime(&e, t0, t1));
            sum += e;
        }
        f = sum / reps;
        return A3D_OK;
    };
    // first pass: every candidate of each kind, three timed launches
    std::vector<std::pair<float, Tune>> timed[2];
    for (int k = 0; k < kinds; ++k) {
        for (const Tune &tc : cand) {
            float f = -1.0f;
            const int rt = time_cand(k, tc, f, 3, nullptr);
            if (rt) return rt;
            if (f >= 0.0f) timed[k].push_back({f, tc});
        }
        if (timed[k].empty()) return fail(A3D_E_CUDA, "no launch configuration of kernel kind %d runs", k);
        std::sort(timed[k].begin(), timed[k].end(), [](const auto &x, const auto &y) { return x.first < y.first; });
        tune[k] = timed[k][0].second;
        tune[k].ms = timed[k][0].first;
    }
    // second pass: the four fastest of each kind (and, for the 1st-order engines, each
    // with the rotated z-tile order) with ten timed launches each, alternating with
    // the other sweep's current choice as in the time loop: the leading candidates
    // often lie within a few percent of each other
    for (int k = 0; k < kinds; ++k) {
        std::vector<Tune> fin;
        for (size_t i = 0; i < timed[k].size() && i < 4; ++i) {
            fin.push_back(timed[k][i].second);
            if (c.physics != A3D_2ORDER && !fp64) {
                Tune r = timed[k][i].second;
                r.rot = 1;
                fin.push_back(r);
            }
        }
        if (nbatch > 1) {  // multi-shot sweeps: each finalist with tile blocks of 1, one x
            // column, 4 and 16 columns, and the whole grid (Sweep::sblk)
            const int ntz = (g.nnz - 2 * MM + 31) / 32;
            std::vector<Tune> more;
            for (const Tune &f : fin) {
                const int T = ntz * ((g.nnx - 2 * MM + f.tx - 1) / f.tx);
                for (int b : {1, ntz, 4 * ntz, 16 * ntz, T}) {
                    if (b > T && b != T) continue;
                    Tune t = f;
                    t.sblk = b;
                    more.push_back(t);
                }
            }
            fin.swap(more);
        }
        const Tune other = kinds == 2 ? tune[1 - k] : Tune{};
        float best = 1e30f;
        for (const Tune &tc : fin) {
            float f = -1.0f;
            const int rt = time_cand(k, tc, f, 10, kinds == 2 ? &other : nullptr);
            if (rt) return rt;
            if (f >= 0.0f && f < best) {
                best = f;
                tune[k] = tc;
                tune[k].ms = f;
            }
        }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    tuned = true;
    return check_kernel_error(this);
}

// snapshot ring: slot 0 reuses the crop buffer allocated at setup; pinned host
// buffers, the copy stream and the events are made at the first snapshot
int a3d_engine::snap_setup() {
    if (snap_st) return A3D_OK;
    const size_t bytes = (size_t)cfg.nx * cfg.ny * cfg.nz * 4;
    for (int k = 0; k < NSNAP; ++k) {
        snap_ring_dev[k] = k == 0 ? snap_dev : (float *)dalloc(bytes);
        if (!snap_ring_dev[k]) return fail(A3D_E_NOMEM, "snapshot buffer allocation failed");
        CUDA_TRY(cudaMallocHost(&snap_ring_host[k], bytes));
        CUDA_TRY(cudaEventCreateWithFlags(&snap_cropped[k], cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&snap_copied[k], cudaEventDisableTiming));
    }
    CUDA_TRY(cudaStreamCreateWithFlags(&snap_st, cudaStreamNonBlocking));
    return A3D_OK;
}

// Runs loop() between ev0 and ev1 on the engine stream.  With use_graph it is
// captured into a CUDA graph first and the graph is launched once, so the steps go
// to the GPU as one submission.
static int timed_loop(a3d_engine *e, bool use_graph, const std::function<int()> &loop) {
    cudaStream_t st = e->st;
    if (!use_graph) {
        CUDA_TRY(cudaEventRecord(e->ev0, st));
        int r = loop();
        if (r) return r;
        CUDA_TRY(cudaEventRecord(e->ev1, st));
        return A3D_OK;
    }
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    const int r = loop();
    cudaGraph_t gr = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &gr);
    if (r || ec != cudaSuccess) {
        if (gr) cudaGraphDestroy(gr);
        return r ? r : fail(A3D_E_CUDA, "stream capture of the time loop failed: %s", cudaGetErrorString(ec));
    }
    cudaGraphExec_t ge = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&ge, gr, 0);
    cudaGraphDestroy(gr);
    if (ei != cudaSuccess) return fail(A3D_E_CUDA, "cudaGraphInstantiate failed: %s", cudaGetErrorString(ei));
    cudaError_t el = cudaEventRecord(e->ev0, st);
    if (el == cudaSuccess) el = cudaGraphLaunch(ge, st);
    if (el == cudaSuccess) el = cudaEventRecord(e->ev1, st);
    if (el == cudaSuccess) el = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(ge);
    if (el != cudaSuccess) return fail(A3D_E_CUDA, "graph launch of the time loop failed: %s", cudaGetErrorString(el));
    return A3D_OK;
}

int a3d_engine::run(const a3d_shot &s, float *rec_dev, const SnapHook *hook, double *ms) {
    const a3d_config &c = cfg;
    if (nbatch > 1) {  // an engine of multi-shot sweeps runs a single shot as a sweep of one
        if (hook && hook->want) return fail(A3D_E_UNSUPPORTED, "snapshots are not taken in multi-shot sweeps");
        int r = run_shots(&s, 1, ms);
        if (!r && rec_dev && rec_dev != rec) {
            cudaError_t ce = cudaMemcpyAsync(rec_dev, rec, (size_t)c.nt * c.nx * c.ny * 4, cudaMemcpyDeviceToDevice, st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
            if (ce != cudaSuccess) r = fail(A3D_E_CUDA, "record copy failed: %s", cudaGetErrorString(ce));
        }
        return r;
    }
    if (s.sx < 0 || s.sx >= c.nx || s.sy < 0 || s.sy >= c.ny || s.sz < 0 || s.sz >= c.nz)
        return fail(A3D_E_ARG, "shot (%d,%d,%d) outside the %dx%dx%d model", s.sx, s.sy, s.sz, c.nx, c.ny, c.nz);
    if (!rec_dev) rec_dev = rec;
    CUDA_TRY(cudaSetDevice(device));
    int rc;
    if (!tuned && (rc = autotune())) return rc;
    CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    const size_t fb = g.elems() * esz;
    // direct-wave mute thresholds for this shot
    std::vector<int> mute;
    if (c.mute) {
        mute.resize((size_t)c.nx * c.ny);
        for (int iy = 0; iy < c.ny; ++iy)
            for (int ix = 0; ix < c.nx; ++ix)
                mute[ix + (size_t)c.nx * iy] = mute_nt(ix, iy, s.sx, s.sy, s.sz, c.dx, c.dy, c.dz, c.dt, c.fm, v_mute);
        CUDA_TRY(cudaMemcpyAsync(d_mute, mute.data(), mute.size() * 4, cudaMemcpyHostToDevice, st));
    }
    // snapshots: crop into ring slot k on the compute stream, copy to pinned host
    // memory on the snapshot stream, hand over (in order) when slot k is needed
    // again or after the loop; the compute stream waits only for the copy that
    // last used the slot's device buffer
    struct Pending { int slot, it; };
    std::vector<Pending> queue;
    size_t qhead = 0;
    int nsnap = 0;
    const size_t win = (size_t)c.nx * c.ny * c.nz;
    auto hand_over = [&](size_t upto) -> int {  // deliver queue[qhead, upto)
        for (; qhead < upto; ++qhead) {
            const Pending &q = queue[qhead];
            CUDA_TRY(cudaEventSynchronize(snap_copied[q.slot]));
            if (hook->take) {
                const int r = hook->take(q.it, snap_ring_host[q.slot]);
                if (r) return r;
            }
        }
        return A3D_OK;
    };
    auto snapshot = [&](int it, const void *field) -> int {
        if (!hook || !hook->want || !hook->want(it)) return A3D_OK;
        int r;
        if ((r = snap_setup())) return r;
        const int k = nsnap % NSNAP;
        if (nsnap >= NSNAP && (r = hand_over(queue.size() - (NSNAP - 1)))) return r;  // slot k's last use
        CUDA_TRY(cudaStreamWaitEvent(st, snap_copied[k], 0));
        const int pad = g.pad;
        const float sc = 1.0f / sig_p;  // exact: sig_p is a power of two
        float *dst = snap_ring_dev[k];
        if (fp64)
            crop_window<double><<<1024, 256, 0, st>>>((const double *)field, dst, c.nx, c.ny, c.nz, pad, g.ldz, g.nnx, sc);
        else if (half == 1)
            crop_window<__nv_bfloat16><<<1024, 256, 0, st>>>((const __nv_bfloat16 *)field, dst, c.nx, c.ny, c.nz, pad, g.ldz, g.nnx, sc);
        else if (half == 2 && !pfloat)  // A3D_FP16V snapshots P, stored as float
            crop_window<__half><<<1024, 256, 0, st>>>((const __half *)field, dst, c.nx, c.ny, c.nz, pad, g.ldz, g.nnx, sc);
        else
            crop_window<float><<<1024, 256, 0, st>>>((const float *)field, dst, c.nx, c.ny, c.nz, pad, g.ldz, g.nnx, sc);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaEventRecord(snap_cropped[k], st));
        CUDA_TRY(cudaStreamWaitEvent(snap_st, snap_cropped[k], 0));
        CUDA_TRY(cudaMemcpyAsync(snap_ring_host[k], dst, win * 4, cudaMemcpyDeviceToHost, snap_st));
        CUDA_TRY(cudaEventRecord(snap_copied[k], snap_st));
        queue.push_back({k, it});
        ++nsnap;
        return A3D_OK;
    };
    // the time loop, bracketed by ev0/ev1 (graph replay when graph mode is on and no
    // snapshot or per-kernel events sit in the loop)
    const bool use_graph = graph && !profiling && !(hook && hook->want);
    auto time_loop = [&](auto &&loop) -> int { return timed_loop(this, use_graph, loop); };
    if (c.physics == A3D_2ORDER) {
        CUDA_TRY(cudaMemsetAsync(field_alloc(X, esz), 0, fb, st));
        CUDA_TRY(cudaMemsetAsync(field_alloc(Y, esz), 0, fb, st));
        const int pad = g.pad;
        const int sxp = s.sx + pad, syp = s.sy + pad, szp = s.sz + pad;
        // step 0's dipole into the zero current level (2O:443)
        const size_t si = g.idx(szp, sxp, syp);
        if (fp64) {
            double d[3] = {(double)w2o[0], 0.0, -(double)w2o[0]};
            CUDA_TRY(cudaMemcpyAsync((double *)X + si, d, sizeof d, cudaMemcpyHostToDevice, st));
        } else {
            float d[3] = {w2o[0], 0.0f, -w2o[0]};
            CUDA_TRY(cudaMemcpyAsync((float *)X + si, d, sizeof d, cudaMemcpyHostToDevice, st));
        }
        K2OLaunch L{};
        const int ti = tune[0].tx == 16 ? 1 : 0;
        L.tx = tune[0].tx;
        L.depth = tune[0].depth;
        L.mode = tune[0].mode;
        L.rows = tune[0].rows;
        L.fp64 = fp64;
        L.grid = 0;
        L.tm_vv = m2o_vv[ti];
        K2OParams &p = L.p;
        p.nnz = g.nnz; p.nnx = g.nnx; p.nny = g.nny; p.ldz = g.ldz;
        p.nx = c.nx; p.ny = c.ny;
        p.gz = pad + c.rec_z; p.rx0 = pad; p.ry0 = pad;
        p.fz = fz; p.fx = fx; p.fy = fy;
        p.dz2 = (float)(1.0 / (double)(c.dz * c.dz));  // 2O:387-389
        p.dx2 = (float)(1.0 / (double)(c.dx * c.dx));
        p.dy2 = (float)(1.0 / (double)(c.dy * c.dy));
        p.s_x = sxp; p.s_y = syp; p.s_z = szp;
        p.rec = rec_dev;
        p.mute_nt = c.mute ? d_mute : nullptr;
        p.nt = c.nt;
        p.err = d_err;
        void *buf[2] = {X, Y};
        if ((rc = prepare_profiling(this, 2))) return rc;
        rc = time_loop([&]() -> int {
            int cur = 0;
            for (int it = 0; it < c.nt; ++it) {
                L.tm_cur = m2o_cur[ti][cur];
                L.tm_prev = m2o_prev[ti][1 - cur];
                L.ybuf = buf[1 - cur];
                p.w_next = it + 1 < c.nt ? w2o[it + 1] : 0.0f;
                p.it = it;
                if (profiling) CUDA_TRY(cudaEventRecord(kev[2 * it], st));
                CUDA_TRY(launch_k2o(L, st));
                if (profiling) CUDA_TRY(cudaEventRecord(kev[2 * it + 1], st));
                int r2 = snapshot(it, buf[cur]);
                if (r2) return r2;
                cur = 1 - cur;
            }
            return A3D_OK;
        });
        if (rc) return rc;
    } else {
        void *fields[15] = {u, v, w, P, Q, px, py, pz, qx, qy, qz, u2, v2, w2, P2};
        for (int k = 0; k < 15; ++k) {
            const bool pr = k >= 3 && k < 11;  // P, Q and split components
            if (fields[k]) CUDA_TRY(cudaMemsetAsync(field_alloc(fields[k], fsize(pr)), 0, g.elems() * fsize(pr), st));
        }
        const int np = npml;
        K1Launch Lv{}, Ls{};
        K1Params p{};
        p.nnz = g.nnz; p.nnx = g.nnx; p.nny = g.nny; p.ldz = g.ldz;
        p.nx = c.nx; p.ny = c.ny; p.npml = np;
        p.dtx = c.dt / c.dx; p.dty = c.dt / c.dy; p.dtz = c.dt / c.dz;
        const float *q = pml;
        p.cx1 = q; p.cx2 = q + g.nnx; p.ax1 = q + 2 * g.nnx; p.ax2 = q + 3 * g.nnx; q += 4 * g.nnx;
        p.cy1 = q; p.cy2 = q + g.nny; p.ay1 = q + 2 * g.nny; p.ay2 = q + 3 * g.nny; q += 4 * g.nny;
        p.cz1 = q; p.cz2 = q + g.nnz; p.az1 = q + 2 * g.nnz; p.az2 = q + 3 * g.nnz;
        p.s_x = s.sx + np - 1; p.s_y = s.sy + np - 1; p.s_z = s.sz + np - 1;  // ..iso..:91-93
        p.taper = taper;
        p.px = px; p.py = py; p.pz = pz; p.qx = qx; p.qy = qy; p.qz = qz;
        for (int a = 0; a < 3; ++a) { p.ulo[a] = ulo[a]; p.uhi[a] = uhi[a]; }
        p.rec = rec_dev;
        p.mute_nt = c.mute ? d_mute : nullptr;
        p.nt = c.nt;
        p.err = d_err;
        p.svp = sig_v / sig_p;  // powers of two: exact
        p.spv = sig_p / sig_v;
        p.rec_scale = 1.0f / sig_p;
        const int kv = c.physics == A3D_ISO ? K1_ISO_VEL : (c.physics == A3D_VTI ? K1_VTI_VEL : K1_TTI_VEL);
        Lv.kind = kv; Ls.kind = kv + 1;
        Lv.maps = mvel[tune[0].tx == 16 ? 1 : 0]; Lv.nmaps = nvel;
        Ls.maps = mstr[tune[1].tx == 16 ? 1 : 0]; Ls.nmaps = nstr;
        Lv.out0 = u; Lv.out1 = v; Lv.out2 = w;
        Ls.out0 = P; Ls.out1 = Q;
        Lv.tx = tune[0].tx; Lv.depth = tune[0].depth; Lv.mode = tune[0].mode; Lv.rows = tune[0].rows;
        Ls.tx = tune[1].tx; Ls.depth = tune[1].depth; Ls.mode = tune[1].mode; Ls.rows = tune[1].rows;
        Lv.rot = tune[0].rot; Ls.rot = tune[1].rot;
        Lv.fp64 = Ls.fp64 = fp64; Lv.half = Ls.half = half; Lv.grid = Ls.grid = 0;
        Lv.pf = Ls.pf = pfloat;
        auto launch = c.physics == A3D_ISO ? launch_iso : (c.physics == A3D_VTI ? launch_vti : launch_tti);
        if (learned && !cl_packed) return fail(A3D_E_ARG, "learned rim without a closure (a3d_engine_set_closure)");
        std::vector<int> tap_slot(tap_out ? c.nt : 0, -1);
        for (size_t k = 0; k < tap_slot.size() && k < tap_steps.size(); ++k)
            if (tap_steps[k] >= 0 && tap_steps[k] < c.nt) tap_slot[tap_steps[k]] = (int)k;
        const long long tbox = (long long)(g.nnz - 2 * tap_off) * (g.nnx - 2 * tap_off) * (g.nny - 2 * tap_off);
        const int per = fused ? 2 : (learned ? 4 : 3);
        if ((rc = prepare_profiling(this, per))) return rc;
        if (fused) {  // one fused sweep per step; the buffer sets alternate
            K1Launch Lf = Lv;
            Lf.kind = K1_ISO_STEP;
            Lf.nmaps = 11;
            const int ti = tune[0].tx == 16 ? 1 : 0;
            rc = time_loop([&]() -> int {
                for (int it = 0; it < c.nt; ++it) {
                    p.it = it;
                    p.inj = inj[it];
                    p.amp0 = amp0[it];
                    p.amp1 = amp1[it];
                    Lf.p = p;
                    const int b = it & 1;
                    Lf.maps = mstep[ti][b];
                    void *nu = b ? u : u2, *nv = b ? v : v2, *nw = b ? w : w2, *np_ = b ? P : P2;
                    Lf.out0 = nu; Lf.out1 = nv; Lf.out2 = nw; Lf.out3 = np_;
                    if (profiling) CUDA_TRY(cudaEventRecord(kev[2 * it], st));
                    CUDA_TRY(launch_iso_step(Lf, st));
                    if (profiling) CUDA_TRY(cudaEventRecord(kev[2 * it + 1], st));
                    if (!tap_slot.empty() && tap_slot[it] >= 0)
                        CUDA_TRY(cl_launch_tap(g.nnz, g.nnx, g.nny, g.ldz, tap_off, (const float *)nu, (const float *)nv,
                                               (const float *)nw, (const float *)np_, tap_out + 4 * tbox * tap_slot[it],
                                               st));
                    int r2 = snapshot(it, np_);
                    if (r2) return r2;
                }
                return A3D_OK;
            });
            if (rc) return rc;
        } else
        rc = time_loop([&]() -> int {
            for (int it = 0; it < c.nt; ++it) {
                p.it = it;
                p.inj = inj[it];
                p.amp0 = amp0[it] * sig_p;  // exact: sig_p is a power of two
                p.amp1 = amp1[it] * sig_p;
                Lv.p = p;
                Ls.p = p;
                if (profiling) CUDA_TRY(cudaEventRecord(kev[per * it], st));
                CUDA_TRY(launch(Lv, st));
                if (profiling) CUDA_TRY(cudaEventRecord(kev[per * it + 1], st));
                CUDA_TRY(launch(Ls, st));
                if (profiling) CUDA_TRY(cudaEventRecord(kev[per * it + 2], st));
                if (learned) {
                    if (cl_simt)
                        CUDA_TRY(cl_launch_apply(clg, (float *)u, (float *)v, (float *)w, (float *)P, cl_zinv, cl_kap,
                                                 cl_packed, cl_h, st));
                    else
                        CUDA_TRY(cl_launch_apply_tc(clg, (float *)u, (float *)v, (float *)w, (float *)P, cl_zinv,
                                                    cl_kap, cl_image, cl_packed + CL_NW1 + CL_NW2, cl_y, d_err, nullptr,
                                                    0, g_sms, st));
                    if (profiling) CUDA_TRY(cudaEventRecord(kev[per * it + 3], st));
                }
                if (!tap_slot.empty() && tap_slot[it] >= 0)
                    CUDA_TRY(cl_launch_tap(g.nnz, g.nnx, g.nny, g.ldz, tap_off, (const float *)u, (const float *)v,
                                           (const float *)w, (const float *)P, tap_out + 4 * tbox * tap_slot[it], st));
                int r2 = snapshot(it, P);
                if (r2) return r2;
            }
            return A3D_OK;
        });
        if (rc) return rc;
    }
    if (hook && (rc = hand_over(queue.size()))) return rc;
    if ((rc = check_kernel_error(this))) return rc;
    if (profiling) {
        const int per = c.physics == A3D_2ORDER || fused ? 2 : (learned ? 4 : 3);
        for (int it = 0; it < c.nt; ++it)
            for (int k = 0; k + 1 < per; ++k) {
                float f = 0;
                CUDA_TRY(cudaEventElapsedTime(&f, kev[per * it + k], kev[per * it + k + 1]));
                if (k < 2) {
                    kms[k] += f;
                    klaunch[k] += 1;
                } else {
                    cl_ms += f;
                    cl_launch += 1;
                }
            }
    }
    if (ms) {
        float f = 0;
        CUDA_TRY(cudaEventElapsedTime(&f, ev0, ev1));
        *ms = f;
    }
    return A3D_OK;
}

// Multi-shot sweeps: k shots of this model advance together, every launch covering
// all of them (their wavefields lie fstride elements apart; their records and mute
// tables follow each other).  The arithmetic of each shot is that of run(), so each
// record equals its one-shot run bit for bit.
int a3d_engine::run_shots(const a3d_shot *shots, int k, double *ms) {
    const a3d_config &c = cfg;
    if (nbatch <= 1) return fail(A3D_E_ARG, "the engine was created without multi-shot sweeps (cfg.batch <= 1)");
    if (!shots || k < 1 || k > nbatch) return fail(A3D_E_ARG, "%d shots for an engine of %d", k, nbatch);
    for (int j = 0; j < k; ++j) {
        const a3d_shot &s = shots[j];
        if (s.sx < 0 || s.sx >= c.nx || s.sy < 0 || s.sy >= c.ny || s.sz < 0 || s.sz >= c.nz)
            return fail(A3D_E_ARG, "shot %d (%d,%d,%d) outside the %dx%dx%d model", j, s.sx, s.sy, s.sz, c.nx, c.ny,
                        c.nz);
    }
    CUDA_TRY(cudaSetDevice(device));
    int rc;
    if (!tuned && (rc = autotune())) return rc;
    CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    const int np = npml;
    std::vector<int4> cells(k);
    for (int j = 0; j < k; ++j)  // ..vti..:63-65: the source cell is (s - 1) + npml
        cells[j] = make_int4(shots[j].sx + np - 1, shots[j].sy + np - 1, shots[j].sz + np - 1, 0);
    CUDA_TRY(cudaMemcpyAsync(d_shots, cells.data(), k * sizeof(int4), cudaMemcpyHostToDevice, st));
    std::vector<int> mute;
    if (c.mute) {
        const size_t ntr = (size_t)c.nx * c.ny;
        mute.resize(ntr * k);
        for (int j = 0; j < k; ++j)
            for (int iy = 0; iy < c.ny; ++iy)
                for (int ix = 0; ix < c.nx; ++ix)
                    mute[j * ntr + ix + (size_t)c.nx * iy] =
                        mute_nt(ix, iy, shots[j].sx, shots[j].sy, shots[j].sz, c.dx, c.dy, c.dz, c.dt, c.fm, v_mute);
        CUDA_TRY(cudaMemcpyAsync(d_mute, mute.data(), mute.size() * 4, cudaMemcpyHostToDevice, st));
    }
    for (void *f : {u, v, w})
        if (f) CUDA_TRY(cudaMemsetAsync(field_alloc(f, esz), 0, fstride * esz * (size_t)k, st));
    for (void *f : {P, Q, px, py, pz, qx, qy, qz})
        if (f) CUDA_TRY(cudaMemsetAsync(field_alloc(f, esz_p), 0, fstride_p * esz_p * (size_t)k, st));
    K1Launch Lv{}, Ls{};
    K1Params p{};
    p.nnz = g.nnz; p.nnx = g.nnx; p.nny = g.nny; p.ldz = g.ldz;
    p.nx = c.nx; p.ny = c.ny; p.npml = np;
    p.dtx = c.dt / c.dx; p.dty = c.dt / c.dy; p.dtz = c.dt / c.dz;
    const float *q = pml;
    p.cx1 = q; p.cx2 = q + g.nnx; p.ax1 = q + 2 * g.nnx; p.ax2 = q + 3 * g.nnx; q += 4 * g.nnx;
    p.cy1 = q; p.cy2 = q + g.nny; p.ay1 = q + 2 * g.nny; p.ay2 = q + 3 * g.nny; q += 4 * g.nny;
    p.cz1 = q; p.cz2 = q + g.nnz; p.az1 = q + 2 * g.nnz; p.az2 = q + 3 * g.nnz;
    p.s_x = p.s_y = p.s_z = -100;  // per shot: p.shots
    p.shots = d_shots;
    p.fstride = fstride;
    p.fstride_p = fstride_p;
    p.rstride = (size_t)c.nt * c.nx * c.ny;
    p.taper = taper;
    p.px = px; p.py = py; p.pz = pz; p.qx = qx; p.qy = qy; p.qz = qz;
    for (int a = 0; a < 3; ++a) { p.ulo[a] = ulo[a]; p.uhi[a] = uhi[a]; }
    p.rec = rec;
    p.mute_nt = c.mute ? d_mute : nullptr;
    p.nt = c.nt;
    p.err = d_err;
    p.svp = sig_v / sig_p;
    p.spv = sig_p / sig_v;
    p.rec_scale = 1.0f / sig_p;
    Lv.kind = K1_VTI_VEL; Ls.kind = K1_VTI_STR;
    Lv.maps = mvel[tune[0].tx == 16 ? 1 : 0]; Lv.nmaps = nvel;
    Ls.maps = mstr[tune[1].tx == 16 ? 1 : 0]; Ls.nmaps = nstr;
    Lv.out0 = u; Lv.out1 = v; Lv.out2 = w;
    Ls.out0 = P; Ls.out1 = Q;
    Lv.tx = tune[0].tx; Lv.depth = tune[0].depth; Lv.mode = tune[0].mode; Lv.rows = tune[0].rows;
    Ls.tx = tune[1].tx; Ls.depth = tune[1].depth; Ls.mode = tune[1].mode; Ls.rows = tune[1].rows;
    Lv.rot = tune[0].rot; Ls.rot = tune[1].rot;
    Lv.fp64 = Ls.fp64 = false; Lv.half = Ls.half = half; Lv.grid = Ls.grid = 0;
    Lv.pf = Ls.pf = pfloat;
    Lv.ms = Ls.ms = 1;
    Lv.nshot = Ls.nshot = k;
    Lv.sblk = tune[0].sblk;
    Ls.sblk = tune[1].sblk;
    if ((rc = prepare_profiling(this, 3))) return rc;
    rc = timed_loop(this, graph && !profiling, [&]() -> int {
        for (int it = 0; it < c.nt; ++it) {
            p.it = it;
            p.inj = inj[it];
            p.amp0 = amp0[it] * sig_p;  // exact: sig_p is a power of two
            p.amp1 = amp1[it] * sig_p;
            Lv.p = p;
            Ls.p = p;
            if (profiling) CUDA_TRY(cudaEventRecord(kev[3 * it], st));
            CUDA_TRY(launch_vti(Lv, st));
            if (profiling) CUDA_TRY(cudaEventRecord(kev[3 * it + 1], st));
            CUDA_TRY(launch_vti(Ls, st));
            if (profiling) CUDA_TRY(cudaEventRecord(kev[3 * it + 2], st));
        }
        return A3D_OK;
    });
    if (rc) return rc;
    if ((rc = check_kernel_error(this))) return rc;
    if (profiling)
        for (int it = 0; it < c.nt; ++it)
            for (int kk = 0; kk < 2; ++kk) {
                float f = 0;
                CUDA_TRY(cudaEventElapsedTime(&f, kev[3 * it + kk], kev[3 * it + kk + 1]));
                kms[kk] += f;
                klaunch[kk] += 1;
            }
    if (ms) {
        float f = 0;
        CUDA_TRY(cudaEventElapsedTime(&f, ev0, ev1));
        *ms = f;
    }
    return A3D_OK;
}

// ---------------------------------------------------------------------------
// C API

static int validate(const a3d_config *c) {
    if (!c) return fail(A3D_E_ARG, "null config");
    if (c->physics < A3D_2ORDER || c->physics > A3D_TTI) return fail(A3D_E_ARG, "unknown physics %d", c->physics);
    if (c->nx < 1 || c->ny < 1 || c->nz < 1 || c->nt < 1)
        return fail(A3D_E_ARG, "grid %dx%dx%d, nt %d must be positive", c->nx, c->ny, c->nz, c->nt);
    if (!(c->dx > 0) || !(c->dy > 0) || !(c->dz > 0) || !(c->dt > 0) || !(c->fm > 0))
        return fail(A3D_E_ARG, "dx, dy, dz, dt and fm must be positive");
    if (c->storage != A3D_FP32 && c->storage != A3D_FP64 &&
        !((c->storage == A3D_BF16 || c->storage == A3D_FP16) && c->physics != A3D_2ORDER) &&
        !(c->storage == A3D_FP16V && (c->physics == A3D_VTI || c->physics == A3D_TTI)))
        return fail(A3D_E_UNSUPPORTED, "storage type %d is not built for this engine", c->storage);
    if (c->physics == A3D_ISO && (c->wtype < 1 || c->wtype > 6))
        return fail(A3D_E_ARG, "wavelet type %d outside 1..6", c->wtype);
    if (c->boundary != A3D_BOUNDARY_PML && c->boundary != A3D_BOUNDARY_LEARNED)
        return fail(A3D_E_ARG, "unknown boundary %d", c->boundary);
    if (c->boundary == A3D_BOUNDARY_LEARNED && (c->physics != A3D_ISO || c->storage != A3D_FP32))
        return fail(A3D_E_UNSUPPORTED, "the learned rim is built for the isotropic engine with FP32 storage");
    if (c->batch > 1 && (c->physics != A3D_VTI || c->storage == A3D_FP64))
        return fail(A3D_E_UNSUPPORTED, "multi-shot sweeps are built for the VTI engine with FP32 or 2-byte storage");
    return A3D_OK;
}

extern "C" int a3d_engine_create(a3d_engine **out, const a3d_config *cfg, const float *vel,
                                 const float *rho, const float *eps, const float *del,
                                 const float *theta, const float *phi, int device) {
    clear_error();
    if (!out) return fail(A3D_E_ARG, "null engine pointer");
    *out = nullptr;
    int rc = validate(cfg);
    if (rc) return rc;
    const int ph = cfg->physics;
    if (!vel || (ph == A3D_ISO && !rho) || (ph == A3D_VTI && (!rho || !eps || !del)) ||
        (ph == A3D_TTI && (!eps || !del || !theta || !phi)))
        return fail(A3D_E_ARG, "a model array the physics reads is null");
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(A3D_E_ARG, "device %d not present (%d devices)", device, ndev);
    CUDA_TRY(cudaSetDevice(device));
    CUDA_TRY(cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, device));
    cudaGetLastError();  // a refused launch configuration of an earlier engine leaves nothing pending here
    a3d_engine *e = new (std::nothrow) a3d_engine;
    if (!e) return fail(A3D_E_NOMEM, "host allocation failed");
    e->cfg = *cfg;
    e->device = device;
    e->fp64 = cfg->storage == A3D_FP64;
    e->half = cfg->storage == A3D_BF16 ? 1 : ((cfg->storage == A3D_FP16 || cfg->storage == A3D_FP16V) ? 2 : 0);
    e->pfloat = cfg->storage == A3D_FP16V;
    e->esz = e->fp64 ? 8 : (e->half ? 2 : 4);
    e->esz_p = e->pfloat ? 4 : e->esz;
    e->tx = 8;
    e->nbatch = cfg->batch > 1 ? cfg->batch : 1;
    if (ph == A3D_2ORDER) {
        e->npml = cfg->npml > 0 ? cfg->npml : 50;  // npd, 2O:19
        if (e->cfg.rec_z < 0) e->cfg.rec_z = 1;    // 2O:159 records at model depth 1
        if (e->cfg.rec_z >= cfg->nz) {
            const int rz = e->cfg.rec_z;
            delete e;
            return fail(A3D_E_ARG, "receiver depth %d outside the model", rz);
        }
        e->g.set(cfg->nx, cfg->ny, cfg->nz, MM + e->npml);
    } else {
        e->learned = cfg->boundary == A3D_BOUNDARY_LEARNED;
        e->npml = cfg->npml > 0 ? cfg->npml : (e->learned ? CL_PAD : (ph == A3D_TTI ? 40 : 20));
        if (e->npml < 6) {
            const int w = e->npml;
            delete e;
            return fail(A3D_E_ARG, "PML width %d below 6 cells", w);
        }
        {
            const char *fz = getenv("A3D_FUSED");
            e->fused_ok = ph == A3D_ISO && cfg->storage == A3D_FP32 && !e->learned && !(fz && fz[0] == '0');
            e->fused = e->fused_ok && fz && fz[0] == '1';
        }
        if (e->learned && e->npml != CL_PAD) {
            const int np = e->npml;
            delete e;
            return fail(A3D_E_ARG, "the learned rim pads by %d cells (npml %d given)", CL_PAD, np);
        }
        e->g.set(cfg->nx, cfg->ny, cfg->nz, e->npml);
    }
    if (e->g.elems() > (size_t)INT32_MAX) {  // kernels index a field with 32-bit offsets
        const size_t n = e->g.elems();
        delete e;
        return fail(A3D_E_ARG, "padded grid of %zu cells exceeds 2^31 - 1", n);
    }
    // one copy of a wavefield per shot of a multi-shot sweep, 256-byte aligned
    e->fstride = (e->g.elems() * e->esz + 255) / 256 * 256 / e->esz;
    e->fstride_p = (e->g.elems() * e->esz_p + 255) / 256 * 256 / e->esz_p;
    if (cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e->ev0) != cudaSuccess || cudaEventCreate(&e->ev1) != cudaSuccess) {
        delete e;
        return fail(A3D_E_CUDA, "stream/event creation failed");
    }
    e->d_err = (int *)e->dalloc(sizeof(int) * 4);
    if (!e->d_err) { delete e; return fail(A3D_E_NOMEM, "device allocation failed"); }
    rc = engine_setup(e, vel, rho, eps, del, theta, phi);
    if (rc) { delete e; return rc; }
    *out = e;
    return A3D_OK;
}

extern "C" int a3d_engine_destroy(a3d_engine *e) {
    delete e;
    return A3D_OK;
}

extern "C" int a3d_engine_run(a3d_engine *e, const a3d_shot *shot, float *rec_host, int snap_every,
                              int snap_skip0, float *snaps_host, double *ms) {
    clear_error();
    if (!e || !shot) return fail(A3D_E_ARG, "null engine or shot");
    if (snap_every < 0) return fail(A3D_E_ARG, "negative snapshot interval");
    SnapHook hook;
    int nsnap = 0;
    const size_t win = (size_t)e->cfg.nx * e->cfg.ny * e->cfg.nz;
    if (snap_every > 0 && snaps_host) {
        hook.want = [&](int it) { return it % snap_every == 0 && !(snap_skip0 && it == 0); };
        hook.take = [&](int, const float *d) {
            memcpy(snaps_host + (size_t)nsnap * win, d, win * 4);
            ++nsnap;
            return A3D_OK;
        };
    }
    int rc = e->run(*shot, nullptr, snap_every > 0 && snaps_host ? &hook : nullptr, ms);
    if (rc) return rc;
    if (rec_host) {
        cudaError_t ce = cudaMemcpy(rec_host, e->rec, (size_t)e->cfg.nt * e->cfg.nx * e->cfg.ny * 4, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) return fail(A3D_E_CUDA, "record copy failed: %s", cudaGetErrorString(ce));
    }
    return A3D_OK;
}

extern "C" int a3d_engine_run_device(a3d_engine *e, const a3d_shot *shot, float *rec_dev, double *ms) {
    clear_error();
    if (!e || !shot) return fail(A3D_E_ARG, "null engine or shot");
    return e->run(*shot, rec_dev, nullptr, ms);
}

extern "C" int a3d_engine_run_shots(a3d_engine *e, const a3d_shot *shots, int k, float *recs_host, double *ms) {
    clear_error();
    if (!e || !shots) return fail(A3D_E_ARG, "null engine or shots");
    int rc = e->run_shots(shots, k, ms);
    if (rc) return rc;
    if (recs_host) {
        cudaError_t ce = cudaMemcpy(recs_host, e->rec, (size_t)k * e->cfg.nt * e->cfg.nx * e->cfg.ny * 4,
                                    cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) return fail(A3D_E_CUDA, "record copy failed: %s", cudaGetErrorString(ce));
    }
    return A3D_OK;
}

extern "C" int a3d_engine_copy_record(a3d_engine *e, int j, float *rec_host) {
    clear_error();
    if (!e || !rec_host) return fail(A3D_E_ARG, "null engine or buffer");
    if (j < 0 || j >= e->nbatch) return fail(A3D_E_ARG, "record %d of an engine holding %d", j, e->nbatch);
    const size_t n = (size_t)e->cfg.nt * e->cfg.nx * e->cfg.ny;
    CUDA_TRY(cudaSetDevice(e->device));
    CUDA_TRY(cudaMemcpy(rec_host, e->rec + (size_t)j * n, n * 4, cudaMemcpyDeviceToHost));
    return A3D_OK;
}

extern "C" float *a3d_engine_record_device(a3d_engine *e) { return e ? e->rec : nullptr; }

extern "C" size_t a3d_engine_device_bytes(const a3d_engine *e) { return e ? e->dev_bytes : 0; }

extern "C" int a3d_forward_host(const a3d_config *cfg, const float *vel, const float *rho, const float *eps,
                                const float *del, const float *theta, const float *phi,
                                const a3d_shot *shots, int nshot, float *recs_host, int device) {
    a3d_engine *e = nullptr;
    int rc = a3d_engine_create(&e, cfg, vel, rho, eps, del, theta, phi, device);
    if (rc) return rc;
    const size_t nrec = (size_t)cfg->nt * cfg->nx * cfg->ny;
    for (int i = 0; i < nshot && !rc; ++i)
        rc = a3d_engine_run(e, &shots[i], recs_host ? recs_host + i * nrec : nullptr, 0, 0, nullptr, nullptr);
    a3d_engine_destroy(e);
    return rc;
}

extern "C" int a3d_engine_set_profiling(a3d_engine *e, int on) {
    if (!e) return fail(A3D_E_ARG, "null engine");
    e->profiling = on != 0;
    e->kms[0] = e->kms[1] = 0;
    e->klaunch[0] = e->klaunch[1] = 0;
    e->cl_ms = 0;
    e->cl_launch = 0;
    return A3D_OK;
}

extern "C" int a3d_engine_closure_times(const a3d_engine *e, double *ms, long long *launches) {
    if (!e) return fail(A3D_E_ARG, "null engine");
    if (ms) *ms = e->cl_ms;
    if (launches) *launches = e->cl_launch;
    return A3D_OK;
}

extern "C" int a3d_engine_set_closure(a3d_engine *e, const float *params, size_t n) {
    clear_error();
    if (!e || !params) return fail(A3D_E_ARG, "null engine or parameters");
    if (!e->learned) return fail(A3D_E_ARG, "the engine was not created with boundary A3D_BOUNDARY_LEARNED");
    if (n != (size_t)CL_NPARAM) return fail(A3D_E_ARG, "the closure takes %d parameters, got %zu", CL_NPARAM, n);
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(params[i])) return fail(A3D_E_ARG, "closure parameter %zu is not finite", i);
    CUDA_TRY(cudaSetDevice(e->device));
    if (!e->cl_packed) {
        e->clg = cl_geom(e->g.nnz, e->g.nnx, e->g.nny, e->g.ldz);
        e->cl_packed = (float *)e->dalloc(CL_NPARAM * sizeof(float));
        e->cl_zinv = (float *)e->dfield(4);
        e->cl_kap = (float *)e->dfield(4);
        const char *simt = getenv("A3D_CLOSURE_SIMT");
        e->cl_simt = simt && simt[0] == '1';
        if (e->cl_simt)
            e->cl_h = (__nv_bfloat16 *)e->dalloc((size_t)e->clg.hoff[6] * CL_CH * sizeof(__nv_bfloat16));
        else {
            e->cl_image = (uint16_t *)e->dalloc(cl_tc_image_halves() * sizeof(uint16_t));
            e->cl_y = (float4 *)e->dalloc((size_t)e->clg.hoff[6] * sizeof(float4));
        }
        if (!e->cl_packed || !e->cl_zinv || !e->cl_kap || (e->cl_simt ? !e->cl_h : (!e->cl_image || !e->cl_y))) {
            e->cl_packed = nullptr;
            return fail(A3D_E_NOMEM, "device allocation failed");
        }
        CUDA_TRY(cl_prepare());
        CUDA_TRY(cl_tc_prepare());
        const a3d_config &c = e->cfg;
        const float courant = c.dt / std::min(c.dx, std::min(c.dy, c.dz));
        CUDA_TRY(cl_launch_scales((const float *)e->field_alloc(e->rho, 4), (const float *)e->field_alloc(e->vp, 4),
                                  courant,
                                  (float *)e->field_alloc(e->cl_zinv, 4), (float *)e->field_alloc(e->cl_kap, 4),
                                  e->g.elems(), e->st));
    }
    std::vector<float> pk(CL_NPARAM);
    cl_pack_params(params, pk.data());
    CUDA_TRY(cudaMemcpyAsync(e->cl_packed, pk.data(), CL_NPARAM * sizeof(float), cudaMemcpyHostToDevice, e->st));
    if (e->cl_image) {
        std::vector<uint16_t> img(cl_tc_image_halves());
        cl_pack_tc(params, img.data());
        CUDA_TRY(cudaMemcpyAsync(e->cl_image, img.data(), img.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, e->st));
    }
    CUDA_TRY(cudaStreamSynchronize(e->st));
    return A3D_OK;
}

extern "C" int a3d_engine_set_tap(a3d_engine *e, const int *steps, int n, int off, float *dev_out) {
    clear_error();
    if (!e) return fail(A3D_E_ARG, "null engine");
    if (n == 0) {
        e->tap_steps.clear();
        e->tap_out = nullptr;
        return A3D_OK;
    }
    if (n < 0 || !steps || !dev_out) return fail(A3D_E_ARG, "taps need steps and an output buffer");
    if (e->cfg.physics == A3D_2ORDER || e->esz != 4) return fail(A3D_E_UNSUPPORTED, "taps are built for 1st-order FP32 engines");
    if (off < 0 || 2 * off >= std::min(e->g.nnz, std::min(e->g.nnx, e->g.nny)))
        return fail(A3D_E_ARG, "tap offset %d leaves an empty box", off);
    e->tap_steps.assign(steps, steps + n);
    e->tap_off = off;
    e->tap_out = dev_out;
    return A3D_OK;
}

extern "C" int a3d_engine_kernel_times(const a3d_engine *e, double *ms, long long *launches) {
    if (!e) return fail(A3D_E_ARG, "null engine");
    for (int k = 0; k < 2; ++k) {
        if (ms) ms[k] = e->kms[k];
        if (launches) launches[k] = e->klaunch[k];
    }
    return A3D_OK;
}

extern "C" int a3d_engine_describe(a3d_engine *e, char *buf, size_t n) {
    if (!e || !buf || n == 0) return fail(A3D_E_ARG, "null engine or buffer");
    if (!e->tuned) {
        CUDA_TRY(cudaSetDevice(e->device));
        int rc = e->autotune();
        if (rc) return rc;
    }
    snprintf(buf, n,
             "{\"grid\": [%d, %d, %d], \"ldz\": %d, \"pad\": %d, \"device_bytes\": %zu, \"fused\": %d, "
             "\"sig_v_log2\": %d, \"sig_p_log2\": %d, "
             "\"kernels\": [{\"tile_x\": %d, \"rows\": %d, \"depth\": %d, \"plan\": %d, \"rot\": %d, \"sblk\": %d, "
             "\"ms\": %.4f}, {\"tile_x\": %d, \"rows\": %d, \"depth\": %d, \"plan\": %d, \"rot\": %d, \"sblk\": %d, "
             "\"ms\": %.4f}]}",
             e->g.nnz, e->g.nnx, e->g.nny, e->g.ldz, e->g.pad, e->dev_bytes, (int)e->fused, ilogbf(e->sig_v),
             ilogbf(e->sig_p), e->tune[0].tx, e->tune[0].rows,
             e->tune[0].depth, e->tune[0].mode, e->tune[0].rot, e->tune[0].sblk, e->tune[0].ms, e->tune[1].tx,
             e->tune[1].rows, e->tune[1].depth, e->tune[1].mode, e->tune[1].rot, e->tune[1].sblk, e->tune[1].ms);
    return A3D_OK;
}

extern "C" const char *a3d_last_error(void) { return a3d::g_err.c_str(); }
