// a3d_noalloc.cu — a 2nd-order time step that allocates no device memory.
//
// For callers that cannot call cudaMalloc — a host framework that owns every
// device allocation through its own pool, or a process whose device memory is
// provisioned up front — this entry point advances one time step on device
// buffers the caller provides.  The step kernel's scratch (the three per-axis
// sponge-factor tables and the kernel error word) lives in the file-scope
// array below instead of in allocations: A3D_NOALLOC_SCRATCH_BYTES (about 97 KB)
// of device memory that every GPU which loads this library holds until exit.
//
// Set-up: the first call on a device, with that device current, looks the
// array's device address up with cudaGetSymbolAddress (the host-side name of a
// __device__ array is only a stand-in, not a device address); make that first
// call before any stream capture.  The address is kept per device together with
// the id of the device's context it was found in; when the application resets the
// device (cudaDeviceReset) the next call sees a new context and looks it up again.
// Every call shares the array and rewrites it (tables recomputed, error word
// cleared), so calls that overlap on the GPU race.
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/acoustic3d.h"
#include "a3d_engine.h"

namespace a3d {

constexpr int NOALLOC_TABLE_OFF = 256;  // error word, then the tables
static __device__ __align__(256) unsigned char g_noalloc_scratch[A3D_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64];                 // device address of the scratch array, per device
static unsigned long long g_noalloc_ctx[64];   // id of the context it was looked up in

// id of the current context (unique for the process's lifetime, never reused), 0 if
// the driver cannot tell; through the runtime's driver entry points, no extra link
static unsigned long long current_context_id() {
    static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_cur || !get_id || get_cur(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// sponge factor tables of the three padded axes, as hi/lo floats (setup, FP64)
__global__ void noalloc_sponge_tables(float2 *fz, float2 *fx, float2 *fy, int nz, int nx, int ny,
                                      int npd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n3[3] = {nz, nx, ny};
    float2 *t3[3] = {fz, fx, fy};
    const float qp = -0.25f;
    for (int a = 0; a < 3; ++a) {
        const int nn = n3[a] + 2 * MM + 2 * npd;
        if (i >= nn) continue;
        double F = 0.0;
        if (i < npd) {
            const double r = (double)(npd - i) / (1.0 * npd);
            F = (double)qp * (r * r) + 1;
        } else if (i >= 2 * MM + npd + n3[a]) {
            const double r = (double)(i - 2 * MM - npd - n3[a]) / (1.0 * npd);
            F = (double)qp * (r * r) + 1;
        }
        const float hi = (float)F;
        t3[a][i] = make_float2(hi, (float)(F - (double)hi));
    }
}

// with `device` current: the scratch array's device address on it
static int noalloc_setup(int device, void **out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_noalloc_ptr[device] || ctx == 0 || ctx != g_noalloc_ctx[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(A3D_E_CUDA, "cudaGetSymbolAddress of the step scratch failed: %s", cudaGetErrorString(e));
        g_noalloc_ptr[device] = p;
        g_noalloc_ctx[device] = ctx;
    }
    *out = g_noalloc_ptr[device];
    return A3D_OK;
}

// makes `device` current for the call's lifetime and gives the caller's current
// device back on every return path
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int device) {
        if ((err = cudaGetDevice(&prev)) != cudaSuccess) { prev = -1; return; }
        if (prev != device) err = cudaSetDevice(device);
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace a3d

using namespace a3d;

extern "C" int a3d_2order_step_noalloc(const float *cur, float *prev_next, const float *vv, float *rec,
                                       int nx, int ny, int nz, int npd, int ldz, float dx, float dy,
                                       float dz, int sx, int sy, int sz, float w_next, int rec_z, int it,
                                       int nt, int device) {
    clear_error();
    if (device < 0 || device >= 64) return fail(A3D_E_ARG, "device %d out of range", device);
    if (!cur || !prev_next || !vv) return fail(A3D_E_ARG, "null field pointer");
    if (nx < 1 || ny < 1 || nz < 1 || npd < 1 || nt < 1 || it < 0 || it >= nt)
        return fail(A3D_E_ARG, "bad sizes (nx %d ny %d nz %d npd %d it %d nt %d)", nx, ny, nz, npd, it, nt);
    const int pad = MM + npd, nnx = nx + 2 * pad, nny = ny + 2 * pad, nnz = nz + 2 * pad;
    if (nnx > A3D_NOALLOC_MAX_AXIS || nny > A3D_NOALLOC_MAX_AXIS || nnz > A3D_NOALLOC_MAX_AXIS)
        return fail(A3D_E_ARG, "padded grid %dx%dx%d exceeds the %d-cell axis limit of the no-allocation step",
                    nnz, nnx, nny, A3D_NOALLOC_MAX_AXIS);
    if (ldz < nnz || ldz % 4 != 0) return fail(A3D_E_ARG, "ldz %d must be >= %d and a multiple of 4", ldz, nnz);
    // the step kernel indexes a field with 32-bit offsets, as the engine does
    if ((unsigned long long)ldz * (unsigned long long)nnx * (unsigned long long)nny > (unsigned long long)INT32_MAX)
        return fail(A3D_E_ARG, "padded grid of %llu cells (ldz %d x %d x %d) exceeds the 2^31 - 1 cell limit",
                    (unsigned long long)ldz * nnx * nny, ldz, nnx, nny);
    if (((uintptr_t)cur | (uintptr_t)prev_next | (uintptr_t)vv) % 16 != 0)
        return fail(A3D_E_ARG, "field pointers must be 16-byte aligned");
    if (sx < 0 || sx >= nx || sy < 0 || sy >= ny || sz < 0 || sz >= nz || rec_z < 0 || rec_z >= nz)
        return fail(A3D_E_ARG, "shot or receiver depth outside the model");
    DeviceScope scope(device);
    cudaError_t ce = scope.err;
    if (ce != cudaSuccess) return fail(A3D_E_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(ce));
    void *scratch = nullptr;
    int rc = noalloc_setup(device, &scratch);
    if (rc) return rc;
    int *err = (int *)scratch;
    float2 *fz = (float2 *)((unsigned char *)scratch + NOALLOC_TABLE_OFF);
    float2 *fx = fz + A3D_NOALLOC_MAX_AXIS, *fy = fx + A3D_NOALLOC_MAX_AXIS;
    if ((ce = cudaMemsetAsync(err, 0, sizeof(int), 0)) != cudaSuccess)
        return fail(A3D_E_CUDA, "clearing the error word: %s", cudaGetErrorString(ce));
    const int nmax = nnz > nnx ? (nnz > nny ? nnz : nny) : (nnx > nny ? nnx : nny);
    noalloc_sponge_tables<<<(nmax + 255) / 256, 256>>>(fz, fx, fy, nz, nx, ny, npd);
    // tensor maps over the caller's buffers (host-side descriptors, no allocation)
    Grid g;
    g.nx = nx; g.ny = ny; g.nz = nz; g.pad = pad;
    g.nnx = nnx; g.nny = nny; g.nnz = nnz; g.ldz = ldz;
    K2OLaunch L{};
    L.tx = 8;
    L.rows = 2;
    L.fp64 = false;
    if ((rc = make_field_map(&L.tm_cur, cur, false, g, 40, L.tx + 8)) ||
        (rc = make_field_map(&L.tm_prev, prev_next, false, g, 32, L.tx)) ||
        (rc = make_field_map(&L.tm_vv, vv, false, g, 32, L.tx)))
        return rc;
    L.ybuf = prev_next;
    K2OParams &p = L.p;
    p.nnz = nnz; p.nnx = nnx; p.nny = nny; p.ldz = ldz;
    p.nx = nx; p.ny = ny;
    p.gz = pad + rec_z; p.rx0 = pad; p.ry0 = pad;
    p.fz = fz; p.fx = fx; p.fy = fy;
    p.dz2 = (float)(1.0 / (double)(dz * dz));
    p.dx2 = (float)(1.0 / (double)(dx * dx));
    p.dy2 = (float)(1.0 / (double)(dy * dy));
    p.s_x = sx + pad; p.s_y = sy + pad; p.s_z = sz + pad;
    p.w_next = w_next;
    p.rec = rec;
    p.mute_nt = nullptr;
    p.it = it;
    p.nt = nt;
    p.err = err;
    if (!rec) p.gz = -1;  // no receiver row: nothing is recorded
    if ((ce = launch_k2o(L, 0)) != cudaSuccess) return fail(A3D_E_CUDA, "step launch: %s", cudaGetErrorString(ce));
    int herr = 0;
    if ((ce = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, 0)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(0)) != cudaSuccess)
        return fail(A3D_E_CUDA, "step: %s", cudaGetErrorString(ce));
    if (herr) return fail(A3D_E_KERNEL, "the step kernel gave up a bounded wait (code %d)", herr);
    return A3D_OK;
}
