// a3d_legacy.cpp — the reference's four extern "C" entry points, file in / file out.
//
// Each call: read the raw float32 model files (bulk reads over a few host threads
// instead of the reference's per-element fread), upload, run the shot(s) on the
// device, decimate the record on the device into the file's order, and write it
// through the pinned staging ring (one chunk copied while host threads write the
// previous one) — the reference copies the whole record to the host and writes it
// one float at a time (..iso..:589-598); snapshots in the reference's byte layout.
// Differences from the reference, all on error paths: no exit(), no fread on a
// null FILE*, no division by a zero snapshot interval, no endless loop on a zero
// decimation step; each of those returns a status instead (message on stderr).
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "a3d_engine.h"

using namespace a3d;

namespace {

// Phase timing: with A3D_LEGACY_TIMING set, each drop-in call prints one JSON line
// to stderr with the seconds spent reading the model files, creating the engine
// (upload, padding, set-up, tuning when the grid is new), in the time loops and in
// writing the records — the counterpart of the reference's clock() print (2O:479).
struct PhaseClock {
    using clk = std::chrono::steady_clock;
    bool on = getenv("A3D_LEGACY_TIMING") != nullptr;
    clk::time_point t = clk::now();
    double read = 0, create = 0, loop = 0, write = 0;
    double lap() {
        const clk::time_point n = clk::now();
        const double d = std::chrono::duration<double>(n - t).count();
        t = n;
        return d;
    }
    void print(const char *entry) const {
        if (on)
            fprintf(stderr, "{\"entry\": \"%s\", \"read_s\": %.4f, \"create_s\": %.4f, \"loop_s\": %.4f, "
                            "\"write_s\": %.4f}\n", entry, read, create, loop, write);
    }
};
thread_local PhaseClock *g_phase = nullptr;  // the current call's clock (legacy entry points only)
struct PhaseScope {  // one per drop-in call: installs the clock, prints it on the way out
    PhaseClock clock;
    const char *entry;
    explicit PhaseScope(const char *e) : entry(e) {
        if (clock.on) g_phase = &clock;
    }
    ~PhaseScope() {
        if (g_phase == &clock) {
            clock.print(entry);
            g_phase = nullptr;
        }
    }
};

// runs f(lo, hi) over [0, n) split into up to `maxth` ranges of at least `min_part`
// units, one per host thread (this thread takes the first); returns the first error
template <class F>
int par_ranges(size_t n, size_t min_part, size_t maxth, F f) {
    size_t nth = std::min<size_t>(maxth, std::max<size_t>(1, n / std::max<size_t>(min_part, 1)));
    nth = std::min<size_t>(nth, std::max(1u, std::thread::hardware_concurrency()));
    const size_t part = (n + nth - 1) / nth;
    std::vector<int> rc(nth, A3D_OK);
    std::vector<std::thread> ts;
    size_t k = 1;
    try {
        for (; k < nth; ++k) {
            const size_t lo = k * part, hi = std::min(n, lo + part);
            if (lo >= hi) break;
            ts.emplace_back([&, k, lo, hi] { rc[k] = f(lo, hi); });
        }
    } catch (...) {  // a thread could not be started: this thread takes what is left
    }
    rc[0] = f(0, std::min(n, part));
    if (!rc[0] && k < nth && k * part < n) rc[0] = f(k * part, n);
    for (auto &t : ts) t.join();
    for (int r : rc)
        if (r) return r;
    return A3D_OK;
}

// whole-file read of n floats: pread over up to 8 host threads for large files
int read_model(const char *fn, size_t n, std::vector<float> &out) {
    const int fd = fn ? open(fn, O_RDONLY) : -1;
    if (fd < 0) {
        printf("error open <%s>!\n", fn ? fn : "(null)");  // ..iso..:246
        return fail(A3D_E_IO, "cannot open model file <%s>", fn ? fn : "(null)");
    }
    out.resize(n);
    const size_t bytes = n * 4;
    char *dst = reinterpret_cast<char *>(out.data());
    size_t short_at = bytes;  // first byte a thread could not read (bytes: none)
    std::mutex mu;
    par_ranges(bytes, size_t(16) << 20, 8, [&](size_t lo, size_t hi) {
        size_t off = lo;
        while (off < hi) {
            const ssize_t got = pread(fd, dst + off, hi - off, (off_t)off);
            if (got < 0 && errno == EINTR) continue;
            if (got <= 0) break;
            off += (size_t)got;
        }
        if (off < hi) {
            std::lock_guard<std::mutex> lk(mu);
            short_at = std::min(short_at, off);
        }
        return A3D_OK;
    });
    close(fd);
    if (short_at < bytes)
        return fail(A3D_E_IO, "model file <%s> holds %zu of %zu floats", fn, short_at / 4, n);
    return A3D_OK;
}

// receivers (iy step jy, ix step jx) and samples (it step jt) of the record
// [ny][nx][nt] into the file's order, it fastest (..iso..:590-598 / 2O:483-490)
__global__ void gather_record(const float *__restrict__ rec, float *__restrict__ out, int nx, int nt, int jx,
                              int jy, int jt, int ndx, int ndt, size_t total) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int itd = (int)(i % ndt);
        const size_t tr = i / ndt;
        const int ixd = (int)(tr % ndx), iyd = (int)(tr / ndx);
        out[i] = rec[((size_t)iyd * jy * nx + (size_t)ixd * jx) * nt + (size_t)itd * jt];
    }
}

// writes the decimated record of the device record rec_dev ([ny][nx][nt]) at byte
// offset is*nt*nx*ny*4 of the file (the reference's fseek, ..iso..:591): the gather
// runs on the device, the bytes come through the pinned staging ring, and up to 4
// host threads write each chunk with pwrite while the next one is copied
int write_record(FILE *f, const float *rec_dev, int is, int nx, int ny, int nt, int jx, int jy, int jt,
                 cudaStream_t st) {
    const int ndx = (nx + jx - 1) / jx, ndy = (ny + jy - 1) / jy, ndt = (nt + jt - 1) / jt;
    const size_t total = (size_t)ndx * ndy * ndt;
    const float *src = rec_dev;
    float *tmp = nullptr;
    if (jx != 1 || jy != 1 || jt != 1) {
        if (cudaMalloc(&tmp, total * 4) != cudaSuccess) return fail(A3D_E_NOMEM, "record gather buffer");
        gather_record<<<1024, 256, 0, st>>>(rec_dev, tmp, nx, nt, jx, jy, jt, ndx, ndt, total);
        if (cudaGetLastError() != cudaSuccess) {
            cudaFree(tmp);
            return fail(A3D_E_CUDA, "record gather launch failed");
        }
        src = tmp;
    }
    if (fflush(f) != 0) {
        cudaFree(tmp);
        return fail(A3D_E_IO, "shot record write failed");
    }
    const int fd = fileno(f);
    const off_t base = (off_t)is * nt * nx * ny * (off_t)sizeof(float);
    const int rc = stage_from_device(src, total * 4, st, [&](const unsigned char *p, size_t off, size_t n) {
        return par_ranges(n, size_t(4) << 20, 4, [&](size_t lo, size_t hi) {
            while (lo < hi) {
                const ssize_t w = pwrite(fd, p + lo, hi - lo, base + (off_t)(off + lo));
                if (w < 0 && errno == EINTR) continue;
                if (w <= 0) return fail(A3D_E_IO, "shot record write failed");
                lo += (size_t)w;
            }
            return A3D_OK;
        });
    });
    if (tmp) cudaFree(tmp);
    return rc;
}

// Call trace: with A3D_LEGACY_TRACE set to a file name, every drop-in call appends
// one JSON line with its entry point and each argument as the library received it,
// before any other work (so a caller's argument marshalling can be checked on a
// machine without a GPU).  Off when the variable is unset.
struct Trace {
    std::string s;
    bool on = false;
    explicit Trace(const char *entry) {
        on = getenv("A3D_LEGACY_TRACE") != nullptr;
        if (on) s = std::string("{\"entry\": \"") + entry + "\"";
    }
    Trace &str(const char *k, const char *v) {
        if (!on) return *this;
        s += std::string(", \"") + k + "\": ";
        if (!v) { s += "null"; return *this; }
        s += "\"";
        for (const char *c = v; *c; ++c) {
            if (*c == '"' || *c == '\\') s += '\\';
            if ((unsigned char)*c >= 0x20) s += *c;
        }
        s += "\"";
        return *this;
    }
    Trace &i(const char *k, long long v) {
        if (on) s += std::string(", \"") + k + "\": " + std::to_string(v);
        return *this;
    }
    Trace &f(const char *k, float v) {
        if (!on) return *this;
        char b[64];
        snprintf(b, sizeof b, "%.9g", (double)v);
        s += std::string(", \"") + k + "\": " + b;
        return *this;
    }
    Trace &b(const char *k, bool v) {
        if (on) s += std::string(", \"") + k + "\": " + (v ? "true" : "false");
        return *this;
    }
    ~Trace() {
        if (!on) return;
        if (FILE *t = fopen(getenv("A3D_LEGACY_TRACE"), "a")) {
            fprintf(t, "%s}\n", s.c_str());
            fclose(t);
        }
    }
};

// the geometry arguments every entry point shares, in the reference's order
void trace_geometry(Trace &t, int is, int ns, int nx, int ny, int nz, float dx, float dy, float dz, int sxbeg,
                    int sybeg, int szbeg, int jsx, int jsy, int jsz, float dgx, float dgy, float dgt, int nt) {
    t.i("is", is).i("ns", ns).i("nx", nx).i("ny", ny).i("nz", nz).f("dx", dx).f("dy", dy).f("dz", dz);
    t.i("sxbeg", sxbeg).i("sybeg", sybeg).i("szbeg", szbeg).i("jsx", jsx).i("jsy", jsy).i("jsz", jsz);
    t.f("dgx", dgx).f("dgy", dgy).f("dgt", dgt).i("nt", nt);
}

int steps(float dg, float d, const char *what, int &j) {
    j = (int)(dg / d);
    if (j <= 0) return fail(A3D_E_ARG, "%s sampling step %g / %g rounds to %d", what, dg, d, j);
    return A3D_OK;
}

struct Snapper {
    std::string prefix;  // FNsnap
    const char *fmt;     // "ishot_%d_it_%d.bin" or "ishot_%dit_%d.bin"
    int is = 0;
    int nbytes = 0;
    bool io_error = false;
    int write(int it, const float *d) {
        char name[64];
        snprintf(name, sizeof name, fmt, is, it);
        std::string path = prefix + name;
        FILE *f = fopen(path.c_str(), "wb");
        if (!f) {
            printf("cannot write snapfile\n");  // ..iso..:578
            io_error = true;
            return A3D_OK;
        }
        if (fwrite(d, 1, (size_t)nbytes, f) != (size_t)nbytes) io_error = true;
        fclose(f);
        return A3D_OK;
    }
};

int run_legacy(const a3d_config &cfg, const std::vector<const float *> &m, int device,
               const std::vector<a3d_shot> &shots, const std::vector<int> &shot_index, FILE *fshot,
               int jx, int jy, int jt, Snapper *snap, std::function<bool(int, int)> want) {
    a3d_engine *e = nullptr;
    if (g_phase) g_phase->read += g_phase->lap();
    int rc = a3d_engine_create(&e, &cfg, m[0], m[1], m[2], m[3], m[4], m[5], device);
    if (rc) return rc;
    if (g_phase) g_phase->create += g_phase->lap();
    for (size_t k = 0; k < shots.size() && !rc; ++k) {
        const int is = shot_index[k];
        SnapHook hook;
        if (snap) {
            snap->is = is;
            hook.want = [&](int it) { return want(is, it); };
            hook.take = [&](int it, const float *d) { return snap->write(it, d); };
        }
        rc = e->run(shots[k], nullptr, snap ? &hook : nullptr, nullptr);
        if (rc) break;
        if (g_phase) g_phase->loop += g_phase->lap();
        rc = write_record(fshot, e->rec, is, cfg.nx, cfg.ny, cfg.nt, jx, jy, jt, e->st);
        if (g_phase) g_phase->write += g_phase->lap();
    }
    a3d_engine_destroy(e);
    if (!rc && snap && snap->io_error) rc = fail(A3D_E_IO, "a snapshot file could not be written");
    return rc;
}

a3d_config base_cfg(int physics, int nx, int ny, int nz, float dx, float dy, float dz, int nt, float dt,
                    float fm) {
    a3d_config c{};
    c.physics = physics;
    c.nx = nx; c.ny = ny; c.nz = nz;
    c.dx = dx; c.dy = dy; c.dz = dz;
    c.nt = nt; c.dt = dt; c.fm = fm;
    c.wtype = 1;
    c.npml = 0;    // the reference's width
    c.rec_z = -1;  // the reference's depth
    c.storage = A3D_FP32;
    return c;
}

}  // namespace

extern "C" int cuda_3dfd(char *FNvel, char *FNsnap, char *FNshot, int is, int ns, int nx, int ny, int nz,
                         float dx, float dy, float dz, int sxbeg, int sybeg, int szbeg, int jsx, int jsy,
                         int jsz, float dgx, float dgy, float dgt, int nt, int kt, float dt, float fm,
                         bool show_snapshot, bool cut_directwave, int snap_interval, int cudaDevicei) {
    (void)ns; (void)kt; (void)cut_directwave; (void)snap_interval;  // unused by the reference too
    {
        Trace t("cuda_3dfd");
        t.str("FNvel", FNvel).str("FNsnap", FNsnap).str("FNshot", FNshot);
        trace_geometry(t, is, ns, nx, ny, nz, dx, dy, dz, sxbeg, sybeg, szbeg, jsx, jsy, jsz, dgx, dgy, dgt, nt);
        t.i("kt", kt).f("dt", dt).f("fm", fm).b("show_snapshot", show_snapshot).b("cut_directwave", cut_directwave);
        t.i("snap_interval", snap_interval).i("cudaDevicei", cudaDevicei);
    }
    PhaseScope phase("cuda_3dfd");
    clear_error();
    int jx, jy, jt, rc;
    if ((rc = steps(dgx, dx, "receiver x", jx)) || (rc = steps(dgy, dy, "receiver y", jy)) ||
        (rc = steps(dgt, dt, "time", jt)))
        return rc;
    std::vector<float> vel;
    if ((rc = read_model(FNvel, (size_t)nx * ny * nz, vel))) return rc;
    FILE *fshot = fopen(FNshot, "wb");
    if (!fshot) return fail(A3D_E_IO, "cannot open shot file <%s>", FNshot ? FNshot : "(null)");
    a3d_config c = base_cfg(A3D_2ORDER, nx, ny, nz, dx, dy, dz, nt, dt, fm);
    // cuda_set_s (2O:45-52): shot `is` sits at (szbeg+is*jsz, sxbeg+is*jsx, sybeg+is*jsy)
    std::vector<a3d_shot> shots{{sxbeg + is * jsx, sybeg + is * jsy, szbeg + is * jsz}};
    Snapper sn{FNsnap ? FNsnap : "", "ishot_%d_it_%d.bin"};
    sn.nbytes = nx * ny * nz * 4;
    rc = run_legacy(c, {vel.data(), nullptr, nullptr, nullptr, nullptr, nullptr}, cudaDevicei, shots, {is},
                    fshot, jx, jy, jt, show_snapshot ? &sn : nullptr,
                    [](int, int it) { return it % 500 == 0; });  // 2O:456
    fclose(fshot);
    return rc;
}

static int run_first_order(int physics, const char *FNvel, const char *FNrho, const char *FNeps,
                           const char *FNdel, const char *FNsnap, const char *FNshot, int ns, int nx,
                           int ny, int nz, float dx, float dy, float dz, int sxbeg, int sybeg, int szbeg,
                           int jsx, int jsy, float dgx, float dgy, float dgt, int nt, float dt, int wtype,
                           float fm, bool show_snapshot, bool cut_directwave, int snap_interval,
                           int device) {
    clear_error();
    int jx, jy, jt, rc;
    if ((rc = steps(dgx, dx, "receiver x", jx)) || (rc = steps(dgy, dy, "receiver y", jy)) ||
        (rc = steps(dgt, dt, "time", jt)))
        return rc;
    if (show_snapshot && snap_interval <= 0)
        return fail(A3D_E_ARG, "snapshot interval %d must be positive", snap_interval);
    if (ns < 1) return fail(A3D_E_ARG, "ns = %d", ns);
    FILE *fshot = fopen(FNshot, "wb");
    if (!fshot) return fail(A3D_E_IO, "cannot open shot file <%s>", FNshot ? FNshot : "(null)");
    const size_t n = (size_t)nx * ny * nz;
    std::vector<float> vel, rho, eps, del;
    rc = read_model(FNvel, n, vel);
    if (!rc) rc = read_model(FNrho, n, rho);
    if (!rc && physics == A3D_VTI) rc = read_model(FNeps, n, eps);
    if (!rc && physics == A3D_VTI) rc = read_model(FNdel, n, del);
    if (rc) { fclose(fshot); return rc; }
    a3d_config c = base_cfg(physics, nx, ny, nz, dx, dy, dz, nt, dt, fm);
    c.wtype = physics == A3D_ISO ? wtype : 1;  // VTI forces the Ricker (..vti..:413)
    c.mute = cut_directwave;
    // shots is = 0..ns-1 at (sxbeg + is*jsx, sybeg, szbeg) (..iso..:500, 63-64 with nsx = ns)
    std::vector<a3d_shot> shots;
    std::vector<int> idx;
    for (int k = 0; k < ns; ++k) {
        shots.push_back({sxbeg + (k % ns) * jsx, sybeg + (k / ns) * jsy, szbeg});
        idx.push_back(k);
    }
    Snapper sn{FNsnap ? FNsnap : "", physics == A3D_ISO ? "ishot_%dit_%d.bin" : "ishot_%d_it_%d.bin"};
    sn.nbytes = nx * ny * nz * 4;
    rc = run_legacy(c, {vel.data(), rho.data(), physics == A3D_VTI ? eps.data() : nullptr,
                        physics == A3D_VTI ? del.data() : nullptr, nullptr, nullptr},
                    device, shots, idx, fshot, jx, jy, jt, show_snapshot ? &sn : nullptr,
                    [snap_interval](int, int it) { return it % snap_interval == 0; });
    fclose(fshot);
    return rc;
}

extern "C" int cuda_3dfd_1order(char *FNvel, char *FNrho, char *FNsnap, char *FNshot, int is, int ns,
                                int nx, int ny, int nz, float dx, float dy, float dz, int sxbeg, int sybeg,
                                int szbeg, int jsx, int jsy, int jsz, float dgx, float dgy, float dgt, int nt,
                                float dt, int wtype, float fm, bool show_snapshot, bool cut_directwave,
                                int snap_interval, int cudaDevicei) {
    (void)is; (void)jsz;  // the reference's shot loop overwrites `is` (..iso..:500)
    {
        Trace t("cuda_3dfd_1order");
        t.str("FNvel", FNvel).str("FNrho", FNrho).str("FNsnap", FNsnap).str("FNshot", FNshot);
        trace_geometry(t, is, ns, nx, ny, nz, dx, dy, dz, sxbeg, sybeg, szbeg, jsx, jsy, jsz, dgx, dgy, dgt, nt);
        t.f("dt", dt).i("wtype", wtype).f("fm", fm).b("show_snapshot", show_snapshot);
        t.b("cut_directwave", cut_directwave).i("snap_interval", snap_interval).i("cudaDevicei", cudaDevicei);
    }
    PhaseScope phase("cuda_3dfd_1order");
    return run_first_order(A3D_ISO, FNvel, FNrho, nullptr, nullptr, FNsnap, FNshot, ns, nx, ny, nz, dx, dy, dz,
                           sxbeg, sybeg, szbeg, jsx, jsy, dgx, dgy, dgt, nt, dt, wtype, fm, show_snapshot,
                           cut_directwave, snap_interval, cudaDevicei);
}

extern "C" int cuda_3dfd_vti(char *FNvel, char *FNrho, char *FNepsilon, char *FNdelta, char *FNsnap,
                             char *FNshot, int is, int ns, int nx, int ny, int nz, float dx, float dy,
                             float dz, int sxbeg, int sybeg, int szbeg, int jsx, int jsy, int jsz, float dgx,
                             float dgy, float dgt, int nt, float dt, float fm, bool show_snapshot,
                             bool cut_directwave, int snap_interval, int cudaDevicei) {
    (void)is; (void)jsz;
    {
        Trace t("cuda_3dfd_vti");
        t.str("FNvel", FNvel).str("FNrho", FNrho).str("FNepsilon", FNepsilon).str("FNdelta", FNdelta);
        t.str("FNsnap", FNsnap).str("FNshot", FNshot);
        trace_geometry(t, is, ns, nx, ny, nz, dx, dy, dz, sxbeg, sybeg, szbeg, jsx, jsy, jsz, dgx, dgy, dgt, nt);
        t.f("dt", dt).f("fm", fm).b("show_snapshot", show_snapshot).b("cut_directwave", cut_directwave);
        t.i("snap_interval", snap_interval).i("cudaDevicei", cudaDevicei);
    }
    PhaseScope phase("cuda_3dfd_vti");
    return run_first_order(A3D_VTI, FNvel, FNrho, FNepsilon, FNdelta, FNsnap, FNshot, ns, nx, ny, nz, dx, dy,
                           dz, sxbeg, sybeg, szbeg, jsx, jsy, dgx, dgy, dgt, nt, dt, 1, fm, show_snapshot,
                           cut_directwave, snap_interval, cudaDevicei);
}

extern "C" int cuda_3dfd_tti(char *FNvel, char *FNrho, char *FNepsilon, char *FNdelta, char *FNtheta,
                             char *FNpsi, char *FNsnap, char *FNshot, int is, int ns, int nx, int ny, int nz,
                             float dx, float dy, float dz, int sxbeg, int sybeg, int szbeg, int jsx, int jsy,
                             int jsz, float dgx, float dgy, float dgt, int nt, float dt, float fm,
                             bool show_snapshot, bool cut_directwave, int snap_interval, int cudaDevicei) {
    (void)FNrho; (void)is; (void)ns; (void)jsx; (void)jsy; (void)jsz; (void)show_snapshot; (void)snap_interval;
    {
        Trace t("cuda_3dfd_tti");
        t.str("FNvel", FNvel).str("FNrho", FNrho).str("FNepsilon", FNepsilon).str("FNdelta", FNdelta);
        t.str("FNtheta", FNtheta).str("FNpsi", FNpsi).str("FNsnap", FNsnap).str("FNshot", FNshot);
        trace_geometry(t, is, ns, nx, ny, nz, dx, dy, dz, sxbeg, sybeg, szbeg, jsx, jsy, jsz, dgx, dgy, dgt, nt);
        t.f("dt", dt).f("fm", fm).b("show_snapshot", show_snapshot).b("cut_directwave", cut_directwave);
        t.i("snap_interval", snap_interval).i("cudaDevicei", cudaDevicei);
    }
    PhaseScope phase("cuda_3dfd_tti");
    clear_error();
    FILE *fshot = FNshot ? fopen(FNshot, "wb") : nullptr;
    if (!fshot) {  // ..tti..:429-432
        printf("cannot write shot file");
        fail(A3D_E_IO, "cannot open shot file <%s>", FNshot ? FNshot : "(null)");
        return 1;
    }
    int jx, jy, jt, rc;
    if ((rc = steps(dgx, dx, "receiver x", jx)) || (rc = steps(dgy, dy, "receiver y", jy)) ||
        (rc = steps(dgt, dt, "time", jt))) {
        fclose(fshot);
        return rc;
    }
    const size_t n = (size_t)nx * ny * nz;
    std::vector<float> vel, eps, del, th, ph;
    rc = read_model(FNvel, n, vel);
    if (!rc) rc = read_model(FNepsilon, n, eps);
    if (!rc) rc = read_model(FNdelta, n, del);
    if (!rc) rc = read_model(FNtheta, n, th);
    if (!rc) rc = read_model(FNpsi, n, ph);
    if (rc) { fclose(fshot); return rc; }
    a3d_config c = base_cfg(A3D_TTI, nx, ny, nz, dx, dy, dz, nt, dt, fm);
    c.mute = cut_directwave;
    Snapper sn{FNsnap ? FNsnap : "", "ishot_%d_it_%d.bin"};
    sn.nbytes = nx * ny * nz * 4;
    // ns is forced to 1 (..tti..:439); snapshots every 100 steps, it != 0 (..tti..:593)
    rc = run_legacy(c, {vel.data(), nullptr, eps.data(), del.data(), th.data(), ph.data()}, cudaDevicei,
                    {{sxbeg, sybeg, szbeg}}, {0}, fshot, jx, jy, jt, &sn,
                    [](int s, int it) { return s == 0 && it != 0 && it % 100 == 0; });
    fclose(fshot);
    return rc;
}
