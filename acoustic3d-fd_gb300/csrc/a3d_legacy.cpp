// a3d_legacy.cpp — the reference's four extern "C" entry points, file in / file out.
//
// Each call: read the raw float32 model files (one bulk read per file instead of
// the reference's per-element fread), upload, run the shot(s) on the device,
// write the decimated record and the snapshots in the reference's byte layout.
// Differences from the reference, all on error paths: no exit(), no fread on a
// null FILE*, no division by a zero snapshot interval, no endless loop on a zero
// decimation step; each of those returns a status instead (message on stderr).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "a3d_engine.h"

using namespace a3d;

namespace {

int read_model(const char *fn, size_t n, std::vector<float> &out) {
    FILE *f = fn ? fopen(fn, "rb") : nullptr;
    if (!f) {
        printf("error open <%s>!\n", fn ? fn : "(null)");  // ..iso..:246
        return fail(A3D_E_IO, "cannot open model file <%s>", fn ? fn : "(null)");
    }
    out.resize(n);
    const size_t got = fread(out.data(), 4, n, f);
    fclose(f);
    if (got != n) return fail(A3D_E_IO, "model file <%s> holds %zu of %zu floats", fn, got, n);
    return A3D_OK;
}

// decimated record write, ..iso..:590-598 / 2O:483-490: offset is*nt*nx*ny floats,
// loops iy (step dgy/dy), ix (step dgx/dx), it (step dgt/dt), it fastest
int write_record(FILE *f, const std::vector<float> &rec, int is, int nx, int ny, int nt, int jx,
                 int jy, int jt) {
    std::vector<float> out;
    out.reserve((size_t)((nx + jx - 1) / jx) * ((ny + jy - 1) / jy) * ((nt + jt - 1) / jt));
    for (int iy = 0; iy < ny; iy += jy)
        for (int ix = 0; ix < nx; ix += jx)
            for (int it = 0; it < nt; it += jt) out.push_back(rec[(size_t)iy * nx * nt + (size_t)ix * nt + it]);
    if (fseek(f, (long)is * nt * nx * ny * (long)sizeof(float), SEEK_SET) != 0 ||
        fwrite(out.data(), 4, out.size(), f) != out.size())
        return fail(A3D_E_IO, "shot record write failed");
    return A3D_OK;
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
    int rc = a3d_engine_create(&e, &cfg, m[0], m[1], m[2], m[3], m[4], m[5], device);
    if (rc) return rc;
    std::vector<float> rec((size_t)cfg.nt * cfg.nx * cfg.ny);
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
        if (cudaMemcpy(rec.data(), e->rec, rec.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = fail(A3D_E_CUDA, "record copy failed");
            break;
        }
        rc = write_record(fshot, rec, is, cfg.nx, cfg.ny, cfg.nt, jx, jy, jt);
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
