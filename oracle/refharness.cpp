// refharness.cpp — runs the reference's own CUDA kernels on a GPU machine.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles the reference's four
// .cu files (device code only) into oracle/_ref/*.cubin; this program loads those
// cubins with the CUDA runtime's library API and replays each engine's host loop
// (the extern "C" drivers of the reference, restated here: host code compiled on
// the x86 build machine does not run on the aarch64 GPU machine, there is no
// aarch64 cross compiler on the build machine, and the reference sources are not
// present on the GPU machine, so only the device code travels, as cubins).  Its
// outputs are the golden records that pin the CPU oracle, and its timings are the
// "reference kernels rebuilt for sm_103a" GPU baseline.
//
// Usage: refharness CUBIN_DIR CASE_DIR [timing_steps]
//   CASE_DIR/case.txt  "key value" lines: engine (2o|iso|vti|tti) nx ny nz dx dy dz
//                      sx sy sz nt dt fm wtype mute
//   CASE_DIR/{vel,rho,eps,del,theta,phi}.bin   raw float32 models, z fastest
//   optional key "sync 0" drops the device synchronisations the reference's host
//   loops make after their launches (ISO: 5 per step, ..iso..:523-565; VTI: 4,
//   ..vti..:557-598; TTI and 2O: none); by default they are made, as the reference
//   makes them, so the loop time is that of the reference's own host loop.
// Writes CASE_DIR/rec_ref.bin: the full record rec[it + nt*(ix + nx*iy)] (float32),
// before the direct-wave mute, and, when mute is 1, CASE_DIR/rec_mute.bin after it;
// prints one line "refharness <engine> ms=<loop time> steps=<n>".
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#define CK(x)                                                                             \
    do {                                                                                  \
        cudaError_t e_ = (x);                                                             \
        if (e_ != cudaSuccess) {                                                          \
            fprintf(stderr, "refharness: %s failed: %s (line %d)\n", #x,                  \
                    cudaGetErrorString(e_), __LINE__);                                    \
            exit(3);                                                                      \
        }                                                                                 \
    } while (0)

static const int MM = 4;

struct Lib {
    cudaLibrary_t lib{};
    std::vector<cudaKernel_t> ks;
    std::vector<std::string> names;
    void load(const std::string &path) {
        CK(cudaLibraryLoadFromFile(&lib, path.c_str(), nullptr, nullptr, 0, nullptr, nullptr, 0));
        unsigned n = 0;
        CK(cudaLibraryGetKernelCount(&n, lib));
        ks.resize(n);
        CK(cudaLibraryEnumerateKernels(ks.data(), n, lib));
        for (auto k : ks) {
            const char *nm = nullptr;
            CK(cudaFuncGetName(&nm, (const void *)k));
            names.emplace_back(nm ? nm : "");
        }
    }
    // kernels are C++ functions: match the Itanium-mangled prefix "_Z<len><name>"
    cudaKernel_t get(const char *name) {
        std::string pre = "_Z" + std::to_string(strlen(name)) + name;
        for (size_t i = 0; i < ks.size(); ++i)
            if (names[i].compare(0, pre.size(), pre) == 0) return ks[i];
        fprintf(stderr, "refharness: kernel %s not found\n", name);
        exit(3);
    }
};

template <class... A>
static void launch(cudaKernel_t k, dim3 g, dim3 b, A... args) {
    void *argv[] = {(void *)&args...};
    CK(cudaLaunchKernel((const void *)k, g, b, argv, 0, 0));
}

struct Case {
    std::map<std::string, std::string> kv;
    std::string dir;
    int i(const char *k) const { return atoi(kv.at(k).c_str()); }
    float f(const char *k) const { return (float)atof(kv.at(k).c_str()); }
    std::string s(const char *k) const { return kv.at(k); }
};

static std::vector<float> read_model(const Case &c, const char *name, size_t n) {
    std::vector<float> v(n);
    std::string p = c.dir + "/" + name + ".bin";
    FILE *f = fopen(p.c_str(), "rb");
    if (!f || fread(v.data(), 4, n, f) != n) {
        fprintf(stderr, "refharness: cannot read %s\n", p.c_str());
        exit(2);
    }
    fclose(f);
    return v;
}

// interior copy + edge replication, as read_file + pad_vv (ISO:198-260) produce
static std::vector<float> pad(const std::vector<float> &m, int nx, int ny, int nz, int p) {
    int nnx = nx + 2 * p, nny = ny + 2 * p, nnz = nz + 2 * p;
    std::vector<float> o((size_t)nnx * nny * nnz);
    for (int iy = 0; iy < nny; ++iy)
        for (int ix = 0; ix < nnx; ++ix)
            for (int iz = 0; iz < nnz; ++iz) {
                int cy = std::min(std::max(iy - p, 0), ny - 1);
                int cx = std::min(std::max(ix - p, 0), nx - 1);
                int cz = std::min(std::max(iz - p, 0), nz - 1);
                o[iz + (size_t)nnz * (ix + (size_t)nnx * iy)] = m[cz + (size_t)nz * (cx + (size_t)nx * cy)];
            }
    return o;
}

static void write_rec(const std::string &op, const std::vector<float> &rec) {
    FILE *f = fopen(op.c_str(), "wb");
    if (!f || fwrite(rec.data(), 4, rec.size(), f) != rec.size()) {
        fprintf(stderr, "refharness: cannot write %s\n", op.c_str());
        exit(2);
    }
    fclose(f);
}

static float *dalloc(size_t n) {
    float *p;
    CK(cudaMalloc(&p, n * 4));
    CK(cudaMemset(p, 0, n * 4));
    return p;
}
static float *dupload(const std::vector<float> &h) {
    float *p = dalloc(h.size());
    CK(cudaMemcpy(p, h.data(), h.size() * 4, cudaMemcpyHostToDevice));
    return p;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: refharness CUBIN_DIR CASE_DIR [timing_steps]\n");
        return 1;
    }
    std::string cub = argv[1];
    Case c;
    c.dir = argv[2];
    {
        std::string p = c.dir + "/case.txt";
        FILE *f = fopen(p.c_str(), "r");
        if (!f) { fprintf(stderr, "refharness: no %s\n", p.c_str()); return 2; }
        char k[64], v[256];
        while (fscanf(f, "%63s %255s", k, v) == 2) c.kv[k] = v;
        fclose(f);
    }
    const std::string eng = c.s("engine");
    const int nx = c.i("nx"), ny = c.i("ny"), nz = c.i("nz");
    const float dx = c.f("dx"), dy = c.f("dy"), dz = c.f("dz");
    const int sx = c.i("sx"), sy = c.i("sy"), sz = c.i("sz");
    int nt = c.i("nt");
    const float dt = c.f("dt"), fm = c.f("fm");
    const int wtype = c.kv.count("wtype") ? c.i("wtype") : 1;
    const int mute = c.kv.count("mute") ? c.i("mute") : 0;
    const bool refsync = c.kv.count("sync") ? c.i("sync") != 0 : true;
    auto sync = [&]() { if (refsync) CK(cudaDeviceSynchronize()); };
    const int steps = argc > 3 ? atoi(argv[3]) : nt;  // timing runs may stop early
    const size_t nm = (size_t)nx * ny * nz;
    const int is = 0, ns = 1, jsx = 1, jsy = 1, jsz = 1;
    std::vector<float> rec((size_t)nt * nx * ny);
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float ms = 0;
    Lib L;

    if (eng == "2o") {  // cuda_3dfd, Toa_3dfd_cuda.cu:366-508 (npd = 50 compiled in)
        L.load(cub + "/ref_2order.cubin");
        const int npd = 50, pd = MM + npd;
        const int nnz = nz + 2 * pd, nnx = nx + 2 * pd, nny = ny + 2 * pd, ng = nx * ny;
        auto v0 = read_model(c, "vel", nm);
        auto vv = pad(v0, nx, ny, nz, pd);
        for (auto &x : vv) { float t = x * dt; x = t * t; }
        float _dz2 = 1.0 / (dz * dz), _dx2 = 1.0 / (dx * dx), _dy2 = 1.0 / (dy * dy);
        size_t tot = (size_t)nnz * nnx * nny;
        float *d_wlt = dalloc(nt), *d_vv = dupload(vv), *d_p0 = dalloc(tot), *d_p1 = dalloc(tot);
        float *d_xy = dalloc(ng), *d_txy = dalloc((size_t)ng * nt);
        int *d_s, *d_g;
        CK(cudaMalloc(&d_s, ns * 4));
        CK(cudaMalloc(&d_g, ng * 4));
        dim3 dimg((nnz + 15) / 16, (nnx + 15) / 16), dimb(16, 16);
        launch(L.get("cuda_ricker_wavelet"), dim3((nt + 511) / 512), dim3(512), d_wlt, fm, dt, nt);
        launch(L.get("cuda_set_s"), dim3(1), dim3(ns), d_s, sz, sx, sy, jsz, jsx, jsy, ns, nz, nx, ny);
        launch(L.get("cuda_set_g"), dim3((ng + 511) / 512), dim3(512), d_g, ng, nz, nx, ny);
        auto kdip = L.get("cuda_add_dipole"), kstep = L.get("cuda_step_fd3d"),
             kabs = L.get("cuda_absorb_bndr"), krec = L.get("cuda_record"),
             ktr = L.get("cuda_trans_xy2txy");
        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(e0));
        for (int it = 0; it < steps; ++it) {
            launch(kdip, dim3(1), dim3(1), d_p1, d_wlt + it, d_s + is, 1);
            launch(kstep, dimg, dimb, d_p0, d_p1, d_vv, _dz2, _dx2, _dy2, nz, nx, ny);
            std::swap(d_p0, d_p1);
            launch(kabs, dimg, dimb, d_p0, nz, nx, ny, -0.25f);
            launch(kabs, dimg, dimb, d_p1, nz, nx, ny, -0.25f);
            launch(krec, dim3((ng + 511) / 512), dim3(512), d_p0, d_xy, d_g, ng);
            launch(ktr, dim3((ng + 511) / 512), dim3(512), d_xy, d_txy, it, nt, ng);
        }
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        CK(cudaMemcpy(rec.data(), d_txy, rec.size() * 4, cudaMemcpyDeviceToHost));
        write_rec(c.dir + "/rec_ref.bin", rec);
        if (mute) {  // the reference leaves this call commented out (2O:474-477)
            dim3 xg((nnx + 15) / 16, (nny + 15) / 16);
            launch(L.get("mute_directwave"), xg, dimb, nx, ny, nt, dt, fm, dx, dy, dz, sx, sy, jsx,
                   jsy, sz, is, v0[1], d_txy, 60, ns);
        }
        CK(cudaMemcpy(rec.data(), d_txy, rec.size() * 4, cudaMemcpyDeviceToHost));
    } else {  // 1st-order engines: ISO:372-671, VTI:389-688, TTI:390-676
        const bool iso = eng == "iso", vti = eng == "vti", tti = eng == "tti";
        if (!iso && !vti && !tti) { fprintf(stderr, "refharness: bad engine\n"); return 1; }
        L.load(cub + (iso ? "/ref_1order.cubin" : vti ? "/ref_vti.cubin" : "/ref_tti.cubin"));
        const int npml = tti ? 40 : 20;
        const float pfac = iso ? 10000.0f : 10.0f;
        const int wt = iso ? wtype : 1;
        const int nnx = nx + 2 * npml, nny = ny + 2 * npml, nnz = nz + 2 * npml;
        const size_t tot = (size_t)nnx * nny * nnz;
        auto vp_h = pad(read_model(c, "vel", nm), nx, ny, nz, npml);
        float *vp = dupload(vp_h), *rho = nullptr, *eps = nullptr, *del = nullptr,
              *th = nullptr, *ph = nullptr;
        if (!tti) rho = dupload(pad(read_model(c, "rho", nm), nx, ny, nz, npml));
        if (!iso) {
            eps = dupload(pad(read_model(c, "eps", nm), nx, ny, nz, npml));
            del = dupload(pad(read_model(c, "del", nm), nx, ny, nz, npml));
        }
        if (tti) {
            th = dupload(pad(read_model(c, "theta", nm), nx, ny, nz, npml));
            ph = dupload(pad(read_model(c, "phi", nm), nx, ny, nz, npml));
        }
        float *u0 = dalloc(tot), *u1 = dalloc(tot), *v0 = dalloc(tot), *v1 = dalloc(tot),
              *w0 = dalloc(tot), *w1 = dalloc(tot), *P = dalloc(tot), *Q = dalloc(tot);
        float *px0 = dalloc(tot), *px1 = dalloc(tot), *py0 = dalloc(tot), *py1 = dalloc(tot),
              *pz0 = dalloc(tot), *pz1 = dalloc(tot);
        float *qx0 = nullptr, *qx1 = nullptr, *qy0 = nullptr, *qy1 = nullptr, *qz0 = nullptr,
              *qz1 = nullptr;
        if (!iso) {
            qx0 = dalloc(tot); qx1 = dalloc(tot); qy0 = dalloc(tot);
            qy1 = dalloc(tot); qz0 = dalloc(tot); qz1 = dalloc(tot);
        }
        float *cx1 = dalloc(nnx), *cx2 = dalloc(nnx), *cy1 = dalloc(nny), *cy2 = dalloc(nny),
              *cz1 = dalloc(nnz), *cz2 = dalloc(nnz);
        float *ax1 = dalloc(nnx), *ax2 = dalloc(nnx), *ay1 = dalloc(nny), *ay2 = dalloc(nny),
              *az1 = dalloc(nnz), *az2 = dalloc(nnz);
        float *shot = dalloc((size_t)nt * nx * ny);
        dim3 dimg((nnz + 15) / 16, (nnx + 15) / 16), dimb(16, 16);
        launch(L.get("get_d0"), dim3(1), dim3(1), dx, dy, dz, nnx, nny, nnz, npml, vp);
        auto kc = L.get("initial_coffe");
        launch(kc, dim3((nnx + 511) / 512), dim3(512), dt, nx, cx1, cx2, ax1, ax2, npml);
        launch(kc, dim3((nny + 511) / 512), dim3(512), dt, ny, cy1, cy2, ay1, ay2, npml);
        launch(kc, dim3((nnz + 511) / 512), dim3(512), dt, nz, cz1, cz2, az1, az2, npml);
        auto ksrc = L.get("add_source"), kvel = L.get("update_vel"),
             kstr = L.get("update_stress"), krec = L.get("shot_record");
        const int nsx = ns, fsx = sx, fsy = sy, zs = sz, dsx = jsx, dsy = jsy;
        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(e0));
        float t = dt;
        for (int it = 0; it < steps; ++it, t += dt) {
            if (iso) {
                launch(ksrc, dim3(1), dim3(1), -pfac, fsx, fsy, zs, nx, ny, nz, nnx, nny, nnz, dt,
                       t, fm, wt, npml, is, dsx, dsy, P, nsx);
                sync();
                launch(ksrc, dim3(1), dim3(1), pfac, fsx, fsy, zs + 2, nx, ny, nz, nnx, nny, nnz,
                       dt, t, fm, wt, npml, is, dsx, dsy, P, nsx);
                sync();
                launch(kvel, dimg, dimb, nx, ny, nz, nnx, nny, nnz, npml, dt, dx, dy, dz, u0, v0, w0,
                       u1, v1, w1, P, cx1, cx2, cy1, cy2, cz1, cz2, rho);
                sync();
                launch(kstr, dimg, dimb, nx, ny, nz, nnx, nny, nnz, dt, dx, dy, dz, u1, v1, w1, P,
                       vp, rho, npml, px1, px0, py1, py0, pz1, pz0, ax1, ax2, ay1, ay2, az1, az2,
                       fsx, dsx, fsy, dsy, zs, is, nsx);
                sync();
            } else if (vti) {
                launch(ksrc, dim3(1), dim3(1), pfac, fsx, fsy, zs, nx, ny, nz, nnx, nny, nnz, dt, t,
                       fm, wt, npml, is, dsx, dsy, P, Q, nsx);
                sync();
                launch(kvel, dimg, dimb, nx, ny, nz, nnx, nny, nnz, npml, dt, dx, dy, dz, u0, v0, w0,
                       u1, v1, w1, P, Q, cx1, cx2, cy1, cy2, cz1, cz2, rho);
                sync();
                launch(kstr, dimg, dimb, nx, ny, nz, nnx, nny, nnz, dt, dx, dy, dz, u1, v1, w1, P, Q,
                       vp, rho, npml, px1, px0, py1, py0, pz1, pz0, qx1, qx0, qy1, qy0, qz1, qz0,
                       ax1, ax2, ay1, ay2, az1, az2, del, eps, fsx, dsx, fsy, dsy, zs, is, nsx, true);
                sync();
            } else {
                launch(ksrc, dim3(1), dim3(1), pfac, fsx, fsy, zs, nx, ny, nz, nnx, nny, nnz, dt, t,
                       fm, wt, npml, is, dsx, dsy, P, Q, nsx);
                launch(kvel, dimg, dimb, nx, ny, nz, nnx, nny, nnz, npml, dt, dx, dy, dz, u0, v0, w0,
                       u1, v1, w1, P, Q, cx1, cx2, cy1, cy2, cz1, cz2, th, ph);
                launch(kstr, dimg, dimb, nx, ny, nz, nnx, nny, nnz, dt, dx, dy, dz, u1, v1, w1, P, Q,
                       vp, npml, px1, px0, py1, py0, pz1, pz0, qx1, qx0, qy1, qy0, qz1, qz0, ax1,
                       ax2, ay1, ay2, az1, az2, del, eps, fsx, dsx, fsy, dsy, zs, is, nsx, true, th,
                       ph);
            }
            if (tti) {  // TTI:580-588 assigns instead of swapping
                u0 = u1; v0 = v1; w0 = w1; px0 = px1; py0 = py1; pz0 = pz1;
                qx0 = qx1; qy0 = qy1; qz0 = qz1;
            } else {
                std::swap(u0, u1); std::swap(v0, v1); std::swap(w0, w1);
                std::swap(px0, px1); std::swap(py0, py1); std::swap(pz0, pz1);
                if (vti) { std::swap(qx0, qx1); std::swap(qy0, qy1); std::swap(qz0, qz1); }
            }
            launch(krec, dim3((nx * ny + 511) / 512), dim3(512), nnx, nny, nnz, nx, ny, nz, npml, it,
                   nt, P, shot);
            if (!tti) sync();
        }
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        CK(cudaMemcpy(rec.data(), shot, rec.size() * 4, cudaMemcpyDeviceToHost));
        write_rec(c.dir + "/rec_ref.bin", rec);
        if (mute) {
            dim3 xg((nnx + 15) / 16, (nny + 15) / 16);
            auto km = L.get("mute_directwave");
            if (iso)
                launch(km, xg, dimb, nx, ny, nt, dt, fm, dx, dy, dz, fsx, fsy, dsx, dsy, zs, is, vp,
                       shot, 60, nsx);
            else
                launch(km, xg, dimb, nx, ny, nt, dt, fm, dx, dy, dz, fsx, fsy, dsx, dsy, zs, is, vp,
                       eps, shot, 60, nsx);
        }
        CK(cudaMemcpy(rec.data(), shot, rec.size() * 4, cudaMemcpyDeviceToHost));
    }
    CK(cudaDeviceSynchronize());
    if (mute) write_rec(c.dir + "/rec_mute.bin", rec);
    printf("refharness %s ms=%.3f steps=%d\n", eng.c_str(), ms, steps);
    return 0;
}
