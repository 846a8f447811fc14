// a3d_batch.cu — a3d_run_batch: every shot of a survey on one device.
//
// The reference drives a survey from Python with a process pool, one process
// and one full library call per shot (readmodel.py:186-204; each call reads the
// model files, allocates, runs, writes and frees).  Here one call keeps an engine
// (model resident in HBM, tensor maps built, launch shapes tuned) for as long as
// consecutive shots use the same window, and carries the tuned launch shapes
// over to the engines of later windows.  With cfg.batch = K > 1 (VTI) consecutive
// shots on the same window run K at a time as multi-shot sweeps (one launch per
// kernel and step for all K), each shot's record the same as its single run.
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "a3d_engine.h"

using namespace a3d;

namespace {

bool same_window(const a3d_window &a, const a3d_window &b) {
    return a.x0 == b.x0 && a.y0 == b.y0 && a.z0 == b.z0 && a.nx == b.nx && a.ny == b.ny && a.nz == b.nz;
}

// the window [x0, x0+nx) x [y0, y0+ny) x [z0, z0+nz) of a model array (z fastest,
// then x, then y) as a dense array of the same order
void crop(const float *m, const a3d_config &c, const a3d_window &w, float *out) {
    for (int iy = 0; iy < w.ny; ++iy)
        for (int ix = 0; ix < w.nx; ++ix)
            memcpy(&out[((size_t)iy * w.nx + ix) * w.nz],
                   m + (size_t)w.z0 + (size_t)c.nz * ((size_t)(w.x0 + ix) + (size_t)c.nx * (w.y0 + iy)),
                   (size_t)w.nz * sizeof(float));
}

}  // namespace

extern "C" int a3d_run_batch(const a3d_problem *pb, const a3d_shot *shots, int nshot, const a3d_opts *o) {
    clear_error();
    if (!pb || !o || nshot < 0 || (nshot > 0 && !shots)) return fail(A3D_E_ARG, "null problem, shots or options");
    const a3d_config &c = pb->cfg;
    const a3d_window whole{0, 0, 0, c.nx, c.ny, c.nz};
    // check every window and shot before any work
    for (int i = 0; i < nshot; ++i) {
        const a3d_window w = (o->windows && o->windows[i].nx != 0) ? o->windows[i] : whole;
        if (w.nx < 1 || w.ny < 1 || w.nz < 1 || w.x0 < 0 || w.y0 < 0 || w.z0 < 0 || w.x0 + w.nx > c.nx ||
            w.y0 + w.ny > c.ny || w.z0 + w.nz > c.nz)
            return fail(A3D_E_ARG, "shot %d: window (%d,%d,%d)+(%d,%d,%d) outside the %dx%dx%d model", i, w.x0,
                        w.y0, w.z0, w.nx, w.ny, w.nz, c.nx, c.ny, c.nz);
        const a3d_shot &s = shots[i];
        if (s.sx < w.x0 || s.sx >= w.x0 + w.nx || s.sy < w.y0 || s.sy >= w.y0 + w.ny || s.sz < w.z0 ||
            s.sz >= w.z0 + w.nz)
            return fail(A3D_E_ARG, "shot %d at (%d,%d,%d) lies outside its window", i, s.sx, s.sy, s.sz);
    }
    const float *arrays[6] = {pb->vel, pb->rho, pb->eps, pb->del, pb->theta, pb->phi};
    std::vector<float> cropped[6];
    a3d_engine *e = nullptr;
    a3d_window cur{};
    a3d_engine::Tune tune[2];
    bool have_tune = false, fused = false;
    size_t off = 0;
    int rc = A3D_OK;
    const int K = c.batch > 1 ? c.batch : 1;
    for (int i = 0; i < nshot && rc == A3D_OK;) {
        const a3d_window w = (o->windows && o->windows[i].nx != 0) ? o->windows[i] : whole;
        if (!e || !same_window(w, cur)) {
            if (e) a3d_engine_destroy(e);
            e = nullptr;
            a3d_config wc = c;
            wc.nx = w.nx;
            wc.ny = w.ny;
            wc.nz = w.nz;
            const float *wa[6];
            std::vector<std::thread> ts;  // one host thread per model array to crop
            bool oom = false;
            for (int k = 0; k < 6 && !oom; ++k) {
                if (!arrays[k] || same_window(w, whole)) {
                    wa[k] = arrays[k];
                    continue;
                }
                try {
                    cropped[k].resize((size_t)w.nx * w.ny * w.nz);
                } catch (...) {
                    oom = true;
                    break;
                }
                wa[k] = cropped[k].data();
                try {
                    ts.emplace_back(crop, arrays[k], std::cref(c), std::cref(w), cropped[k].data());
                } catch (...) {  // no thread: crop here
                    crop(arrays[k], c, w, cropped[k].data());
                }
            }
            for (auto &t : ts) t.join();
            if (oom) {
                rc = fail(A3D_E_NOMEM, "host allocation of a %dx%dx%d window failed", w.nx, w.ny, w.nz);
                break;
            }
            rc = a3d_engine_create(&e, &wc, wa[0], wa[1], wa[2], wa[3], wa[4], wa[5], o->device);
            if (rc) break;
            if (have_tune) {  // launch shapes (and the isotropic step's form) tuned on the first engine
                e->tune[0] = tune[0];
                e->tune[1] = tune[1];
                e->tuned = true;
                if (fused && e->fused_ok) e->fused = true;
                else if ((rc = e->drop_fused())) break;
            }
            cur = w;
        }
        e->graph = o->graph != 0;
        // this shot and the following ones on the same window, up to K of them
        int k = 1;
        while (k < K && i + k < nshot &&
               same_window((o->windows && o->windows[i + k].nx != 0) ? o->windows[i + k] : whole, w))
            ++k;
        std::vector<a3d_shot> rel(k);
        for (int j = 0; j < k; ++j)
            rel[j] = a3d_shot{shots[i + j].sx - w.x0, shots[i + j].sy - w.y0, shots[i + j].sz - w.z0};
        double ms = 0;
        if (K > 1)
            rc = a3d_engine_run_shots(e, rel.data(), k, o->recs_host ? o->recs_host + off : nullptr, &ms);
        else
            rc = a3d_engine_run(e, &rel[0], o->recs_host ? o->recs_host + off : nullptr, 0, 0, nullptr, &ms);
        if (rc) break;
        if (!have_tune) {
            tune[0] = e->tune[0];
            tune[1] = e->tune[1];
            fused = e->fused;
            have_tune = true;
        }
        for (int j = 0; j < k; ++j) {  // a sweep's device time is shared evenly by its shots
            if (o->rec_offsets) o->rec_offsets[i + j] = off;
            if (o->ms) o->ms[i + j] = ms / k;
            off += (size_t)c.nt * w.nx * w.ny;
        }
        i += k;
    }
    if (e) a3d_engine_destroy(e);
    return rc;
}
