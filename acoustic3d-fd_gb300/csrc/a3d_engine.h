// a3d_engine.h — the engine object behind the C ABI.
#pragma once
#include <functional>
#include <string>
#include <vector>

#include "../../include/acoustic3d.h"
#include "a3d_closure.h"
#include "a3d_k1.cuh"
#include "a3d_setup.h"

namespace a3d {

// thread-local last-error text; fail() records it, prints it and returns code
int fail(int code, const char *fmt, ...);
void clear_error();

// copy of a large pageable host buffer to the device through a pinned staging ring
// (a3d_stage.cu); waits for the copy (stream st) and returns an A3D_* code
int stage_to_device(void *dst, const void *src, size_t bytes, cudaStream_t st);

// copy of a device buffer to the host through the same pinned ring, handing each
// chunk (host pointer, byte offset, bytes) to sink while the next chunk is copied;
// returns the first non-zero sink result or an A3D_* code
int stage_from_device(const void *src, size_t bytes, cudaStream_t st,
                      const std::function<int(const unsigned char *, size_t, size_t)> &sink);

// tensor map over a padded field (dims nnz, nnx, nny; rows of g.ldz elements)
// dtype: 0 float, 1 bfloat16, 2 float16, 3 double
int make_field_map(CUtensorMap *m, const void *base, int dtype, const Grid &g, int box0, int box1);

// snapshot hook: want(it) says whether a snapshot is taken after step it;
// take(it, window) receives the model window (nz*nx*ny floats, z fastest)
struct SnapHook {
    std::function<bool(int)> want;
    std::function<int(int, const float *)> take;
};

}  // namespace a3d

struct a3d_engine {
    a3d_config cfg{};
    a3d::Grid g;
    int device = 0;
    int npml = 0;          // absorber cells (1st order) or sponge width npd (2nd order)
    int tx = 8;
    bool fp64 = false;
    int half = 0;          // 2-byte wavefields: 1 bfloat16, 2 float16 (isotropic and VTI engines)
    size_t esz = 4;        // bytes per wavefield element
    // multi-shot sweeps (VTI, cfg.batch = K > 1): every wavefield and split
    // component holds K copies fstride elements apart (4-D tensor maps over them),
    // K records and K mute tables follow each other, d_shots the shots' source cells
    int nbatch = 1;
    size_t fstride = 0, fstride_p = 0;  // u, v, w / P, Q and split components (elements)
    // A3D_FP16V (VTI, TTI): u, v, w float16 (half = 2, esz = 2), P, Q and split components float
    bool pfloat = false;
    size_t esz_p = 4;      // bytes per element of P, Q and the split components
    int4 *d_shots = nullptr;
    // power-of-two storage scales of 2-byte wavefields: sig_v for u, v, w, sig_p for P
    // and its split components (1 otherwise)
    float sig_v = 1.0f, sig_p = 1.0f;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int *d_err = nullptr;
    std::vector<void *> allocs;
    size_t dev_bytes = 0;

    // model parameters on the device (float, padded layout)
    float *vv = nullptr, *vp = nullptr, *rho = nullptr, *rinv = nullptr, *eps = nullptr, *del = nullptr;
    float *tct = nullptr, *tst = nullptr, *tcp = nullptr, *tsp = nullptr;  // TTI trig
    float v_mute = 0.0f;   // direct-wave mute velocity

    // wavefields
    void *X = nullptr, *Y = nullptr;                          // 2nd order
    void *u = nullptr, *v = nullptr, *w = nullptr, *P = nullptr, *Q = nullptr;
    // fused isotropic step (FP32, PML): a second set of u, v, w, P; step it reads set
    // it & 1 and writes the other (set 0 = u, v, w, P)
    bool fused_ok = false;  // the fused step is built for this engine (buffers, maps)
    bool fused = false;     // chosen: A3D_FUSED=1 forces it, =0 rules it out, else the autotuner decides
    void *u2 = nullptr, *v2 = nullptr, *w2 = nullptr, *P2 = nullptr;
    CUtensorMap mstep[2][2][11];  // [tile width][set read]
    void *px = nullptr, *py = nullptr, *pz = nullptr, *qx = nullptr, *qy = nullptr, *qz = nullptr;

    // coefficients
    float2 *fz = nullptr, *fx = nullptr, *fy = nullptr;       // 2nd-order sponge
    float *pml = nullptr;  // cx1 cx2 ax1 ax2 | cy1 cy2 ay1 ay2 | cz1 cz2 az1 az2 blocks
    int ulo[3] = {0, 0, 0}, uhi[3] = {0, 0, 0};  // pressure-undamped interval per axis (x, y, z)
    float2 *taper = nullptr;
    std::vector<float> w2o;                    // 2nd-order Ricker samples
    std::vector<float> amp0, amp1;             // 1st-order injected amplitudes per step
    std::vector<int> inj;                      // 1st-order: inject at step it

    float *rec = nullptr;   // [ny][nx][nt]
    int *d_mute = nullptr;  // first unmuted sample per trace
    // snapshot pipeline: the model window is cropped on the device into one of
    // NSNAP buffers, copied on a second stream into pinned host memory, and handed
    // to the caller when a later snapshot needs the slot or the shot ends, so the
    // time loop does not stop for it
    static constexpr int NSNAP = 3;
    float *snap_dev = nullptr;               // crop buffer of slot 0 (the others are allocated lazily)
    float *snap_ring_dev[NSNAP] = {nullptr, nullptr, nullptr};
    float *snap_ring_host[NSNAP] = {nullptr, nullptr, nullptr};  // pinned
    cudaStream_t snap_st = nullptr;
    cudaEvent_t snap_cropped[NSNAP] = {nullptr, nullptr, nullptr}, snap_copied[NSNAP] = {nullptr, nullptr, nullptr};
    int snap_setup();

    // tensor maps for the two tile widths (index 0: 32x8 tiles, 1: 32x16)
    CUtensorMap m2o_cur[2][2], m2o_prev[2][2], m2o_vv[2];  // [tile][buffer]
    CUtensorMap mvel[2][9], mstr[2][18];
    int nvel = 0, nstr = 0;

    // launch configuration per kernel kind ([0] velocity / 2nd-order step, [1] stress),
    // chosen by the autotuner on the first run unless fixed by the config
    struct Tune { int tx = 8; int depth = 0; int mode = 0; int rows = 2; float ms = 0; int rot = 0; int sblk = 1; };
    Tune tune[2];
    bool tuned = false;
    int autotune();
    int autotune_form();  // tunes the kernels of the current form (two sweeps, or the fused step)
    int drop_fused();     // settle on the two-sweep form and free the fused step's buffers

    // learned rim (boundary A3D_BOUNDARY_LEARNED): undamped 6-cell rim, corrected
    // after every step by the closure (bfloat16-rounded weights in the kernels'
    // layout, 1/(rho vp) and vp dt / min(d) on the padded grid, hidden activations)
    bool learned = false;
    a3d::ClGeom clg{};
    float *cl_packed = nullptr, *cl_zinv = nullptr, *cl_kap = nullptr;
    __nv_bfloat16 *cl_h = nullptr;   // CUDA-core path (A3D_CLOSURE_SIMT=1)
    uint16_t *cl_image = nullptr;    // tensor-core path: per-face bfloat16 weight images
    float4 *cl_y = nullptr;          // and per-face outputs
    bool cl_simt = false;
    double cl_ms = 0;
    long long cl_launch = 0;

    // teacher taps: after step tap_steps[k], u, v, w, P over [tap_off, nn - tap_off)
    // go to tap_out + 4 k box cells
    std::vector<int> tap_steps;
    int tap_off = 0;
    float *tap_out = nullptr;

    // replay each shot's time loop as one CUDA graph (ignored with snapshots or
    // per-kernel timing)
    bool graph = false;

    // optional per-kernel timing: events around every launch of each kernel kind
    bool profiling = false;
    std::vector<cudaEvent_t> kev;  // 3 per step (1st order) or 2 per step (2nd order)
    double kms[2] = {0, 0};        // summed device ms: [0] velocity / 2nd-order step, [1] stress
    long long klaunch[2] = {0, 0};

    ~a3d_engine();
    void *dalloc(size_t bytes);  // zeroed; null on failure
    void *dfield(size_t esz);    // zeroed padded field; returns its base (allocation + zoff)
    // nbatch copies of a wavefield (pressure: P, Q or a split component), fstride /
    // fstride_p elements apart; returns the first copy's base
    void *dfield_batch(bool pressure);
    size_t fsize(bool pressure) const { return pressure ? esz_p : esz; }
    size_t field_bytes(size_t esz) const { return g.elems() * esz; }
    void *field_alloc(void *base, size_t es) const { return (char *)base - a3d::Grid::zoff * es; }
    int run(const a3d_shot &s, float *rec_dev, const a3d::SnapHook *hook, double *ms);
    int run_shots(const a3d_shot *shots, int k, double *ms);  // multi-shot sweeps (nbatch > 1)
};
