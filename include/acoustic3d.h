/*
 * acoustic3d.h — C ABI of the GB300 (sm_103a) acoustic finite-difference engines.
 *
 * Two layers:
 *
 * 1. Drop-in entry points with the names and argument lists of the reference's
 *    four shared libraries (paths relative to the reference project).  The build
 *    produces lib/acoustic2order.so, lib/acoustic1order.so, lib/acoustic1vti.so and
 *    lib/acoustic1tti.so; each exports all four symbols, so readmodel.py's
 *    cdll.LoadLibrary('./lib/<name>.so') + <symbol>(...) calls work unchanged.
 *    They read the same raw float32 model files and write byte-identical shot
 *    records and snapshots.  Unlike the reference they never exit() the process:
 *    they return an int status (0 ok, A3D_E_* otherwise, message on stderr); a
 *    ctypes caller that sets no restype ignores it, as it ignored the void.
 *
 * 2. An in-memory engine API (a3d_*) used by the tests and benchmarks: the model
 *    is uploaded once into device memory and any number of shots run against it.
 *
 * Model arrays are float32, nx*ny*nz, z fastest, then x, then y (the reference's
 * file order, readmodel.py / ..iso..:249-257).  Records are float32
 * [ny][nx][nt], time fastest (the reference's internal record layout).
 */
#ifndef ACOUSTIC3D_H
#define ACOUSTIC3D_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- statuses */
#define A3D_OK 0
#define A3D_E_ARG 1         /* invalid argument or geometry                         */
#define A3D_E_IO 2          /* model, record or snapshot file could not be opened/read/written */
#define A3D_E_CUDA 3        /* CUDA runtime error (message names the call)          */
#define A3D_E_NOMEM 4       /* host or device allocation failed                     */
#define A3D_E_KERNEL 5      /* a kernel gave up a bounded wait (error word set)     */
#define A3D_E_UNSUPPORTED 6 /* combination not built (e.g. storage type for physics) */

/* ------------------------------------------------- drop-in entry points */

/* Replaces cuda_3dfd, src/Toa_3dfd_cuda.cu:366-370 (lib/acoustic2order.so).
 * 2nd-order 8th-order-Laplacian leap-frog, 50-cell sponge, z-dipole source,
 * receivers on every surface node at model depth 1.  As in the reference,
 * kt, snap_interval and cut_directwave are ignored (readmodel.py passes the last
 * two in swapped positions, readmodel.py:335-338) and snapshots, when
 * show_snapshot is set, are taken every 500 steps as FNsnap"ishot_<is>_it_<it>.bin". */
int cuda_3dfd(char *FNvel, char *FNsnap, char *FNshot, int is, int ns, int nx, int ny, int nz,
              float dx, float dy, float dz, int sxbeg, int sybeg, int szbeg, int jsx, int jsy,
              int jsz, float dgx, float dgy, float dgt, int nt, int kt, float dt, float fm,
              bool show_snapshot, bool cut_directwave, int snap_interval, int cudaDevicei);

/* Replaces cuda_3dfd_1order, src/Toa_gpu_3diso_fd_1orderfunciton.cu:372-377
 * (lib/acoustic1order.so).  Staggered-grid pressure/particle-velocity with
 * density, 20-cell split PML, dipole source (wavelet wtype 1..6), receivers at
 * model depth 0, optional direct-wave mute; ns shots along x (is = 0..ns-1), each
 * record written at byte offset is*nt*nx*ny*4.  Snapshots every snap_interval
 * steps as FNsnap"ishot_<is>it_<it>.bin" (no underscore, as the reference). */
int cuda_3dfd_1order(char *FNvel, char *FNrho, char *FNsnap, char *FNshot, int is, int ns,
                     int nx, int ny, int nz, float dx, float dy, float dz, int sxbeg, int sybeg,
                     int szbeg, int jsx, int jsy, int jsz, float dgx, float dgy, float dgt, int nt,
                     float dt, int wtype, float fm, bool show_snapshot, bool cut_directwave,
                     int snap_interval, int cudaDevicei);

/* Replaces cuda_3dfd_vti, src/Toa_gpu_3dvti_fd_1orderfunciton.cu:389-395
 * (lib/acoustic1vti.so).  Pseudo-acoustic VTI (P, Q) with density, epsilon,
 * delta, SV-suppression ball round the source, 20-cell PML, Ricker monopole into
 * P and Q.  Snapshots as FNsnap"ishot_<is>_it_<it>.bin". */
int cuda_3dfd_vti(char *FNvel, char *FNrho, char *FNepsilon, char *FNdelta, char *FNsnap,
                  char *FNshot, int is, int ns, int nx, int ny, int nz, float dx, float dy,
                  float dz, int sxbeg, int sybeg, int szbeg, int jsx, int jsy, int jsz, float dgx,
                  float dgy, float dgt, int nt, float dt, float fm, bool show_snapshot,
                  bool cut_directwave, int snap_interval, int cudaDevicei);

/* Replaces cuda_3dfd_tti, src/Toa_gpu_3dtti_fd_1orderfunciton.cu:390-398
 * (lib/acoustic1tti.so).  Pseudo-acoustic TTI with tilt theta and azimuth psi
 * (radians), no density (FNrho is ignored), 40-cell PML, ns forced to 1;
 * snapshots every 100 steps for it != 0 whatever show_snapshot says.
 * Returns 1 when the shot file cannot be opened, as the reference does. */
int cuda_3dfd_tti(char *FNvel, char *FNrho, char *FNepsilon, char *FNdelta, char *FNtheta,
                  char *FNpsi, char *FNsnap, char *FNshot, int is, int ns, int nx, int ny, int nz,
                  float dx, float dy, float dz, int sxbeg, int sybeg, int szbeg, int jsx, int jsy,
                  int jsz, float dgx, float dgy, float dgt, int nt, float dt, float fm,
                  bool show_snapshot, bool cut_directwave, int snap_interval, int cudaDevicei);

/* ------------------------------------------------------- engine API */

enum a3d_physics { A3D_2ORDER = 0, A3D_ISO = 1, A3D_VTI = 2, A3D_TTI = 3 };
enum a3d_storage { A3D_FP32 = 0, A3D_BF16 = 1, A3D_FP16 = 2, A3D_FP64 = 3, A3D_FP16V = 4 };

typedef struct {
    int physics;       /* enum a3d_physics                                        */
    int nx, ny, nz;    /* model grid                                              */
    float dx, dy, dz;  /* spacing (m)                                             */
    int nt;            /* time steps                                              */
    float dt, fm;      /* step (s), Ricker peak frequency (Hz)                    */
    int wtype;         /* isotropic source wavelet 1..6 (others use 1)            */
    int npml;          /* absorber cells; <= 0 selects the reference's value:
                          50 (2nd-order sponge), 20 (iso, VTI), 40 (TTI)          */
    int rec_z;         /* 2nd order: receiver depth in model cells; < 0: 1        */
    int mute;          /* zero the direct wave in the record                      */
    int storage;       /* enum a3d_storage of the wavefields: FP32, FP64 (the FP64
                          error-reference run), BF16 / FP16 (isotropic, VTI and TTI:
                          2-byte fields, float arithmetic), or FP16V (VTI: u, v, w
                          as float16, P, Q and the split components as float: VTI
                          and TTI; long records stay stable with it where the
                          all-2-byte forms diverge)                               */
    int tile_x;        /* kernel tile width along x: 8 or 16 fixes it, 0 lets the
                          autotuner choose, < 0 disables the autotuner (32x8 tiles) */
    int boundary;      /* enum a3d_boundary: A3D_BOUNDARY_PML (0, the physics' own
                          absorber) or A3D_BOUNDARY_LEARNED (isotropic, FP32: a 6-cell
                          undamped rim corrected by the closure set with
                          a3d_engine_set_closure; npml must be 10 or <= 0)          */
    int batch;         /* VTI, FP32 / BF16 / FP16: the most shots one launch advances
                          together (multi-shot sweeps, a3d_engine_run_shots); the
                          engine holds that many copies of every wavefield and
                          record.  <= 1: one shot per launch                        */
} a3d_config;

enum a3d_boundary { A3D_BOUNDARY_PML = 0, A3D_BOUNDARY_LEARNED = 1 };

typedef struct {
    int sx, sy, sz;    /* shot position in model cells (sxbeg, sybeg, szbeg)      */
} a3d_shot;

typedef struct a3d_engine a3d_engine;

/* Create an engine on `device` and upload the model.  Arrays the physics does
 * not read may be NULL (2nd order: vel; iso: vel, rho; VTI: vel, rho, eps, del;
 * TTI: vel, eps, del, theta, phi). */
int a3d_engine_create(a3d_engine **out, const a3d_config *cfg, const float *vel,
                      const float *rho, const float *eps, const float *del, const float *theta,
                      const float *phi, int device);
int a3d_engine_destroy(a3d_engine *e);

/* Run one shot.  rec_host: nt*nx*ny floats (or NULL).  If snap_every > 0, a
 * snapshot (model window, nz*nx*ny floats, z fastest) is copied into snaps_host
 * after every step with it % snap_every == 0 (it != 0 too when snap_skip0).
 * *ms (optional) receives the device time of the time loop (CUDA events). */
int a3d_engine_run(a3d_engine *e, const a3d_shot *shot, float *rec_host, int snap_every,
                   int snap_skip0, float *snaps_host, double *ms);

/* Run one shot leaving the record on the device: rec_dev is a device pointer to
 * nt*nx*ny floats (or NULL to keep the engine's own buffer); no host copies. */
int a3d_engine_run_device(a3d_engine *e, const a3d_shot *shot, float *rec_dev, double *ms);

/* Multi-shot sweeps: no counterpart in the reference, which runs one shot per
 * library call in its own process (readmodel.py:186-204; each call a full
 * cuda_3dfd_vti, ..vti..:389-688).  On an engine created with cfg.batch = K > 1,
 * run k <= K shots of the same model together: every launch advances all k shots
 * by one step, the CTAs that hold one tile of the grid for the different shots run
 * side by side, so each tile's model parameters come from HBM once per step for
 * all shots.  Each shot's record equals its one-shot run (a3d_engine_run) bit for
 * bit.  recs_host: k * nt*nx*ny floats, shot after shot (or NULL); *ms (optional)
 * the device time of the whole time loop.  Snapshots are not taken. */
int a3d_engine_run_shots(a3d_engine *e, const a3d_shot *shots, int k, float *recs_host, double *ms);

/* Copy the record of shot j (0-based, in the order of the last run's shots; 0 for
 * a one-shot run) to rec_host (nt*nx*ny floats). */
int a3d_engine_copy_record(a3d_engine *e, int j, float *rec_host);

/* Device pointer of the engine's record buffer ([ny][nx][nt] floats; an engine
 * with cfg.batch = K holds K of them, shot after shot). */
float *a3d_engine_record_device(a3d_engine *e);

/* Bytes the engine holds in device memory. */
size_t a3d_engine_device_bytes(const a3d_engine *e);

/* Everything in one call from host buffers: create, run the shots, copy their
 * records into recs_host (nshot * nt*nx*ny floats), destroy. */
int a3d_forward_host(const a3d_config *cfg, const float *vel, const float *rho, const float *eps,
                     const float *del, const float *theta, const float *phi,
                     const a3d_shot *shots, int nshot, float *recs_host, int device);

/* ------------------------------------------------- batched multi-shot API */
/* The batched entry point the reference's Python driver would feed instead of one
 * process per shot (readmodel.py:186-204 runs a process pool over the shot list,
 * each process calling one of the four entry points above once).  One call runs
 * every shot of a survey on one device: the model is uploaded once per window
 * shape, the autotuned launch shapes are kept for the whole batch, and each shot's
 * record lands in recs_host. */
typedef struct {
    a3d_config cfg;    /* physics, whole-model grid, time axis, absorber, storage, tile */
    const float *vel, *rho, *eps, *del, *theta, *phi;  /* host model arrays, nx*ny*nz
                                                          each (NULL where not read) */
} a3d_problem;

typedef struct {
    int x0, y0, z0;    /* window origin in model cells                              */
    int nx, ny, nz;    /* window size; nx == 0 selects the whole model              */
} a3d_window;

typedef struct {
    int device;                 /* CUDA device                                         */
    const a3d_window *windows;  /* one per shot, or NULL (every shot sees the whole
                                   model).  A windowed shot runs on the model cropped to
                                   its window, with the window's own absorber; its
                                   position stays in model cells and must lie inside   */
    int graph;                  /* 1: replay each shot's time loop as one CUDA graph   */
    float *recs_host;           /* out (or NULL): the records one after another, shot i
                                   taking nt * wnx * wny floats ([wny][wnx][nt])        */
    size_t *rec_offsets;        /* out (or NULL): nshot float offsets into recs_host   */
    double *ms;                 /* out (or NULL): nshot device times of the time loops
                                   (a multi-shot sweep's time shared evenly by its shots) */
} a3d_opts;

/* Run nshot shots.  Returns A3D_OK, or the first failure (later shots not run). */
int a3d_run_batch(const a3d_problem *pb, const a3d_shot *shots, int nshot, const a3d_opts *opts);

/* Per-kernel device timing (CUDA events around every launch, on the engine's
 * stream).  After runs with profiling on, ms[0]/launches[0] sum the velocity
 * sweeps (1st order) or the fused steps (2nd order), ms[1]/launches[1] the stress
 * sweeps.  Turning profiling on resets the sums. */
int a3d_engine_set_profiling(a3d_engine *e, int on);
int a3d_engine_kernel_times(const a3d_engine *e, double *ms, long long *launches);

/* JSON description of the engine (grid, layout, bytes held, the power-of-two
 * scales of float16 storage as log2 — sig_v_log2 for u, v, w, sig_p_log2 for P, Q,
 * 0 for other storage — and the autotuned launch configuration of each kernel
 * kind); runs the autotuner if it has not run. */
int a3d_engine_describe(a3d_engine *e, char *buf, size_t n);

/* Message of the last failure on the calling thread ("" if none). */
const char *a3d_last_error(void);

/* ------------------------------------------------- learned absorbing rim */
/* No counterpart in the reference, whose absorber is the split PML of
 * ..iso..:263-291 (20 cells per face).  The learned rim pads the model by 10 cells
 * per face: the outer 4 are never updated (as in every engine) and the inner 6 are
 * updated without damping, then corrected after every step by a small network:
 *
 *   x      = [u, v, w, P/(rho vp), k u, k v, k w, k P/(rho vp)],  k = vp dt / min(d)
 *   h_f    = relu(W1 * x)        3x3x3 conv, 8 -> 32 channels, no bias, on face f's box
 *                                (depth -1..5 along its normal, zero outside)
 *   y_f    = W2_f * h_f          3x3x3 conv, 32 -> 4 channels, one kernel per face
 *   (u, v, w, P) += sum over the faces whose rim holds the cell of
 *                   G_f[depth] . y_f  (channel 3 times rho vp)
 *
 * A3D_CLOSURE_NPARAM floats in this order: W1 [32][8][27], W2 [6][4][32][27],
 * G [6][6][4]; a 3x3x3 tap index is ((dy+1)*3 + (dx+1))*3 + (dz+1); face
 * f = 2*axis + side (axis 0 z, 1 x, 2 y; side 0 low, 1 high).  The kernels use
 * the weights rounded to bfloat16, store h as bfloat16 and accumulate in float. */
#define A3D_CLOSURE_NPARAM 27792

/* Install the closure of an engine created with boundary = A3D_BOUNDARY_LEARNED
 * (required before its first run). */
int a3d_engine_set_closure(a3d_engine *e, const float *params, size_t n);

/* Teacher taps: after each listed step (0-based, ascending or not) the engine
 * copies u, v, w and P over the box [off, nn - off) of its padded grid, z fastest,
 * into dev_out (device memory; step k of the list at dev_out + 4 * k * box cells).
 * FP32 storage only.  n = 0 removes the taps. */
int a3d_engine_set_tap(a3d_engine *e, const int *steps, int n, int off, float *dev_out);

/* Device ms and launch pairs of the closure summed over runs with profiling on. */
int a3d_engine_closure_times(const a3d_engine *e, double *ms, long long *launches);

/* Training object: teacher state pairs on the rim grid of an nx*ny*nz model
 * (model + 10 cells per face, dense, z fastest), the loss
 *   sum over rim cells of |correction - (S_t+1 - step(S_t))|^2 / E,
 * channel 3 divided by rho vp and E the rim energy of step(S_t) in the same units,
 * where step is the engine's undamped update on the rim grid (zeros in its outer 4
 * cells), and Adam on float master weights (bfloat16 rounding in every forward). */
typedef struct a3d_closure a3d_closure;
int a3d_closure_create(a3d_closure **out, int nx, int ny, int nz, int device);
int a3d_closure_destroy(a3d_closure *c);
int a3d_closure_set_params(a3d_closure *c, const float *params, size_t n);
int a3d_closure_get_params(const a3d_closure *c, float *params, size_t n);
/* a model (vel, rho: nx*ny*nz host arrays) and its time step; *model receives its id */
int a3d_closure_add_model(a3d_closure *c, const float *vel, const float *rho, float dx, float dy, float dz,
                          float dt, int *model);
/* one teacher pair: device arrays of 4 rim-grid fields each (u, v, w, P), e.g. two
 * consecutive taps of a wide-PML engine with off = its npml - 10, or a learned-rim
 * engine's own state (off = 0) and the wide-PML state one step later.  A pair whose
 * rim energy is not finite is refused (A3D_E_ARG). */
int a3d_closure_add_sample(a3d_closure *c, int model, const float *state0_dev, const float *state1_dev);
int a3d_closure_num_samples(const a3d_closure *c);
/* device buffer owned by the object for nstates rim-grid states (4 fields each),
 * e.g. the tap target of a wide-PML engine; NULL on failure.  A larger request
 * replaces the buffer. */
float *a3d_closure_staging(a3d_closure *c, int nstates);
/* decoupled weight decay of W1 and W2 (w -= lr * decay * w every Adam step; 0 off) */
int a3d_closure_set_decay(a3d_closure *c, float decay);
/* epochs over the samples in seeded random order, minibatches of `batch` samples;
 * loss_per_epoch (or NULL) receives the mean minibatch loss of each epoch */
int a3d_closure_train(a3d_closure *c, int epochs, int batch, float lr, unsigned long long seed,
                      float *loss_per_epoch);
/* one sample: the correction of step(S_t) (4 rim-grid fields, zero off the rim),
 * the gradient of its loss (A3D_CLOSURE_NPARAM) and the loss; any may be NULL */
int a3d_closure_eval(a3d_closure *c, int sample, float *delta_host, float *grad_host, float *loss);
/* the same correction computed by the engine's tensor-core kernels (tcgen05
 * MMAs, bfloat16 operands, float accumulation) instead of the CUDA-core ones */
int a3d_closure_eval_tc(a3d_closure *c, int sample, float *delta_host);
/* step(S_t) and S_t+1 of one sample (4 rim-grid fields each; either may be NULL) */
int a3d_closure_teacher(const a3d_closure *c, int sample, float *x_host, float *t_host);

/* ------------------------------------------- 2nd-order step without allocation */

/* No counterpart in the reference.  One 2nd-order time step on device buffers the
 * caller owns, for callers that cannot call cudaMalloc: a host framework that
 * hands out all device memory from its own pool, or a process whose device memory
 * is provisioned up front.  The call allocates nothing; the step kernel's scratch
 * (three per-axis sponge-factor tables and an error word) lives in one fixed
 * array of A3D_NOALLOC_SCRATCH_BYTES (about 97 KB) that every GPU which loads the
 * library holds until the process exits.  Padded axes above A3D_NOALLOC_MAX_AXIS
 * cells, and padded grids above 2^31 - 1 cells (ldz * nnx * nny; the step indexes
 * a field with 32-bit offsets, as the engine does), are rejected with A3D_E_ARG
 * before any GPU work.
 *
 * Buffers (device, float, 16-byte aligned): the padded grid has nnz = nz + 8 +
 * 2*npd cells along z (likewise x, y) and element (iz, ix, iy) at
 * iz + ldz*(ix + nnx*iy), ldz >= nnz a multiple of 4.  `cur` is the current level
 * including this step's dipole (before the first step set cur at the source cell
 * (sz+4+npd, sx+4+npd, sy+4+npd) to w[0] and two cells deeper to -w[0]);
 * `prev_next` holds the previous level on entry and the next level on return,
 * with the next step's dipole amplitude w_next already added, so the two buffers
 * swap roles every step.  `vv` is (v dt)^2 edge-padded.  `rec` ([ny][nx][nt]
 * floats, receivers at model depth rec_z) receives sample `it`, or is NULL.
 * The computation is the engine's 2nd-order step with the direct-wave mute off,
 * bit for bit; the step applies no mute, so callers that want one zero the early
 * samples of `rec` themselves.
 *
 * The first call on a device sets up the scratch address for that device (it is
 * looked up again after the device's context is re-created, e.g. by
 * cudaDeviceReset); make that first call before any stream capture.  Every call
 * runs on the legacy default stream, waits for the step to finish, and leaves the
 * caller's current device as it found it.  All calls share the scratch array (tables
 * recomputed and error word cleared on each call), so calls that overlap on the
 * GPU — from several host threads, say — race. */
#define A3D_NOALLOC_MAX_AXIS 4096
#define A3D_NOALLOC_SCRATCH_BYTES (256 + 3 * A3D_NOALLOC_MAX_AXIS * 8)
int a3d_2order_step_noalloc(const float *cur, float *prev_next, const float *vv, float *rec,
                            int nx, int ny, int nz, int npd, int ldz, float dx, float dy,
                            float dz, int sx, int sy, int sz, float w_next, int rec_z, int it,
                            int nt, int device);

#ifdef __cplusplus
}
#endif
#endif
