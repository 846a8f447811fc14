/*
 * a3d_oracle.h — CPU restatement of the reference forward-modelling engines.
 *
 * TEST INFRASTRUCTURE ONLY.  These functions are the oracle the CUDA engines are
 * tested against: the tests, the smoke check and the CPU-baseline leg of the
 * benchmark call them.  The product path never links, loads or calls them.
 *
 * Each engine runs one shot on the host, OpenMP-parallel over y-planes, and
 * returns the full (undecimated) receiver record in the reference's internal
 * layout rec[it + nt*(ix + nx*iy)] (it fastest), with the direct-wave mute
 * applied when cfg->mute is set, plus optional snapshots (model window,
 * z fastest, then x, then y; one nz*nx*ny block per snapshot taken).
 *
 * Two arithmetic forms:
 *   form 0 — "literal": the reference's own arithmetic, operation by operation
 *            (split PML fields px,py,pz (qx,qy,qz) everywhere, P = px+py+pz,
 *            source added into P and then overwritten).
 *   form 1 — "engine": the arithmetic of the CUDA engines (unsplit P/Q in the
 *            undamped interior, split components only on PML-damped axes,
 *            source injected into the velocity update's view of P only, the
 *            velocity update multiplied by the float reciprocal of density).
 *            The CUDA kernels reproduce this form bit for bit.
 * For the 2nd-order engine the two forms coincide.
 *
 * The _f32 variants compute the wavefield in float; the _f64 variants compute
 * the wavefield in double from the same float-valued coefficients, source
 * samples and model (the FP64 oracle run) and write double records/snapshots.
 */
#ifndef A3D_ORACLE_H
#define A3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny, nz;        /* model grid; files are z fastest, then x, then y  */
    float dx, dy, dz;      /* grid spacing (m)                                  */
    int sx, sy, sz;        /* shot position in model cells (sxbeg,sybeg,szbeg)  */
    int nt;                /* time steps                                        */
    float dt, fm;          /* time step (s), peak frequency (Hz)                */
    int wtype;             /* source wavelet 1..6 (1st-order isotropic only)    */
    int npml;              /* absorber width: PML cells (1st order) or sponge
                              cells npd (2nd order, reference value 50)         */
    int rec_z;             /* 2nd order only: receiver depth in model cells
                              (reference records at model z = 1)                */
    int mute;              /* apply the direct-wave mute to the record          */
    int snap_every;        /* 0: no snapshots; else take one when it%snap_every==0 */
    int snap_skip0;        /* 1: never take a snapshot at it == 0               */
    int form;              /* 0 literal, 1 engine                               */
    int threads;           /* OpenMP threads (0 = runtime default)              */
    int store;             /* float oracle, engine form, 1st-order engines: the
                              CUDA engine's wavefield storage emulated — 0 float;
                              1 bfloat16 (every field); 2 float16 of 2^k x (every
                              field: k = sig_v_log2 for u, v, w, sig_p_log2 for P,
                              Q and split components); 4 (VTI, TTI) float16 u, v,
                              w at 2^sig_v_log2, P, Q float (FP16V).  Formats no
                              engine stores yet, for measuring them: 5 every field
                              a 24-bit float (float with the low 8 significand bits
                              rounded off); 6 u, v, w 24-bit, P, Q float          */
    int sig_v_log2;        /* the engine's scales of store 2 / 4 (log2)         */
    int sig_p_log2;
} a3d_oracle_cfg;

/* Return 0 on success, negative on bad arguments / allocation failure. */
int a3d_oracle_2o_f32(const a3d_oracle_cfg *c, const float *vel, float *rec, float *snaps);
int a3d_oracle_2o_f64(const a3d_oracle_cfg *c, const float *vel, double *rec, double *snaps);

int a3d_oracle_iso_f32(const a3d_oracle_cfg *c, const float *vel, const float *rho,
                       float *rec, float *snaps);
int a3d_oracle_iso_f64(const a3d_oracle_cfg *c, const float *vel, const float *rho,
                       double *rec, double *snaps);

int a3d_oracle_vti_f32(const a3d_oracle_cfg *c, const float *vel, const float *rho,
                       const float *eps, const float *del, float *rec, float *snaps);
int a3d_oracle_vti_f64(const a3d_oracle_cfg *c, const float *vel, const float *rho,
                       const float *eps, const float *del, double *rec, double *snaps);

int a3d_oracle_tti_f32(const a3d_oracle_cfg *c, const float *vel, const float *eps,
                       const float *del, const float *theta, const float *phi,
                       float *rec, float *snaps);
int a3d_oracle_tti_f64(const a3d_oracle_cfg *c, const float *vel, const float *eps,
                       const float *del, const float *theta, const float *phi,
                       double *rec, double *snaps);

/* Setup pieces, exported so tests can check them on their own. */
float a3d_oracle_ricker2o(int it, float dt, float fm);               /* Toa_3dfd_cuda.cu:34-43 */
float a3d_oracle_round_f16(float x);  /* x rounded to float16 (ties to even), as float  */
float a3d_oracle_round_bf16(float x); /* x rounded to bfloat16 (ties to even), as float */
float a3d_oracle_round_f24(float x);  /* x rounded to a 24-bit float (ties to even)     */
float a3d_oracle_wavelet(int wtype, float t, float fm);              /* ..iso..:52-87          */
float a3d_oracle_d0(const float *vp_padded, int nnx, int nny, int nnz, int npml,
                    float dx, float dy, float dz);                   /* ..iso..:193-195        */
void  a3d_oracle_pml(float dt, float d0, int n, int npml,
                     float *c1, float *c2, float *a1, float *a2);    /* ..iso..:263-291        */
int   a3d_oracle_mute_nt(int ix, int iy, int sx, int sy, int sz, float dx, float dy,
                         float dz, float dt, float fm, float v0);    /* ..iso..:322-347        */

#ifdef __cplusplus
}
#endif
#endif
