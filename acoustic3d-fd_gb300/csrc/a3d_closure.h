// a3d_closure.h — learned absorbing rim for the isotropic engine: geometry of the
// rim and of its face boxes, the parameter layout, and the launchers the engine's
// time loop calls.
//
// The model is padded by 10 cells per face: the outer 4 are never updated (the
// stencil's reach, as in every engine) and the inner 6 form the rim.  The engine
// updates the rim with the undamped equations; after every step the closure adds a
// correction to u, v, w and P in the rim cells:
//
//   x(c)   = [u, v, w, P / (rho vp), kappa u, kappa v, kappa w, kappa P / (rho vp)]
//            (kappa = vp dt / min(dx, dy, dz), the cell's Courant number)
//   h_f(c) = relu(W1 * x)(c)                  3x3x3 conv, 8 -> 32 channels, no bias
//   y_f(c) = (W2_f * h_f)(c)                  3x3x3 conv, 32 -> 4 channels, per face f
//   delta  = sum over the faces f whose rim holds c of G_f[depth_f(c)] . y_f(c)
//   (u, v, w, P) += (delta_0, delta_1, delta_2, rho vp delta_3)
//
// Both layers are positively homogeneous (no biases, relu), so the correction
// scales with the wavefield.  Weights and hidden activations are bfloat16 values,
// accumulation is float.  Face f = 2 * axis + side (axis 0 z, 1 x, 2 y; side 0 the
// low face, 1 the high face).  h_f lives on the face box: depth -1 .. 5 along the
// face normal (depth 0 touches the interior) by the full updated extent [4, nn - 4)
// of the two other axes; h is zero outside the box.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace a3d {

constexpr int CL_PAD = 10, CL_RIM = 6, CL_CIN = 8, CL_CH = 32, CL_COUT = 4;
constexpr int CL_NW1 = CL_CH * CL_CIN * 27;              // W1 [j][i][tap]
constexpr int CL_NW2 = 6 * CL_COUT * CL_CH * 27;         // W2 [f][o][j][tap]
constexpr int CL_NG = 6 * CL_RIM * CL_COUT;              // G  [f][depth][o]
constexpr int CL_NPARAM = CL_NW1 + CL_NW2 + CL_NG;       // 27792
// tap = ((dy + 1) * 3 + (dx + 1)) * 3 + (dz + 1), the cell offset of a 3x3x3 kernel

struct ClGeom {
    int nn[3];            // padded extents (z, x, y)
    long long ldz;        // row pitch: element (iz, ix, iy) at iz + ldz * (ix + nn[1] * iy)
    int T1[6], T2[6];     // face f's tangential extents (nn - 8 of its first / second other axis)
    long long hoff[7];    // first cell of face f's box in the hidden buffer; hoff[6] = total
    int blo[6][3], bext[6][3];  // the rim as six disjoint boxes (z, x, y)
    long long roff[7];    // first cell of each box; roff[6] = rim cells
};

// geometry of a grid padded by CL_PAD cells per face (nn >= 2 * CL_PAD + 1 per axis)
ClGeom cl_geom(int nnz, int nnx, int nny, long long ldz);

// canonical parameters (float, CL_NPARAM) -> the kernels' layouts, each value
// rounded to bfloat16: W1c [tap][i][j], W2c [f][tap][j][o], Gc [f][depth][o]
void cl_pack_params(const float *canon, float *packed /* CL_NPARAM */);
float cl_round_bf16(float x);

// zinv = 1 / (rho vp) (0 where rho vp is not positive), kappa = vp * courant over n elements
cudaError_t cl_launch_scales(const float *rho, const float *vp, float courant, float *zinv, float *kap,
                             size_t n, cudaStream_t st);

// sets the kernels' shared-memory limit on the current device (once per device,
// before the first launch or stream capture)
cudaError_t cl_prepare();

// the two layers: hidden activations of every face-box cell into h, then the
// correction of every rim cell (added in place, or written to dout when set)
cudaError_t cl_launch_hidden(const ClGeom &g, const float *u, const float *v, const float *w, const float *P,
                             const float *zinv, const float *kap, const float *packed, __nv_bfloat16 *h,
                             cudaStream_t st);
cudaError_t cl_launch_correct(const ClGeom &g, float *u, float *v, float *w, float *P, const float *zinv,
                              const float *packed, const __nv_bfloat16 *h, float *dout, long long dstride,
                              cudaStream_t st);

// one application of the closure to the fields (in place); h: hoff[6] * 32 bfloat16
cudaError_t cl_launch_apply(const ClGeom &g, float *u, float *v, float *w, float *P, const float *zinv,
                            const float *kap, const float *packed, __nv_bfloat16 *h, cudaStream_t st);

// tensor-core inference (a3d_closure_tc.cu): the weights as six per-face bfloat16
// images, both layers fused per face-box block into y (float4 per face-box cell),
// then the per-cell combination over faces, added to the fields (or written to
// dout, four fields of stride dstride).  err: kernel error word.
size_t cl_tc_image_halves();
void cl_pack_tc(const float *canon, uint16_t *image);
cudaError_t cl_tc_prepare();
cudaError_t cl_launch_apply_tc(const ClGeom &g, float *u, float *v, float *w, float *P, const float *zinv,
                               const float *kap, const uint16_t *image, const float *Gc, float4 *y, int *err,
                               float *dout, long long dstride, int nsm, cudaStream_t st);

// dense copy (z fastest) of the box [off, nn - off) of four fields of a padded grid
// (extents nnz, nnx, nny; row pitch ldz) into out: u, v, w, P one after another
cudaError_t cl_launch_tap(int nnz, int nnx, int nny, long long ldz, int off, const float *u, const float *v,
                          const float *w, const float *P, float *out, cudaStream_t st);

}  // namespace a3d
