// a3d_setup.h — host-side setup of a shot: model padding into the device
// layout, source wavelets, PML profiles, sponge factors, SV taper, mute.
// Every formula follows the reference operation by operation (double where the
// reference computes in double), so the device sees the same coefficient values.
#pragma once
#include <cstddef>
#include <vector>

namespace a3d {

// Device layout of a padded field: element (iz, ix, iy) at base + idx(iz, ix, iy),
// base = allocation + zoff elements.  zoff = 28 puts the first updated cell of a
// row (iz = 4) on a 128-byte boundary, and ldz (a multiple of 32 elements) keeps
// every row so, which is what makes the kernels' 32-wide TMA boxes whole sectors.
struct Grid {
    static constexpr int zoff = 28;
    int nx = 0, ny = 0, nz = 0;  // model
    int pad = 0;                 // cells added on every face
    int nnx = 0, nny = 0, nnz = 0, ldz = 0;
    void set(int nx_, int ny_, int nz_, int pad_) {
        nx = nx_; ny = ny_; nz = nz_; pad = pad_;
        nnx = nx + 2 * pad; nny = ny + 2 * pad; nnz = nz + 2 * pad;
        ldz = (zoff + nnz + 31) / 32 * 32;
    }
    size_t elems() const { return (size_t)ldz * nnx * nny; }  // allocation, in elements
    size_t idx(int iz, int ix, int iy) const {
        return (size_t)iz + (size_t)ldz * ((size_t)ix + (size_t)nnx * iy);
    }
};

float ricker2o(int it, float dt, float fm);          // Toa_3dfd_cuda.cu:34-43
float wavelet1(int wtype, float t, float favg);      // ..iso..:52-87
float pml_d0(float vmid, int npml, float dx, float dy, float dz);  // ..iso..:193-195
void pml_profile(float dt, float d0, int n, int npml, float *c1, float *c2, float *a1,
                 float *a2);                         // ..iso..:263-291
int mute_nt(int ix, int iy, int sx, int sy, int sz, float dx, float dy, float dz, float dt,
            float fm, float v0);                     // ..iso..:322-347
// sponge factor of one face position as (hi, lo) floats; (0,0) outside the sponge
void sponge_factors(int n, int npd, float *hi_lo /* 2*(n + 2*4 + 2*npd) */);  // 2O:123-154
// SV-ball taper factor for r^2 = 0..225 as (hi, lo) floats   ..vti..:154-175
void sv_taper_table(float *hi_lo /* 2*226 */);

}  // namespace a3d
