// rt_common.cuh -- shared device-side definitions of the GB300 raytracer path.
//
// Device layout (HBM): every 6D field is stored UNPADDED, x fastest
// (Fortran column-major order of the interior of the reference arrays,
// for_src/main_module.f90:135-193).  Ghost cells are not stored: the
// boundary conditions of integrate.f90:14-94 and reflection_condition
// (parallel_mpi.f90:798-876) are applied as index maps when a neighbour is
// read (clamp = open outflow, z-mirror with reversed m = reflection).
//
// A face velocity v_a of the reference lives on faces f = 0..n_a of axis a
// (superbee_fluxes.f90:18 etc. loop over faces s-1..e).  Face f >= 1 is
// stored in the cell-shaped field vel[a] at cell c_a = f-1 ("right face of
// the cell"); face 0 is stored in the plane vel_lo[a], the cell shape with
// axis a collapsed to one.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define RT_ONX 2

namespace rt {

struct Dims {
  int n[6];            // nx ny nz nk nl nm
  long long s[6];      // strides of the unpadded 6D arrays (s[0] = 1)
  long long ps[6][6];  // ps[a][b]: stride along b of the face-0 plane of axis a
  long long ncell;     // product of n
  long long nvol3;     // nx*ny*nz
  long long nspec;     // nk*nl*nm
  int upper_refl;      // enable_upper_reflection (main_module.f90:30)
  int lower_refl;      // enable_lower_reflection (main_module.f90:31)
};

// 1D grids on the padded index range (Fortran index f at position f+1).
struct Grid {
  const double* d[6];  // dxt dyt dzt dkt dlt dmt
  const double* kt;
  const double* lt;
  const double* mt;
};

// padded 3D background fields, Fortran order (x fastest), index f+1 per axis
struct Background {
  const double* Nsqr;
  const double* U;
  const double* V;
  int px, py;          // padded extents in x and y
};

__host__ __device__ __forceinline__ int pidx(int f) { return f + RT_ONX - 1; }

// stride of the plane vel_lo[a] along axis b (axis a collapsed)
__host__ __device__ __forceinline__ long long plane_stride_calc(const Dims& d, int a, int b) {
  return b < a ? d.s[b] : (b == a ? 0 : d.s[b] / d.n[a]);
}
__host__ __device__ __forceinline__ long long plane_stride(const Dims& d, int a, int b) {
  return d.ps[a][b];
}
// fill d.ps from d.n and d.s (host side, once per handle)
__host__ __forceinline__ void fill_plane_strides(Dims& d) {
  for (int a = 0; a < 6; a++)
    for (int b = 0; b < 6; b++) d.ps[a][b] = plane_stride_calc(d, a, b);
}

// ---- exact binary64 arithmetic (never contracted into FMA) --------------
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
// gfortran MAX/MIN of two reals as used by the reference: a > b ? a : b
__device__ __forceinline__ double fmax2(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double fmin2(double a, double b) { return a < b ? a : b; }

// Neighbour coordinate along axis a for a stencil offset, applying the
// reference's ghost-cell rules.  Returns the (possibly mirrored) coordinate;
// mflip is set when the z-reflection reverses the m index
// (parallel_mpi.f90:839, :869).  Open boundaries copy the edge cell
// (integrate.f90:24-94).
__device__ __forceinline__ int map_coord(const Dims& d, int a, int c, int& mflip) {
  const int n = d.n[a];
  if (c >= 0 && c < n) return c;
  if (a == 2) {
    if (c >= n && d.upper_refl) { mflip ^= 1; return 2 * n - 1 - c; }
    if (c < 0 && d.lower_refl) { mflip ^= 1; return -c - 1; }
  }
  return c < 0 ? 0 : n - 1;
}

}  // namespace rt
