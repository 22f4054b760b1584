// rt_split.cu -- two-pass binary64 step (variant RT_VARIANT_SPLIT).
//
// The binary64 form is bound by the FP64 pipe, and most of its work is the
// superbee flux of superbee_fluxes.f90:19-30 (one correctly rounded
// division each).  The fused kernels evaluate each z, k, l and m face twice
// (once from each side); this form evaluates every face once, as the
// reference does:
//   pass 1  split_flux_kernel: per cell, the right-face flux of each axis
//           (and, at c_a = 0, the face-0 flux) into binary64 flux fields;
//   pass 2  split_update_kernel: flux divergence in the axis order x,y,z,
//           k,l,m (integrate.f90:105-200), mean-flow term (:202-252) and the
//           update (:255-268).
// Both passes use the fused kernels' arithmetic (flux_fp64u with the cached
// uCFL, the same boundary maps), so the result is bit-identical to them and
// to the oracle.  Six flux fields of the cell shape and six face-0 planes
// (axes with n > 1 only) are the price: 48 B per cell more device memory and
// about 100 B per cell more HBM traffic, which the FP64-bound step can
// afford (it uses a few percent of the bandwidth).
#include "rt_kernels.h"
#include "rt_step.cuh"

namespace rt {

namespace {

__device__ __forceinline__ void cell_coords(const Dims& d, long long v3, long long sp, int c[6]) {
  c[0] = (int)(v3 % d.n[0]);
  long long r = v3 / d.n[0];
  c[1] = (int)(r % d.n[1]);
  c[2] = (int)(r / d.n[1]);
  c[3] = (int)(sp % d.n[3]);
  r = sp / d.n[3];
  c[4] = (int)(r % d.n[4]);
  c[5] = (int)(r / d.n[4]);
}

// one thread per (x,y,z) cell, blocks over the (k,l,m) planes
dim3 cells_grid(const Dims& d) {
  const long long bx = (d.nvol3 + 255) / 256;
  const long long by = d.nspec < 65535 ? d.nspec : 65535;
  return dim3((unsigned)bx, (unsigned)by, 1);
}

__global__ void __launch_bounds__(256) split_flux_kernel(StepArgs<double> A, SplitFluxes F) {
  const Dims& d = A.d;
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= d.nvol3) return;
  for (long long sp = blockIdx.y; sp < d.nspec; sp += gridDim.y) {
    int c[6];
    cell_coords(d, v3, sp, c);
    const long long p = v3 + sp * d.nvol3;
    const double e0 = A.E[p];
#pragma unroll
    for (int a = 0; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const int ca = c[a];
      const double Em1 = A.E[nb_index(d, p, a, ca, -1, c[5])];
      const double Ep1 = A.E[nb_index(d, p, a, ca, +1, c[5])];
      const double Ep2 = A.E[nb_index(d, p, a, ca, +2, c[5])];
      // face ca+1: E(ca-1), E(ca), E(ca+1), E(ca+2)
      F.f[a][p] = flux_fp64u(__ldcs(A.vel[a] + p), __ldcs(A.uc[a] + p), Em1, e0, Ep1, Ep2);
      if (ca == 0) {  // face 0: E(-2), E(-1), E(0), E(1) through the boundary maps
        const long long q = plane_index(d, a, c);
        const double Em2 = A.E[nb_index(d, p, a, ca, -2, c[5])];
        F.f0[a][q] = flux_fp64u(A.vlo[a][q], A.ucl[a][q], Em2, Em1, e0, Ep1);
      }
    }
  }
}

__global__ void __launch_bounds__(256) split_update_kernel(StepArgs<double> A, SplitFluxes F) {
  const Dims& d = A.d;
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= d.nvol3) return;
  for (long long sp = blockIdx.y; sp < d.nspec; sp += gridDim.y) {
    int c[6];
    cell_coords(d, v3, sp, c);
    const long long p = v3 + sp * d.nvol3;
    const double e0 = A.E[p];
    double dE = 0.;
#pragma unroll
    for (int a = 0; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const int ca = c[a];
      const double fr = F.f[a][p];
      const double fl = ca > 0 ? F.f[a][p - d.s[a]] : F.f0[a][plane_index(d, a, c)];
      dE = dsub(dE, ddiv(dsub(fr, fl), A.g.d[a][pidx(ca + 1)]));
    }
    double mf = 0.;
    if (d.n[0] > 1) mf = dadd(mf, dmul(e0, __ldcs(A.lam[0] + p)));
    if (d.n[1] > 1) mf = dadd(mf, dmul(e0, __ldcs(A.lam[1] + p)));
    if (d.n[2] > 1) mf = dadd(mf, dmul(e0, __ldcs(A.lam[2] + p)));
    __stcs(A.Enew + p, dadd(e0, dmul(A.dt, dsub(dE, mf))));
  }
}

}  // namespace

cudaError_t launch_step_split(const StepArgs<double>& A, const SplitFluxes& F, cudaStream_t st) {
  const dim3 g = cells_grid(A.d);
  split_flux_kernel<<<g, 256, 0, st>>>(A, F);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  split_update_kernel<<<g, 256, 0, st>>>(A, F);
  return cudaGetLastError();
}

}  // namespace rt
