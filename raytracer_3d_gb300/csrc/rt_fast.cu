// rt_fast.cu -- fast binary64 step (variant RT_VARIANT_FAST).
//
// The same two passes as the two-pass bit-exact step (rt_split.cu): every
// face flux is evaluated once into the binary64 flux fields, then a second
// pass forms the divergence, the mean-flow term and the update.  What
// changes is the arithmetic (rt_fast.cuh): no division and no binary64
// comparison anywhere, because GB300's binary64 pipe is the limit of this
// form (about 0.5 T operations/s against tens of T for binary32):
//
//   pass 1   F = v*E_up + h*psi                 4 binary64 ops per face
//            (psi selected on the integer pipes; h cached per face)
//   pass 2   E_new = E*mu + sum_a c_a*(F_l - F_r)   2 per axis + 1
//            mu = 1 - dt*(lambda_x + lambda_y + lambda_z)  (cached per cell)
//            c_a = dt/d_a                          (per-axis table)
//
// which is the reference's E + dt*(dE - meanfl) (integrate.f90:105-262)
// with dE = -sum_a (F_r - F_l)/d_a, regrouped.  About 37 binary64
// operations per cell against roughly 290 for the bit-exact sequence
// (twelve correctly rounded divisions, limiter comparisons).  Results
// agree with the reference to a few units in the last place of the terms
// per step; the parity tests hold them to the plain form's bound of 1e-12
// relative L-infinity per step.
//
// Cached fields: h of every face in the handle's uCFL fields (the uCFL of
// the bit-exact kernels is recomputed when one of them runs next), mu
// (8 B per cell) and the table c_a.
#include "rt_fast.cuh"
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

// resident CTAs per SM the two passes are compiled for (register budget:
// 64 per thread).  Both passes wait on scattered loads of E and the flux
// fields; at 32^6 four CTAs per SM measured 119 ms per step, three 128 ms,
// two (96 registers) 157 ms
#ifndef RT_FAST_MINB_FLUX
#define RT_FAST_MINB_FLUX 4
#endif
#ifndef RT_FAST_MINB_UPD
#define RT_FAST_MINB_UPD 4
#endif

dim3 cells_grid(const Dims& d) {
  const long long bx = (d.nvol3 + 255) / 256;
  const long long by = d.nspec < 65535 ? d.nspec : 65535;
  return dim3((unsigned)bx, (unsigned)by, 1);
}

// The u-th spectral plane (k,l,m) in band order: bands of B values of m,
// l outer inside a band, m inner, k fastest (B = 1: the natural order).
// The CTAs that run together then read the m +-1, +-2 neighbour planes of E
// (pass 1) and the m-1 flux planes (pass 2) from L2 instead of HBM.
__device__ __forceinline__ long long band_plane(const Dims& d, long long u, int B) {
  const int nk = d.n[3], nl = d.n[4], nm = d.n[5];
  const long long per_band = (long long)nk * nl * B;
  const long long b = u / per_band;
  long long r = u - b * per_band;
  const int bs = (b + 1) * B > nm ? nm - (int)b * B : B;   // the last band may be shorter
  const int k = (int)(r % nk);
  r /= nk;
  const int m = (int)b * B + (int)(r % bs);
  const int l = (int)(r / bs);
  return k + (long long)nk * (l + (long long)nl * m);
}

// h = |v|/2 * (1 - |v*dt/d(f)|) of every face of axis a: right faces
// f = c_a + 1 into hr, the face-0 plane into hl (spacing d(0)), the faces
// and spacings of the reference's uCFL (superbee_fluxes.f90:19)
__global__ void fast_h_kernel(Dims d, Grid g, int a, double dt, const double* vel, const double* vlo,
                              double* hr, double* hl) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < d.ncell; p += stride) {
    const int ca = (int)((p / d.s[a]) % d.n[a]);
    const double v = vel[p];
    hr[p] = 0.5 * fabs(v) * (1.0 - fabs(v * dt / g.d[a][pidx(ca + 1)]));
  }
  const long long np = d.ncell / d.n[a];
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < np; q += stride) {
    const double v = vlo[q];
    hl[q] = 0.5 * fabs(v) * (1.0 - fabs(v * dt / g.d[a][pidx(0)]));
  }
}

// mu = 1 - dt*(lambda_x[nx>1] + lambda_y[ny>1] + lambda_z[nz>1]) per cell
// (the growth-rate terms of integrate.f90:202-252), and the per-axis
// tables c_a(f) = dt/d_a(f) on the padded index range
__global__ void fast_mu_kernel(Dims d, Grid g, double dt, const double* lx, const double* ly, const double* lz,
                               double* mu, double* tab, long long toff1, long long toff2, long long toff3,
                               long long toff4, long long toff5) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long p = t0; p < d.ncell; p += stride) {
    double s = 0.0;
    if (d.n[0] > 1) s += lx[p];
    if (d.n[1] > 1) s += ly[p];
    if (d.n[2] > 1) s += lz[p];
    mu[p] = 1.0 - dt * s;
  }
  const long long off[7] = {0, toff1, toff2, toff3, toff4, toff5, toff5 + d.n[5] + 2 * RT_ONX};
  for (long long i = t0; i < off[6]; i += stride) {
    int a = 0;
    while (i >= off[a + 1]) a++;
    tab[i] = dt / g.d[a][i - off[a]];
  }
}

// pass 1: the right-face flux of every axis with n > 1 (and the face-0
// flux at c_a = 0), one thread per cell
// ones: ~0 (see sel64)
__global__ void __launch_bounds__(256, RT_FAST_MINB_FLUX) fast_flux_kernel(StepArgs<double> A, SplitFluxes F,
                                                                            int band, unsigned long long ones) {
  const Dims& d = A.d;
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= d.nvol3) return;
  for (long long u = blockIdx.y; u < d.nspec; u += gridDim.y) {
    const long long sp = band_plane(d, u, band);
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
      __stcs(F.f[a] + p, flux_fast64(__ldcs(A.vel[a] + p), __ldcs(A.uc[a] + p), Em1, e0, Ep1, Ep2, ones));
      if (ca == 0) {  // face 0: E(-2), E(-1), E(0), E(1) through the boundary maps
        const long long q = plane_index(d, a, c);
        const double Em2 = A.E[nb_index(d, p, a, ca, -2, c[5])];
        F.f0[a][q] = flux_fast64(A.vlo[a][q], A.ucl[a][q], Em2, Em1, e0, Ep1, ones);
      }
    }
  }
}

// pass 2: E_new = E*mu + sum_a c_a*(F_l - F_r), axis order x,y,z,k,l,m
__global__ void __launch_bounds__(256, RT_FAST_MINB_UPD) fast_update_kernel(StepArgs<double> A, SplitFluxes F,
                                                                            const double* mu, FastTab T, int band) {
  const Dims& d = A.d;
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= d.nvol3) return;
  for (long long u = blockIdx.y; u < d.nspec; u += gridDim.y) {
    const long long sp = band_plane(d, u, band);
    int c[6];
    cell_coords(d, v3, sp, c);
    const long long p = v3 + sp * d.nvol3;
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const int ca = c[a];
      const double fr = F.f[a][p];   // also the left flux of cell p + s_a: kept in L2
      const double fl = ca > 0 ? F.f[a][p - d.s[a]] : F.f0[a][plane_index(d, a, c)];
      acc = __fma_rn(T.c[a][pidx(ca + 1)], __dsub_rn(fl, fr), acc);
    }
    __stcs(A.Enew + p, __fma_rn(__ldcs(A.E + p), __ldcs(mu + p), acc));
  }
}

}  // namespace

cudaError_t launch_fast_prepare(const Dims& d, const Grid& g, double dt, const double* const* vel,
                                const double* const* vlo, const double* const* lam, double* const* hr,
                                double* const* hl, double* mu, double* tab, const long long* toff,
                                cudaStream_t st) {
  for (int a = 0; a < 6; a++) {
    if (d.n[a] <= 1) continue;
    fast_h_kernel<<<8 * 152, 256, 0, st>>>(d, g, a, dt, vel[a], vlo[a], hr[a], hl[a]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  fast_mu_kernel<<<8 * 152, 256, 0, st>>>(d, g, dt, lam[0], lam[1], lam[2], mu, tab, toff[1], toff[2], toff[3],
                                         toff[4], toff[5]);
  return cudaGetLastError();
}

cudaError_t launch_step_fast(const StepArgs<double>& A, const SplitFluxes& F, const double* mu, const FastTab& T,
                             int band, cudaStream_t st) {
  const dim3 g = cells_grid(A.d);
  const int B = band < 1 ? 1 : (band > A.d.n[5] ? A.d.n[5] : band);
  fast_flux_kernel<<<g, 256, 0, st>>>(A, F, B, ~0ull);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  fast_update_kernel<<<g, 256, 0, st>>>(A, F, mu, T, B);
  return cudaGetLastError();
}

}  // namespace rt
