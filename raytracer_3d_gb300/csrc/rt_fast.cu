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

// 32-bit index geometry of the two passes (the host rejects fields of 2^31
// cells or more; their flux fields alone would exceed the device memory):
// strides, the divisors of the cell and band coordinates, and the band
// shape.  Band order of the spectral planes: bands of B values of m, l
// outer inside a band, m inner, k fastest; B divides nm.  The CTAs that
// run together then read the m +-1, +-2 neighbour planes of E (pass 1) and
// the m-1 flux planes (pass 2) from L2 instead of HBM.
struct FastGeom {
  int s[6];                  // strides of the 6D fields
  int ps[6][6];              // strides of the face-0 planes
  unsigned nvol3, nspec;
  DivU32 nx, ny;             // v3 -> x, y, z
  DivU32 per_band, nk, B;    // u -> band, k, m in band, l
};

FastGeom make_geom(const Dims& d, int B) {
  FastGeom G;
  for (int a = 0; a < 6; a++) {
    G.s[a] = (int)d.s[a];
    for (int b = 0; b < 6; b++) G.ps[a][b] = (int)d.ps[a][b];
  }
  G.nvol3 = (unsigned)d.nvol3;
  G.nspec = (unsigned)d.nspec;
  G.nx = make_div((unsigned)d.n[0]);
  G.ny = make_div((unsigned)d.n[1]);
  G.per_band = make_div((unsigned)(d.n[3] * d.n[4] * B));
  G.nk = make_div((unsigned)d.n[3]);
  G.B = make_div((unsigned)B);
  return G;
}

// coordinates of cell (v3, u) and its index: u is the plane's position in
// band order
__device__ __forceinline__ int cell_at(const Dims& d, const FastGeom& G, unsigned v3, unsigned u, int c[6]) {
  const unsigned q = G.nx.div(v3);
  c[0] = (int)(v3 - q * G.nx.d);
  c[2] = (int)G.ny.div(q);
  c[1] = (int)(q - (unsigned)c[2] * G.ny.d);
  const unsigned b = G.per_band.div(u);
  const unsigned r = u - b * G.per_band.d;
  const unsigned r2 = G.nk.div(r);
  c[3] = (int)(r - r2 * G.nk.d);
  c[4] = (int)G.B.div(r2);
  c[5] = (int)(b * G.B.d + (r2 - (unsigned)c[4] * G.B.d));
  const unsigned sp = (unsigned)c[3] + (unsigned)d.n[3] * ((unsigned)c[4] + (unsigned)d.n[4] * (unsigned)c[5]);
  return (int)(v3 + sp * G.nvol3);
}

// nb_index in 32-bit arithmetic
__device__ __forceinline__ int nb32(const Dims& d, const FastGeom& G, int p, int a, int c, int off, int cm) {
  int flip = 0;
  const int c2 = map_coord(d, a, c + off, flip);
  int q = p + (c2 - c) * G.s[a];
  if (flip) q += ((d.n[5] - 1 - cm) - cm) * G.s[5];
  return q;
}

__device__ __forceinline__ int plane32(const FastGeom& G, int a, const int c[6]) {
  int q = 0;
#pragma unroll
  for (int b = 0; b < 6; b++) q += c[b] * G.ps[a][b];
  return q;
}

// resident CTAs per SM the two passes are compiled for (register budgets
// 40 and 32 per thread, no spills).  Both passes wait on scattered loads
// of E and the flux fields, so warps in flight pay: at 32^6 the pair
// measured 108.1 ms per step at 4/4 CTAs, 102.1 at 5/5, 98.8 at 6/6 and
// 97.1 at 6/8 (the 64-bit index form at 4/4: 120.7 ms)
#ifndef RT_FAST_MINB_FLUX
#define RT_FAST_MINB_FLUX 6
#endif
#ifndef RT_FAST_MINB_UPD
#define RT_FAST_MINB_UPD 8
#endif

dim3 cells_grid(const Dims& d) {
  const long long bx = (d.nvol3 + 255) / 256;
  const long long by = d.nspec < 65535 ? d.nspec : 65535;
  return dim3((unsigned)bx, (unsigned)by, 1);
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

// Face 0 of an axis whose lower boundary copies the edge cell (every axis
// but z with the lower reflection): E(-2) = E(-1) = E(0), so Rj = 0, the
// limited slope is 0 and the flux is v*E(0) exactly.  The update pass forms
// it from the cell's own E (one multiply); only the reflected z face 0 (a
// whole plane of cells) is evaluated in full by the flux pass.  Along x the
// cells with c_x = 0 are one lane of every warp: a full flux evaluation
// there would occupy the binary64 pipe for the whole warp's issue slots.
__device__ __forceinline__ bool face0_is_copy(const Dims& d, int a) { return a != 2 || !d.lower_refl; }

// pass 1: the right-face flux of every axis with n > 1 (and the reflected
// z face 0), one thread per cell.
// XW: x rows are whole segments of a warp (nx divides 32; CTAs of 256
// threads start on a row).  The x faces then share their differences:
// lane x forms D(x) = E(x+1) - E(x) once, the upwind difference of face
// x+1/2 is D(x-1) or D(x+1) from the neighbouring lane, and E(x+1) comes
// from the next lane too -- one binary64 subtraction per x face instead of
// two, and no x-neighbour loads.  The operands and operations are those of
// flux_fast64, so the fluxes are the same bits; beyond the row ends the
// ghost cells copy the edge, so D(-1) = D(nx-1) = D(nx) = 0 there.  Lanes
// past the last cell run on a clamped cell (the shuffles need every lane)
// and store nothing.
template <bool XW>
__global__ void __launch_bounds__(256, RT_FAST_MINB_FLUX) fast_flux_kernel(StepArgs<double> A, SplitFluxes F,
                                                                            FastGeom G) {
  const Dims& d = A.d;
  const unsigned v3raw = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = v3raw < G.nvol3;
  if (!XW && !valid) return;
  const unsigned v3 = valid ? v3raw : G.nvol3 - 1;
  const int nx = d.n[0];
  for (unsigned u = blockIdx.y; u < G.nspec; u += gridDim.y) {
    int c[6];
    const int p = cell_at(d, G, v3, u, c);
    const double e0 = A.E[p];
#pragma unroll
    for (int a = 0; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const int ca = c[a];
      if (XW && a == 0) {
        const double Ep1 = __shfl_down_sync(0xffffffffu, e0, 1, nx);   // the row's last lane: its own E
        const double Rj = __dsub_rn(Ep1, e0);
        const double Dm = __shfl_up_sync(0xffffffffu, Rj, 1, nx);
        const double Dp = __shfl_down_sync(0xffffffffu, Rj, 1, nx);
        const double v = __ldcs(A.vel[0] + p), h = __ldcs(A.uc[0] + p);
        const bool pos = f64_pos(v);
        const double up = pos ? (ca > 0 ? Dm : 0.0) : (ca < nx - 1 ? Dp : 0.0);
        const double Fx = __fma_rn(h, superbee_slope64(Rj, up), __dmul_rn(v, pos ? e0 : Ep1));
        if (valid) __stcs(F.f[0] + p, Fx);
        continue;
      }
      const double Em1 = A.E[nb32(d, G, p, a, ca, -1, c[5])];
      const double Ep1 = A.E[nb32(d, G, p, a, ca, +1, c[5])];
      const double Ep2 = A.E[nb32(d, G, p, a, ca, +2, c[5])];
      const double Fa = flux_fast64(__ldcs(A.vel[a] + p), __ldcs(A.uc[a] + p), Em1, e0, Ep1, Ep2);
      if (valid) __stcs(F.f[a] + p, Fa);
      if (valid && ca == 0 && !face0_is_copy(d, a)) {  // E(-2), E(-1), E(0), E(1) through the boundary maps
        const int q = plane32(G, a, c);
        const double Em2 = A.E[nb32(d, G, p, a, ca, -2, c[5])];
        F.f0[a][q] = flux_fast64(A.vlo[a][q], A.ucl[a][q], Em2, Em1, e0, Ep1);
      }
    }
  }
}

// pass 2: E_new = E*mu + sum_a c_a*(F_l - F_r), axis order x,y,z,k,l,m
__global__ void __launch_bounds__(256, RT_FAST_MINB_UPD) fast_update_kernel(StepArgs<double> A, SplitFluxes F,
                                                                            const double* mu, FastTab T, FastGeom G) {
  const Dims& d = A.d;
  const unsigned v3 = blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= G.nvol3) return;
  for (unsigned u = blockIdx.y; u < G.nspec; u += gridDim.y) {
    int c[6];
    const int p = cell_at(d, G, v3, u, c);
    const double e0 = __ldcs(A.E + p);
    double acc = 0.0;
#pragma unroll
    for (int a = 0; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const int ca = c[a];
      const double fr = F.f[a][p];   // also the left flux of cell p + s_a: kept in L2
      double fl;
      if (ca > 0) {
        fl = F.f[a][p - G.s[a]];
      } else {
        const int q = plane32(G, a, c);
        fl = face0_is_copy(d, a) ? __dmul_rn(A.vlo[a][q], e0) : F.f0[a][q];
      }
      acc = __fma_rn(T.c[a][pidx(ca + 1)], __dsub_rn(fl, fr), acc);
    }
    __stcs(A.Enew + p, __fma_rn(e0, __ldcs(mu + p), acc));
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
  const Dims& d = A.d;
  if (d.ncell >= (1ll << 31)) return cudaErrorInvalidValue;
  // the band: the largest divisor of nm not above the requested width
  int B = band < 1 ? 1 : (band > d.n[5] ? d.n[5] : band);
  while (d.n[5] % B) B--;
  const FastGeom G = make_geom(d, B);
  const dim3 g = cells_grid(d);
  if (d.n[0] >= 2 && 32 % d.n[0] == 0) fast_flux_kernel<true><<<g, 256, 0, st>>>(A, F, G);
  else fast_flux_kernel<false><<<g, 256, 0, st>>>(A, F, G);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  fast_update_kernel<<<g, 256, 0, st>>>(A, F, mu, T, G);
  return cudaGetLastError();
}

}  // namespace rt
