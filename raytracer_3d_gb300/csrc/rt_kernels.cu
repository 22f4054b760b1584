// rt_kernels.cu -- sm_103a kernels of the time-stepping path:
//   coefficient kernels   calc_parameter.f90:13-261
//   fused step kernel     superbee_fluxes.f90 + integrate.f90:102-268
//   budget kernels        diagnose.f90:46-329 (reductions)
#include "rt_kernels.h"

#include "rt_coeff.cuh"
#include "rt_step.cuh"
#include "rt_step2.cuh"
#include "rt_step3.cuh"
#include "rt_step4.cuh"

namespace rt {

// ---------------------------------------------------------------------------
// index helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void decode(const Dims& d, long long v3, long long sp, int c[6]) {
  c[0] = (int)(v3 % d.n[0]);
  long long r = v3 / d.n[0];
  c[1] = (int)(r % d.n[1]);
  c[2] = (int)(r / d.n[1]);
  c[3] = (int)(sp % d.n[3]);
  r = sp / d.n[3];
  c[4] = (int)(r % d.n[4]);
  c[5] = (int)(r / d.n[4]);
}

// ---------------------------------------------------------------------------
// coefficients
// ---------------------------------------------------------------------------
// One thread per interior cell: the six right-face velocities and the three
// growth rates, binary64.
__global__ void __launch_bounds__(128) coeff_cells_kernel(Dims d, Background bg, Grid g, Phys ph,
                                                          CoeffOut64 out) {
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= d.nvol3) return;
  for (long long sp = blockIdx.y; sp < d.nspec; sp += gridDim.y) {
    int c0[6];
    decode(d, v3, sp, c0);
    int c[6];
#pragma unroll
    for (int b = 0; b < 6; b++) c[b] = c0[b] + 1;  // Fortran indices
    const long long p = v3 + sp * d.nvol3;
    double v[6];
    for (int a = 0; a < 6; a++) {
      v[a] = face_velocity(d, bg, g, ph, a, c);
      out.vel[a][p] = v[a];
    }
    double lx, ly, lz;
    growth_rates(bg, g, ph, c, v[0], v[1], v[2], lx, ly, lz);
    out.lam[0][p] = lx;
    out.lam[1][p] = ly;
    out.lam[2][p] = lz;
  }
}

// One thread per cell of the face-0 plane of axis a.
__global__ void __launch_bounds__(128) coeff_planes_kernel(Dims d, Background bg, Grid g, Phys ph,
                                                           int a, double* out) {
  long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nplane = d.ncell / d.n[a];
  if (q >= nplane) return;
  int c[6];
  long long r = q;
  for (int b = 0; b < 6; b++) {
    if (b == a) { c[b] = 0; continue; }
    c[b] = (int)(r % d.n[b]) + 1;
    r /= d.n[b];
  }
  out[q] = face_velocity(d, bg, g, ph, a, c);
}

// max over interior cells of sum_a max(|v_a(F-1)|,|v_a(F)|)/d_a(F): the
// CFL rate that defines dt for the CFL-specified workloads.
__global__ void __launch_bounds__(256) max_rate_kernel(Dims d, Grid g, ConstCoeff64 cf,
                                                       double* partial) {
  __shared__ double red[256];
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double best = 0.0;
  if (v3 < d.nvol3) {
    for (long long sp = blockIdx.y; sp < d.nspec; sp += gridDim.y) {
      int c[6];
      decode(d, v3, sp, c);
      const long long p = v3 + sp * d.nvol3;
      double r = 0.0;
      for (int a = 0; a < 6; a++) {
        if (d.n[a] <= 1) continue;
        const double vr = cf.vel[a][p];
        const double vl = c[a] > 0 ? cf.vel[a][p - d.s[a]] : cf.vlo[a][plane_index(d, a, c)];
        r = dadd(r, ddiv(fmax2(fabs(vl), fabs(vr)), g.d[a][pidx(c[a] + 1)]));
      }
      best = fmax2(best, r);
    }
  }
  red[threadIdx.x] = best;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax2(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

__global__ void max_reduce_kernel(const double* partial, long long n, double* out) {
  __shared__ double red[256];
  double best = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) best = fmax2(best, partial[i]);
  red[threadIdx.x] = best;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax2(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// binary64 -> binary32 copy of the coefficient fields; the binary32 form
// keeps one combined growth rate lam = lambda_x[nx>1] + lambda_y[ny>1] +
// lambda_z[nz>1], summed in binary64 before rounding.
__global__ void to_fp32_kernel(const double* src, float* dst, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    dst[i] = __double2float_rn(src[i]);
}

__global__ void lam_combine_kernel(const double* lx, const double* ly, const double* lz, int ux,
                                   int uy, int uz, float* dst, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    if (ux) s += lx[i];
    if (uy) s += ly[i];
    if (uz) s += lz[i];
    dst[i] = __double2float_rn(s);
  }
}

// uCFL = |v*dt/d(f)| of every face of axis a (binary64 form), in the order of
// superbee_fluxes.f90:19: right faces f = c_a + 1 and the face-0 plane
__global__ void ucfl_kernel(Dims d, Grid g, int a, double dt, const double* vel, const double* vlo,
                            double* uc, double* ucl) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < d.ncell; p += stride) {
    const int ca = (int)((p / d.s[a]) % d.n[a]);
    uc[p] = fabs(ddiv(dmul(vel[p], dt), g.d[a][pidx(ca + 1)]));
  }
  const long long np = d.ncell / d.n[a];
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < np; q += stride)
    ucl[q] = fabs(ddiv(dmul(vlo[q], dt), g.d[a][pidx(0)]));
}

cudaError_t launch_ucfl(const Dims& d, const Grid& g, double dt, const double* const* vel,
                        const double* const* vlo, double* const* uc, double* const* ucl,
                        cudaStream_t st) {
  for (int a = 0; a < 6; a++) {
    ucfl_kernel<<<8 * 152, 256, 0, st>>>(d, g, a, dt, vel[a], vlo[a], uc[a], ucl[a]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// fused step
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T update(T e0, T dE, T mf, double dt);
template <>
__device__ __forceinline__ double update<double>(double e0, double dE, double mf, double dt) {
  // dE = dE - meanfl; E = E + dt*dE  (integrate.f90:261-262)
  return dadd(e0, dmul(dt, dsub(dE, mf)));
}
template <>
__device__ __forceinline__ float update<float>(float e0, float dE, float mf, double dt) {
  return e0 + (float)dt * (dE - mf);
}

template <class T>
__global__ void __launch_bounds__(256) step_kernel(StepArgs<T> A) {
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= A.d.nvol3) return;
  for (long long sp = blockIdx.y; sp < A.d.nspec; sp += gridDim.y) {
    int c[6];
    decode(A.d, v3, sp, c);
    const long long p = v3 + sp * A.d.nvol3;
    const T e0 = A.E[p];
    if constexpr (sizeof(T) == 4) {
      A.Enew[p] = cell_step32(A, p, c, e0);
      if (blockIdx.x == 0 && sp == 0) advance_seed(A.seed_in, A.seed_out, 0);
    } else {
      const CellTerms<T> t = cell_terms<T>(A, p, c, e0);
      A.Enew[p] = update<T>(e0, t.dE, t.meanfl, A.dt);
    }
  }
}

// ---------------------------------------------------------------------------
// budget (diagnose.f90:46-329)
// ---------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T tsub(T a, T b);
template <>
__device__ __forceinline__ double tsub<double>(double a, double b) { return dsub(a, b); }
template <>
__device__ __forceinline__ float tsub<float>(float a, float b) { return a - b; }

// scalar sums and maxima over interior cells, diagnose.f90:46-68
// partial layout: [block][DIAG_CELL_NV]
template <class T>
__global__ void __launch_bounds__(256) diag_cells_kernel(StepArgs<T> A, const T* Ecur,
                                                         double* partial) {
  __shared__ double red[256];
  const Dims& d = A.d;
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double acc[DIAG_CELL_NV];
  for (int k = 0; k < DIAG_CELL_NV; k++) acc[k] = 0.0;
  if (v3 < d.nvol3) {
    for (long long sp = blockIdx.y; sp < d.nspec; sp += gridDim.y) {
      int c[6];
      decode(d, v3, sp, c);
      const long long p = v3 + sp * d.nvol3;
      const T e0 = A.E[p];
      const CellTerms<T> t = cell_terms<T>(A, p, c, e0);
      const double dEv = (double)tsub<T>(t.dE, t.meanfl);  // dE after the mean-flow term
      double fxa = g_d(A.g, 0, c[0]);
      fxa = dmul(fxa, g_d(A.g, 1, c[1]));
      fxa = dmul(fxa, g_d(A.g, 2, c[2]));
      fxa = dmul(fxa, g_d(A.g, 3, c[3]));
      fxa = dmul(fxa, g_d(A.g, 4, c[4]));
      fxa = dmul(fxa, g_d(A.g, 5, c[5]));
      acc[0] = dadd(acc[0], dmul(dEv, fxa));
      acc[1] = dadd(acc[1], dmul((double)t.meanfl, fxa));
      acc[2] = fmax2(acc[2], ddiv(fabs((double)t.meanfl), fmax2(RT_LIT_1EM12, (double)Ecur[p])));
      for (int a = 0; a < 6; a++) acc[3 + a] = fmax2(acc[3 + a], fabs((double)A.vel[a][p]));
    }
  }
  const int blk = blockIdx.y * gridDim.x + blockIdx.x;
  for (int k = 0; k < DIAG_CELL_NV; k++) {
    red[threadIdx.x] = acc[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w)
        red[threadIdx.x] = (k < 2) ? dadd(red[threadIdx.x], red[threadIdx.x + w])
                                   : fmax2(red[threadIdx.x], red[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[(long long)blk * DIAG_CELL_NV + k] = red[0];
    __syncthreads();
  }
}

// flux through face 0 (lo) or face n (hi) of axis a at a boundary-plane
// cell; c[] holds 0-based coordinates with c[a] = 0 or n-1
template <class T>
__device__ __forceinline__ double boundary_flux(const StepArgs<T>& A, const int c[6], int a, bool hi);

template <>
__device__ __forceinline__ double boundary_flux<double>(const StepArgs<double>& A, const int c[6],
                                                        int a, bool hi) {
  const Dims& d = A.d;
  long long p = 0;
  for (int b = 0; b < 6; b++) p += (long long)c[b] * d.s[b];
  const int ca = c[a];
  if (!hi) {  // face 0: E(-1), E(0), E(1), E(2) -> cells -2, -1, 0, 1
    const double Ea = A.E[nb_index(d, p, a, ca, -2, c[5])];
    const double Eb = A.E[nb_index(d, p, a, ca, -1, c[5])];
    const double Ec = A.E[p];
    const double Ed = A.E[nb_index(d, p, a, ca, +1, c[5])];
    return flux_fp64(A.vlo[a][plane_index(d, a, c)], A.g.d[a][pidx(0)], A.dt, Ea, Eb, Ec, Ed);
  }
  // face n: E(n-1), E(n), E(n+1), E(n+2) -> cells n-2, n-1, n, n+1
  const double Ea = A.E[nb_index(d, p, a, ca, -1, c[5])];
  const double Eb = A.E[p];
  const double Ec = A.E[nb_index(d, p, a, ca, +1, c[5])];
  const double Ed = A.E[nb_index(d, p, a, ca, +2, c[5])];
  return flux_fp64(A.vel[a][p], A.g.d[a][pidx(d.n[a])], A.dt, Ea, Eb, Ec, Ed);
}

template <>
__device__ __forceinline__ double boundary_flux<float>(const StepArgs<float>& A, const int c[6],
                                                       int a, bool hi) {
  const Dims& d = A.d;
  long long p = 0;
  for (int b = 0; b < 6; b++) p += (long long)c[b] * d.s[b];
  const int ca = c[a];
  if (!hi) {
    const float Ea = A.E[nb_index(d, p, a, ca, -2, c[5])];
    const float Eb = A.E[nb_index(d, p, a, ca, -1, c[5])];
    const float Ec = A.E[p];
    const float Ed = A.E[nb_index(d, p, a, ca, +1, c[5])];
    return (double)flux_fp32(A.vlo[a][plane_index(d, a, c)], A.t32.hcfl[a][pidx(0)], Ea, Eb, Ec, Ed);
  }
  const float Ea = A.E[nb_index(d, p, a, ca, -1, c[5])];
  const float Eb = A.E[p];
  const float Ec = A.E[nb_index(d, p, a, ca, +1, c[5])];
  const float Ed = A.E[nb_index(d, p, a, ca, +2, c[5])];
  return (double)flux_fp32(A.vel[a][p], A.t32.hcfl[a][pidx(d.n[a])], Ea, Eb, Ec, Ed);
}

// boundary-flux integrals bfl_{a}{s,e}, diagnose.f90:102-277.  blockIdx.z
// = axis; partial layout [axis][block][2]
template <class T>
__global__ void __launch_bounds__(256) diag_planes_kernel(StepArgs<T> A, long long nblk,
                                                          double* partial) {
  __shared__ double red[2][256];
  const Dims& d = A.d;
  const int a = blockIdx.z;
  double acc_lo = 0.0, acc_hi = 0.0;
  if (d.n[a] > 1) {
    const long long nplane = d.ncell / d.n[a];
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < nplane;
         q += (long long)gridDim.x * blockDim.x) {
      int c[6];
      long long r = q;
      for (int b = 0; b < 6; b++) {
        if (b == a) { c[b] = 0; continue; }
        c[b] = (int)(r % d.n[b]);
        r /= d.n[b];
      }
      // area element: product of the other five grid spacings in axis
      // order, left to right (diagnose.f90:109 etc.)
      double area = 0.0;
      bool first = true;
      for (int b = 0; b < 6; b++) {
        if (b == a) continue;
        const double db = g_d(A.g, b, c[b]);
        area = first ? db : dmul(area, db);
        first = false;
      }
      const double flo = boundary_flux<T>(A, c, a, false);
      c[a] = d.n[a] - 1;
      const double fhi = boundary_flux<T>(A, c, a, true);
      acc_lo = dadd(acc_lo, dmul(flo, area));
      acc_hi = dadd(acc_hi, dmul(fhi, area));
    }
  }
  red[0][threadIdx.x] = acc_lo;
  red[1][threadIdx.x] = acc_hi;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[0][threadIdx.x] = dadd(red[0][threadIdx.x], red[0][threadIdx.x + w]);
      red[1][threadIdx.x] = dadd(red[1][threadIdx.x], red[1][threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[((long long)a * nblk + blockIdx.x) * 2 + 0] = red[0][0];
    partial[((long long)a * nblk + blockIdx.x) * 2 + 1] = red[1][0];
  }
}

// Wavenumber integrals on each spatial cell, in the reference's summation
// order (diagnose.f90:84-98 and :186-277): E_int, meanfl_int, diss_ks,
// diss_ke, diss_ls, diss_le, diss_ms, diss_me.  out layout [8][nvol3].
template <class T>
__device__ __forceinline__ double meanfl_of(const StepArgs<T>& A, long long p, T e0);
template <>
__device__ __forceinline__ double meanfl_of<double>(const StepArgs<double>& A, long long p, double e0) {
  double mf = 0.;
  if (A.d.n[0] > 1) mf = dadd(mf, dmul(e0, A.lam[0][p]));
  if (A.d.n[1] > 1) mf = dadd(mf, dmul(e0, A.lam[1][p]));
  if (A.d.n[2] > 1) mf = dadd(mf, dmul(e0, A.lam[2][p]));
  return mf;
}
template <>
__device__ __forceinline__ double meanfl_of<float>(const StepArgs<float>& A, long long p, float e0) {
  return (double)(e0 * A.lam[0][p]);
}

template <class T>
__global__ void __launch_bounds__(128) diag_vol3_kernel(StepArgs<T> A, const T* Ecur, double* out) {
  const Dims& d = A.d;
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= d.nvol3) return;
  const int nk = d.n[3], nl = d.n[4], nm = d.n[5];
  int c[6];
  decode(d, v3, 0, c);
  // E_int and meanfl_int: loops m, n(l-axis), l(k-axis)
  double eint = 0., mint = 0.;
  for (int m = 0; m < nm; m++)
    for (int n = 0; n < nl; n++)
      for (int l = 0; l < nk; l++) {
        const long long p = v3 + d.nvol3 * (l + (long long)nk * (n + (long long)nl * m));
        const double dk = g_d(A.g, 3, l), dl = g_d(A.g, 4, n), dm = g_d(A.g, 5, m);
        eint = dadd(eint, dmul(dmul(dmul((double)Ecur[p], dl), dm), dk));
        const double mf = meanfl_of<T>(A, p, A.E[p]);
        mint = dadd(mint, dmul(dmul(dmul(mf, dk), dl), dm));
      }
  out[0 * d.nvol3 + v3] = eint;
  out[1 * d.nvol3 + v3] = mint;
  // diss_ks / diss_ke: k faces 0 and nk, loops m, n
  double ks = 0., ke = 0., ls = 0., le = 0., ms = 0., me = 0.;
  if (nk > 1) {
    for (int m = 0; m < nm; m++)
      for (int n = 0; n < nl; n++) {
        c[3] = 0; c[4] = n; c[5] = m;
        const double flo = boundary_flux<T>(A, c, 3, false);
        c[3] = nk - 1;
        const double fhi = boundary_flux<T>(A, c, 3, true);
        const double dl = g_d(A.g, 4, n), dm = g_d(A.g, 5, m);
        ks = dadd(ks, dmul(dmul(flo, dl), dm));
        ke = dadd(ke, dmul(dmul(fhi, dl), dm));
      }
  }
  if (nl > 1) {  // l faces, loops m, l(k-axis)
    for (int m = 0; m < nm; m++)
      for (int l = 0; l < nk; l++) {
        c[3] = l; c[4] = 0; c[5] = m;
        const double flo = boundary_flux<T>(A, c, 4, false);
        c[4] = nl - 1;
        const double fhi = boundary_flux<T>(A, c, 4, true);
        const double dk = g_d(A.g, 3, l), dm = g_d(A.g, 5, m);
        ls = dadd(ls, dmul(dmul(flo, dk), dm));
        le = dadd(le, dmul(dmul(fhi, dk), dm));
      }
  }
  if (nm > 1) {  // m faces, loops n(l-axis), l(k-axis)
    for (int n = 0; n < nl; n++)
      for (int l = 0; l < nk; l++) {
        c[3] = l; c[4] = n; c[5] = 0;
        const double flo = boundary_flux<T>(A, c, 5, false);
        c[5] = nm - 1;
        const double fhi = boundary_flux<T>(A, c, 5, true);
        const double dk = g_d(A.g, 3, l), dl = g_d(A.g, 4, n);
        ms = dadd(ms, dmul(dmul(flo, dk), dl));
        me = dadd(me, dmul(dmul(fhi, dk), dl));
      }
  }
  out[2 * d.nvol3 + v3] = ks;
  out[3 * d.nvol3 + v3] = ke;
  out[4 * d.nvol3 + v3] = ls;
  out[5 * d.nvol3 + v3] = le;
  out[6 * d.nvol3 + v3] = ms;
  out[7 * d.nvol3 + v3] = me;
}

// final fixed-order reduction of the partials (one block)
__global__ void diag_finish_kernel(const double* pc, long long ncb, const double* pp, long long npb,
                                   double* out) {
  __shared__ double red[256];
  // cell partials
  for (int k = 0; k < DIAG_CELL_NV; k++) {
    double acc = 0.0;
    for (long long i = threadIdx.x; i < ncb; i += blockDim.x) {
      const double x = pc[i * DIAG_CELL_NV + k];
      acc = (k < 2) ? dadd(acc, x) : fmax2(acc, x);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w)
        red[threadIdx.x] = (k < 2) ? dadd(red[threadIdx.x], red[threadIdx.x + w])
                                   : fmax2(red[threadIdx.x], red[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) out[k] = red[0];
    __syncthreads();
  }
  // plane partials: 6 axes x {lo, hi}
  for (int k = 0; k < 12; k++) {
    const int a = k / 2, side = k % 2;
    double acc = 0.0;
    for (long long i = threadIdx.x; i < npb; i += blockDim.x)
      acc = dadd(acc, pp[((long long)a * npb + i) * 2 + side]);
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] = dadd(red[threadIdx.x], red[threadIdx.x + w]);
      __syncthreads();
    }
    if (threadIdx.x == 0) out[DIAG_CELL_NV + k] = red[0];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static dim3 cell_grid(const Dims& d, int threads) {
  const long long bx = (d.nvol3 + threads - 1) / threads;
  long long by = d.nspec < 65535 ? d.nspec : 65535;
  return dim3((unsigned)bx, (unsigned)by, 1);
}

cudaError_t launch_coeff(const Dims& d, const Background& bg, const Grid& g, const Phys& ph,
                         const CoeffOut64& out, cudaStream_t st) {
  coeff_cells_kernel<<<cell_grid(d, 128), 128, 0, st>>>(d, bg, g, ph, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (int a = 0; a < 6; a++) {
    const long long nplane = d.ncell / d.n[a];
    coeff_planes_kernel<<<(unsigned)((nplane + 127) / 128), 128, 0, st>>>(d, bg, g, ph, a, out.vlo[a]);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

long long max_rate_partials(const Dims& d) {
  dim3 gr = cell_grid(d, 256);
  return (long long)gr.x * gr.y;
}

cudaError_t launch_max_rate(const Dims& d, const Grid& g, const ConstCoeff64& cf, double* partial,
                            double* out, cudaStream_t st) {
  dim3 gr = cell_grid(d, 256);
  max_rate_kernel<<<gr, 256, 0, st>>>(d, g, cf, partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  max_reduce_kernel<<<1, 256, 0, st>>>(partial, (long long)gr.x * gr.y, out);
  return cudaGetLastError();
}

// ---- padded host array <-> unpadded device field, read / written by the GPU
// through the host's page tables (devices with pageable memory access) ----
// A warp moves one x row: row r of the interior is (y, z, k, l, m) in x-fastest
// order; the host array is padded by RT_ONX on every axis (Fortran order).
template <bool TO_DEVICE, class T>
__global__ void host_rows_kernel(const double* __restrict__ hsrc, double* __restrict__ hdst,
                                 const T* __restrict__ dsrc, T* __restrict__ ddst, Dims d) {
  long long P[6];
#pragma unroll
  for (int a = 0; a < 6; a++) P[a] = d.n[a] + 2 * RT_ONX;
  const long long rows = d.ncell / d.n[0];
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarp = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = warp; r < rows; r += nwarp) {
    long long q = r;
    const int j = (int)(q % d.n[1]); q /= d.n[1];
    const int k = (int)(q % d.n[2]); q /= d.n[2];
    const int l = (int)(q % d.n[3]); q /= d.n[3];
    const int n = (int)(q % d.n[4]);
    const int m = (int)(q / d.n[4]);
    const long long h0 = RT_ONX + P[0] * ((j + RT_ONX) + P[1] * ((k + RT_ONX) + P[2] *
                         ((l + RT_ONX) + P[3] * ((n + RT_ONX) + P[4] * (long long)(m + RT_ONX)))));
    const long long d0 = r * d.n[0];
    for (int x = lane; x < d.n[0]; x += 32) {
      if (TO_DEVICE) ddst[d0 + x] = (T)hsrc[h0 + x];
      else hdst[h0 + x] = (double)dsrc[d0 + x];
    }
  }
}

template <class T>
cudaError_t launch_host_gather(const double* host, T* dst, const Dims& d, cudaStream_t st) {
  host_rows_kernel<true, T><<<8 * 152, 256, 0, st>>>(host, nullptr, nullptr, dst, d);
  return cudaGetLastError();
}
template <class T>
cudaError_t launch_host_scatter(const T* src, double* host, const Dims& d, cudaStream_t st) {
  host_rows_kernel<false, T><<<8 * 152, 256, 0, st>>>(nullptr, host, src, nullptr, d);
  return cudaGetLastError();
}
template cudaError_t launch_host_gather<double>(const double*, double*, const Dims&, cudaStream_t);
template cudaError_t launch_host_gather<float>(const double*, float*, const Dims&, cudaStream_t);
template cudaError_t launch_host_scatter<double>(const double*, double*, const Dims&, cudaStream_t);
template cudaError_t launch_host_scatter<float>(const float*, double*, const Dims&, cudaStream_t);

cudaError_t launch_to_fp32(const double* src, float* dst, long long n, cudaStream_t st) {
  to_fp32_kernel<<<4 * 152, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

cudaError_t launch_lam_combine(const double* lx, const double* ly, const double* lz, int ux, int uy,
                               int uz, float* dst, long long n, cudaStream_t st) {
  lam_combine_kernel<<<4 * 152, 256, 0, st>>>(lx, ly, lz, ux, uy, uz, dst, n);
  return cudaGetLastError();
}

PlaneSched make_sched(const Dims& d, const StepTuning& tn, int gz) {
  PlaneSched S;
  S.sweep = tn.sweep ? 1 : 0;
  const int nb = S.sweep ? d.n[4] : d.n[5];
  S.band = tn.band > 0 ? tn.band : 8;
  if (S.band > nb) S.band = nb;
  S.nband = (nb + S.band - 1) / S.band;
  S.gz = gz > 0 ? gz : 1;
  S.nunits = (long long)((d.n[2] + S.gz - 1) / S.gz) * d.n[3];
  return S;
}
PlaneSched make_sched(const Dims& d, const StepTuning& tn) { return make_sched(d, tn, 1); }

template <class T>
size_t group_path_smem(const Dims& d, int G) { return group_smem<T>(d, G); }
template size_t group_path_smem<double>(const Dims&, int);
template size_t group_path_smem<float>(const Dims&, int);

// z planes per item: about one cell per thread, at most nz, at most 4096
// cells per item (the coordinate multiply), shared memory within 200 KB
template <class T>
int group_size(const Dims& d, const StepTuning& tn) {
  const long long nxy = (long long)d.n[0] * d.n[1];
  if (!tma_ok<T>(d) || nxy > 4096) return 0;
  int G = tn.group > 0 ? tn.group : (int)(tn.threads / nxy);
  if (G < 1) G = 1;
  if (G > d.n[2]) G = d.n[2];
  while (G > 1 && ((long long)(G + 1) * nxy > 4096 || group_smem<T>(d, G) > 200 * 1024)) G--;
  if ((long long)(G + 1) * nxy > 4096 * 2 || group_smem<T>(d, G) > 200 * 1024) return 0;
  return G;
}
template int group_size<double>(const Dims&, const StepTuning&);
template int group_size<float>(const Dims&, const StepTuning&);

long long sched_items(const Dims& d, const PlaneSched& S) {
  const int nouter = S.sweep ? d.n[5] : d.n[4];
  return (long long)S.nband * nouter * S.band * S.nunits;
}

template <class T>
size_t plane_smem(const Dims& d) { return (size_t)3 * d.n[0] * d.n[1] * sizeof(T); }

template <class T>
bool plane_ok(const Dims& d) { return plane_smem<T>(d) <= 48 * 1024; }
template size_t plane_smem<double>(const Dims&);
template size_t plane_smem<float>(const Dims&);
template bool plane_ok<double>(const Dims&);
template bool plane_ok<float>(const Dims&);

// the TMA path: planes a multiple of 16 bytes, shared memory within 200 KB,
// at most 4096 cells per plane (the coordinate multiply of tma_item), and at
// most RT_TMA_MAXC cells per thread for the largest CTA (checked again for
// the CTA size actually launched)
template <class T>
bool tma_path_ok(const Dims& d) {
  const long long nxy = (long long)d.n[0] * d.n[1];
  return tma_ok<T>(d) && tma_smem<T>(d) <= 200 * 1024 && nxy <= 4096 && nxy <= RT_TMA_MAXC * 1024LL;
}
// cells per thread of the TMA kernels for a CTA of nt threads
static int tma_maxc(long long nxy, int nt) { return (int)((nxy + nt - 1) / nt); }
template <class T>
size_t tma_path_smem(const Dims& d) { return tma_smem<T>(d); }
template bool tma_path_ok<double>(const Dims&);
template bool tma_path_ok<float>(const Dims&);
template size_t tma_path_smem<double>(const Dims&);
template size_t tma_path_smem<float>(const Dims&);

template <class T, int NT, class K>
static cudaError_t set_smem(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <class T, int NT, int MAXC>
static cudaError_t launch_tma_nt_c(const StepArgs<T>& A, const PlaneSched& S, long long nblk,
                                   cudaStream_t st) {
  const size_t sm = tma_smem<T>(A.d);
  cudaError_t e = set_smem<T, NT>(step_tma_kernel<T, NT, MAXC>, sm);
  if (e != cudaSuccess) return e;
  step_tma_kernel<T, NT, MAXC><<<(unsigned)nblk, NT, sm, st>>>(A, S);
  return cudaGetLastError();
}

template <class T, int NT>
static cudaError_t launch_tma_nt(const StepArgs<T>& A, const PlaneSched& S, long long nblk,
                                 cudaStream_t st) {
  const int mc = tma_maxc((long long)A.d.n[0] * A.d.n[1], NT);
  if (mc <= 1) return launch_tma_nt_c<T, NT, 1>(A, S, nblk, st);
  if (mc <= 2) return launch_tma_nt_c<T, NT, 2>(A, S, nblk, st);
  return launch_tma_nt_c<T, NT, 4>(A, S, nblk, st);
}

template <class T, int NT>
static cudaError_t launch_group_nt(const StepArgs<T>& A, const PlaneSched& S, long long nblk,
                                   cudaStream_t st) {
  const size_t sm = group_smem<T>(A.d, S.gz);
  cudaError_t e = set_smem<T, NT>(step_group_kernel<T, NT>, sm);
  if (e != cudaSuccess) return e;
  step_group_kernel<T, NT><<<(unsigned)nblk, NT, sm, st>>>(A, S);
  return cudaGetLastError();
}

template <class T>
cudaError_t launch_step(const StepArgs<T>& A, const StepTuning& tn, cudaStream_t st) {
  if constexpr (sizeof(T) == 4) {
    bool done = false;
    cudaError_t e = launch_persist(A, tn, st, done);
    if (done) return e;
  }
  if (tn.variant == RT_VARIANT_GROUP) {
    const int G = group_size<T>(A.d, tn);
    if (G > 0) {
      const PlaneSched S = make_sched(A.d, tn, G);
      const long long nblk = sched_items(A.d, S);
      if (tn.threads == 128) return launch_group_nt<T, 128>(A, S, nblk, st);
      if (tn.threads == 512) return launch_group_nt<T, 512>(A, S, nblk, st);
      if (tn.threads == 1024) return launch_group_nt<T, 1024>(A, S, nblk, st);
      return launch_group_nt<T, 256>(A, S, nblk, st);
    }
  }
  if ((tn.variant == RT_VARIANT_TMA || tn.variant >= RT_VARIANT_W3) &&
      tma_path_ok<T>(A.d) &&
      tma_maxc((long long)A.d.n[0] * A.d.n[1], tn.threads) <= RT_TMA_MAXC) {
    const PlaneSched S = make_sched(A.d, tn);
    const long long nblk = sched_items(A.d, S);
    if (tn.threads == 128) return launch_tma_nt<T, 128>(A, S, nblk, st);
    if (tn.threads == 512) return launch_tma_nt<T, 512>(A, S, nblk, st);
    if (tn.threads == 1024) return launch_tma_nt<T, 1024>(A, S, nblk, st);
    return launch_tma_nt<T, 256>(A, S, nblk, st);
  }
  if ((tn.variant != RT_VARIANT_CELL) && plane_ok<T>(A.d)) {
    const PlaneSched S = make_sched(A.d, tn);
    const long long nblk = sched_items(A.d, S);
    const size_t sm = plane_smem<T>(A.d);
    if (tn.threads == 128)
      step_plane_kernel<T, 128><<<(unsigned)nblk, 128, sm, st>>>(A, S);
    else if (tn.threads >= 512)
      step_plane_kernel<T, 512><<<(unsigned)nblk, 512, sm, st>>>(A, S);
    else
      step_plane_kernel<T, 256><<<(unsigned)nblk, 256, sm, st>>>(A, S);
    return cudaGetLastError();
  }
  step_kernel<T><<<cell_grid(A.d, 256), 256, 0, st>>>(A);
  return cudaGetLastError();
}
template cudaError_t launch_step<double>(const StepArgs<double>&, const StepTuning&, cudaStream_t);
template cudaError_t launch_step<float>(const StepArgs<float>&, const StepTuning&, cudaStream_t);

template <class T>
cudaError_t launch_batch(const void* members, const long long* first, int nmem, size_t smem,
                         int threads, int grid, cudaStream_t st) {
  const BatchMember<T>* mem = (const BatchMember<T>*)members;
  if (threads == 128)
    batch_plane_kernel<T, 128><<<grid, 128, smem, st>>>(mem, first, nmem);
  else if (threads >= 512)
    batch_plane_kernel<T, 512><<<grid, 512, smem, st>>>(mem, first, nmem);
  else
    batch_plane_kernel<T, 256><<<grid, 256, smem, st>>>(mem, first, nmem);
  return cudaGetLastError();
}
template cudaError_t launch_batch<double>(const void*, const long long*, int, size_t, int, int, cudaStream_t);
template cudaError_t launch_batch<float>(const void*, const long long*, int, size_t, int, int, cudaStream_t);

template <class T, int NT>
static int occ_batch(bool tma, size_t smem, bool group = false) {
  int nb = 0;
  cudaError_t e;
  if (group) {
    e = set_smem<T, NT>(batch_group_kernel<T, NT>, smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_group_kernel<T, NT>, NT, smem);
  } else if (tma) {
    // one MAXC for the occupancy query: register use differs little
    e = set_smem<T, NT>(batch_tma_kernel<T, NT, 1>, smem);
    if (e == cudaSuccess) e = set_smem<T, NT>(batch_tma_kernel<T, NT, 2>, smem);
    if (e == cudaSuccess) e = set_smem<T, NT>(batch_tma_kernel<T, NT, 4>, smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_tma_kernel<T, NT, 4>, NT, smem);
  } else {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_plane_kernel<T, NT>, NT, smem);
  }
  if (e != cudaSuccess) { cudaGetLastError(); return 0; }
  return nb;
}

template <class T>
int batch_blocks_per_sm(int threads, size_t smem, bool tma, bool group) {
  if (threads == 128) return occ_batch<T, 128>(tma, smem, group);
  if (threads == 512) return occ_batch<T, 512>(tma, smem, group);
  if (threads == 1024) return (tma || group) ? occ_batch<T, 1024>(tma, smem, group) : 0;
  return occ_batch<T, 256>(tma, smem, group);
}
template int batch_blocks_per_sm<double>(int, size_t, bool, bool);
template int batch_blocks_per_sm<float>(int, size_t, bool, bool);

template <class T>
cudaError_t launch_batch_group(const void* members, const long long* first, int nmem, size_t smem,
                               int threads, int grid, cudaStream_t st) {
  const BatchMember<T>* mem = (const BatchMember<T>*)members;
  if (threads == 128) batch_group_kernel<T, 128><<<grid, 128, smem, st>>>(mem, first, nmem);
  else if (threads == 512) batch_group_kernel<T, 512><<<grid, 512, smem, st>>>(mem, first, nmem);
  else if (threads == 1024) batch_group_kernel<T, 1024><<<grid, 1024, smem, st>>>(mem, first, nmem);
  else batch_group_kernel<T, 256><<<grid, 256, smem, st>>>(mem, first, nmem);
  return cudaGetLastError();
}
template cudaError_t launch_batch_group<double>(const void*, const long long*, int, size_t, int, int, cudaStream_t);
template cudaError_t launch_batch_group<float>(const void*, const long long*, int, size_t, int, int, cudaStream_t);

template <class T, int NT>
static void batch_tma_nt(const BatchMember<T>* mem, const long long* first, int nmem, size_t smem,
                         int maxc, int grid, cudaStream_t st) {
  if (maxc <= 1) batch_tma_kernel<T, NT, 1><<<grid, NT, smem, st>>>(mem, first, nmem);
  else if (maxc <= 2) batch_tma_kernel<T, NT, 2><<<grid, NT, smem, st>>>(mem, first, nmem);
  else batch_tma_kernel<T, NT, 4><<<grid, NT, smem, st>>>(mem, first, nmem);
}

template <class T>
cudaError_t launch_batch_tma(const void* members, const long long* first, int nmem, size_t smem,
                             int threads, int grid, long long max_nxy, cudaStream_t st) {
  const BatchMember<T>* mem = (const BatchMember<T>*)members;
  const int mc = tma_maxc(max_nxy, threads);
  if (mc > RT_TMA_MAXC) return cudaErrorInvalidConfiguration;
  if (threads == 128) batch_tma_nt<T, 128>(mem, first, nmem, smem, mc, grid, st);
  else if (threads == 512) batch_tma_nt<T, 512>(mem, first, nmem, smem, mc, grid, st);
  else if (threads == 1024) batch_tma_nt<T, 1024>(mem, first, nmem, smem, mc, grid, st);
  else batch_tma_nt<T, 256>(mem, first, nmem, smem, mc, grid, st);
  return cudaGetLastError();
}
template cudaError_t launch_batch_tma<double>(const void*, const long long*, int, size_t, int, int, long long, cudaStream_t);
template cudaError_t launch_batch_tma<float>(const void*, const long long*, int, size_t, int, int, long long, cudaStream_t);

size_t batch_member_bytes(int precision_fp64) {
  return precision_fp64 ? sizeof(BatchMember<double>) : sizeof(BatchMember<float>);
}

DiagSizes diag_sizes(const Dims& d) {
  DiagSizes s;
  dim3 gr = cell_grid(d, 256);
  s.cell_blocks = (long long)gr.x * gr.y;
  s.plane_blocks = 4 * 152;
  return s;
}

template <class T>
cudaError_t launch_diag(const StepArgs<T>& A, const T* Ecur, double* scratch, double* vol3,
                        double* result, cudaStream_t st) {
  const DiagSizes s = diag_sizes(A.d);
  double* pc = scratch;
  double* pp = scratch + s.cell_blocks * DIAG_CELL_NV;
  diag_cells_kernel<T><<<cell_grid(A.d, 256), 256, 0, st>>>(A, Ecur, pc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  diag_planes_kernel<T><<<dim3((unsigned)s.plane_blocks, 1, 6), 256, 0, st>>>(A, s.plane_blocks, pp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  diag_vol3_kernel<T><<<(unsigned)((A.d.nvol3 + 127) / 128), 128, 0, st>>>(A, Ecur, vol3);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  diag_finish_kernel<<<1, 256, 0, st>>>(pc, s.cell_blocks, pp, s.plane_blocks, result);
  return cudaGetLastError();
}
template cudaError_t launch_diag<double>(const StepArgs<double>&, const double*, double*, double*,
                                         double*, cudaStream_t);
template cudaError_t launch_diag<float>(const StepArgs<float>&, const float*, double*, double*,
                                        double*, cudaStream_t);

// the module arrays dE and meanfl that integrate leaves behind
// (integrate.f90:202-262): per cell of the state A.E, dE after the mean-flow
// term and meanfl, widened to binary64; unpadded, x fastest
template <class T>
__global__ void __launch_bounds__(256) tendency_kernel(StepArgs<T> A, double* dE, double* meanfl) {
  const long long v3 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v3 >= A.d.nvol3) return;
  for (long long sp = blockIdx.y; sp < A.d.nspec; sp += gridDim.y) {
    int c[6];
    decode(A.d, v3, sp, c);
    const long long p = v3 + sp * A.d.nvol3;
    const CellTerms<T> t = cell_terms<T>(A, p, c, A.E[p]);
    dE[p] = (double)tsub<T>(t.dE, t.meanfl);
    meanfl[p] = (double)t.meanfl;
  }
}

template <class T>
cudaError_t launch_tendency(const StepArgs<T>& A, double* dE, double* meanfl, cudaStream_t st) {
  tendency_kernel<T><<<cell_grid(A.d, 256), 256, 0, st>>>(A, dE, meanfl);
  return cudaGetLastError();
}
template cudaError_t launch_tendency<double>(const StepArgs<double>&, double*, double*, cudaStream_t);
template cudaError_t launch_tendency<float>(const StepArgs<float>&, double*, double*, cudaStream_t);

}  // namespace rt
