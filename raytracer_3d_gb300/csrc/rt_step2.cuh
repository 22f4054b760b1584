// rt_step2.cuh -- plane-tiled fused step (the production step kernel).
//
// One CTA updates one "plane": all nx*ny cells of one (z, k) pair at one
// (l, m).  The plane of E is staged in shared memory, the x and y face
// fluxes are evaluated once per face and shared through shared memory, the
// z, k, l and m faces are evaluated from neighbour loads.  CTAs are numbered
// in band order
//     for band of Bm m-values: for l: for m in band: for (z, k)
// so that the CTAs resident at any moment cover whole (x,y,z,k) slabs of a
// few neighbouring (l, m) and the +-2 neighbour planes along z, k, l and m
// are still in L2 when they are re-read.  The state that is read once
// (x and y velocities, growth rate) and the new state are streamed with
// evict-first cache hints so that they do not push the reused E planes and
// the z/k/l/m velocities (re-read as the left face of the next cell along
// their axis) out of L2.
//
// Arithmetic is the same as rt_step.cuh (binary64: reference order, bit
// for bit; binary32: division-free limiter).  The divergence is accumulated
// in the reference's axis order x, y, z, k, l, m.
#pragma once
#include "rt_step.cuh"

namespace rt {

template <class T> __device__ __forceinline__ T ld_stream(const T* p) { return __ldcs(p); }
template <class T> __device__ __forceinline__ void st_stream(T* p, T v) { __stcs(p, v); }

// flux of face 0 of an open axis: the ghost cells copy cell 0, so
// Rj = E(0)-E(-1) = 0 and the superbee diffusive term vanishes; the flux is
// v*(E0+E0)*0.5 = v*E0 exactly (also in binary64, where the scaling by 2
// and 0.5 is exact and a zero sign cannot change a later nonzero sum).
template <class T> __device__ __forceinline__ T open_face0_flux(T v, T e0);
template <> __device__ __forceinline__ double open_face0_flux<double>(double v, double e0) {
  return dmul(v, e0);
}
template <> __device__ __forceinline__ float open_face0_flux<float>(float v, float e0) {
  return v * e0;
}

template <class T> __device__ __forceinline__ T face_flux(const StepArgs<T>& A, int a, int F, T v,
                                                          T Ea, T Eb, T Ec, T Ed);
template <> __device__ __forceinline__ double face_flux<double>(const StepArgs<double>& A, int a,
                                                               int F, double v, double Ea,
                                                               double Eb, double Ec, double Ed) {
  return flux_fp64(v, A.g.d[a][pidx(F)], A.dt, Ea, Eb, Ec, Ed);
}
template <> __device__ __forceinline__ float face_flux<float>(const StepArgs<float>& A, int a, int F,
                                                             float v, float Ea, float Eb, float Ec,
                                                             float Ed) {
  return flux_fp32(v, A.t32.hcfl[a][pidx(F)], Ea, Eb, Ec, Ed);
}

// binary64: dE -= (fr - fl) / d(F); binary32: acc += (fl - fr) * dt/d(F)
// (div32, the two-term constant)
template <class T> __device__ __forceinline__ T div_acc(const StepArgs<T>& A, int a, int F, T dE,
                                                        T fr, T fl);
template <> __device__ __forceinline__ double div_acc<double>(const StepArgs<double>& A, int a,
                                                             int F, double dE, double fr,
                                                             double fl) {
  return dsub(dE, ddiv(dsub(fr, fl), A.g.d[a][pidx(F)]));
}
template <> __device__ __forceinline__ float div_acc<float>(const StepArgs<float>& A, int a, int F,
                                                           float dE, float fr, float fl) {
  return div32(dE, fr, fl, A.t32.chi[a][pidx(F)], A.t32.clo[a][pidx(F)]);
}

// Band schedule of the plane items.  sweep = 0: for band of `band` m
// values: for l: for m in band: for (z,k).  sweep = 1: the roles of l and m
// exchanged (bands of l values, m outer within a band).
struct PlaneSched {
  int band;          // values per band of the banded axis
  int nband;         // ceil(n_banded / band)
  int sweep;         // 0: bands over m, 1: bands over l
  int gz;            // z planes per item (1 for the plane kernels)
  long long nunits;  // ceil(nz / gz) * nk
};

// Update one work item (one (z,k) plane at one (l,m)) of the band-ordered
// schedule.  All threads of the CTA call it with the same item; it
// synchronises the CTA internally and returns with shared memory free.
template <class T, int NT>
__device__ __forceinline__ void plane_item(const StepArgs<T>& A, const PlaneSched& S, long long item,
                                           unsigned char* smem_raw) {
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1], nz = d.n[2], nl = d.n[4], nm = d.n[5];
  const int nxy = nx * ny;
  // binary32: this step's rounding seed; item 0 also writes the next one
  unsigned seed = 0;
  if constexpr (sizeof(T) == 4) {
    seed = *A.seed_in;
    advance_seed(A.seed_in, A.seed_out, item);
  }
  T* sE = reinterpret_cast<T*>(smem_raw);
  T* sFx = sE + nxy;
  T* sFy = sFx + nxy;

  // ---- decode the work item (band order) ----
  long long i = item;
  const int u = (int)(i % S.nunits);
  i /= S.nunits;
  const int inner = (int)(i % S.band);
  i /= S.band;
  const int nouter = S.sweep ? nm : nl;
  const int outer = (int)(i % nouter);
  const int b = (int)(i / nouter);
  const int banded = b * S.band + inner;
  const int l = S.sweep ? banded : outer;
  const int m = S.sweep ? outer : banded;
  if ((S.sweep ? l >= nl : m >= nm)) return;  // tail of the last band; uniform over the CTA
  const int z = u % nz;
  const int k = u / nz;
  const long long p0 = (long long)z * d.s[2] + (long long)k * d.s[3] + (long long)l * d.s[4] +
                       (long long)m * d.s[5];

  // ---- stage the plane of E ----
  for (int q = threadIdx.x; q < nxy; q += NT) sE[q] = A.E[p0 + q];
  __syncthreads();

  // ---- x and y right-face fluxes, once per face ----
  for (int q = threadIdx.x; q < nxy; q += NT) {
    const int x = q % nx, y = q / nx;
    if (nx > 1) {
      const int xm = x > 0 ? x - 1 : 0, xp = x + 1 < nx ? x + 1 : nx - 1,
                xpp = x + 2 < nx ? x + 2 : nx - 1;
      const T v = ld_stream(A.vel[0] + p0 + q);
      sFx[q] = face_flux<T>(A, 0, x + 1, v, sE[y * nx + xm], sE[q], sE[y * nx + xp], sE[y * nx + xpp]);
    }
    if (ny > 1) {
      const int ym = y > 0 ? y - 1 : 0, yp = y + 1 < ny ? y + 1 : ny - 1,
                ypp = y + 2 < ny ? y + 2 : ny - 1;
      const T v = ld_stream(A.vel[1] + p0 + q);
      sFy[q] = face_flux<T>(A, 1, y + 1, v, sE[ym * nx + x], sE[q], sE[yp * nx + x], sE[ypp * nx + x]);
    }
  }
  __syncthreads();

  // ---- divergence in axis order, mean-flow term, update ----
  for (int q = threadIdx.x; q < nxy; q += NT) {
    const int x = q % nx, y = q / nx;
    const long long p = p0 + q;
    const T e0 = sE[q];
    T dE = T(0);
    if (nx > 1) {
      // face 0: plane of x face 0 (x collapsed); p0 is a multiple of nx*ny
      const T fl = x > 0 ? sFx[q - 1] : open_face0_flux<T>(A.vlo[0][p0 / nx + y], e0);
      dE = div_acc<T>(A, 0, x + 1, dE, sFx[q], fl);
    }
    if (ny > 1) {
      // face 0: plane of y face 0 (y collapsed)
      const T fl = y > 0 ? sFy[q - nx] : open_face0_flux<T>(A.vlo[1][p0 / ny + x], e0);
      dE = div_acc<T>(A, 1, y + 1, dE, sFy[q], fl);
    }
    int c[6] = {x, y, z, k, l, m};
#pragma unroll
    for (int a = 2; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const int ca = c[a];
      const T Em2 = A.E[nb_index(d, p, a, ca, -2, m)];
      const T Em1 = A.E[nb_index(d, p, a, ca, -1, m)];
      const T Ep1 = A.E[nb_index(d, p, a, ca, +1, m)];
      const T Ep2 = A.E[nb_index(d, p, a, ca, +2, m)];
      const T vr = A.vel[a][p];
      const T vl = ca > 0 ? A.vel[a][p - d.s[a]] : A.vlo[a][plane_index(d, a, c)];
      const T fr = face_flux<T>(A, a, ca + 1, vr, Em1, e0, Ep1, Ep2);
      const T fl = face_flux<T>(A, a, ca, vl, Em2, Em1, e0, Ep1);
      dE = div_acc<T>(A, a, ca + 1, dE, fr, fl);
    }
    if constexpr (sizeof(T) == 8) {
      // meanfl = ((0 + E*lx) + E*ly) + E*lz, integrate.f90:202-252
      double mf = 0.;
      if (nx > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[0] + p)));
      if (ny > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[1] + p)));
      if (nz > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[2] + p)));
      st_stream(A.Enew + p, dadd(e0, dmul(A.dt, dsub(dE, mf))));
    } else {
      st_stream(A.Enew + p, upd32(e0, dE, e0 * ld_stream(A.lam[0] + p), A.dthi, A.dtlo, sr_bits(p, seed)));
    }
  }
  __syncthreads();  // shared memory is reused by the next item
}

// one CTA per work item of one field
template <class T, int NT>
__global__ void __launch_bounds__(NT) step_plane_kernel(StepArgs<T> A, PlaneSched S) {
  extern __shared__ unsigned char smem_raw[];
  plane_item<T, NT>(A, S, blockIdx.x, smem_raw);
}

// Batched ensemble: one persistent launch advances every member by one step.
// The work list is the concatenation of the members' band-ordered items
// (member 0 first); CTA b takes items b, b + gridDim.x, ...  Member j owns
// items [first[j], first[j+1]).
template <class T>
struct BatchMember {
  StepArgs<T> A;
  PlaneSched S;
};

template <class T, int NT>
__global__ void __launch_bounds__(NT) batch_plane_kernel(const BatchMember<T>* __restrict__ mem,
                                                         const long long* __restrict__ first,
                                                         int nmem) {
  extern __shared__ unsigned char smem_raw[];
  const long long total = first[nmem];
  int j = 0;
  for (long long it = blockIdx.x; it < total; it += gridDim.x) {
    while (it >= first[j + 1]) j++;  // items are visited in increasing order
    plane_item<T, NT>(mem[j].A, mem[j].S, it - first[j], smem_raw);
  }
}

}  // namespace rt
