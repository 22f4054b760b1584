// rt_step3.cuh -- TMA-staged plane step (sm_103a).
//
// Same work decomposition and band order as rt_step2.cuh (one CTA per
// (z,k) plane of (x,y) at one (l,m)), but the 17 planes of E that the stencil
// reads -- the centre and the +-1, +-2 neighbours along z, k, l and m, with
// the boundary maps applied per plane -- are copied into shared memory by
// the bulk-copy engine (cp.async.bulk, completion on an mbarrier), issued by
// one thread.  Everything the per-cell code needs besides the in-plane index
// (neighbour plane slots, the face-0 planes, grid constants) is uniform over
// the CTA and computed once.  Velocities and the growth rate are read once
// per cell straight into registers with evict-first hints.
//
// Every wait on the mbarrier is bounded: after RT_WAIT_LIMIT polls the CTA
// raises bit 0 of *status, waits once more (bounded) for its copies, and
// leaves the item unwritten; the host turns the flag into an error.
#pragma once
#include <cstdint>

#include "rt_step2.cuh"

namespace rt {

#define RT_WAIT_LIMIT (1u << 22)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bulk copy global -> shared, completion counted on the mbarrier; dst, src
// and bytes are multiples of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// bounded wait; returns false (and raises the status flag) on timeout
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status) {
  for (uint32_t it = 0; it < RT_WAIT_LIMIT; it++)
    if (mbar_try_wait(bar, parity)) return true;
  if (threadIdx.x == 0) atomicOr(status, 1);
  for (uint32_t it = 0; it < RT_WAIT_LIMIT; it++)  // let copies in flight land
    if (mbar_try_wait(bar, parity)) break;
  return false;
}

// planes staged per item: E centre, then z, k, l, m neighbours at -2,-1,+1,+2
#define RT_NPLANE 17

// true when the TMA path applies: plane bytes a multiple of 16
template <class T>
__host__ __device__ __forceinline__ bool tma_ok(const Dims& d) {
  return ((long long)d.n[0] * d.n[1] * (long long)sizeof(T)) % 16 == 0;
}
template <class T>
__host__ __device__ __forceinline__ size_t tma_smem(const Dims& d) {
  return 16 + (size_t)(RT_NPLANE + 2) * d.n[0] * d.n[1] * sizeof(T);
}

// coordinate of a neighbour plane after the boundary maps (same rules as
// map_coord); returns the plane's linear offset
__device__ __forceinline__ long long nb_plane(const Dims& d, const int c[6], int a, int off) {
  int flip = 0;
  const int ca = map_coord(d, a, c[a] + off, flip);
  long long p = 0;
#pragma unroll
  for (int b = 2; b < 6; b++) {
    int cb = c[b];
    if (b == a) cb = ca;
    if (b == 5 && flip) cb = d.n[5] - 1 - cb;
    p += (long long)cb * d.s[b];
  }
  return p;
}

// returns false only when a bounded wait timed out (status raised)
template <class T, int NT>
__device__ __forceinline__ bool tma_item(const StepArgs<T>& A, const PlaneSched& S, long long item,
                                         unsigned char* smem_raw, uint32_t phase) {
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1], nz = d.n[2], nl = d.n[4], nm = d.n[5];
  const int nxy = nx * ny;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  T* sP = reinterpret_cast<T*>(smem_raw + 16);   // RT_NPLANE planes
  T* sFx = sP + (size_t)RT_NPLANE * nxy;
  T* sFy = sFx + nxy;

  // ---- decode the work item (band order, as rt_step2.cuh) ----
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
  if ((S.sweep ? l >= nl : m >= nm)) return true;
  const int z = u % nz;
  const int k = u / nz;
  const int c[6] = {0, 0, z, k, l, m};
  const long long p0 = (long long)z * d.s[2] + (long long)k * d.s[3] + (long long)l * d.s[4] +
                       (long long)m * d.s[5];

  // ---- stage the 17 E planes with the bulk-copy engine ----
  const uint32_t pbytes = (uint32_t)(nxy * sizeof(T));
  if (threadIdx.x == 0) {
    // order the CTA's earlier generic-proxy reads of these buffers before the
    // async-proxy writes below (the preceding __syncthreads made them complete)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    uint32_t nplanes = 1;
    for (int a = 2; a < 6; a++)
      if (d.n[a] > 1) nplanes += 4;
    mbar_arrive_expect_tx(bar, nplanes * pbytes);
    bulk_g2s(sP, A.E + p0, pbytes, bar);
    int slot = 1;
    for (int a = 2; a < 6; a++) {
      if (d.n[a] <= 1) { slot += 4; continue; }
      const int offs[4] = {-2, -1, 1, 2};
      for (int j = 0; j < 4; j++)
        bulk_g2s(sP + (size_t)(slot + j) * nxy, A.E + nb_plane(d, c, a, offs[j]), pbytes, bar);
      slot += 4;
    }
  }
  // uniform per-CTA data while the copies fly
  const T* vlft[6];
  long long vlft_off[6];
#pragma unroll
  for (int a = 2; a < 6; a++) {
    if (c[a] > 0) { vlft[a] = A.vel[a]; vlft_off[a] = p0 - d.s[a]; }
    else {  // face 0 plane: (x,y) contiguous at the plane index of (0,0,c[2..5])
      long long q = 0;
      for (int bb = 2; bb < 6; bb++) q += (long long)c[bb] * plane_stride(d, a, bb);
      vlft[a] = A.vlo[a];
      vlft_off[a] = q;
    }
  }

  if (!mbar_wait_bounded(bar, phase, A.status)) return false;

  const T* sE = sP;
  // ---- x and y right-face fluxes, once per face ----
  for (int q = threadIdx.x; q < nxy; q += NT) {
    const int y = q / nx, x = q - y * nx;
    if (nx > 1) {
      const int r = y * nx;
      const int xm = x > 0 ? x - 1 : 0, xp = x + 1 < nx ? x + 1 : nx - 1,
                xpp = x + 2 < nx ? x + 2 : nx - 1;
      const T v = ld_stream(A.vel[0] + p0 + q);
      sFx[q] = face_flux<T>(A, 0, x + 1, v, sE[r + xm], sE[q], sE[r + xp], sE[r + xpp]);
    }
    if (ny > 1) {
      const int ym = y > 0 ? y - 1 : 0, yp = y + 1 < ny ? y + 1 : ny - 1,
                ypp = y + 2 < ny ? y + 2 : ny - 1;
      const T v = ld_stream(A.vel[1] + p0 + q);
      sFy[q] = face_flux<T>(A, 1, y + 1, v, sE[ym * nx + x], sE[q], sE[yp * nx + x], sE[ypp * nx + x]);
    }
  }
  __syncthreads();

  // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
  for (int q = threadIdx.x; q < nxy; q += NT) {
    const int y = q / nx, x = q - y * nx;
    const long long p = p0 + q;
    const T e0 = sE[q];
    T dE = T(0);
    if (nx > 1) {
      const T fl = x > 0 ? sFx[q - 1] : open_face0_flux<T>(A.vlo[0][p0 / nx + y], e0);
      dE = div_acc<T>(A, 0, x + 1, dE, sFx[q], fl);
    }
    if (ny > 1) {
      const T fl = y > 0 ? sFy[q - nx] : open_face0_flux<T>(A.vlo[1][p0 / ny + x], e0);
      dE = div_acc<T>(A, 1, y + 1, dE, sFy[q], fl);
    }
#pragma unroll
    for (int a = 2; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const T* sN = sP + (size_t)(1 + 4 * (a - 2)) * nxy;
      const T Em2 = sN[q], Em1 = sN[nxy + q], Ep1 = sN[2 * nxy + q], Ep2 = sN[3 * nxy + q];
      const T vr = A.vel[a][p];
      const T vl = vlft[a][vlft_off[a] + q];
      const T fr = face_flux<T>(A, a, c[a] + 1, vr, Em1, e0, Ep1, Ep2);
      const T fl = face_flux<T>(A, a, c[a], vl, Em2, Em1, e0, Ep1);
      dE = div_acc<T>(A, a, c[a] + 1, dE, fr, fl);
    }
    if constexpr (sizeof(T) == 8) {
      double mf = 0.;
      if (nx > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[0] + p)));
      if (ny > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[1] + p)));
      if (nz > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[2] + p)));
      st_stream(A.Enew + p, dadd(e0, dmul(A.dt, dsub(dE, mf))));
    } else {
      const T mf = e0 * ld_stream(A.lam[0] + p);
      st_stream(A.Enew + p, (T)(e0 + (T)A.dt * (dE - mf)));
    }
  }
  __syncthreads();  // shared memory and the barrier are reused by the next item
  return true;
}

template <class T, int NT>
__global__ void __launch_bounds__(NT) step_tma_kernel(StepArgs<T> A, PlaneSched S) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  tma_item<T, NT>(A, S, blockIdx.x, smem_raw, 0);
}

// persistent batched form: the mbarrier is re-armed for every item, the
// phase bit alternates
template <class T, int NT>
__global__ void __launch_bounds__(NT) batch_tma_kernel(const BatchMember<T>* __restrict__ mem,
                                                       const long long* __restrict__ first,
                                                       int nmem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const long long total = first[nmem];
  int j = 0;
  uint32_t phase = 0;
  for (long long it = blockIdx.x; it < total; it += gridDim.x) {
    while (it >= first[j + 1]) j++;
    const BatchMember<T>& M = mem[j];
    // items past the end of the last band skip the copies: keep the phase
    long long ii = it - first[j];
    const long long per = (long long)M.S.nunits * M.S.band * (M.S.sweep ? M.A.d.n[5] : M.A.d.n[4]);
    const int banded = (int)(ii / per) * M.S.band + (int)((ii / M.S.nunits) % M.S.band);
    if (banded >= (M.S.sweep ? M.A.d.n[4] : M.A.d.n[5])) continue;
    if (!tma_item<T, NT>(M.A, M.S, ii, smem_raw, phase)) return;
    phase ^= 1;
  }
}

}  // namespace rt
