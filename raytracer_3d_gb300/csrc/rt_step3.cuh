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

// bounded wait; returns false (and raises the status flag) on timeout.
// LIMIT polls (the failure-detection self-test uses a short one).  After a
// timeout the caller's copies get a second LIMIT polls to land; a copy that
// has not landed by then is abandoned when the CTA leaves (its shared memory
// may be handed to another CTA), so the flagged launch's results, and those
// of any launch that overlaps it, are invalid -- which is what the raised
// status tells the host.  No CTA issues a copy after one of its own waits
// has timed out.
template <uint32_t LIMIT = RT_WAIT_LIMIT>
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* status) {
  for (uint32_t it = 0; it < LIMIT; it++)
    if (mbar_try_wait(bar, parity)) return true;
  if (threadIdx.x == 0) atomicOr(status, 1);
  for (uint32_t it = 0; it < LIMIT; it++)  // let copies in flight land
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
// per-item values that every thread needs, computed by thread 0 while it
// issues the copies and published through shared memory
template <class T>
struct ItemDesc {
  long long vloff[6];     // offset of the left-face velocities of (x,y)=(0,0), axes 2..5
  T kcfl_r[6], kch_r[6], kcl_r[6], kcfl_l[6];   // binary32 grid constants of the two faces
  double d_r[6], d_l[6];               // binary64 grid spacings of the two faces
};
// shared-memory bytes of the descriptor, rounded to the 16-byte alignment of
// the planes that follow it
template <class T>
__host__ __device__ constexpr size_t desc_bytes() { return (sizeof(ItemDesc<T>) + 15) / 16 * 16; }

template <class T>
__host__ __device__ __forceinline__ size_t tma_smem(const Dims& d) {
  return 16 + desc_bytes<T>() + (size_t)(RT_NPLANE + 2) * d.n[0] * d.n[1] * sizeof(T);
}

// most cells one thread owns in the TMA kernels
#define RT_TMA_MAXC 4

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

// grid constants of one face: binary32 form keeps dt/(2d) and dt/d (as
// chi + clo), binary64 keeps d (the reference divides)
template <class T> struct FaceK;
template <> struct FaceK<float> {
  float cfl, chi, clo;
  __device__ __forceinline__ void load(const StepArgs<float>& A, int a, int F, bool with_div) {
    cfl = A.t32.hcfl[a][pidx(F)];
    chi = with_div ? A.t32.chi[a][pidx(F)] : 0.f;
    clo = with_div ? A.t32.clo[a][pidx(F)] : 0.f;
  }
};
template <> struct FaceK<double> {
  double d;
  __device__ __forceinline__ void load(const StepArgs<double>& A, int a, int F, bool) {
    d = A.g.d[a][pidx(F)];
  }
};
// u: the cached uCFL of the face (binary64 form); the binary32 form forms
// |v|*dt/(2d) from its table instead
__device__ __forceinline__ float kflux(const StepArgs<float>&, const FaceK<float>& k, float v, float,
                                       float Ea, float Eb, float Ec, float Ed) {
  return flux_fp32(v, k.cfl, Ea, Eb, Ec, Ed);
}
__device__ __forceinline__ double kflux(const StepArgs<double>&, const FaceK<double>&, double v,
                                        double u, double Ea, double Eb, double Ec, double Ed) {
  return flux_fp64u(v, u, Ea, Eb, Ec, Ed);
}
// cached uCFL of the binary64 form (zero for binary32, where it is unused)
template <class T>
__device__ __forceinline__ T ucfl_at(const T* base, long long i) {
  if constexpr (sizeof(T) == 8) return base[i];
  else return T(0);
}
// binary64: dE -= (fr - fl)/d; binary32: acc += (fl - fr)*dt/d (div32),
// with the right face's constants
__device__ __forceinline__ float kdiv(const FaceK<float>& kr, float dE, float fr, float fl) {
  return div32(dE, fr, fl, kr.chi, kr.clo);
}
__device__ __forceinline__ double kdiv(const FaceK<double>& kr, double dE, double fr, double fl) {
  return dsub(dE, ddiv(dsub(fr, fl), kr.d));
}

// Update one work item.  MAXC = most cells one thread owns (nx*ny <= MAXC*NT).
// Returns false only when a bounded wait timed out (status raised).
template <class T, int NT, int MAXC>
__device__ __forceinline__ bool tma_item(const StepArgs<T>& A, const PlaneSched& S, long long item,
                                         unsigned char* smem_raw, uint32_t phase) {
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1], nz = d.n[2], nl = d.n[4], nm = d.n[5];
  const int nxy = nx * ny;
  // binary32: this step's rounding seed; item 0 also writes the next one
  unsigned seed = 0;
  if constexpr (sizeof(T) == 4) {
    seed = *A.seed_in;
    advance_seed(A.seed_in, A.seed_out, item);
  }
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  ItemDesc<T>* desc = reinterpret_cast<ItemDesc<T>*>(smem_raw + 16);
  T* sP = reinterpret_cast<T*>(smem_raw + 16 + desc_bytes<T>());   // RT_NPLANE planes
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

  // ---- while the copies fly: thread 0 fills the item descriptor ----
  if (threadIdx.x == 0) {
#pragma unroll
    for (int a = 2; a < 6; a++) {
      long long off;
      if (c[a] > 0) {
        off = p0 - d.s[a];
      } else {  // face-0 plane: (x,y) contiguous at the plane index of (0,0,c[2..5])
        off = 0;
        for (int bb = 2; bb < 6; bb++) off += (long long)c[bb] * plane_stride(d, a, bb);
      }
      desc->vloff[a] = off;
      if (d.n[a] > 1) {
        if constexpr (sizeof(T) == 4) {
          desc->kcfl_r[a] = A.t32.hcfl[a][pidx(c[a] + 1)];
          desc->kch_r[a] = A.t32.chi[a][pidx(c[a] + 1)];
          desc->kcl_r[a] = A.t32.clo[a][pidx(c[a] + 1)];
          desc->kcfl_l[a] = A.t32.hcfl[a][pidx(c[a])];
        } else {
          desc->d_r[a] = A.g.d[a][pidx(c[a] + 1)];
          desc->d_l[a] = A.g.d[a][pidx(c[a])];
        }
      }
    }
  }
  __syncthreads();
  FaceK<T> kr[6], kl[6];
  long long vloff[6];
#pragma unroll
  for (int a = 2; a < 6; a++) {
    vloff[a] = desc->vloff[a];
    if constexpr (sizeof(T) == 4) {
      kr[a].cfl = desc->kcfl_r[a];
      kr[a].chi = desc->kch_r[a];
      kr[a].clo = desc->kcl_r[a];
      kl[a].cfl = desc->kcfl_l[a];
      kl[a].chi = 0.f;
      kl[a].clo = 0.f;
    } else {
      kr[a].d = desc->d_r[a];
      kl[a].d = desc->d_l[a];
    }
  }
  // q -> (x, y) by multiplying with ceil(2^32/nx): exact for q*nx <= 2^32,
  // which holds because nx*ny <= 4096 on this path
  const unsigned long long ymul = ((1ull << 32) + (unsigned)nx - 1) / (unsigned)nx;

  if (!mbar_wait_bounded(bar, phase, A.status)) return false;

  const T* sE = sP;
  // ---- x and y right-face fluxes, once per face ----
#pragma unroll 1
  for (int j = 0; j < MAXC; j++) {
    const int q = threadIdx.x + j * NT;
    if (q < nxy) {
      const int y = (int)(((unsigned long long)q * ymul) >> 32), x = q - y * nx;
      if (nx > 1) {
        const int r = y * nx;
        const int xm = x > 0 ? x - 1 : 0, xp = x + 1 < nx ? x + 1 : nx - 1,
                  xpp = x + 2 < nx ? x + 2 : nx - 1;
        FaceK<T> kx;
        kx.load(A, 0, x + 1, false);
        sFx[q] = kflux(A, kx, ld_stream(A.vel[0] + p0 + q), ucfl_at<T>(A.uc[0], p0 + q), sE[r + xm], sE[q],
                       sE[r + xp], sE[r + xpp]);
      }
      if (ny > 1) {
        const int ym = y > 0 ? y - 1 : 0, yp = y + 1 < ny ? y + 1 : ny - 1,
                  ypp = y + 2 < ny ? y + 2 : ny - 1;
        FaceK<T> ky;
        ky.load(A, 1, y + 1, false);
        sFy[q] = kflux(A, ky, ld_stream(A.vel[1] + p0 + q), ucfl_at<T>(A.uc[1], p0 + q), sE[ym * nx + x],
                       sE[q], sE[yp * nx + x], sE[ypp * nx + x]);
      }
    }
  }
  __syncthreads();

  // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
#pragma unroll 1
  for (int j = 0; j < MAXC; j++) {
    const int q = threadIdx.x + j * NT;
    if (q < nxy) {
      const int y = (int)(((unsigned long long)q * ymul) >> 32), x = q - y * nx;
      // the cell's face velocities and rate, loaded together
      T vr[4], vl[4], ur[4], ul[4];
#pragma unroll
      for (int a = 2; a < 6; a++) {
        const bool act = d.n[a] > 1;
        vr[a - 2] = act ? A.vel[a][p0 + q] : T(0);
        vl[a - 2] = act ? (c[a] > 0 ? A.vel[a][vloff[a] + q] : A.vlo[a][vloff[a] + q]) : T(0);
        ur[a - 2] = act ? ucfl_at<T>(A.uc[a], p0 + q) : T(0);
        ul[a - 2] = act ? (c[a] > 0 ? ucfl_at<T>(A.uc[a], vloff[a] + q) : ucfl_at<T>(A.ucl[a], vloff[a] + q))
                        : T(0);
      }
      const T e0 = sE[q];
      T dE = T(0);
      if (nx > 1) {
        FaceK<T> kx;
        kx.load(A, 0, x + 1, true);
        const T fl = x > 0 ? sFx[q - 1] : open_face0_flux<T>(A.vlo[0][p0 / nx + y], e0);
        dE = kdiv(kx, dE, sFx[q], fl);
      }
      if (ny > 1) {
        FaceK<T> ky;
        ky.load(A, 1, y + 1, true);
        const T fl = y > 0 ? sFy[q - nx] : open_face0_flux<T>(A.vlo[1][p0 / ny + x], e0);
        dE = kdiv(ky, dE, sFy[q], fl);
      }
#pragma unroll
      for (int a = 2; a < 6; a++) {
        if (d.n[a] <= 1) continue;
        const T* sN = sP + (size_t)(1 + 4 * (a - 2)) * nxy;
        const T Em2 = sN[q], Em1 = sN[nxy + q], Ep1 = sN[2 * nxy + q], Ep2 = sN[3 * nxy + q];
        const T fr = kflux(A, kr[a], vr[a - 2], ur[a - 2], Em1, e0, Ep1, Ep2);
        const T fl = kflux(A, kl[a], vl[a - 2], ul[a - 2], Em2, Em1, e0, Ep1);
        dE = kdiv(kr[a], dE, fr, fl);
      }
      if constexpr (sizeof(T) == 8) {
        // meanfl = ((0 + E*lx) + E*ly) + E*lz, integrate.f90:202-252
        double mf = 0.;
        if (nx > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[0] + p0 + q)));
        if (ny > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[1] + p0 + q)));
        if (nz > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[2] + p0 + q)));
        st_stream(A.Enew + p0 + q, dadd(e0, dmul(A.dt, dsub(dE, mf))));
      } else {
        st_stream(A.Enew + p0 + q,
                  upd32(e0, dE, e0 * ld_stream(A.lam[0] + p0 + q), A.dthi, A.dtlo, sr_bits(p0 + q, seed)));
      }
    }
  }
  __syncthreads();  // shared memory and the barrier are reused by the next item
  return true;
}

// registers are left to the compiler (a cap of 64 made the binary32 kernel
// spill and run slower)
template <class T, int NT>
struct TmaMinBlocks { static constexpr int value = 1; };

template <class T, int NT, int MAXC>
__global__ void __launch_bounds__(NT, (TmaMinBlocks<T, NT>::value))
    step_tma_kernel(StepArgs<T> A, PlaneSched S) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  tma_item<T, NT, MAXC>(A, S, blockIdx.x, smem_raw, 0);
}

// persistent batched form: the mbarrier is re-armed for every item, the
// phase bit alternates
template <class T, int NT, int MAXC>
__global__ void __launch_bounds__(NT, (TmaMinBlocks<T, NT>::value))
    batch_tma_kernel(const BatchMember<T>* __restrict__ mem,
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
    if (!tma_item<T, NT, MAXC>(M.A, M.S, ii, smem_raw, phase)) return;
    phase ^= 1;
  }
}

}  // namespace rt
