// rt_step4.cuh -- z-group TMA step: one work item = G consecutive z planes.
//
// Generalises the plane item of rt_step3.cuh for small (x,y) planes: an item
// covers the cells (x, y, z0..z0+G-1) at one (k, l, m), so a CTA of NT
// threads stays busy when nx*ny is much smaller than NT (the ensemble and
// serving workloads mix planes of 64 to 1024 cells).  Staged by the
// bulk-copy engine into shared memory (completion on an mbarrier with a
// bounded wait):
//   * the z window z0-2 .. z0+G+1 of E (in-range planes in one copy, the
//     boundary-mapped ghost planes one copy each),
//   * for k, l and m the G-plane blocks at -2, -1, +1, +2 (contiguous),
// at most 17 copies per item.  Face fluxes along x, y and z are evaluated
// once per face and shared through shared memory; k, l, m faces per cell.
// Arithmetic is that of rt_step.cuh, the divergence in the reference's axis
// order, so results are bit-identical to the other step kernels.
#pragma once
#include "rt_step3.cuh"

namespace rt {

template <class T>
struct GroupDesc {
  long long vloff[6];      // axes 3..5: left-face velocity offset of (0,0,z0)
  long long zvoff[2];      // z face 0 of the group: offset into vel[2] (or vlo[2] when z0 == 0)
  T kcfl_r[6], kch_r[6], kcl_r[6], kcfl_l[6];
  double d_r[6], d_l[6];
};

template <class T>
__host__ __device__ constexpr size_t gdesc_bytes() { return (sizeof(GroupDesc<T>) + 15) / 16 * 16; }

// planes of shared memory for a group of G: z window (G+4), k/l/m blocks
// (12G), x/y fluxes (2G), z faces (G+1)
__host__ __device__ __forceinline__ long long group_planes(int G) { return 16LL * G + 5; }

template <class T>
__host__ __device__ __forceinline__ size_t group_smem(const Dims& d, int G) {
  return 16 + gdesc_bytes<T>() + (size_t)group_planes(G) * d.n[0] * d.n[1] * sizeof(T);
}

// offset of the (x,y) plane at (z, k, l, m) after the boundary map of axis a
// applied to coordinate c[a] + off (z may reflect and flip m)
__device__ __forceinline__ long long mapped_plane(const Dims& d, const int c[6], int a, int off) {
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
__device__ __forceinline__ bool group_item(const StepArgs<T>& A, const PlaneSched& S, long long item,
                                           unsigned char* smem_raw, uint32_t phase) {
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1], nz = d.n[2], nl = d.n[4], nm = d.n[5];
  const int nxy = nx * ny;
  const int G = S.gz;
  // binary32: this step's rounding seed; item 0 also writes the next one
  unsigned seed = 0;
  if constexpr (sizeof(T) == 4) {
    seed = *A.seed_in;
    advance_seed(A.seed_in, A.seed_out, item);
  }
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  GroupDesc<T>* desc = reinterpret_cast<GroupDesc<T>*>(smem_raw + 16);
  T* sW = reinterpret_cast<T*>(smem_raw + 16 + gdesc_bytes<T>());  // z window, G+4 planes
  T* sB = sW + (size_t)(G + 4) * nxy;                                 // k,l,m blocks, 12G planes
  T* sFx = sB + (size_t)12 * G * nxy;
  T* sFy = sFx + (size_t)G * nxy;
  T* sFz = sFy + (size_t)G * nxy;                                     // G+1 face planes

  // ---- decode: (z group, k) units, band order over (l, m) ----
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
  const int ngz = (nz + G - 1) / G;
  const int gz = u % ngz;
  const int k = u / ngz;
  const int z0 = gz * G;
  const int Ge = (nz - z0) < G ? (nz - z0) : G;
  const int c[6] = {0, 0, z0, k, l, m};
  const long long p0 = (long long)z0 * d.s[2] + (long long)k * d.s[3] + (long long)l * d.s[4] +
                       (long long)m * d.s[5];
  const int ncell = Ge * nxy;

  // ---- thread 0: descriptor and the bulk copies ----
  const uint32_t pbytes = (uint32_t)(nxy * sizeof(T));
  if (threadIdx.x == 0) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    const bool zact = nz > 1;
    // z window: slots s = 0..Ge+3 hold z = z0-2+s; without a z axis only the
    // centre planes (slots 2..Ge+1) are read
    const int zlo = zact ? z0 - 2 : z0, zhi = zact ? z0 + Ge + 1 : z0 + Ge - 1;
    const int in_lo = zlo < 0 ? 0 : zlo, in_hi = zhi > nz - 1 ? nz - 1 : zhi;
    uint32_t nplanes = (uint32_t)(zhi - zlo + 1);
    for (int a = 3; a < 6; a++)
      if (d.n[a] > 1) nplanes += 4u * Ge;
    mbar_arrive_expect_tx(bar, nplanes * pbytes);
    {
      int cc[6] = {0, 0, in_lo, k, l, m};
      bulk_g2s(sW + (size_t)(in_lo - (z0 - 2)) * nxy, A.E + mapped_plane(d, cc, 2, 0),
               (uint32_t)(in_hi - in_lo + 1) * pbytes, bar);
      for (int z = zlo; z <= zhi; z++) {
        if (z >= 0 && z < nz) continue;
        int cz[6] = {0, 0, z0, k, l, m};
        bulk_g2s(sW + (size_t)(z - (z0 - 2)) * nxy, A.E + mapped_plane(d, cz, 2, z - z0), pbytes, bar);
      }
    }
    for (int a = 3; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const int offs[4] = {-2, -1, 1, 2};
      for (int j = 0; j < 4; j++)
        bulk_g2s(sB + ((size_t)(a - 3) * 4 + j) * G * nxy, A.E + mapped_plane(d, c, a, offs[j]),
                 (uint32_t)Ge * pbytes, bar);
    }
    for (int a = 3; a < 6; a++) {
      long long off;
      if (c[a] > 0) {
        off = p0 - d.s[a];
      } else {
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
    // z face 0 of the group (between z0-1 and z0)
    if (z0 > 0) {
      desc->zvoff[0] = p0 - d.s[2];
      desc->zvoff[1] = 0;
    } else {
      long long off = 0;
      for (int bb = 3; bb < 6; bb++) off += (long long)c[bb] * plane_stride(d, 2, bb);
      desc->zvoff[0] = off;
      desc->zvoff[1] = 1;  // read from the face-0 plane
    }
  }
  __syncthreads();
  FaceK<T> kr[6], kl[6];
  long long vloff[6];
#pragma unroll
  for (int a = 3; a < 6; a++) {
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
  const long long zv0 = desc->zvoff[0];
  const bool zv0_plane = desc->zvoff[1] != 0;
  // q -> (plane j, x, y) by multiplying with ceil(2^32/n): exact for q*n <= 2^32
  const unsigned long long xmul = ((1ull << 32) + (unsigned)nx - 1) / (unsigned)nx;
  const unsigned long long pmul = ((1ull << 32) + (unsigned)nxy - 1) / (unsigned)nxy;

  if (!mbar_wait_bounded(bar, phase, A.status)) return false;

  // ---- phase A: x, y right-face fluxes of every cell; z faces 0..Ge ----
  for (int q = threadIdx.x; q < ncell; q += NT) {
    const int j = (int)(((unsigned long long)q * pmul) >> 32);
    const int r = q - j * nxy;
    const int y = (int)(((unsigned long long)r * xmul) >> 32), x = r - y * nx;
    const T* sE = sW + (size_t)(j + 2) * nxy;
    const long long pc = p0 + q;
    if (nx > 1) {
      const int row = y * nx;
      const int xm = x > 0 ? x - 1 : 0, xp = x + 1 < nx ? x + 1 : nx - 1,
                xpp = x + 2 < nx ? x + 2 : nx - 1;
      FaceK<T> kx;
      kx.load(A, 0, x + 1, false);
      sFx[q] = kflux(A, kx, ld_stream(A.vel[0] + pc), ucfl_at<T>(A.uc[0], pc), sE[row + xm], sE[r],
                     sE[row + xp], sE[row + xpp]);
    }
    if (ny > 1) {
      const int ym = y > 0 ? y - 1 : 0, yp = y + 1 < ny ? y + 1 : ny - 1,
                ypp = y + 2 < ny ? y + 2 : ny - 1;
      FaceK<T> ky;
      ky.load(A, 1, y + 1, false);
      sFy[q] = kflux(A, ky, ld_stream(A.vel[1] + pc), ucfl_at<T>(A.uc[1], pc), sE[ym * nx + x], sE[r],
                     sE[yp * nx + x], sE[ypp * nx + x]);
    }
  }
  if (nz > 1) {
    // face jf (0..Ge) lies between z0+jf-1 and z0+jf (Fortran face z0+jf)
    const int nface = (Ge + 1) * nxy;
    for (int q = threadIdx.x; q < nface; q += NT) {
      const int jf = (int)(((unsigned long long)q * pmul) >> 32);
      const int r = q - jf * nxy;
      T v, uc;
      if (jf > 0) {
        const long long pv = p0 + (long long)(jf - 1) * nxy + r;
        v = A.vel[2][pv];
        uc = ucfl_at<T>(A.uc[2], pv);
      } else if (zv0_plane) {
        v = A.vlo[2][zv0 + r];
        uc = ucfl_at<T>(A.ucl[2], zv0 + r);
      } else {
        v = A.vel[2][zv0 + r];
        uc = ucfl_at<T>(A.uc[2], zv0 + r);
      }
      FaceK<T> kz;
      kz.load(A, 2, z0 + jf, false);
      sFz[q] = kflux(A, kz, v, uc, sW[(size_t)jf * nxy + r], sW[(size_t)(jf + 1) * nxy + r],
                     sW[(size_t)(jf + 2) * nxy + r], sW[(size_t)(jf + 3) * nxy + r]);
    }
  }
  __syncthreads();

  // ---- phase B: divergence (x,y,z,k,l,m), mean-flow term, update ----
  for (int q = threadIdx.x; q < ncell; q += NT) {
    const int j = (int)(((unsigned long long)q * pmul) >> 32);
    const int r = q - j * nxy;
    const int y = (int)(((unsigned long long)r * xmul) >> 32), x = r - y * nx;
    const long long pc = p0 + q;
    T vr[3], vl[3], ur[3], ul[3];
#pragma unroll
    for (int a = 3; a < 6; a++) {
      const bool act = d.n[a] > 1;
      vr[a - 3] = act ? A.vel[a][pc] : T(0);
      vl[a - 3] = act ? (c[a] > 0 ? A.vel[a][vloff[a] + q] : A.vlo[a][vloff[a] + q]) : T(0);
      ur[a - 3] = act ? ucfl_at<T>(A.uc[a], pc) : T(0);
      ul[a - 3] = act ? (c[a] > 0 ? ucfl_at<T>(A.uc[a], vloff[a] + q) : ucfl_at<T>(A.ucl[a], vloff[a] + q))
                      : T(0);
    }
    const T e0 = sW[(size_t)(j + 2) * nxy + r];
    T dE = T(0);
    if (nx > 1) {
      FaceK<T> kx;
      kx.load(A, 0, x + 1, true);
      const T fl = x > 0 ? sFx[q - 1] : open_face0_flux<T>(A.vlo[0][(p0 + (long long)j * nxy) / nx + y], e0);
      dE = kdiv(kx, dE, sFx[q], fl);
    }
    if (ny > 1) {
      FaceK<T> ky;
      ky.load(A, 1, y + 1, true);
      const T fl = y > 0 ? sFy[q - nx] : open_face0_flux<T>(A.vlo[1][(p0 + (long long)j * nxy) / ny + x], e0);
      dE = kdiv(ky, dE, sFy[q], fl);
    }
    if (nz > 1) {
      FaceK<T> kz;
      kz.load(A, 2, z0 + j + 1, true);
      dE = kdiv(kz, dE, sFz[(size_t)(j + 1) * nxy + r], sFz[(size_t)j * nxy + r]);
    }
#pragma unroll
    for (int a = 3; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const T* sN = sB + (size_t)(a - 3) * 4 * G * nxy + (size_t)j * nxy + r;
      const size_t bs = (size_t)G * nxy;
      const T Em2 = sN[0], Em1 = sN[bs], Ep1 = sN[2 * bs], Ep2 = sN[3 * bs];
      const T fr = kflux(A, kr[a], vr[a - 3], ur[a - 3], Em1, e0, Ep1, Ep2);
      const T fl = kflux(A, kl[a], vl[a - 3], ul[a - 3], Em2, Em1, e0, Ep1);
      dE = kdiv(kr[a], dE, fr, fl);
    }
    if constexpr (sizeof(T) == 8) {
      double mf = 0.;
      if (nx > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[0] + pc)));
      if (ny > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[1] + pc)));
      if (nz > 1) mf = dadd(mf, dmul(e0, ld_stream(A.lam[2] + pc)));
      st_stream(A.Enew + pc, dadd(e0, dmul(A.dt, dsub(dE, mf))));
    } else {
      st_stream(A.Enew + pc, upd32(e0, dE, e0 * ld_stream(A.lam[0] + pc), A.dthi, A.dtlo, sr_bits(pc, seed)));
    }
  }
  __syncthreads();
  return true;
}

template <class T, int NT>
__global__ void __launch_bounds__(NT) step_group_kernel(StepArgs<T> A, PlaneSched S) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  group_item<T, NT>(A, S, blockIdx.x, smem_raw, 0);
}

template <class T, int NT>
__global__ void __launch_bounds__(NT) batch_group_kernel(const BatchMember<T>* __restrict__ mem,
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
    const long long ii = it - first[j];
    const long long per = (long long)M.S.nunits * M.S.band * (M.S.sweep ? M.A.d.n[5] : M.A.d.n[4]);
    const int banded = (int)(ii / per) * M.S.band + (int)((ii / M.S.nunits) % M.S.band);
    if (banded >= (M.S.sweep ? M.A.d.n[4] : M.A.d.n[5])) continue;   // no copies issued: keep phase
    if (!group_item<T, NT>(M.A, M.S, ii, smem_raw, phase)) return;
    phase ^= 1;
  }
}

}  // namespace rt
