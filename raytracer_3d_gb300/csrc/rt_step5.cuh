// rt_step5.cuh -- persistent, software-pipelined TMA step (binary32 form).
//
// The plane items of rt_step3.cuh (one (z,k) plane of (x,y) at one (l,m),
// band order over (l,m)) are processed by persistent CTAs, CTA b taking
// items b, b + G, b + 2G, ... so that the CTAs of the GPU still sweep the
// band order together.  While item i is computed:
//   * thread 0 has already issued the 17 bulk copies of item i+G into the
//     second shared-memory stage (two stages, each with its own mbarrier),
//   * every thread has already loaded its cells' face velocities and growth
//     rate of item i+G into registers,
// so the copy and load latency of one item hides behind the arithmetic of
// the previous one.  Waits on the mbarriers are bounded (rt_step3.cuh).
// Arithmetic and axis order are those of the other step kernels: results
// are bit-identical to them.
#pragma once
#include "rt_step3.cuh"

namespace rt {

// item -> (z, k, l, m) in band order without holes: the last band may be
// shorter than S.band
__device__ __forceinline__ void decode_dense(const Dims& d, const PlaneSched& S, long long item,
                                             int c[6]) {
  const int nb_axis = S.sweep ? d.n[4] : d.n[5];
  const int no_axis = S.sweep ? d.n[5] : d.n[4];
  const long long per_full = S.nunits * (long long)no_axis * S.band;
  const long long b = item / per_full;
  long long rem = item - b * per_full;
  int bsize = S.band;
  if ((b + 1) * S.band > nb_axis) bsize = nb_axis - (int)b * S.band;
  const int u = (int)(rem % S.nunits);
  rem /= S.nunits;
  const int inner = (int)(rem % bsize);
  const int outer = (int)(rem / bsize);
  const int banded = (int)b * S.band + inner;
  c[0] = 0;
  c[1] = 0;
  c[2] = u % d.n[2];
  c[3] = u / d.n[2];
  c[4] = S.sweep ? banded : outer;
  c[5] = S.sweep ? outer : banded;
}

__host__ __device__ __forceinline__ long long dense_items(const Dims& d) {
  return (long long)d.n[2] * d.n[3] * d.n[4] * d.n[5];
}

// per-cell values of one item a thread keeps in registers
template <int MAXC>
struct CellRegs {
  float vx[MAXC], vy[MAXC], vr[4][MAXC], vl[4][MAXC], lam[MAXC], b0x[MAXC], b0y[MAXC];
};

__host__ __device__ __forceinline__ size_t pipe_smem(const Dims& d) {
  return 32 + 2 * desc_bytes<float>() + (size_t)(2 * RT_NPLANE + 2) * d.n[0] * d.n[1] * sizeof(float);
}

template <int NT, int MAXC>
__device__ __forceinline__ void pipe_prefetch(const StepArgs<float>& A, const int c[6], long long p0,
                                              unsigned long long ymul, CellRegs<MAXC>& R) {
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1], nxy = nx * ny;
  long long vloff[6];
#pragma unroll
  for (int a = 2; a < 6; a++) {
    if (c[a] > 0) {
      vloff[a] = p0 - d.s[a];
    } else {
      long long off = 0;
#pragma unroll
      for (int bb = 2; bb < 6; bb++) off += (long long)c[bb] * d.ps[a][bb];
      vloff[a] = off;
    }
  }
#pragma unroll
  for (int j = 0; j < MAXC; j++) {
    const int q = threadIdx.x + j * NT;
    if (q < nxy) {
      const int y = (int)(((unsigned long long)q * ymul) >> 32), x = q - y * nx;
      R.vx[j] = nx > 1 ? ld_stream(A.vel[0] + p0 + q) : 0.f;
      R.vy[j] = ny > 1 ? ld_stream(A.vel[1] + p0 + q) : 0.f;
      R.b0x[j] = (nx > 1 && x == 0) ? A.vlo[0][p0 / nx + y] : 0.f;
      R.b0y[j] = (ny > 1 && y == 0) ? A.vlo[1][p0 / ny + x] : 0.f;
#pragma unroll
      for (int a = 2; a < 6; a++) {
        const bool act = d.n[a] > 1;
        R.vr[a - 2][j] = act ? A.vel[a][p0 + q] : 0.f;
        R.vl[a - 2][j] = act ? (c[a] > 0 ? A.vel[a][vloff[a] + q] : A.vlo[a][vloff[a] + q]) : 0.f;
      }
      R.lam[j] = ld_stream(A.lam[0] + p0 + q);
    }
  }
}

// thread 0: descriptor of an item and its 17 bulk copies into a stage
__device__ __forceinline__ void pipe_issue(const StepArgs<float>& A, const int c[6], long long p0,
                                           float* sP, ItemDesc<float>* desc, uint64_t* bar) {
  const Dims& d = A.d;
  const int nxy = d.n[0] * d.n[1];
  const uint32_t pbytes = (uint32_t)(nxy * sizeof(float));
#pragma unroll
  for (int a = 2; a < 6; a++) {
    if (d.n[a] > 1) {
      desc->kcfl_r[a] = A.t32.hcfl[a][pidx(c[a] + 1)];
      desc->kinv_r[a] = A.t32.inv_d[a][pidx(c[a] + 1)];
      desc->kcfl_l[a] = A.t32.hcfl[a][pidx(c[a])];
    }
  }
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

template <int NT, int MAXC>
__global__ void __launch_bounds__(NT, 1) step_pipe_kernel(StepArgs<float> A, PlaneSched S,
                                                          long long nitems) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1], nz = d.n[2], nxy = nx * ny;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);   // bar[0], bar[1]
  ItemDesc<float>* desc = reinterpret_cast<ItemDesc<float>*>(smem_raw + 32);
  float* sP0 = reinterpret_cast<float*>(smem_raw + 32 + 2 * desc_bytes<float>());
  float* sFx = sP0 + (size_t)2 * RT_NPLANE * nxy;
  float* sFy = sFx + nxy;
  (void)nz;

  long long it = blockIdx.x;
  if (it >= nitems) return;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const unsigned long long ymul = ((1ull << 32) + (unsigned)nx - 1) / (unsigned)nx;

  // prologue: first item into stage 0
  int c[6];
  decode_dense(d, S, it, c);
  long long p0 = (long long)c[2] * d.s[2] + (long long)c[3] * d.s[3] + (long long)c[4] * d.s[4] +
                 (long long)c[5] * d.s[5];
  if (threadIdx.x == 0) pipe_issue(A, c, p0, sP0, &desc[0], &bar[0]);
  CellRegs<MAXC> cur, nxt;
  pipe_prefetch<NT, MAXC>(A, c, p0, ymul, cur);
  __syncthreads();   // desc[0] visible to all threads

  uint32_t phases = 0u;   // bit s: parity of the next completion of bar[s]
  for (int k = 0; it < nitems; k++, it += gridDim.x) {
    const int st = k & 1;
    float* sP = sP0 + (size_t)st * RT_NPLANE * nxy;
    // ---- look ahead: copies and register loads of the next item ----
    const long long itn = it + gridDim.x;
    int cn[6];
    long long p0n = 0;
    if (itn < nitems) {
      decode_dense(d, S, itn, cn);
      p0n = (long long)cn[2] * d.s[2] + (long long)cn[3] * d.s[3] + (long long)cn[4] * d.s[4] +
            (long long)cn[5] * d.s[5];
      if (threadIdx.x == 0)
        pipe_issue(A, cn, p0n, sP0 + (size_t)(st ^ 1) * RT_NPLANE * nxy, &desc[st ^ 1], &bar[st ^ 1]);
      pipe_prefetch<NT, MAXC>(A, cn, p0n, ymul, nxt);
    }
    // ---- this item's constants, then its planes ----
    FaceK<float> kr[6], kl[6];
#pragma unroll
    for (int a = 2; a < 6; a++) {
      kr[a].cfl = desc[st].kcfl_r[a];
      kr[a].inv = desc[st].kinv_r[a];
      kl[a].cfl = desc[st].kcfl_l[a];
      kl[a].inv = 0.f;
    }
    if (!mbar_wait_bounded(&bar[st], (phases >> st) & 1u, A.status)) {
      // let the look-ahead copies land before the CTA leaves (bounded)
      if (itn < nitems) mbar_wait_bounded(&bar[st ^ 1], (phases >> (st ^ 1)) & 1u, A.status);
      return;
    }
    phases ^= 1u << st;
    const float* sE = sP;
    // ---- x and y right-face fluxes, once per face ----
#pragma unroll
    for (int j = 0; j < MAXC; j++) {
      const int q = threadIdx.x + j * NT;
      if (q < nxy) {
        const int y = (int)(((unsigned long long)q * ymul) >> 32), x = q - y * nx;
        if (nx > 1) {
          const int r = y * nx;
          const int xm = x > 0 ? x - 1 : 0, xp = x + 1 < nx ? x + 1 : nx - 1,
                    xpp = x + 2 < nx ? x + 2 : nx - 1;
          sFx[q] = flux_fp32(cur.vx[j], A.t32.hcfl[0][pidx(x + 1)], sE[r + xm], sE[q], sE[r + xp], sE[r + xpp]);
        }
        if (ny > 1) {
          const int ym = y > 0 ? y - 1 : 0, yp = y + 1 < ny ? y + 1 : ny - 1,
                    ypp = y + 2 < ny ? y + 2 : ny - 1;
          sFy[q] = flux_fp32(cur.vy[j], A.t32.hcfl[1][pidx(y + 1)], sE[ym * nx + x], sE[q], sE[yp * nx + x],
                             sE[ypp * nx + x]);
        }
      }
    }
    __syncthreads();
    // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
#pragma unroll
    for (int j = 0; j < MAXC; j++) {
      const int q = threadIdx.x + j * NT;
      if (q < nxy) {
        const int y = (int)(((unsigned long long)q * ymul) >> 32), x = q - y * nx;
        const float e0 = sE[q];
        float dE = 0.f;
        if (nx > 1) {
          const float fl = x > 0 ? sFx[q - 1] : open_face0_flux<float>(cur.b0x[j], e0);
          dE -= (sFx[q] - fl) * A.t32.inv_d[0][pidx(x + 1)];
        }
        if (ny > 1) {
          const float fl = y > 0 ? sFy[q - nx] : open_face0_flux<float>(cur.b0y[j], e0);
          dE -= (sFy[q] - fl) * A.t32.inv_d[1][pidx(y + 1)];
        }
#pragma unroll
        for (int a = 2; a < 6; a++) {
          if (d.n[a] <= 1) continue;
          const float* sN = sP + (size_t)(1 + 4 * (a - 2)) * nxy;
          const float Em2 = sN[q], Em1 = sN[nxy + q], Ep1 = sN[2 * nxy + q], Ep2 = sN[3 * nxy + q];
          const float fr = flux_fp32(cur.vr[a - 2][j], kr[a].cfl, Em1, e0, Ep1, Ep2);
          const float fl = flux_fp32(cur.vl[a - 2][j], kl[a].cfl, Em2, Em1, e0, Ep1);
          dE -= (fr - fl) * kr[a].inv;
        }
        const float mf = e0 * cur.lam[j];
        st_stream(A.Enew + p0 + q, e0 + (float)A.dt * (dE - mf));
      }
    }
    __syncthreads();   // stage st, its descriptor and the flux planes are free again
    cur = nxt;
    p0 = p0n;
  }
}

}  // namespace rt
