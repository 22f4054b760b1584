// rt_step6.cuh -- warp-specialised, multi-stage TMA step (binary32 form).
//
// Work items are the (z,k) planes of (x,y) at one (l,m) in band order, as in
// rt_step5.cuh, walked by persistent CTAs (CTA b takes items b, b+G, ...).
// Each CTA has NT consumer threads and one producer warp:
//
//   producer (one warp): decodes the next items, writes their descriptors
//     (plane offset, left-face velocity bases, face-0 bases, grid constants)
//     into shared memory and issues the 17 bulk copies of E of each item into
//     a ring of `ns` stages (2..4, as many as fit).  Stage s is refilled only
//     after every consumer thread has released it (mbarrier empty[s]);
//     copies complete on full[s]; descriptors are published on dful[s].
//   consumers: thread t owns column x = t % nx and R consecutive rows
//     y0 = (t / nx) * R ...; it loads its velocities and growth rate of the
//     NEXT item into registers while it computes the current one.
//     x-face fluxes are computed once per face and passed to the right
//     neighbour with a warp shuffle (the first lane of a warp whose column is
//     not 0 computes its left face itself); y-face fluxes are computed once
//     per face inside the thread's rows, plus the face below the first row.
//
// No CTA-wide barrier runs inside the item loop: warps drift by up to `ns`
// items.  Every mbarrier wait is bounded (status bit 0, no hang).  The
// arithmetic (flux_fp32, axis order x,y,z,k,l,m, divergence and update
// expressions) is that of the other binary32 step kernels: results are
// bit-identical to them.
#pragma once
#include "rt_step5.cuh"

namespace rt {

#define RT_WS_MAXSTAGE 4

// per-item values the producer publishes for the consumers
struct WsDesc {
  long long p0;            // offset of cell (0,0) of the plane
  const float* vl[4];      // left-face velocities at (0,0), axes z..m
  const float* b0x;        // face-0 x velocities of the plane (index y)
  const float* b0y;        // face-0 y velocities of the plane (index x)
  float kcfl_r[4], kinv_r[4], kcfl_l[4];
  int member;              // batched form: index of the member the item belongs to
};

__host__ __device__ constexpr size_t ws_desc_bytes() { return (sizeof(WsDesc) + 15) / 16 * 16; }
__host__ __device__ constexpr size_t ws_head_bytes() { return 128 + RT_WS_MAXSTAGE * ws_desc_bytes(); }
__host__ __device__ __forceinline__ size_t ws_stage_bytes(const Dims& d) {
  return (size_t)RT_NPLANE * d.n[0] * d.n[1] * sizeof(float);
}
__host__ __device__ __forceinline__ size_t ws_smem(const Dims& d, int ns) {
  return ws_head_bytes() + (size_t)ns * ws_stage_bytes(d);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// bounded wait from any thread; raises status bit 0 on timeout
template <uint32_t LIMIT = RT_WAIT_LIMIT>
__device__ __forceinline__ bool ws_wait(uint64_t* bar, uint32_t parity, int* status) {
  for (uint32_t it = 0; it < LIMIT; it++)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(status, 1);
  return false;
}

// bounded wait of a whole warp: lane 0 polls, the result is broadcast, and
// __syncwarp orders the other lanes' later accesses after lane 0's acquire
template <uint32_t LIMIT = RT_WAIT_LIMIT>
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, int* status) {
  bool ok = true;
  if ((threadIdx.x & 31) == 0) ok = ws_wait<LIMIT>(bar, parity, status);
  ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
  __syncwarp();
  return ok;
}

// item -> (z,k,l,m) in band order without holes, 32-bit arithmetic (the
// launcher checks that the item count is below 2^31)
__device__ __forceinline__ void ws_decode(const Dims& d, const PlaneSched& S, unsigned item, int c[6]) {
  const unsigned nb_axis = S.sweep ? d.n[4] : d.n[5];
  const unsigned no_axis = S.sweep ? d.n[5] : d.n[4];
  const unsigned nunits = (unsigned)S.nunits;
  const unsigned per_full = nunits * no_axis * (unsigned)S.band;
  const unsigned b = item / per_full;
  unsigned rem = item - b * per_full;
  unsigned bsize = S.band;
  if ((b + 1) * (unsigned)S.band > nb_axis) bsize = nb_axis - b * (unsigned)S.band;
  const unsigned u = rem % nunits;
  rem /= nunits;
  const unsigned inner = rem % bsize;
  const unsigned outer = rem / bsize;
  const int banded = (int)(b * (unsigned)S.band + inner);
  c[0] = 0;
  c[1] = 0;
  c[2] = (int)(u % (unsigned)d.n[2]);
  c[3] = (int)(u / (unsigned)d.n[2]);
  c[4] = S.sweep ? banded : (int)outer;
  c[5] = S.sweep ? (int)outer : banded;
}

// column -> (k,l,m) in the band order of ws_decode with units = k only
// (PlaneSched made with gz = nz: nunits = nk); c[2] is left to the caller
__device__ __forceinline__ void ws_decode_col(const Dims& d, const PlaneSched& S, unsigned col, int c[6]) {
  const unsigned nb_axis = S.sweep ? d.n[4] : d.n[5];
  const unsigned no_axis = S.sweep ? d.n[5] : d.n[4];
  const unsigned nk = (unsigned)d.n[3];
  const unsigned per_full = nk * no_axis * (unsigned)S.band;
  const unsigned b = col / per_full;
  unsigned rem = col - b * per_full;
  unsigned bsize = S.band;
  if ((b + 1) * (unsigned)S.band > nb_axis) bsize = nb_axis - b * (unsigned)S.band;
  const unsigned k = rem % nk;
  rem /= nk;
  const unsigned inner = rem % bsize;
  const unsigned outer = rem / bsize;
  const int banded = (int)(b * (unsigned)S.band + inner);
  c[0] = 0;
  c[1] = 0;
  c[3] = (int)k;
  c[4] = S.sweep ? banded : (int)outer;
  c[5] = S.sweep ? (int)outer : banded;
}

// A CTA's sequence of work items.  Plain: items b, b+G, b+2G, ... of the
// band order (count = items).  Z-march: whole z columns -- columns b, b+G,
// ... of the band order over (k,l,m), each column's planes z = 0..nz-1 in
// turn (count = columns), so consecutive items of a CTA are z neighbours.
template <bool ZM>
struct ItemWalk {
  long long it;   // item (plain) or column (z-march)
  int z;          // z-march: plane within the column
  __device__ __forceinline__ void start() { it = blockIdx.x; z = 0; }
  __device__ __forceinline__ bool valid(long long count) const { return it < count; }
  __device__ __forceinline__ void next(int nz) {
    if (ZM) {
      if (++z == nz) { z = 0; it += gridDim.x; }
    } else {
      it += gridDim.x;
    }
  }
  __device__ __forceinline__ void decode(const Dims& d, const PlaneSched& S, int c[6]) const {
    if (ZM) {
      ws_decode_col(d, S, (unsigned)it, c);
      c[2] = z;
    } else {
      ws_decode(d, S, (unsigned)it, c);
    }
  }
};

// producer: the 32 lanes of the last warp.  All lanes decode the next item
// and work out their part while the stage is still in use; once it is free,
// lanes 0 and 2..5 write the descriptor, lane 0 arms the stage, and lane
// j < 17 issues the bulk copy of plane j (0 = centre, 1 + 4(a-2) + i =
// neighbour i of axis a).
template <bool ZM = false>
__device__ __forceinline__ void ws_produce(const StepArgs<float>& A, const PlaneSched& S, long long nitems,
                                           int ns, uint64_t* full, uint64_t* empty, uint64_t* dful,
                                           WsDesc* desc, float* stage0) {
  const Dims& d = A.d;
  const int lane = threadIdx.x & 31;
  const int nxy = d.n[0] * d.n[1];
  const uint32_t pbytes = (uint32_t)(nxy * sizeof(float));
  uint32_t nplanes = 1;
  for (int a = 2; a < 6; a++)
    if (d.n[a] > 1) nplanes += 4;
  int s = 0;
  uint32_t rnd = 0;   // completed passes over the ring
  long long issued = 0;
  ItemWalk<ZM> w;
  for (w.start(); w.valid(nitems); w.next(d.n[2])) {
    // ---- before the stage is free: decode, the lane's copy and its share
    // of the descriptor (lanes 2..5: axis `lane`; lane 0: offsets) ----
    int c[6];
    w.decode(d, S, c);
    const long long p0 = (long long)c[2] * d.s[2] + (long long)c[3] * d.s[3] + (long long)c[4] * d.s[4] +
                         (long long)c[5] * d.s[5];
    const float* vlp = nullptr;
    float kr = 0.f, ki = 0.f, kl = 0.f;
    if (lane >= 2 && lane < 6) {
      const int a = lane;
      if (c[a] > 0) {
        vlp = A.vel[a] + (p0 - d.s[a]);
      } else {
        long long off = 0;
#pragma unroll
        for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[a][b];
        vlp = A.vlo[a] + off;
      }
      if (d.n[a] > 1) {
        kr = A.t32.hcfl[a][pidx(c[a] + 1)];
        ki = A.t32.inv_d[a][pidx(c[a] + 1)];
        kl = A.t32.hcfl[a][pidx(c[a])];
      }
    }
    long long o0 = 0, o1 = 0;
    if (lane == 0) {
#pragma unroll
      for (int b = 2; b < 6; b++) {
        o0 += (long long)c[b] * d.ps[0][b];
        o1 += (long long)c[b] * d.ps[1][b];
      }
    }
    // z-march past the column's first plane: the left z face flux is carried
    // by the consumers, so the z-2 plane (lane 1) is not needed
    const bool skip_zm2 = ZM && w.z > 0;
    const float* src = nullptr;
    if (lane < RT_NPLANE) {
      long long off = p0;
      bool go = true;
      if (lane > 0) {
        const int a = 2 + (lane - 1) / 4, i = (lane - 1) % 4;
        go = d.n[a] > 1 && !(lane == 1 && skip_zm2);
        if (go) off = nb_plane(d, c, a, i < 2 ? i - 2 : i - 1);
      }
      if (go) src = A.E + off;
    }
    // ---- stage s is free once every consumer thread released its previous item ----
    if (rnd > 0 && !warp_wait(&empty[s], (rnd - 1) & 1u, A.status)) break;
    WsDesc& D = desc[s];
    if (lane >= 2 && lane < 6) {
      D.vl[lane - 2] = vlp;
      D.kcfl_r[lane - 2] = kr;
      D.kinv_r[lane - 2] = ki;
      D.kcfl_l[lane - 2] = kl;
    }
    if (lane == 0) {
      D.p0 = p0;
      D.b0x = A.vlo[0] + o0;
      D.b0y = A.vlo[1] + o1;
    }
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&dful[s]);   // release: the descriptor (ordered by the __syncwarp) is visible to waiters
      mbar_arrive_expect_tx(&full[s], (nplanes - (skip_zm2 && d.n[2] > 1 ? 1u : 0u)) * pbytes);
    }
    __syncwarp();
    if (src) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_g2s(stage0 + (size_t)s * RT_NPLANE * nxy + (size_t)lane * nxy, src, pbytes, &full[s]);
    }
    issued++;
    if (++s == ns) { s = 0; rnd++; }
  }
  // copies still in flight (only after a timeout) land before the CTA can
  // leave: wait, bounded, for the last completion of every used stage
  for (int j = 0; j < ns; j++) {
    const long long uses = issued / ns + (j < issued % ns ? 1 : 0);
    if (uses == 0) continue;
    for (uint32_t w = 0; w < RT_WAIT_LIMIT; w++)
      if (mbar_try_wait(&full[j], (uint32_t)((uses - 1) & 1))) break;
  }
}

// a consumer thread's per-item values
template <int R>
struct WsRegs {
  float vx[R], vy[R], vr[4][R], vl[4][R], lam[R];
  float xl[R];   // x == 0: face-0 velocity; first lane with x > 0: velocity of face x
  float yb;      // y0 == 0: face-0 velocity; else velocity of face y0 (below row y0)
};

template <int R>
__device__ __forceinline__ void ws_load(const StepArgs<float>& A, const WsDesc& D, int x, int y0,
                                        const int yrow[R], int lane, WsRegs<R>& G) {
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1];
  const long long p0 = D.p0;
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int q = yrow[r] * nx + x;
    const long long o = p0 + q;
    G.vx[r] = ld_stream(A.vel[0] + o);
    G.vy[r] = ld_stream(A.vel[1] + o);
#pragma unroll
    for (int a = 2; a < 6; a++) {
      const bool act = d.n[a] > 1;
      G.vr[a - 2][r] = act ? A.vel[a][o] : 0.f;
      G.vl[a - 2][r] = act ? D.vl[a - 2][q] : 0.f;
    }
    G.lam[r] = ld_stream(A.lam[0] + o);
    G.xl[r] = x == 0 ? D.b0x[yrow[r]] : (lane == 0 ? A.vel[0][o - 1] : 0.f);
  }
  G.yb = y0 == 0 ? D.b0y[x] : (y0 < ny ? A.vel[1][p0 + (long long)(y0 - 1) * nx + x] : 0.f);
}

template <int NT, int R>
struct WsMinBlocks { static constexpr int value = (NT <= 256 && R <= 2) ? 2 : 1; };

// PF = 1: the next item's velocities are loaded into registers while the
// current item is computed; PF = 0: they are loaded at the start of the item
// (fewer registers; the other warps cover the latency)
template <int NT, int R, int PF>
__global__ void __launch_bounds__(NT + 32, (WsMinBlocks<NT, R>::value))
    step_ws_kernel(StepArgs<float> A, PlaneSched S, long long nitems, int ns) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + RT_WS_MAXSTAGE;
  uint64_t* dful = empty + RT_WS_MAXSTAGE;
  WsDesc* desc = reinterpret_cast<WsDesc*>(smem_raw + 128);
  float* stage0 = reinterpret_cast<float*>(smem_raw + ws_head_bytes());
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1], nxy = nx * ny;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ns; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NT);
      mbar_init(&dful[s], 1);
    }
    fence_mbar_init();
  }
  __syncthreads();
  if (blockIdx.x >= nitems) return;

  if (threadIdx.x >= NT) {
    ws_produce(A, S, nitems, ns, full, empty, dful, desc, stage0);
    return;
  }

  // ---- consumer: the thread's column and rows, fixed for every item ----
  const int t = threadIdx.x, lane = t & 31;
  const int x = t % nx, y0 = (t / nx) * R;
  int yrow[R];
#pragma unroll
  for (int r = 0; r < R; r++) yrow[r] = y0 + r < ny ? y0 + r : ny - 1;
  const int xm = x > 0 ? x - 1 : 0, xp = x + 1 < nx ? x + 1 : nx - 1, xpp = x + 2 < nx ? x + 2 : nx - 1,
            xmm = x > 1 ? x - 2 : 0;
  const float cx = A.t32.hcfl[0][pidx(x + 1)], ix = A.t32.inv_d[0][pidx(x + 1)];
  const float cxl = A.t32.hcfl[0][pidx(x)];
  float cy[R], iy[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    cy[r] = A.t32.hcfl[1][pidx(yrow[r] + 1)];
    iy[r] = A.t32.inv_d[1][pidx(yrow[r] + 1)];
  }
  const float cyb = A.t32.hcfl[1][pidx(y0 < ny ? y0 : ny - 1)];
  // smem offsets of the column's rows y0-2 .. y0+R+1 (clamped)
  int ecol[R + 4];
#pragma unroll
  for (int j = 0; j < R + 4; j++) {
    int yy = y0 + j - 2;
    yy = yy < 0 ? 0 : (yy > ny - 1 ? ny - 1 : yy);
    ecol[j] = yy * nx + x;
  }
  const float dt = (float)A.dt;

  WsRegs<R> cur, nxt;
  if (PF) {
    if (!ws_wait(&dful[0], 0, A.status)) return;
    ws_load<R>(A, desc[0], x, y0, yrow, lane, cur);
  }

  int s = 0;
  uint32_t par = 0;
  for (long long it = blockIdx.x; it < nitems; it += gridDim.x) {
    int sn = s + 1;
    uint32_t parn = par;
    if (sn == ns) { sn = 0; parn ^= 1u; }
    if (PF) {
      // ---- look ahead: the next item's registers ----
      if (it + gridDim.x < nitems) {
        if (!ws_wait(&dful[sn], parn, A.status)) return;
        ws_load<R>(A, desc[sn], x, y0, yrow, lane, nxt);
      }
    } else {
      if (!ws_wait(&dful[s], par, A.status)) return;
      ws_load<R>(A, desc[s], x, y0, yrow, lane, cur);
    }
    const WsDesc& D = desc[s];
    const long long p0 = D.p0;
    float kcr[4], kir[4], kcl[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      kcr[a] = D.kcfl_r[a];
      kir[a] = D.kinv_r[a];
      kcl[a] = D.kcfl_l[a];
    }
    if (!ws_wait(&full[s], par, A.status)) return;
    const float* sE = stage0 + (size_t)s * RT_NPLANE * nxy;

    float ec[R + 4];
#pragma unroll
    for (int j = 0; j < R + 4; j++) ec[j] = sE[ecol[j]];
    // ---- x faces: right face here, left face from the lane to the left ----
    float fxr[R], fxl[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int rb = yrow[r] * nx;
      fxr[r] = flux_fp32(cur.vx[r], cx, sE[rb + xm], ec[r + 2], sE[rb + xp], sE[rb + xpp]);
    }
#pragma unroll
    for (int r = 0; r < R; r++) fxl[r] = __shfl_up_sync(0xffffffffu, fxr[r], 1);
    if (x == 0) {
#pragma unroll
      for (int r = 0; r < R; r++) fxl[r] = open_face0_flux<float>(cur.xl[r], ec[r + 2]);
    } else if (lane == 0) {
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int rb = yrow[r] * nx;
        fxl[r] = flux_fp32(cur.xl[r], cxl, sE[rb + xmm], sE[rb + x - 1], ec[r + 2], sE[rb + xp]);
      }
    }
    // ---- y faces: below the first row, then above every row ----
    float fy[R + 1];
    fy[0] = y0 == 0 ? open_face0_flux<float>(cur.yb, ec[2])
                    : flux_fp32(cur.yb, cyb, ec[0], ec[1], ec[2], ec[3]);
#pragma unroll
    for (int r = 0; r < R; r++) fy[r + 1] = flux_fp32(cur.vy[r], cy[r], ec[r + 1], ec[r + 2], ec[r + 3], ec[r + 4]);
    // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float e0 = ec[r + 2];
      const int q = yrow[r] * nx + x;
      float dE = 0.f;
      dE -= (fxr[r] - fxl[r]) * ix;
      dE -= (fy[r + 1] - fy[r]) * iy[r];
#pragma unroll
      for (int a = 2; a < 6; a++) {
        if (d.n[a] <= 1) continue;
        const float* sN = sE + (size_t)(1 + 4 * (a - 2)) * nxy + q;
        const float Em2 = sN[0], Em1 = sN[nxy], Ep1 = sN[2 * nxy], Ep2 = sN[3 * nxy];
        const float fr = flux_fp32(cur.vr[a - 2][r], kcr[a - 2], Em1, e0, Ep1, Ep2);
        const float fl = flux_fp32(cur.vl[a - 2][r], kcl[a - 2], Em2, Em1, e0, Ep1);
        dE -= (fr - fl) * kir[a - 2];
      }
      const float mf = e0 * cur.lam[r];
      if (y0 + r < ny) st_stream(A.Enew + p0 + q, e0 + dt * (dE - mf));
    }
    // ---- release the stage: this thread's reads of it and of its
    // descriptor are done (every consumer thread arrives) ----
    mbar_arrive(&empty[s]);
    if (PF) cur = nxt;
    s = sn;
    par = parn;
  }
}

}  // namespace rt
