// rt_step8.cuh -- warp-specialised step with every operand staged by TMA
// (binary32 form).
//
// As rt_step7.cuh (producer warp, ring of stages, 2-wide cell blocks,
// shuffled x faces, register-chained y faces), but a stage holds everything
// one item reads: the 17 planes of E, the 11 planes of face velocities and
// growth rate (x and y right faces, right and left faces of z,k,l,m, the
// combined rate) and the two face-0 rows of the plane (x faces by y, y
// faces by x).  The consumers issue no global load at all: their operands
// are in shared memory when the stage's mbarrier completes, so no warp
// waits on HBM latency; the producer runs up to ns-1 items ahead.
// Requires nx and ny multiples of 4 (16-byte rows of the face-0 copies).
// Results are bit-identical to the other binary32 step kernels.
#pragma once
#include "rt_step7.cuh"

namespace rt {

// stage layout (floats): E planes [0,17), velocity/rate planes [17,28),
// face-0 x row (ny), face-0 y row (nx)
#define RT_W3_EPL 17
#define RT_W3_NPL 28
#define RT_W3_VX 17
#define RT_W3_VY 18
#define RT_W3_VR 19   // + a-2
#define RT_W3_VL 23   // + a-2
#define RT_W3_LAM 27

__host__ __device__ __forceinline__ size_t w3_stage_floats(const Dims& d) {
  return (size_t)RT_W3_NPL * d.n[0] * d.n[1] + d.n[1] + d.n[0];
}
__host__ __device__ __forceinline__ size_t w3_smem(const Dims& d, int ns) {
  return ws_head_bytes() + (size_t)ns * w3_stage_floats(d) * sizeof(float);
}

// copy `lane` of an item (0..29): what it holds and where it lands.  This
// is the lane map w3_prepare writes out inline; tests/native checks it (bytes
// against w3_tx_bytes, bounds, overlap, alignment, coverage of every plane
// the consumers read).
struct W3Copy {
  bool valid;      // false: the axis is collapsed (no copy)
  int kind;        // 0 E plane, 1 right-face velocities, 2 left-face velocities, 3 x/y velocity or rate, 4 face-0 row
  int a, i;        // axis and neighbour index (kind 0), axis (1, 2), which (3: 0 x, 1 y, 2 rate; 4: 0 x, 1 y)
  long long dst;   // stage offset, floats
  unsigned bytes;
};
__host__ __device__ __forceinline__ W3Copy w3_copy(const Dims& d, int lane) {
  const int nx = d.n[0], ny = d.n[1];
  const long long nxy = (long long)nx * ny;
  W3Copy c{false, 0, 0, 0, 0, (unsigned)(nxy * sizeof(float))};
  if (lane < RT_NPLANE) {
    c.kind = 0;
    if (lane == 0) {
      c.valid = true;
    } else {
      c.a = 2 + (lane - 1) / 4;
      c.i = (lane - 1) % 4;
      c.valid = d.n[c.a] > 1;
    }
    c.dst = lane * nxy;
  } else if (lane < 25) {
    const bool right = lane < 21;
    c.kind = right ? 1 : 2;
    c.a = 2 + (right ? lane - 17 : lane - 21);
    c.valid = d.n[c.a] > 1;
    c.dst = (long long)((right ? RT_W3_VR : RT_W3_VL) + c.a - 2) * nxy;
  } else if (lane < 28) {
    c.kind = 3;
    c.i = lane - 25;
    c.valid = true;
    c.dst = (long long)(c.i == 0 ? RT_W3_VX : (c.i == 1 ? RT_W3_VY : RT_W3_LAM)) * nxy;
  } else if (lane < 30) {
    c.kind = 4;
    c.i = lane - 28;
    c.valid = true;
    c.dst = (long long)RT_W3_NPL * nxy + (c.i == 0 ? 0 : ny);
    c.bytes = (unsigned)((c.i == 0 ? ny : nx) * sizeof(float));
  }
  return c;
}
// bytes the item's mbarrier expects: the sum of the valid copies' bytes
__host__ __device__ __forceinline__ unsigned w3_tx_bytes(const Dims& d) {
  unsigned nact = 0;
  for (int a = 2; a < 6; a++)
    if (d.n[a] > 1) nact++;
  const unsigned pbytes = (unsigned)((long long)d.n[0] * d.n[1] * sizeof(float));
  return (1 + 6 * nact + 3) * pbytes + (unsigned)((d.n[0] + d.n[1]) * sizeof(float));
}

// One item into a stage, by the 32 lanes of the producer warp, in two
// parts.  w3_prepare does everything that does not touch the stage: all
// lanes decode the item, lane j works out copy j (the lane map of w3_copy:
// 0..16 the E planes, 17..20 right and 21..24 left face velocities of z..m,
// 25 x and 26 y velocities, 27 the rate, 28 and 29 the face-0 rows) and
// lanes 2..5 load the grid constants of axis `lane`.  The producer runs it
// while the stage is still in use; once the stage is free, w3_commit
// publishes the descriptor, arms the stage's mbarrier and issues the copies
// (the ring has only two stages for 32x32 planes, so the producer's latency
// after the wait shows in the step time).
struct W3Prep {
  long long p0;
  const float* src;   // null: no copy on this lane
  float* dst;
  uint32_t bytes;
  float kr, kh, ko, kl;   // lanes 2..5: constants of axis `lane`
};
__device__ __forceinline__ W3Prep w3_prepare(const StepArgs<float>& A, const PlaneSched& S, long long li,
                                             float* sP) {
  const Dims& d = A.d;
  const int lane = threadIdx.x & 31;
  int c[6];
  ws_decode(d, S, (unsigned)li, c);
  W3Prep P;
  P.p0 = (long long)c[2] * d.s[2] + (long long)c[3] * d.s[3] + (long long)c[4] * d.s[4] +
         (long long)c[5] * d.s[5];
  const long long p0 = P.p0;
  P.kr = P.kh = P.ko = P.kl = 0.f;
  if (lane >= 2 && lane < 6 && d.n[lane] > 1) {
    P.kr = A.t32.hcfl[lane][pidx(c[lane] + 1)];
    P.kh = A.t32.chi[lane][pidx(c[lane] + 1)];
    P.ko = A.t32.clo[lane][pidx(c[lane] + 1)];
    P.kl = A.t32.hcfl[lane][pidx(c[lane])];
  }
  const int nx = d.n[0], ny = d.n[1];
  const long long nxy = (long long)nx * ny;
  P.src = nullptr;
  P.dst = nullptr;
  P.bytes = (uint32_t)(nxy * sizeof(float));
  if (lane < RT_NPLANE) {
    long long off = p0;
    bool go = true;
    if (lane > 0) {
      const int a = 2 + (lane - 1) / 4, i = (lane - 1) % 4;
      go = d.n[a] > 1;
      if (go) off = nb_plane(d, c, a, i < 2 ? i - 2 : i - 1);
    }
    if (go) { P.src = A.E + off; P.dst = sP + lane * nxy; }
  } else if (lane < 25) {
    const bool right = lane < 21;
    const int a = 2 + (right ? lane - 17 : lane - 21);
    if (d.n[a] > 1) {
      if (right) {
        P.src = A.vel[a] + p0;
      } else if (c[a] > 0) {
        P.src = A.vel[a] + (p0 - d.s[a]);
      } else {
        long long off = 0;
#pragma unroll
        for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[a][b];
        P.src = A.vlo[a] + off;
      }
      P.dst = sP + ((right ? RT_W3_VR : RT_W3_VL) + a - 2) * nxy;
    }
  } else if (lane < 28) {
    const int which = lane - 25;   // x velocity, y velocity, rate
    P.src = (which == 0 ? A.vel[0] : (which == 1 ? A.vel[1] : A.lam[0])) + p0;
    P.dst = sP + (which == 0 ? RT_W3_VX : (which == 1 ? RT_W3_VY : RT_W3_LAM)) * nxy;
  } else if (lane < 30) {
    long long off = 0;
    const int a = lane - 28;   // face-0 x row (by y), face-0 y row (by x)
#pragma unroll
    for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[a][b];
    P.src = A.vlo[a] + off;
    P.dst = sP + RT_W3_NPL * nxy + (a == 0 ? 0 : ny);
    P.bytes = (uint32_t)((a == 0 ? ny : nx) * sizeof(float));
  }
  return P;
}

__device__ __forceinline__ void w3_commit(const W3Prep& P, const Dims& d, int member, WsDesc* D,
                                          uint64_t* fullb, uint64_t* dfulb) {
  const int lane = threadIdx.x & 31;
  if (lane >= 2 && lane < 6) {
    D->kcfl_r[lane - 2] = P.kr;
    D->kch_r[lane - 2] = P.kh;
    D->kcl_r[lane - 2] = P.ko;
    D->kcfl_l[lane - 2] = P.kl;
  }
  if (lane == 0) {
    D->p0 = P.p0;
    D->member = member;
  }
  __syncwarp();
  if (lane == 0) {
    mbar_arrive(dfulb);   // release: lanes 0..5's descriptor writes (ordered by the __syncwarp)
    mbar_arrive_expect_tx(fullb, w3_tx_bytes(d));
  }
  __syncwarp();
  if (P.src) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bulk_g2s(P.dst, P.src, P.bytes, fullb);
  }
}

// producer warp after its last item: copies still in flight (only after a
// timeout) land before the CTA can leave (bounded waits)
__device__ __forceinline__ void ws_drain(uint64_t* full, int ns, long long issued) {
  for (int j = 0; j < ns; j++) {
    const long long uses = issued / ns + (j < issued % ns ? 1 : 0);
    if (uses == 0) continue;
    for (uint32_t w = 0; w < RT_WAIT_LIMIT; w++)
      if (mbar_try_wait(&full[j], (uint32_t)((uses - 1) & 1))) break;
  }
}

// a consumer thread's 2 x R block of an nx x ny plane and the constants it
// needs, fixed for every item of one field
template <int R>
struct W3Geom {
  int nx, ny, nxy, x0, y0, xm, xmm, yb_off;
  bool has_right;
  int yrow[R], ecol[R + 4];
  float cxa, cxb, hxa, hxb, oxa, oxb, cxl, cyb, dthi, dtlo;
  float cy[R], hy[R], oy[R];
  unsigned seed;   // this step's rounding seed of the field
};

template <int R>
__device__ __forceinline__ void w3_geom(const StepArgs<float>& A, int t, W3Geom<R>& g) {
  const int nx = A.d.n[0], ny = A.d.n[1];
  g.nx = nx;
  g.ny = ny;
  g.nxy = nx * ny;
  const int hx = nx >> 1;
  g.x0 = 2 * (t % hx);
  g.y0 = (t / hx) * R;
  const int x0 = g.x0, y0 = g.y0;
#pragma unroll
  for (int r = 0; r < R; r++) g.yrow[r] = y0 + r < ny ? y0 + r : ny - 1;
  g.xm = x0 > 0 ? x0 - 1 : 0;
  g.xmm = x0 > 1 ? x0 - 2 : 0;
  g.has_right = x0 + 2 < nx;
  g.cxa = A.t32.hcfl[0][pidx(x0 + 1)];
  g.cxb = A.t32.hcfl[0][pidx(x0 + 2)];
  g.hxa = A.t32.chi[0][pidx(x0 + 1)];
  g.hxb = A.t32.chi[0][pidx(x0 + 2)];
  g.oxa = A.t32.clo[0][pidx(x0 + 1)];
  g.oxb = A.t32.clo[0][pidx(x0 + 2)];
  g.cxl = A.t32.hcfl[0][pidx(x0)];
#pragma unroll
  for (int r = 0; r < R; r++) {
    g.cy[r] = A.t32.hcfl[1][pidx(g.yrow[r] + 1)];
    g.hy[r] = A.t32.chi[1][pidx(g.yrow[r] + 1)];
    g.oy[r] = A.t32.clo[1][pidx(g.yrow[r] + 1)];
  }
  g.cyb = A.t32.hcfl[1][pidx(y0 < ny ? y0 : ny - 1)];
#pragma unroll
  for (int j = 0; j < R + 4; j++) {
    int yy = y0 + j - 2;
    yy = yy < 0 ? 0 : (yy > ny - 1 ? ny - 1 : yy);
    g.ecol[j] = yy * nx + x0;
  }
  // smem offset of the y velocities below the block (row y0-1) or of the
  // face-0 y row (y0 == 0)
  g.yb_off = y0 == 0 ? RT_W3_NPL * g.nxy + ny + x0
                     : RT_W3_VY * g.nxy + ((y0 - 1 < ny - 1 ? y0 - 1 : ny - 1)) * nx + x0;
  g.dthi = A.dthi;
  g.dtlo = A.dtlo;
  g.seed = *A.seed_in;
}

// one item of one consumer thread from a filled stage
template <int R>
__device__ __forceinline__ void w3_item(const StepArgs<float>& A, const W3Geom<R>& g, const WsDesc& D,
                                        const float* sE, int lane) {
  const Dims& d = A.d;
  const int nx = g.nx, ny = g.ny, nxy = g.nxy, x0 = g.x0, y0 = g.y0;
  const long long p0 = D.p0;
  float kcr[4], khr[4], kor[4], kcl[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    kcr[a] = D.kcfl_r[a];
    khr[a] = D.kch_r[a];
    kor[a] = D.kcl_r[a];
    kcl[a] = D.kcfl_l[a];
  }
  float2 ec[R + 4];
#pragma unroll
  for (int j = 0; j < R + 4; j++) ec[j] = ld2(sE + g.ecol[j]);
  // ---- x faces ----
  float fxa[R], fxb[R], fxl[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int rb = g.yrow[r] * nx;
    const float2 e01 = ec[r + 2];
    const float em = sE[rb + g.xm];
    const float2 e23 = g.has_right ? ld2(sE + rb + x0 + 2) : make_float2(e01.y, e01.y);
    const float2 vx = ld2(sE + RT_W3_VX * nxy + rb + x0);
    fxa[r] = flux_fp32(vx.x, g.cxa, em, e01.x, e01.y, e23.x);
    fxb[r] = flux_fp32(vx.y, g.cxb, e01.x, e01.y, e23.x, e23.y);
  }
#pragma unroll
  for (int r = 0; r < R; r++) fxl[r] = __shfl_up_sync(0xffffffffu, fxb[r], 1);
  if (x0 == 0) {
#pragma unroll
    for (int r = 0; r < R; r++) fxl[r] = open_face0_flux<float>(sE[RT_W3_NPL * nxy + g.yrow[r]], ec[r + 2].x);
  } else if (lane == 0) {
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int rb = g.yrow[r] * nx;
      fxl[r] = flux_fp32(sE[RT_W3_VX * nxy + rb + x0 - 1], g.cxl, sE[rb + g.xmm], sE[rb + x0 - 1], ec[r + 2].x,
                         ec[r + 2].y);
    }
  }
  // ---- y faces (both columns) ----
  float2 fy[R + 1];
  {
    const float2 vb = ld2(sE + g.yb_off);
    if (y0 == 0) {
      fy[0].x = open_face0_flux<float>(vb.x, ec[2].x);
      fy[0].y = open_face0_flux<float>(vb.y, ec[2].y);
    } else {
      fy[0].x = flux_fp32(vb.x, g.cyb, ec[0].x, ec[1].x, ec[2].x, ec[3].x);
      fy[0].y = flux_fp32(vb.y, g.cyb, ec[0].y, ec[1].y, ec[2].y, ec[3].y);
    }
  }
#pragma unroll
  for (int r = 0; r < R; r++) {
    const float2 vy = ld2(sE + RT_W3_VY * nxy + g.yrow[r] * nx + x0);
    fy[r + 1].x = flux_fp32(vy.x, g.cy[r], ec[r + 1].x, ec[r + 2].x, ec[r + 3].x, ec[r + 4].x);
    fy[r + 1].y = flux_fp32(vy.y, g.cy[r], ec[r + 1].y, ec[r + 2].y, ec[r + 3].y, ec[r + 4].y);
  }
  // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
#pragma unroll
  for (int r = 0; r < R; r++) {
    const float2 e0 = ec[r + 2];
    const int q = g.yrow[r] * nx + x0;
    float dEa = div32(0.f, fxa[r], fxl[r], g.hxa, g.oxa);
    float dEb = div32(0.f, fxb[r], fxa[r], g.hxb, g.oxb);
    dEa = div32(dEa, fy[r + 1].x, fy[r].x, g.hy[r], g.oy[r]);
    dEb = div32(dEb, fy[r + 1].y, fy[r].y, g.hy[r], g.oy[r]);
#pragma unroll
    for (int a = 2; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const float* sN = sE + (size_t)(1 + 4 * (a - 2)) * nxy + q;
      const float2 Em2 = ld2(sN), Em1 = ld2(sN + nxy), Ep1 = ld2(sN + 2 * nxy), Ep2 = ld2(sN + 3 * nxy);
      const float2 vr = ld2(sE + (RT_W3_VR + a - 2) * nxy + q), vl = ld2(sE + (RT_W3_VL + a - 2) * nxy + q);
      const float fra = flux_fp32(vr.x, kcr[a - 2], Em1.x, e0.x, Ep1.x, Ep2.x);
      const float fla = flux_fp32(vl.x, kcl[a - 2], Em2.x, Em1.x, e0.x, Ep1.x);
      dEa = div32(dEa, fra, fla, khr[a - 2], kor[a - 2]);
      const float frb = flux_fp32(vr.y, kcr[a - 2], Em1.y, e0.y, Ep1.y, Ep2.y);
      const float flb = flux_fp32(vl.y, kcl[a - 2], Em2.y, Em1.y, e0.y, Ep1.y);
      dEb = div32(dEb, frb, flb, khr[a - 2], kor[a - 2]);
    }
    const float2 lam = ld2(sE + RT_W3_LAM * nxy + q);
    const float mfa = e0.x * lam.x, mfb = e0.y * lam.y;
    if (y0 + r < ny)
      st2_stream(A.Enew + p0 + q, make_float2(upd32(e0.x, dEa, mfa, g.dthi, g.dtlo, sr_bits(p0 + q, g.seed)),
                                              upd32(e0.y, dEb, mfb, g.dthi, g.dtlo, sr_bits(p0 + q + 1, g.seed))));
  }
}

template <int NT, int R>
__global__ void __launch_bounds__(NT + 32, 1) step_w3_kernel(StepArgs<float> A, PlaneSched S, long long nitems,
                                                            int ns) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + RT_WS_MAXSTAGE;
  uint64_t* dful = empty + RT_WS_MAXSTAGE;
  WsDesc* desc = reinterpret_cast<WsDesc*>(smem_raw + 128);
  float* stage0 = reinterpret_cast<float*>(smem_raw + ws_head_bytes());
  const size_t sfl = w3_stage_floats(A.d);

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
    // ---- producer warp ----
    int s = 0;
    uint32_t rnd = 0;
    long long issued = 0;
    for (long long it = blockIdx.x; it < nitems; it += gridDim.x) {
      const W3Prep P = w3_prepare(A, S, it, stage0 + (size_t)s * sfl);
      if (rnd > 0 && !warp_wait(&empty[s], (rnd - 1) & 1u, A.status)) break;
      w3_commit(P, A.d, 0, &desc[s], &full[s], &dful[s]);
      issued++;
      if (++s == ns) { s = 0; rnd++; }
    }
    ws_drain(full, ns, issued);
    return;
  }

  // ---- consumers ----
  const int lane = threadIdx.x & 31;
  W3Geom<R> g;
  w3_geom<R>(A, threadIdx.x, g);
  advance_seed(A.seed_in, A.seed_out, blockIdx.x);   // CTA 0 takes item 0
  int s = 0;
  uint32_t par = 0;
  for (long long it = blockIdx.x; it < nitems; it += gridDim.x) {
    if (!ws_wait(&dful[s], par, A.status)) return;
    if (!ws_wait(&full[s], par, A.status)) return;
    w3_item<R>(A, g, desc[s], stage0 + (size_t)s * sfl, lane);
    mbar_arrive(&empty[s]);
    if (++s == ns) { s = 0; par ^= 1u; }
  }
}

// Batched form: the members' items one after the other (member j owns
// items [first[j], first[j+1]) of its own band order), walked by persistent
// CTAs; stages are sized for the largest member plane (stage_floats).  The
// consumers recompute their block geometry when the member changes.
// The CTA's part as a device function: bid / nb stand for the block index
// and the grid size, so a kernel can give a share of its CTAs to this class
// (batch_fused_kernel, rt_step11.cuh).
template <int NT, int R>
__device__ __forceinline__ void batch_w3_cta(const BatchMember<float>* __restrict__ mem,
                                             const long long* __restrict__ first, int nmem, int ns,
                                             long long stage_floats, long long bid, long long nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + RT_WS_MAXSTAGE;
  uint64_t* dful = empty + RT_WS_MAXSTAGE;
  WsDesc* desc = reinterpret_cast<WsDesc*>(smem_raw + 128);
  float* stage0 = reinterpret_cast<float*>(smem_raw + ws_head_bytes());
  const long long nitems = first[nmem];
  int* status = mem[0].A.status;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ns; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NT);
      mbar_init(&dful[s], 1);
    }
    fence_mbar_init();
  }
  __syncthreads();
  if (bid >= nitems) return;

  if (threadIdx.x >= NT) {
    int s = 0, j = 0;
    uint32_t rnd = 0;
    long long issued = 0;
    for (long long it = bid; it < nitems; it += nb) {
      while (it >= first[j + 1]) j++;
      const W3Prep P = w3_prepare(mem[j].A, mem[j].S, it - first[j], stage0 + (size_t)s * stage_floats);
      if (rnd > 0 && !warp_wait(&empty[s], (rnd - 1) & 1u, status)) break;
      w3_commit(P, mem[j].A.d, j, &desc[s], &full[s], &dful[s]);
      issued++;
      if (++s == ns) { s = 0; rnd++; }
    }
    ws_drain(full, ns, issued);
    return;
  }

  const int lane = threadIdx.x & 31;
  W3Geom<R> g;
  int jc = -1;
  int s = 0;
  uint32_t par = 0;
  for (long long it = bid; it < nitems; it += nb) {
    if (!ws_wait(&dful[s], par, status)) return;
    const int j = desc[s].member;
    const StepArgs<float>& A = mem[j].A;
    if (j != jc) {
      w3_geom<R>(A, threadIdx.x, g);
      jc = j;
    }
    advance_seed(A.seed_in, A.seed_out, it - first[j]);   // the member's item 0
    if (!ws_wait(&full[s], par, status)) return;
    w3_item<R>(A, g, desc[s], stage0 + (size_t)s * stage_floats, lane);
    mbar_arrive(&empty[s]);
    if (++s == ns) { s = 0; par ^= 1u; }
  }
}

template <int NT, int R>
__global__ void __launch_bounds__(NT + 32, 1)
    batch_w3_kernel(const BatchMember<float>* __restrict__ mem, const long long* __restrict__ first, int nmem,
                    int ns, long long stage_floats) {
  batch_w3_cta<NT, R>(mem, first, nmem, ns, stage_floats, blockIdx.x, gridDim.x);
}

}  // namespace rt
