// rt_step9.cuh -- persistent multi-stage step, producer folded into warp 0,
// 2-wide cell blocks with register look-ahead (binary32 form).
//
// The kernel of rt_step7.cuh without the extra producer warp: the CTA is
// NT threads, all consumers, and warp 0 also feeds the ring of stages.  At
// the start of its item k, warp 0 issues item k+ns-1 into the stage that
// item k-1 used (after every thread released it): all 32 lanes decode the
// item, lane 0 publishes the descriptor and arms the stage's mbarrier, and
// lanes 0..16 issue one bulk copy of an E plane each.  Dropping the 33rd
// warp raises the register budget of a 512-thread CTA from 96 to 128 per
// thread, enough to hold the next item's velocities in registers while the
// current item is computed.  The other warps run up to ns-1 items ahead of
// warp 0.  Every wait is bounded.  Results are bit-identical to the other
// binary32 step kernels.  Requires nx even.
#pragma once
#include "rt_step8.cuh"

namespace rt {

// warp 0: issue work item `it` into stage `s` (round `rnd` of that stage)
__device__ __forceinline__ bool w4_issue(const StepArgs<float>& A, const PlaneSched& S, long long it, int s,
                                         uint32_t rnd, uint64_t* full, uint64_t* empty, uint64_t* dful,
                                         WsDesc* desc, float* stage0) {
  const Dims& d = A.d;
  const int lane = threadIdx.x & 31;
  const int nxy = d.n[0] * d.n[1];
  const uint32_t pbytes = (uint32_t)(nxy * sizeof(float));
  // the stage is free once every thread released its previous item
  if (rnd > 0 && !warp_wait(&empty[s], (rnd - 1) & 1u, A.status)) return false;
  int c[6];
  ws_decode(d, S, (unsigned)it, c);
  const long long p0 = (long long)c[2] * d.s[2] + (long long)c[3] * d.s[3] + (long long)c[4] * d.s[4] +
                       (long long)c[5] * d.s[5];
  if (lane == 0) {
    WsDesc& D = desc[s];
    D.p0 = p0;
    long long o0 = 0, o1 = 0;
#pragma unroll
    for (int b = 2; b < 6; b++) {
      o0 += (long long)c[b] * d.ps[0][b];
      o1 += (long long)c[b] * d.ps[1][b];
    }
    D.b0x = A.vlo[0] + o0;
    D.b0y = A.vlo[1] + o1;
    uint32_t nplanes = 1;
#pragma unroll
    for (int a = 2; a < 6; a++) {
      if (c[a] > 0) {
        D.vl[a - 2] = A.vel[a] + (p0 - d.s[a]);
      } else {
        long long off = 0;
#pragma unroll
        for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[a][b];
        D.vl[a - 2] = A.vlo[a] + off;
      }
      const bool act = d.n[a] > 1;
      D.kcfl_r[a - 2] = act ? A.t32.hcfl[a][pidx(c[a] + 1)] : 0.f;
      D.kinv_r[a - 2] = act ? A.t32.inv_d[a][pidx(c[a] + 1)] : 0.f;
      D.kcfl_l[a - 2] = act ? A.t32.hcfl[a][pidx(c[a])] : 0.f;
      if (act) nplanes += 4;
    }
    mbar_arrive(&dful[s]);
    mbar_arrive_expect_tx(&full[s], nplanes * pbytes);
  }
  __syncwarp();
  // lane j copies plane j: 0 = centre, 1 + 4(a-2) + i = neighbour i of axis a
  if (lane < RT_NPLANE) {
    bool go = true;
    long long off = p0;
    if (lane > 0) {
      const int a = 2 + (lane - 1) / 4, i = (lane - 1) % 4;
      const int o = i < 2 ? i - 2 : i - 1;   // -2, -1, +1, +2
      go = d.n[a] > 1;
      if (go) off = nb_plane(d, c, a, o);
    }
    if (go) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_g2s(stage0 + (size_t)s * RT_NPLANE * nxy + (size_t)lane * nxy, A.E + off, pbytes, &full[s]);
    }
  }
  return true;
}

// warp 0 after a timeout: let the copies of items [k, issued) land (bounded)
__device__ __forceinline__ void w4_drain(uint64_t* full, int ns, long long k, long long issued) {
  for (long long j = k; j < issued; j++)
    for (uint32_t w = 0; w < RT_WAIT_LIMIT; w++)
      if (mbar_try_wait(&full[j % ns], (uint32_t)((j / ns) & 1))) break;
}

template <int NT, int R>
__global__ void __launch_bounds__(NT, 1) step_w4_kernel(StepArgs<float> A, PlaneSched S, long long nitems,
                                                       int ns) {
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
  const bool producer = threadIdx.x < 32;
  const long long G = gridDim.x;

  // ---- warp 0: the first ns-1 items ----
  long long issued = 0;   // items issued by warp 0 (local count)
  long long k = 0;        // items consumed by this thread (local count)
  if (producer) {
    for (int j = 0; j < ns - 1; j++) {
      const long long it = blockIdx.x + j * G;
      if (it >= nitems) break;
      if (!w4_issue(A, S, it, j, 0, full, empty, dful, desc, stage0)) {
        w4_drain(full, ns, 0, issued);
        return;
      }
      issued++;
    }
  }

  // ---- consumer geometry (as rt_step7.cuh) ----
  const int t = threadIdx.x, lane = t & 31;
  const int hx = nx >> 1;
  const int x0 = 2 * (t % hx), y0 = (t / hx) * R;
  int yrow[R];
#pragma unroll
  for (int r = 0; r < R; r++) yrow[r] = y0 + r < ny ? y0 + r : ny - 1;
  const int xm = x0 > 0 ? x0 - 1 : 0, xmm = x0 > 1 ? x0 - 2 : 0;
  const bool has_right = x0 + 2 < nx;
  const float cxa = A.t32.hcfl[0][pidx(x0 + 1)], cxb = A.t32.hcfl[0][pidx(x0 + 2)];
  const float ixa = A.t32.inv_d[0][pidx(x0 + 1)], ixb = A.t32.inv_d[0][pidx(x0 + 2)];
  const float cxl = A.t32.hcfl[0][pidx(x0)];
  float cy[R], iy[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    cy[r] = A.t32.hcfl[1][pidx(yrow[r] + 1)];
    iy[r] = A.t32.inv_d[1][pidx(yrow[r] + 1)];
  }
  const float cyb = A.t32.hcfl[1][pidx(y0 < ny ? y0 : ny - 1)];
  int ecol[R + 4];
#pragma unroll
  for (int j = 0; j < R + 4; j++) {
    int yy = y0 + j - 2;
    yy = yy < 0 ? 0 : (yy > ny - 1 ? ny - 1 : yy);
    ecol[j] = yy * nx + x0;
  }
  const float dt = (float)A.dt;

  W2Regs<R> cur, nxt;
  if (!ws_wait(&dful[0], 0, A.status)) {
    if (producer) w4_drain(full, ns, 0, issued);
    return;
  }
  w2_load<R>(A, desc[0], x0, y0, yrow, lane, cur);

  int s = 0;          // stage of item k
  uint32_t par = 0;   // its parity
  int si = ns - 1;    // stage of item k+ns-1 (issued by warp 0 at item k)
  uint32_t ri = 0;    // its round
  for (long long it = blockIdx.x; it < nitems; it += G, k++) {
    // ---- warp 0: refill the stage of item k-1 with item k+ns-1 ----
    if (producer) {
      const long long iti = it + (long long)(ns - 1) * G;
      if (iti < nitems) {
        if (!w4_issue(A, S, iti, si, ri, full, empty, dful, desc, stage0)) {
          w4_drain(full, ns, k, issued);
          return;
        }
        issued++;
      }
    }
    if (++si == ns) { si = 0; ri++; }
    int sn = s + 1;
    uint32_t parn = par;
    if (sn == ns) { sn = 0; parn ^= 1u; }
    // ---- look ahead: the next item's velocities ----
    if (it + G < nitems) {
      if (!ws_wait(&dful[sn], parn, A.status)) {
        if (producer) w4_drain(full, ns, k, issued);
        return;
      }
      w2_load<R>(A, desc[sn], x0, y0, yrow, lane, nxt);
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
    if (!ws_wait(&full[s], par, A.status)) {
      if (producer) w4_drain(full, ns, k, issued);
      return;
    }
    const float* sE = stage0 + (size_t)s * RT_NPLANE * nxy;

    float2 ec[R + 4];
#pragma unroll
    for (int j = 0; j < R + 4; j++) ec[j] = ld2(sE + ecol[j]);
    float fxa[R], fxb[R], fxl[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int rb = yrow[r] * nx;
      const float2 e01 = ec[r + 2];
      const float em = sE[rb + xm];
      const float2 e23 = has_right ? ld2(sE + rb + x0 + 2) : make_float2(e01.y, e01.y);
      fxa[r] = flux_fp32(cur.vx[r].x, cxa, em, e01.x, e01.y, e23.x);
      fxb[r] = flux_fp32(cur.vx[r].y, cxb, e01.x, e01.y, e23.x, e23.y);
    }
#pragma unroll
    for (int r = 0; r < R; r++) fxl[r] = __shfl_up_sync(0xffffffffu, fxb[r], 1);
    if (x0 == 0) {
#pragma unroll
      for (int r = 0; r < R; r++) fxl[r] = open_face0_flux<float>(cur.xl[r], ec[r + 2].x);
    } else if (lane == 0) {
#pragma unroll
      for (int r = 0; r < R; r++) {
        const int rb = yrow[r] * nx;
        fxl[r] = flux_fp32(cur.xl[r], cxl, sE[rb + xmm], sE[rb + x0 - 1], ec[r + 2].x, ec[r + 2].y);
      }
    }
    float2 fy[R + 1];
    if (y0 == 0) {
      fy[0].x = open_face0_flux<float>(cur.yb.x, ec[2].x);
      fy[0].y = open_face0_flux<float>(cur.yb.y, ec[2].y);
    } else {
      fy[0].x = flux_fp32(cur.yb.x, cyb, ec[0].x, ec[1].x, ec[2].x, ec[3].x);
      fy[0].y = flux_fp32(cur.yb.y, cyb, ec[0].y, ec[1].y, ec[2].y, ec[3].y);
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      fy[r + 1].x = flux_fp32(cur.vy[r].x, cy[r], ec[r + 1].x, ec[r + 2].x, ec[r + 3].x, ec[r + 4].x);
      fy[r + 1].y = flux_fp32(cur.vy[r].y, cy[r], ec[r + 1].y, ec[r + 2].y, ec[r + 3].y, ec[r + 4].y);
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 e0 = ec[r + 2];
      const int q = yrow[r] * nx + x0;
      float dEa = 0.f, dEb = 0.f;
      dEa -= (fxa[r] - fxl[r]) * ixa;
      dEb -= (fxb[r] - fxa[r]) * ixb;
      dEa -= (fy[r + 1].x - fy[r].x) * iy[r];
      dEb -= (fy[r + 1].y - fy[r].y) * iy[r];
#pragma unroll
      for (int a = 2; a < 6; a++) {
        if (d.n[a] <= 1) continue;
        const float* sN = sE + (size_t)(1 + 4 * (a - 2)) * nxy + q;
        const float2 Em2 = ld2(sN), Em1 = ld2(sN + nxy), Ep1 = ld2(sN + 2 * nxy), Ep2 = ld2(sN + 3 * nxy);
        const float2 vr = cur.vr[a - 2][r], vl = cur.vl[a - 2][r];
        const float fra = flux_fp32(vr.x, kcr[a - 2], Em1.x, e0.x, Ep1.x, Ep2.x);
        const float fla = flux_fp32(vl.x, kcl[a - 2], Em2.x, Em1.x, e0.x, Ep1.x);
        dEa -= (fra - fla) * kir[a - 2];
        const float frb = flux_fp32(vr.y, kcr[a - 2], Em1.y, e0.y, Ep1.y, Ep2.y);
        const float flb = flux_fp32(vl.y, kcl[a - 2], Em2.y, Em1.y, e0.y, Ep1.y);
        dEb -= (frb - flb) * kir[a - 2];
      }
      const float mfa = e0.x * cur.lam[r].x, mfb = e0.y * cur.lam[r].y;
      if (y0 + r < ny) st2_stream(A.Enew + p0 + q, make_float2(e0.x + dt * (dEa - mfa), e0.y + dt * (dEb - mfb)));
    }
    mbar_arrive(&empty[s]);
    cur = nxt;
    s = sn;
    par = parn;
  }
  // warp 0: nothing is left in flight (every issued item was consumed above)
}

}  // namespace rt
