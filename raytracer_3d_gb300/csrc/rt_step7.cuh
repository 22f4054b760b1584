// rt_step7.cuh -- the production binary32 step: warp-specialised, multi-stage,
// 2-wide cell blocks, CTAs marching along z.
//
// Producer, stage ring and descriptors are those of rt_step6.cuh; each CTA
// walks whole z columns of one (k,l,m) (columns in band order over (k,l,m)),
// so the flux a cell computes on its right z face is its left z-face flux on
// the next plane (same inputs: carried in a register, bit-identical), and
// neither the left z velocities nor the z-2 plane are fetched after a
// column's first plane.
// A consumer thread owns a block of 2 (x) by R (y) cells: columns
// x0 = 2*(t % (nx/2)), x0+1 and rows y0 = (t / (nx/2))*R ... y0+R-1, so
// every shared-memory and global access of the block is an 8-byte pair.
// x faces: the thread computes the right faces of both columns; the left
// face of x0 comes from the lane to the left by a warp shuffle (face 0 is
// the open-boundary flux; the first lane of a warp with x0 > 0 computes it).
// y faces: once per face inside the rows, plus the face below row y0.
// The arithmetic per face and per cell (flux_fp32, axis order x,y,z,k,l,m,
// divergence and update) is that of the other binary32 kernels, so results
// are bit-identical to them.  Requires nx even.
#pragma once
#include "rt_step6.cuh"

namespace rt {

__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ float2 ld2_stream(const float* p) {
  return __ldcs(reinterpret_cast<const float2*>(p));
}
__device__ __forceinline__ void st2_stream(float* p, float2 v) { __stcs(reinterpret_cast<float2*>(p), v); }

template <int R>
struct W2Regs {
  float2 vx[R], vy[R], vr[4][R], vl[4][R], lam[R];
  float xl[R];   // x0 == 0: face-0 velocity of the row; first lane with x0 > 0: velocity of face x0
  float2 yb;     // y0 == 0: face-0 velocities of both columns; else velocities of face y0
};

template <int R>
// skip_vlz: the left z-face velocities are not needed (z-march, carried flux)
__device__ __forceinline__ void w2_load(const StepArgs<float>& A, const WsDesc& D, int x0, int y0,
                                        const int yrow[R], int lane, W2Regs<R>& G, bool skip_vlz = false) {
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1];
  const long long p0 = D.p0;
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int q = yrow[r] * nx + x0;
    const long long o = p0 + q;
    G.vx[r] = ld2_stream(A.vel[0] + o);
    G.vy[r] = ld2_stream(A.vel[1] + o);
#pragma unroll
    for (int a = 2; a < 6; a++) {
      const bool act = d.n[a] > 1;
      G.vr[a - 2][r] = act ? ld2(A.vel[a] + o) : make_float2(0.f, 0.f);
      G.vl[a - 2][r] = (act && !(a == 2 && skip_vlz)) ? ld2(D.vl[a - 2] + q) : make_float2(0.f, 0.f);
    }
    G.lam[r] = ld2_stream(A.lam[0] + o);
    G.xl[r] = x0 == 0 ? D.b0x[yrow[r]] : (lane == 0 ? A.vel[0][o - 1] : 0.f);
  }
  G.yb = y0 == 0 ? ld2(D.b0y + x0)
                 : (y0 < ny ? ld2(A.vel[1] + p0 + (long long)(y0 - 1) * nx + x0) : make_float2(0.f, 0.f));
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
// The next item of a z column is the next z plane: every per-cell operand of
// the consumer (velocities, growth rate; the left-face bases of k, l, m move
// with z as well) lies one plane (nx*ny values) further on.  Asking L2 for
// those lines now turns the next item's loads from HBM latency into L2
// latency, without holding anything in registers.
template <int R>
__device__ __forceinline__ void w2_prefetch_next(const StepArgs<float>& A, const WsDesc& D, int x0,
                                                 const int yrow[R]) {
  const Dims& d = A.d;
  const int nx = d.n[0];
  const long long nxy = (long long)nx * d.n[1];
#pragma unroll
  for (int r = 0; r < R; r++) {
    const int q = yrow[r] * nx + x0;
    const long long o = D.p0 + nxy + q;
    prefetch_l2(A.vel[0] + o);
    prefetch_l2(A.vel[1] + o);
    prefetch_l2(A.lam[0] + o);
#pragma unroll
    for (int a = 2; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      prefetch_l2(A.vel[a] + o);
      if (a > 2) prefetch_l2(D.vl[a - 2] + nxy + q);
    }
  }
}

// nitems counts the (k,l,m) columns; the walk (ItemWalk) visits z = 0..nz-1
// of each
// PK: the pair arithmetic on the packed f32x2 instructions (same results);
// PFN: prefetch the next plane's operands into L2 (no effect on results)
template <int NT, int R, bool PK, bool PFN = false>
__global__ void __launch_bounds__(NT + 32, 1)
    step_w2z_kernel(StepArgs<float> A, PlaneSched S, long long nitems, int ns) {
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
    ws_produce<true>(A, S, nitems, ns, full, empty, dful, desc, stage0);
    return;
  }

  // ---- consumer: the thread's 2 x R block, fixed for every item ----
  const int t = threadIdx.x, lane = t & 31;
  const int hx = nx >> 1;
  const int x0 = 2 * (t % hx), y0 = (t / hx) * R;
  int yrow[R];
#pragma unroll
  for (int r = 0; r < R; r++) yrow[r] = y0 + r < ny ? y0 + r : ny - 1;
  // x offsets: x0-1 and x0-2 (clamped), the pair at x0+2 (absent at the right edge)
  const int xm = x0 > 0 ? x0 - 1 : 0, xmm = x0 > 1 ? x0 - 2 : 0;
  const bool has_right = x0 + 2 < nx;
  const float cxa = A.t32.hcfl[0][pidx(x0 + 1)], cxb = A.t32.hcfl[0][pidx(x0 + 2)];
  const float hxa = A.t32.chi[0][pidx(x0 + 1)], hxb = A.t32.chi[0][pidx(x0 + 2)];
  const float oxa = A.t32.clo[0][pidx(x0 + 1)], oxb = A.t32.clo[0][pidx(x0 + 2)];
  const float cxl = A.t32.hcfl[0][pidx(x0)];
  float cy[R], hy[R], oy[R];
#pragma unroll
  for (int r = 0; r < R; r++) {
    cy[r] = A.t32.hcfl[1][pidx(yrow[r] + 1)];
    hy[r] = A.t32.chi[1][pidx(yrow[r] + 1)];
    oy[r] = A.t32.clo[1][pidx(yrow[r] + 1)];
  }
  const float cyb = A.t32.hcfl[1][pidx(y0 < ny ? y0 : ny - 1)];
  int ecol[R + 4];   // rows y0-2 .. y0+R+1 (clamped), column pair x0
#pragma unroll
  for (int j = 0; j < R + 4; j++) {
    int yy = y0 + j - 2;
    yy = yy < 0 ? 0 : (yy > ny - 1 ? ny - 1 : yy);
    ecol[j] = yy * nx + x0;
  }
  const float dthi = A.dthi, dtlo = A.dtlo;
  const unsigned seed = *A.seed_in;            // this step's rounding seed
  advance_seed(A.seed_in, A.seed_out, blockIdx.x);   // CTA 0 takes column 0

  W2Regs<R> cur;
  int s = 0;
  uint32_t par = 0;
  float2 zcarry[R];   // the right z face flux of the previous plane of the column, per row
  ItemWalk<true> wk;
  for (wk.start(); wk.valid(nitems); wk.next(d.n[2])) {
    int sn = s + 1;
    uint32_t parn = par;
    if (sn == ns) { sn = 0; parn ^= 1u; }
    if (!ws_wait(&dful[s], par, A.status)) return;
    w2_load<R>(A, desc[s], x0, y0, yrow, lane, cur, wk.z > 0);
    if (PFN && wk.z + 1 < d.n[2]) w2_prefetch_next<R>(A, desc[s], x0, yrow);
    const WsDesc& D = desc[s];
    const long long p0 = D.p0;
    float kcr[4], khr[4], kor[4], kcl[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      kcr[a] = D.kcfl_r[a];
      khr[a] = D.kch_r[a];
      kor[a] = D.kcl_r[a];
      kcl[a] = D.kcfl_l[a];
    }
    if (!ws_wait(&full[s], par, A.status)) return;
    const float* sE = stage0 + (size_t)s * RT_NPLANE * nxy;

    float2 ec[R + 4];
#pragma unroll
    for (int j = 0; j < R + 4; j++) ec[j] = ld2(sE + ecol[j]);
    // ---- x faces: the right faces of both columns as one pair ----
    float2 fx[R];   // (face x0+1, face x0+2)
    float fxl[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int rb = yrow[r] * nx;
      const float2 e01 = ec[r + 2];
      const float em = sE[rb + xm];
      const float2 e23 = has_right ? ld2(sE + rb + x0 + 2) : make_float2(e01.y, e01.y);
      fx[r] = flux2<PK>(cur.vx[r], make_float2(cxa, cxb), make_float2(em, e01.x), e01, make_float2(e01.y, e23.x),
                        e23);
    }
#pragma unroll
    for (int r = 0; r < R; r++) fxl[r] = __shfl_up_sync(0xffffffffu, fx[r].y, 1);
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
    // ---- y faces (both columns) ----
    float2 fy[R + 1];
    if (y0 == 0) {
      fy[0].x = open_face0_flux<float>(cur.yb.x, ec[2].x);
      fy[0].y = open_face0_flux<float>(cur.yb.y, ec[2].y);
    } else {
      fy[0] = flux2<PK>(cur.yb, make_float2(cyb, cyb), ec[0], ec[1], ec[2], ec[3]);
    }
#pragma unroll
    for (int r = 0; r < R; r++)
      fy[r + 1] = flux2<PK>(cur.vy[r], make_float2(cy[r], cy[r]), ec[r + 1], ec[r + 2], ec[r + 3], ec[r + 4]);
    // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 e0 = ec[r + 2];
      const int q = yrow[r] * nx + x0;
      float2 acc = div2<PK>(make_float2(0.f, 0.f), fx[r], make_float2(fxl[r], fx[r].x), make_float2(hxa, hxb),
                            make_float2(oxa, oxb));
      acc = div2<PK>(acc, fy[r + 1], fy[r], make_float2(hy[r], hy[r]), make_float2(oy[r], oy[r]));
#pragma unroll
      for (int a = 2; a < 6; a++) {
        if (d.n[a] <= 1) continue;
        const float* sN = sE + (size_t)(1 + 4 * (a - 2)) * nxy + q;
        const float2 Em1 = ld2(sN + nxy), Ep1 = ld2(sN + 2 * nxy), Ep2 = ld2(sN + 3 * nxy);
        const float2 kc = make_float2(kcr[a - 2], kcr[a - 2]);
        const float2 fr = flux2<PK>(cur.vr[a - 2][r], kc, Em1, e0, Ep1, Ep2);
        float2 fl;
        if (a == 2 && wk.z > 0) {   // left z face = the previous plane's right z face
          fl = zcarry[r];
        } else {
          const float2 Em2 = ld2(sN);
          fl = flux2<PK>(cur.vl[a - 2][r], make_float2(kcl[a - 2], kcl[a - 2]), Em2, Em1, e0, Ep1);
        }
        if (a == 2) zcarry[r] = fr;
        acc = div2<PK>(acc, fr, fl, make_float2(khr[a - 2], khr[a - 2]), make_float2(kor[a - 2], kor[a - 2]));
      }
      if (y0 + r < ny)
        st2_stream(A.Enew + p0 + q, upd2<PK>(e0, acc, cur.lam[r], dthi, dtlo,
                                             make_uint2(sr_bits(p0 + q, seed), sr_bits(p0 + q + 1, seed))));
    }
    mbar_arrive(&empty[s]);
    s = sn;
    par = parn;
  }
}

}  // namespace rt
