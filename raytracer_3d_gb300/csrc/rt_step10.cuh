// rt_step10.cuh -- warp-specialised step over row chunks of a plane, every
// operand staged by TMA, several consumer groups per CTA (binary32 form).
//
// A work item is a chunk of HR rows of one (z,k) plane at one (l,m):
// items are (plane item in band order) x (row chunk, fastest), walked by
// persistent CTAs (CTA b takes items b, b+G, ...).  A stage holds all that
// one chunk reads, each piece a contiguous row range copied by one bulk copy:
//   E of the plane, rows y0-2 .. y1+1 (clamped)          (x and y stencils)
//   E of the 16 neighbour planes along z,k,l,m, rows y0 .. y1-1
//   x velocities, right and left face velocities of z,k,l,m and the growth
//     rate, rows y0 .. y1-1; y velocities rows y0-1 .. y1-1 (the face below
//     the chunk); the face-0 x velocities of rows y0 .. y1-1 and the face-0
//     y velocities of the plane.
// The producer warp (one bulk copy per lane) fills a ring of `ns` stages; NG consumer
// groups of GT threads take the CTA's items in turn (group g: local items
// g, g+NG, ...), each thread a 2 (x) by R (y) block as in rt_step7.cuh, with
// x faces passed between lanes by shuffle and y faces chained in registers.
// Consumers issue no global load; no CTA-wide barrier runs in the loop; all
// waits are bounded.  Arithmetic and order per face and per cell are those
// of the other binary32 kernels: results are bit-identical to them.
// Requires nx, ny and HR multiples of 4.
#pragma once
#include "rt_step9.cuh"

namespace rt {

struct W5Desc {
  long long p0;     // cell (0,0) of the plane
  int y0, y1;       // rows of the chunk
  float kcfl_r[4], kinv_r[4], kcfl_l[4];
};
__host__ __device__ constexpr size_t w5_desc_bytes() { return (sizeof(W5Desc) + 15) / 16 * 16; }
__host__ __device__ constexpr size_t w5_head_bytes() { return 128 + RT_WS_MAXSTAGE * w5_desc_bytes(); }

// stage layout, in floats, for chunks of at most HR rows of an nx-wide plane
struct W5Layout {
  int nx, hr;
  __host__ __device__ int ec() const { return 0; }                               // (hr+4) rows
  __host__ __device__ int en(int j) const { return (hr + 4) * nx + j * hr * nx; }  // 16 x hr rows
  __host__ __device__ int vx() const { return (hr + 4 + 16 * hr) * nx; }          // hr rows
  __host__ __device__ int vr(int a) const { return vx() + (1 + (a - 2)) * hr * nx; }
  __host__ __device__ int vl(int a) const { return vx() + (5 + (a - 2)) * hr * nx; }
  __host__ __device__ int lam() const { return vx() + 9 * hr * nx; }
  __host__ __device__ int vy() const { return vx() + 10 * hr * nx; }             // hr+1 rows
  __host__ __device__ int b0x() const { return vy() + (hr + 1) * nx; }            // hr
  __host__ __device__ int b0y() const { return b0x() + hr; }                       // nx
  __host__ __device__ int floats() const { return b0y() + nx; }
};

__host__ __device__ __forceinline__ size_t w5_smem(const Dims& d, int hr, int ns) {
  W5Layout L{d.n[0], hr};
  return w5_head_bytes() + (size_t)ns * L.floats() * sizeof(float);
}

// producer: the 32 lanes of the last warp; lane 0 publishes the descriptor
// and arms the stage, lane j issues copy j: 0 the plane's E rows, 1..16 the
// neighbour rows, 17..20 right and 21..24 left face velocities of z..m,
// 25 x velocities, 26 rate, 27 y velocities, 28 and 29 the face-0 rows
__device__ __forceinline__ void w5_produce(const StepArgs<float>& A, const PlaneSched& S, long long nitems,
                                           int nyc, int hr, int ns, uint64_t* full, uint64_t* empty,
                                           uint64_t* dful, W5Desc* desc, float* stage0) {
  const Dims& d = A.d;
  const int lane = threadIdx.x & 31;
  const int nx = d.n[0], ny = d.n[1];
  const W5Layout L{nx, hr};
  const int sfl = L.floats();
  const uint32_t rowb = (uint32_t)(nx * sizeof(float));
  uint32_t nact = 0;
  for (int a = 2; a < 6; a++)
    if (d.n[a] > 1) nact++;
  int s = 0;
  uint32_t rnd = 0;
  long long issued = 0;
  for (long long it = blockIdx.x; it < nitems; it += gridDim.x) {
    if (rnd > 0 && !warp_wait(&empty[s], (rnd - 1) & 1u, A.status)) break;
    const long long pit = it / nyc;
    const int yc = (int)(it - pit * nyc);
    int c[6];
    ws_decode(d, S, (unsigned)pit, c);
    const long long p0 = (long long)c[2] * d.s[2] + (long long)c[3] * d.s[3] + (long long)c[4] * d.s[4] +
                         (long long)c[5] * d.s[5];
    const int y0 = yc * hr, y1 = y0 + hr < ny ? y0 + hr : ny;
    const int rows = y1 - y0;
    const int ea = y0 - 2 > 0 ? y0 - 2 : 0, eb = y1 + 2 < ny ? y1 + 2 : ny;   // E rows of the plane
    const int va = y0 > 0 ? y0 - 1 : 0;                                        // first y-velocity row
    const uint32_t cb = (uint32_t)rows * rowb;   // bytes of one chunk-rows copy
    if (lane == 0) {
      W5Desc& D = desc[s];
      D.p0 = p0;
      D.y0 = y0;
      D.y1 = y1;
#pragma unroll
      for (int a = 2; a < 6; a++) {
        const bool act = d.n[a] > 1;
        D.kcfl_r[a - 2] = act ? A.t32.hcfl[a][pidx(c[a] + 1)] : 0.f;
        D.kinv_r[a - 2] = act ? A.t32.inv_d[a][pidx(c[a] + 1)] : 0.f;
        D.kcfl_l[a - 2] = act ? A.t32.hcfl[a][pidx(c[a])] : 0.f;
      }
      mbar_arrive(&dful[s]);
      const uint32_t tx = (uint32_t)(eb - ea) * rowb + (4 * nact + 2 * nact + 2) * cb +
                          (uint32_t)(y1 - va) * rowb + (uint32_t)(rows * sizeof(float)) + rowb;
      mbar_arrive_expect_tx(&full[s], tx);
    }
    __syncwarp();
    float* sP = stage0 + (size_t)s * sfl;
    const long long r0 = (long long)y0 * nx;
    const float* src = nullptr;
    float* dst = nullptr;
    uint32_t bytes = cb;
    if (lane == 0) {
      src = A.E + p0 + (long long)ea * nx;
      dst = sP + L.ec() + (ea - y0 + 2) * nx;
      bytes = (uint32_t)(eb - ea) * rowb;
    } else if (lane < RT_NPLANE) {
      const int a = 2 + (lane - 1) / 4, i = (lane - 1) % 4;
      if (d.n[a] > 1) {
        src = A.E + nb_plane(d, c, a, i < 2 ? i - 2 : i - 1) + r0;
        dst = sP + L.en(lane - 1);
      }
    } else if (lane < 25) {
      const bool right = lane < 21;
      const int a = 2 + (right ? lane - 17 : lane - 21);
      if (d.n[a] > 1) {
        if (right) {
          src = A.vel[a] + p0 + r0;
        } else if (c[a] > 0) {
          src = A.vel[a] + (p0 - d.s[a]) + r0;
        } else {
          long long off = 0;
#pragma unroll
          for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[a][b];
          src = A.vlo[a] + off + r0;
        }
        dst = sP + (right ? L.vr(a) : L.vl(a));
      }
    } else if (lane == 25) {
      src = A.vel[0] + p0 + r0;
      dst = sP + L.vx();
    } else if (lane == 26) {
      src = A.lam[0] + p0 + r0;
      dst = sP + L.lam();
    } else if (lane == 27) {
      src = A.vel[1] + p0 + (long long)va * nx;
      dst = sP + L.vy() + (va - y0 + 1) * nx;
      bytes = (uint32_t)(y1 - va) * rowb;
    } else if (lane < 30) {
      const int a = lane - 28;   // face-0 x rows of the chunk (by y), face-0 y row (by x)
      long long off = 0;
#pragma unroll
      for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[a][b];
      src = A.vlo[a] + off + (a == 0 ? y0 : 0);
      dst = sP + (a == 0 ? L.b0x() : L.b0y());
      bytes = a == 0 ? (uint32_t)(rows * sizeof(float)) : rowb;
    }
    if (src) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      bulk_g2s(dst, src, bytes, &full[s]);
    }
    issued++;
    if (++s == ns) { s = 0; rnd++; }
  }
  for (int j = 0; j < ns; j++) {
    const long long uses = issued / ns + (j < issued % ns ? 1 : 0);
    if (uses == 0) continue;
    for (uint32_t w = 0; w < RT_WAIT_LIMIT; w++)
      if (mbar_try_wait(&full[j], (uint32_t)((uses - 1) & 1))) break;
  }
}

template <int GT, int NG, int R>
__global__ void __launch_bounds__(GT * NG + 32, 1)
    step_w5_kernel(StepArgs<float> A, PlaneSched S, long long nitems, int nyc, int hr, int ns) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + RT_WS_MAXSTAGE;
  uint64_t* dful = empty + RT_WS_MAXSTAGE;
  W5Desc* desc = reinterpret_cast<W5Desc*>(smem_raw + 128);
  float* stage0 = reinterpret_cast<float*>(smem_raw + w5_head_bytes());
  const Dims& d = A.d;
  const int nx = d.n[0], ny = d.n[1];
  const W5Layout L{nx, hr};
  const int sfl = L.floats();
  constexpr int NT = GT * NG;

  if (threadIdx.x == 0) {
    for (int s = 0; s < ns; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], GT);
      mbar_init(&dful[s], 1);
    }
    fence_mbar_init();
  }
  __syncthreads();
  if (blockIdx.x >= nitems) return;
  if (threadIdx.x >= NT) {
    w5_produce(A, S, nitems, nyc, hr, ns, full, empty, dful, desc, stage0);
    return;
  }

  // ---- consumer: group g, the thread's 2 x R block inside the chunk ----
  const int g = threadIdx.x / GT, gt = threadIdx.x % GT, lane = threadIdx.x & 31;
  const int hx = nx >> 1;
  const int x0 = 2 * (gt % hx), yl0 = (gt / hx) * R;   // first row, relative to the chunk
  const int xm = x0 > 0 ? x0 - 1 : 0, xmm = x0 > 1 ? x0 - 2 : 0;
  const bool has_right = x0 + 2 < nx;
  const float cxa = A.t32.hcfl[0][pidx(x0 + 1)], cxb = A.t32.hcfl[0][pidx(x0 + 2)];
  const float ixa = A.t32.inv_d[0][pidx(x0 + 1)], ixb = A.t32.inv_d[0][pidx(x0 + 2)];
  const float cxl = A.t32.hcfl[0][pidx(x0)];
  const float dt = (float)A.dt;
  const long long G = gridDim.x;

  // local items g, g+NG, ... of this CTA: stage (k % ns), parity (k / ns) & 1
  int s = g % ns;
  uint32_t par = (uint32_t)((g / ns) & 1);
  for (long long it = blockIdx.x + g * G; it < nitems; it += NG * G) {
    if (!ws_wait(&dful[s], par, A.status)) return;
    const W5Desc& D = desc[s];
    const long long p0 = D.p0;
    const int y0 = D.y0, y1 = D.y1;
    float kcr[4], kir[4], kcl[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
      kcr[a] = D.kcfl_r[a];
      kir[a] = D.kinv_r[a];
      kcl[a] = D.kcfl_l[a];
    }
    // rows of the block (clamped into the chunk for the dead ones)
    int yr[R];
    float cy[R], iy[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int y = y0 + yl0 + r;
      yr[r] = y < y1 ? y : y1 - 1;
      cy[r] = A.t32.hcfl[1][pidx(yr[r] + 1)];
      iy[r] = A.t32.inv_d[1][pidx(yr[r] + 1)];
    }
    const int yb = y0 + yl0 < y1 ? y0 + yl0 : y1 - 1;   // first row (clamped)
    const float cyb = A.t32.hcfl[1][pidx(yb)];
    if (!ws_wait(&full[s], par, A.status)) return;
    const float* sP = stage0 + (size_t)s * sfl;
    const float* sEC = sP + L.ec() + (2 - y0) * nx;   // row y of the plane at sEC + y*nx

    // centre column rows yb-2 .. yb+R+1, clamped to the plane
    float2 ec[R + 4];
#pragma unroll
    for (int j = 0; j < R + 4; j++) {
      int yy = yb + j - 2;
      yy = yy < 0 ? 0 : (yy > ny - 1 ? ny - 1 : yy);
      ec[j] = ld2(sEC + yy * nx + x0);
    }
    // ---- x faces ----
    float fxa[R], fxb[R], fxl[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float* row = sEC + yr[r] * nx;
      const float2 e01 = ec[r + 2];
      const float em = row[xm];
      const float2 e23 = has_right ? ld2(row + x0 + 2) : make_float2(e01.y, e01.y);
      const float2 vx = ld2(sP + L.vx() + (yr[r] - y0) * nx + x0);
      fxa[r] = flux_fp32(vx.x, cxa, em, e01.x, e01.y, e23.x);
      fxb[r] = flux_fp32(vx.y, cxb, e01.x, e01.y, e23.x, e23.y);
    }
#pragma unroll
    for (int r = 0; r < R; r++) fxl[r] = __shfl_up_sync(0xffffffffu, fxb[r], 1);
    if (x0 == 0) {
#pragma unroll
      for (int r = 0; r < R; r++)
        fxl[r] = open_face0_flux<float>(sP[L.b0x() + (yr[r] - y0)], ec[r + 2].x);
    } else if (lane == 0) {
#pragma unroll
      for (int r = 0; r < R; r++) {
        const float* row = sEC + yr[r] * nx;
        fxl[r] = flux_fp32(sP[L.vx() + (yr[r] - y0) * nx + x0 - 1], cxl, row[xmm], row[x0 - 1], ec[r + 2].x,
                           ec[r + 2].y);
      }
    }
    // ---- y faces: below the first row, then above every row ----
    const float* sVY = sP + L.vy() + (1 - y0) * nx;   // row y of the y velocities at sVY + y*nx
    float2 fy[R + 1];
    if (yb == 0) {
      const float2 vb = ld2(sP + L.b0y() + x0);
      fy[0].x = open_face0_flux<float>(vb.x, ec[2].x);
      fy[0].y = open_face0_flux<float>(vb.y, ec[2].y);
    } else {
      const float2 vb = ld2(sVY + (yb - 1) * nx + x0);
      fy[0].x = flux_fp32(vb.x, cyb, ec[0].x, ec[1].x, ec[2].x, ec[3].x);
      fy[0].y = flux_fp32(vb.y, cyb, ec[0].y, ec[1].y, ec[2].y, ec[3].y);
    }
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 vy = ld2(sVY + yr[r] * nx + x0);
      fy[r + 1].x = flux_fp32(vy.x, cy[r], ec[r + 1].x, ec[r + 2].x, ec[r + 3].x, ec[r + 4].x);
      fy[r + 1].y = flux_fp32(vy.y, cy[r], ec[r + 1].y, ec[r + 2].y, ec[r + 3].y, ec[r + 4].y);
    }
    // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 e0 = ec[r + 2];
      const int ql = (yr[r] - y0) * nx + x0;   // offset inside the chunk
      float dEa = 0.f, dEb = 0.f;
      dEa -= (fxa[r] - fxl[r]) * ixa;
      dEb -= (fxb[r] - fxa[r]) * ixb;
      dEa -= (fy[r + 1].x - fy[r].x) * iy[r];
      dEb -= (fy[r + 1].y - fy[r].y) * iy[r];
#pragma unroll
      for (int a = 2; a < 6; a++) {
        if (d.n[a] <= 1) continue;
        const float* sN = sP + L.en(4 * (a - 2)) + ql;
        const int hn = hr * nx;
        const float2 Em2 = ld2(sN), Em1 = ld2(sN + hn), Ep1 = ld2(sN + 2 * hn), Ep2 = ld2(sN + 3 * hn);
        const float2 vr = ld2(sP + L.vr(a) + ql), vl = ld2(sP + L.vl(a) + ql);
        const float fra = flux_fp32(vr.x, kcr[a - 2], Em1.x, e0.x, Ep1.x, Ep2.x);
        const float fla = flux_fp32(vl.x, kcl[a - 2], Em2.x, Em1.x, e0.x, Ep1.x);
        dEa -= (fra - fla) * kir[a - 2];
        const float frb = flux_fp32(vr.y, kcr[a - 2], Em1.y, e0.y, Ep1.y, Ep2.y);
        const float flb = flux_fp32(vl.y, kcl[a - 2], Em2.y, Em1.y, e0.y, Ep1.y);
        dEb -= (frb - flb) * kir[a - 2];
      }
      const float2 lam = ld2(sP + L.lam() + ql);
      const float mfa = e0.x * lam.x, mfb = e0.y * lam.y;
      if (y0 + yl0 + r < y1)
        st2_stream(A.Enew + p0 + (long long)yr[r] * nx + x0,
                   make_float2(e0.x + dt * (dEa - mfa), e0.y + dt * (dEb - mfb)));
    }
    mbar_arrive(&empty[s]);
    // next local item of the group: k + NG
#pragma unroll
    for (int j = 0; j < NG; j++)
      if (++s == ns) { s = 0; par ^= 1u; }
  }
}

}  // namespace rt
