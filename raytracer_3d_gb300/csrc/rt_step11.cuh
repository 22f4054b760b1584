// rt_step11.cuh -- warp-specialised staged step for small x-y planes:
// G consecutive z slices per work item (binary32 form).
//
// For planes of a few hundred cells a CTA of NT consumer threads (2 cells
// each) would idle on one plane, so a work item is G = 2*NT/(nx*ny) slices
// z0 .. z0+G-1 of one (k,l,m), in band order over (l,m) with (z group, k)
// inside (PlaneSched with gz = G).  A stage holds all that the G slices
// read, each piece one bulk copy of a whole plane (or face-0 row), issued by
// the producer warp, 32 copies at a time:
//   E at z0-2 .. z0+G+1 (boundary maps applied per plane; the z window is
//   shared by the slices), the 12 k,l,m neighbour planes of every slice,
//   the 11 velocity / rate planes of every slice, the face-0 rows of every
//   slice.
// Consumer thread t owns the cell pair (x0, x0+1) of row y of slice g, with
// x faces passed between lanes by shuffle.  Slices past nz (last group) are
// computed from clamped planes and not stored.  The arithmetic per face and
// per cell (flux_fp32, axis order x,y,z,k,l,m, divergence, update) is that
// of the other binary32 kernels: results are bit-identical to them.
// Requires nx, ny multiples of 4 and every axis z..m longer than one.
// The same kernel steps one field or, over a member list, an ensemble.
#pragma once
#include "rt_step8.cuh"

namespace rt {

#define RT_W6_MAXG 16

struct W6Desc {
  long long p0;   // cell (0,0) of slice z0
  int member, z0;
  // dt/(2d) of the right face, dt/d of the cell as hi + lo, dt/(2d) of the left face
  float kr[4], kh[4], ko[4], kl[4];                                    // k,l,m faces (index a-2)
  float zr[RT_W6_MAXG], zh[RT_W6_MAXG], zo[RT_W6_MAXG], zl[RT_W6_MAXG];  // z faces of every slice
};
__host__ __device__ constexpr size_t w6_desc_bytes() { return (sizeof(W6Desc) + 15) / 16 * 16; }
// the producer's shared-memory copy of the current member's arguments
// (batched form: read once per member instead of from global memory per item)
__host__ __device__ constexpr size_t w6_member_bytes() { return (sizeof(BatchMember<float>) + 15) / 16 * 16; }
__host__ __device__ constexpr size_t w6_head_bytes() {
  return 128 + RT_WS_MAXSTAGE * w6_desc_bytes() + w6_member_bytes();
}

// Stage layout, in floats, for G slices of an nx x ny plane (P = nx*ny):
// the z window, then every k/l/m neighbour plane and every velocity / rate
// plane with its G slices consecutive (z-consecutive planes of one (k,l,m)
// are consecutive in HBM too, so each group is one bulk copy), then the
// face-0 rows of the slices.
struct W6Layout {
  int P, G, nx, ny;
  __host__ __device__ int ez(int zz) const { return zz * P; }   // zz = z - z0 + 2
  __host__ __device__ int en(int g, int a, int i) const { return (G + 4 + ((a - 3) * 4 + i) * G + g) * P; }
  // k: 0 x, 1 y, 2..5 right faces of z..m, 6..9 left faces of z..m, 10 rate
  __host__ __device__ int v(int g, int k) const { return (G + 4 + 12 * G + k * G + g) * P; }
  __host__ __device__ int b0x(int g) const { return (24 * G + 4) * P + g * ny; }
  __host__ __device__ int b0y(int g) const { return (24 * G + 4) * P + G * ny + g * nx; }
  __host__ __device__ int floats() const { return (24 * G + 4) * P + G * (nx + ny); }
};

__host__ __device__ __forceinline__ W6Layout w6_layout(const Dims& d, int G) {
  return W6Layout{d.n[0] * d.n[1], G, d.n[0], d.n[1]};
}

// Copy j (0..30) of the item whose first slice is z0: what it holds and
// where it lands.  Only the live slices (z < nz) are copied; slots of dead
// slices keep stale data and their results are not stored.
//   0      E of the z window inside [0, nz) (one range)
//   1..4   E at z0-2, z0-1, nz, nz+1 when in the window and outside [0, nz)
//          (boundary-mapped planes)
//   5..16  k,l,m neighbours (a, i) of all live slices
//   17..27 velocity / rate planes k = j-17 of all live slices (k = 6, the
//          left z faces: slices z >= 1 only when z0 == 0)
//   28     left z faces of slice 0 when z0 == 0 (the face-0 plane of z)
//   29, 30 face-0 x rows and y rows of the live slices
#define RT_W6_NCOPY 31
struct W6Copy {
  bool valid;
  int kind;        // 0 z range, 1 mapped z plane, 2 neighbour, 3 velocity / rate, 4 face-0 z plane, 5 face-0 rows
  int a, i, k;     // neighbour axis and offset index; velocity plane; absolute z (kind 0: first z, 1: z)
  int dst;         // stage offset, floats
  unsigned bytes;
};
__host__ __device__ __forceinline__ W6Copy w6_copy(const W6Layout& L, int j, int z0, int nz) {
  const int G = L.G;
  const int gl = z0 + G < nz ? G : nz - z0;   // live slices
  const unsigned pb = (unsigned)(L.P * sizeof(float));
  W6Copy c{false, 0, 0, 0, 0, 0, 0u};
  if (j == 0) {
    const int zs = z0 - 2 > 0 ? z0 - 2 : 0, ze = z0 + G + 2 < nz ? z0 + G + 2 : nz;
    c.valid = ze > zs;
    c.kind = 0;
    c.k = zs;
    c.dst = L.ez(zs - z0 + 2);
    c.bytes = (unsigned)(ze - zs) * pb;
  } else if (j <= 4) {
    const int za = j == 1 ? z0 - 2 : (j == 2 ? z0 - 1 : (j == 3 ? nz : nz + 1));
    c.valid = (za < 0 || za >= nz) && za >= z0 - 2 && za < z0 + G + 2;
    c.kind = 1;
    c.k = za;
    c.dst = L.ez(za - z0 + 2);
    c.bytes = pb;
  } else if (j <= 16) {
    c.valid = true;
    c.kind = 2;
    c.a = 3 + (j - 5) / 4;
    c.i = (j - 5) % 4;
    c.dst = L.en(0, c.a, c.i);
    c.bytes = (unsigned)gl * pb;
  } else if (j <= 27) {
    c.kind = 3;
    c.k = j - 17;
    const int first = (c.k == 6 && z0 == 0) ? 1 : 0;
    c.valid = gl > first;
    c.dst = L.v(first, c.k);
    c.bytes = (unsigned)(gl - first) * pb;
  } else if (j == 28) {
    c.valid = z0 == 0;
    c.kind = 4;
    c.dst = L.v(0, 6);
    c.bytes = pb;
  } else if (j <= 30) {
    c.valid = true;
    c.kind = 5;
    c.i = j - 29;
    c.dst = c.i == 0 ? L.b0x(0) : L.b0y(0);
    c.bytes = (unsigned)(gl * (c.i == 0 ? L.ny : L.nx)) * (unsigned)sizeof(float);
  }
  return c;
}
// bytes an item's mbarrier expects: the sum of its valid copies' bytes
__host__ __device__ __forceinline__ unsigned w6_tx_bytes(const W6Layout& L, int z0, int nz) {
  unsigned t = 0;
  for (int j = 0; j < RT_W6_NCOPY; j++) {
    const W6Copy c = w6_copy(L, j, z0, nz);
    if (c.valid) t += c.bytes;
  }
  return t;
}

// item -> (z0, k, l, m) for z groups of G slices (band order of rt_step6.cuh)
__device__ __forceinline__ void w6_decode(const Dims& d, const PlaneSched& S, unsigned item, int c[6]) {
  const unsigned ngz = (unsigned)((d.n[2] + S.gz - 1) / S.gz);
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
  c[2] = (int)(u % ngz) * S.gz;
  c[3] = (int)(u / ngz);
  c[4] = S.sweep ? banded : (int)outer;
  c[5] = S.sweep ? (int)outer : banded;
}

__host__ __device__ __forceinline__ long long w6_items(const Dims& d, int G) {
  return (long long)((d.n[2] + G - 1) / G) * d.n[3] * d.n[4] * d.n[5];
}

// One item into a stage, by the 32 lanes of the producer warp, split as in
// rt_step8.cuh: w6_prepare (before the stage is free) decodes the item, works
// out each lane's copy (w6_copy) and loads the descriptor's constants,
// lane-distributed (lane g < G: the z faces of slice g; lanes 16..18: axes
// k, l, m); w6_commit writes the descriptor, arms the stage and issues the
// copies.
struct W6Prep {
  long long p0;
  int z0;
  const float* src;   // null: no copy on this lane
  int dst;
  unsigned bytes, tx;
  float c0, c1, c3, c2;   // this lane's descriptor constants
};
__device__ __forceinline__ W6Prep w6_prepare(const StepArgs<float>& A, const PlaneSched& S, long long li) {
  const Dims& d = A.d;
  const int lane = threadIdx.x & 31;
  const int G = S.gz;
  const W6Layout L = w6_layout(d, G);
  const int nz = d.n[2];
  int c[6];
  w6_decode(d, S, (unsigned)li, c);
  const int z0 = c[2];
  const long long p0 = (long long)z0 * d.s[2] + (long long)c[3] * d.s[3] + (long long)c[4] * d.s[4] +
                       (long long)c[5] * d.s[5];
  W6Prep P;
  P.p0 = p0;
  P.z0 = z0;
  P.c0 = P.c1 = P.c3 = P.c2 = 0.f;
  if (lane < G) {
    const int z = z0 + lane < nz ? z0 + lane : nz - 1;
    P.c0 = A.t32.hcfl[2][pidx(z + 1)];
    P.c1 = A.t32.chi[2][pidx(z + 1)];
    P.c3 = A.t32.clo[2][pidx(z + 1)];
    P.c2 = A.t32.hcfl[2][pidx(z)];
  } else if (lane >= 16 && lane < 19) {
    const int a = lane - 13;
    P.c0 = A.t32.hcfl[a][pidx(c[a] + 1)];
    P.c1 = A.t32.chi[a][pidx(c[a] + 1)];
    P.c3 = A.t32.clo[a][pidx(c[a] + 1)];
    P.c2 = A.t32.hcfl[a][pidx(c[a])];
  }
  const W6Copy cp = w6_copy(L, lane, z0, nz);
  P.dst = cp.dst;
  P.bytes = cp.bytes;
  // the item's bytes (= w6_tx_bytes), summed across the lanes' own copies
  P.tx = __reduce_add_sync(0xffffffffu, (lane < RT_W6_NCOPY && cp.valid) ? cp.bytes : 0u);
  P.src = nullptr;
  if (lane < RT_W6_NCOPY && cp.valid) {
    if (cp.kind == 0) {   // z range inside the field: planes (z, k, l, m) are consecutive
      P.src = A.E + (p0 + (long long)(cp.k - z0) * d.s[2]);
    } else if (cp.kind == 1) {   // one boundary-mapped z plane
      int flip = 0;
      const int zm = map_coord(d, 2, cp.k, flip);
      const int m = flip ? d.n[5] - 1 - c[5] : c[5];
      P.src = A.E + ((long long)zm * d.s[2] + (long long)c[3] * d.s[3] + (long long)c[4] * d.s[4] +
                     (long long)m * d.s[5]);
    } else if (cp.kind == 2) {   // the k/l/m maps do not depend on z: slices consecutive
      P.src = A.E + nb_plane(d, c, cp.a, cp.i < 2 ? cp.i - 2 : cp.i - 1);
    } else if (cp.kind == 3) {
      const int k = cp.k;
      if (k < 6) {
        P.src = A.vel[k] + p0;
      } else if (k < 10) {
        const int a = k - 4;
        if (a == 2) {
          P.src = A.vel[2] + (z0 > 0 ? p0 - d.s[2] : p0);   // left z faces of slices z >= 1
        } else if (c[a] > 0) {
          P.src = A.vel[a] + (p0 - d.s[a]);
        } else {
          long long off = 0;
#pragma unroll
          for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[a][b];
          P.src = A.vlo[a] + off;
        }
      } else {
        P.src = A.lam[0] + p0;
      }
    } else if (cp.kind == 4) {   // left z faces of slice z = 0: the face-0 plane of z
      long long off = 0;
#pragma unroll
      for (int b = 3; b < 6; b++) off += (long long)c[b] * d.ps[2][b];
      P.src = A.vlo[2] + off;
    } else {   // face-0 x rows (by y) or y rows (by x) of the live slices
      long long off = 0;
#pragma unroll
      for (int b = 2; b < 6; b++) off += (long long)c[b] * d.ps[cp.i][b];
      P.src = A.vlo[cp.i] + off;
    }
  }
  return P;
}

__device__ __forceinline__ void w6_commit(const W6Prep& P, int G, int member, float* sP, W6Desc* D,
                                          uint64_t* fullb, uint64_t* dfulb) {
  const int lane = threadIdx.x & 31;
  if (lane < G) {
    D->zr[lane] = P.c0;
    D->zh[lane] = P.c1;
    D->zo[lane] = P.c3;
    D->zl[lane] = P.c2;
  } else if (lane >= 16 && lane < 19) {
    D->kr[lane - 15] = P.c0;   // axis a = lane - 13 at index a - 2
    D->kh[lane - 15] = P.c1;
    D->ko[lane - 15] = P.c3;
    D->kl[lane - 15] = P.c2;
  }
  if (lane == 0) {
    D->p0 = P.p0;
    D->member = member;
    D->z0 = P.z0;
  }
  __syncwarp();
  if (lane == 0) {
    mbar_arrive(dfulb);
    mbar_arrive_expect_tx(fullb, P.tx);
  }
  __syncwarp();
  if (P.src) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    bulk_g2s(sP + P.dst, P.src, P.bytes, fullb);
  }
}

// a consumer thread's cell pair and its constants, fixed for one field
struct W6Geom {
  int nx, ny, P, G, g, y, x0, xm, xmm;
  bool has_right, active;
  float cxa, cxb, hxa, hxb, oxa, oxb, cxl, cy, hy, oy, cyb, dthi, dtlo;
  unsigned seed;   // this step's rounding seed of the field
};

__device__ __forceinline__ void w6_geom(const StepArgs<float>& A, int G, int t, W6Geom& w) {
  const int nx = A.d.n[0], ny = A.d.n[1];
  w.nx = nx;
  w.ny = ny;
  w.P = nx * ny;
  w.G = G;
  const int hx = nx >> 1, ts = hx * ny;   // threads per slice
  int g = t / ts;
  w.active = g < G;
  if (!w.active) g = G - 1;
  const int rem = t % ts;
  w.g = g;
  w.y = rem / hx;
  w.x0 = 2 * (rem % hx);
  const int x0 = w.x0, y = w.y;
  w.xm = x0 > 0 ? x0 - 1 : 0;
  w.xmm = x0 > 1 ? x0 - 2 : 0;
  w.has_right = x0 + 2 < nx;
  w.cxa = A.t32.hcfl[0][pidx(x0 + 1)];
  w.cxb = A.t32.hcfl[0][pidx(x0 + 2)];
  w.hxa = A.t32.chi[0][pidx(x0 + 1)];
  w.hxb = A.t32.chi[0][pidx(x0 + 2)];
  w.oxa = A.t32.clo[0][pidx(x0 + 1)];
  w.oxb = A.t32.clo[0][pidx(x0 + 2)];
  w.cxl = A.t32.hcfl[0][pidx(x0)];
  w.cy = A.t32.hcfl[1][pidx(y + 1)];
  w.hy = A.t32.chi[1][pidx(y + 1)];
  w.oy = A.t32.clo[1][pidx(y + 1)];
  w.cyb = A.t32.hcfl[1][pidx(y)];
  w.dthi = A.dthi;
  w.dtlo = A.dtlo;
  w.seed = *A.seed_in;
}

__device__ __forceinline__ void w6_item(const StepArgs<float>& A, const W6Geom& w, const W6Desc& D,
                                        const float* sP, int lane) {
  const Dims& d = A.d;
  const int nx = w.nx, ny = w.ny, x0 = w.x0, y = w.y, g = w.g;
  const W6Layout L{w.P, w.G, nx, ny};
  const float* sC = sP + L.ez(g + 2);   // the slice's own E plane
  float2 ec[5];
#pragma unroll
  for (int j = 0; j < 5; j++) {
    int yy = y + j - 2;
    yy = yy < 0 ? 0 : (yy > ny - 1 ? ny - 1 : yy);
    ec[j] = ld2(sC + yy * nx + x0);
  }
  const int q = y * nx + x0;
  // ---- x faces ----
  const float* row = sC + y * nx;
  const float2 e01 = ec[2];
  const float2 e23 = w.has_right ? ld2(row + x0 + 2) : make_float2(e01.y, e01.y);
  const float2 vx = ld2(sP + L.v(g, 0) + q);
  const float fxa = flux_fp32(vx.x, w.cxa, row[w.xm], e01.x, e01.y, e23.x);
  const float fxb = flux_fp32(vx.y, w.cxb, e01.x, e01.y, e23.x, e23.y);
  float fxl = __shfl_up_sync(0xffffffffu, fxb, 1);
  if (x0 == 0)
    fxl = open_face0_flux<float>(sP[L.b0x(g) + y], e01.x);
  else if (lane == 0)
    fxl = flux_fp32(sP[L.v(g, 0) + q - 1], w.cxl, row[w.xmm], row[x0 - 1], e01.x, e01.y);
  // ---- y faces ----
  float2 fyb, fyt;
  if (y == 0) {
    const float2 vb = ld2(sP + L.b0y(g) + x0);
    fyb.x = open_face0_flux<float>(vb.x, e01.x);
    fyb.y = open_face0_flux<float>(vb.y, e01.y);
  } else {
    const float2 vb = ld2(sP + L.v(g, 1) + q - nx);
    fyb.x = flux_fp32(vb.x, w.cyb, ec[0].x, ec[1].x, ec[2].x, ec[3].x);
    fyb.y = flux_fp32(vb.y, w.cyb, ec[0].y, ec[1].y, ec[2].y, ec[3].y);
  }
  {
    const float2 vy = ld2(sP + L.v(g, 1) + q);
    fyt.x = flux_fp32(vy.x, w.cy, ec[1].x, ec[2].x, ec[3].x, ec[4].x);
    fyt.y = flux_fp32(vy.y, w.cy, ec[1].y, ec[2].y, ec[3].y, ec[4].y);
  }
  // ---- divergence (axis order x,y,z,k,l,m), mean-flow term, update ----
  const float2 e0 = e01;
  float dEa = div32(0.f, fxa, fxl, w.hxa, w.oxa);
  float dEb = div32(0.f, fxb, fxa, w.hxb, w.oxb);
  dEa = div32(dEa, fyt.x, fyb.x, w.hy, w.oy);
  dEb = div32(dEb, fyt.y, fyb.y, w.hy, w.oy);
  {
    const float2 Em2 = ld2(sP + L.ez(g) + q), Em1 = ld2(sP + L.ez(g + 1) + q);
    const float2 Ep1 = ld2(sP + L.ez(g + 3) + q), Ep2 = ld2(sP + L.ez(g + 4) + q);
    const float2 vr = ld2(sP + L.v(g, 2) + q), vl = ld2(sP + L.v(g, 6) + q);
    const float cr = D.zr[g], ch = D.zh[g], co = D.zo[g], cl = D.zl[g];
    const float fra = flux_fp32(vr.x, cr, Em1.x, e0.x, Ep1.x, Ep2.x);
    const float fla = flux_fp32(vl.x, cl, Em2.x, Em1.x, e0.x, Ep1.x);
    dEa = div32(dEa, fra, fla, ch, co);
    const float frb = flux_fp32(vr.y, cr, Em1.y, e0.y, Ep1.y, Ep2.y);
    const float flb = flux_fp32(vl.y, cl, Em2.y, Em1.y, e0.y, Ep1.y);
    dEb = div32(dEb, frb, flb, ch, co);
  }
#pragma unroll
  for (int a = 3; a < 6; a++) {
    const float2 Em2 = ld2(sP + L.en(g, a, 0) + q), Em1 = ld2(sP + L.en(g, a, 1) + q);
    const float2 Ep1 = ld2(sP + L.en(g, a, 2) + q), Ep2 = ld2(sP + L.en(g, a, 3) + q);
    const float2 vr = ld2(sP + L.v(g, a) + q), vl = ld2(sP + L.v(g, a + 4) + q);
    const float cr = D.kr[a - 2], ch = D.kh[a - 2], co = D.ko[a - 2], cl = D.kl[a - 2];
    const float fra = flux_fp32(vr.x, cr, Em1.x, e0.x, Ep1.x, Ep2.x);
    const float fla = flux_fp32(vl.x, cl, Em2.x, Em1.x, e0.x, Ep1.x);
    dEa = div32(dEa, fra, fla, ch, co);
    const float frb = flux_fp32(vr.y, cr, Em1.y, e0.y, Ep1.y, Ep2.y);
    const float flb = flux_fp32(vl.y, cl, Em2.y, Em1.y, e0.y, Ep1.y);
    dEb = div32(dEb, frb, flb, ch, co);
  }
  const float2 lam = ld2(sP + L.v(g, 10) + q);
  const float mfa = e0.x * lam.x, mfb = e0.y * lam.y;
  if (w.active && D.z0 + g < d.n[2]) {
    const long long p = D.p0 + (long long)g * d.s[2] + q;
    st2_stream(A.Enew + p, make_float2(upd32(e0.x, dEa, mfa, w.dthi, w.dtlo, sr_bits(p, w.seed)),
                                       upd32(e0.y, dEb, mfb, w.dthi, w.dtlo, sr_bits(p + 1, w.seed))));
  }
}

// one field (mem == nullptr: A, S, nitems) or the members of an ensemble
// (member j owns items [first[j], first[j+1]), its slices per item in
// mem[j].S.gz; nitems = first[nmem])
// The CTA's part as a device function: bid / nb stand for the block index
// and the grid size (batch_fused_kernel gives a share of its CTAs to this
// class).
template <int NT>
__device__ __forceinline__ void step_w6_cta(const StepArgs<float>& A, const PlaneSched& S,
                                            const BatchMember<float>* __restrict__ mem,
                                            const long long* __restrict__ first, int nmem, long long nitems, int ns,
                                            long long stage_floats, long long bid, long long nb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + RT_WS_MAXSTAGE;
  uint64_t* dful = empty + RT_WS_MAXSTAGE;
  W6Desc* desc = reinterpret_cast<W6Desc*>(smem_raw + 128);
  float* stage0 = reinterpret_cast<float*>(smem_raw + w6_head_bytes());
  int* status = mem ? mem[0].A.status : A.status;
  if (mem) nitems = first[nmem];

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
    int s = 0, j = 0, jcached = -1;
    long long first_j = 0, first_next = mem ? first[1] : 0;
    BatchMember<float>* mc =
        reinterpret_cast<BatchMember<float>*>(smem_raw + 128 + RT_WS_MAXSTAGE * w6_desc_bytes());
    uint32_t rnd = 0;
    long long issued = 0;
    for (long long it = bid; it < nitems; it += nb) {
      if (mem) {
        while (it >= first_next) {
          j++;
          first_j = first_next;
          first_next = first[j + 1];
        }
        if (j != jcached) {   // the 32 lanes copy the member's arguments into shared memory
          const unsigned* src = reinterpret_cast<const unsigned*>(&mem[j]);
          unsigned* dst = reinterpret_cast<unsigned*>(mc);
          const int words = (int)(sizeof(BatchMember<float>) / sizeof(unsigned));
          for (int k = threadIdx.x & 31; k < words; k += 32) dst[k] = src[k];
          __syncwarp();
          jcached = j;
        }
      }
      const StepArgs<float>& Aj = mem ? mc->A : A;
      const PlaneSched& Sj = mem ? mc->S : S;
      const W6Prep P = w6_prepare(Aj, Sj, mem ? it - first_j : it);
      if (rnd > 0 && !warp_wait(&empty[s], (rnd - 1) & 1u, status)) break;
      w6_commit(P, Sj.gz, j, stage0 + (size_t)s * stage_floats, &desc[s], &full[s], &dful[s]);
      issued++;
      if (++s == ns) { s = 0; rnd++; }
    }
    ws_drain(full, ns, issued);
    return;
  }

  const int lane = threadIdx.x & 31;
  W6Geom w;
  int jc = -1;
  int s = 0;
  uint32_t par = 0;
  for (long long it = bid; it < nitems; it += nb) {
    if (!ws_wait(&dful[s], par, status)) return;
    const int j = desc[s].member;
    const StepArgs<float>& Aj = mem ? mem[j].A : A;
    if (j != jc) {
      w6_geom(Aj, mem ? mem[j].S.gz : S.gz, threadIdx.x, w);
      jc = j;
    }
    advance_seed(Aj.seed_in, Aj.seed_out, mem ? it - first[j] : it);   // the field's item 0
    if (!ws_wait(&full[s], par, status)) return;
    w6_item(Aj, w, desc[s], stage0 + (size_t)s * stage_floats, lane);
    mbar_arrive(&empty[s]);
    if (++s == ns) { s = 0; par ^= 1u; }
  }
}

template <int NT>
__global__ void __launch_bounds__(NT + 32, 1)
    step_w6_kernel(StepArgs<float> A, PlaneSched S, const BatchMember<float>* __restrict__ mem,
                   const long long* __restrict__ first, int nmem, long long nitems, int ns, long long stage_floats) {
  step_w6_cta<NT>(A, S, mem, first, nmem, nitems, ns, stage_floats, blockIdx.x, gridDim.x);
}

}  // namespace rt

namespace rt {

// One launch for a whole batched step of the binary32 ensemble: CTAs
// [0, ga) step the members of the fully staged class (batch_w3_cta, planes
// that fill a CTA), the others the members of the small-plane class
// (step_w6_cta).  The host sizes ga in proportion to the two classes'
// cells (both classes run at about the same cost per cell), so both shares
// of the grid finish together; each CTA keeps one role for the launch, so
// the roles' barriers and shared-memory layouts never mix.
template <int NT, int R>
__global__ void __launch_bounds__(NT + 32, 1)
    batch_fused_kernel(const BatchMember<float>* __restrict__ pmem, const long long* __restrict__ pfirst, int np,
                       int pns, long long pstage, const BatchMember<float>* __restrict__ smem6,
                       const long long* __restrict__ sfirst, int ns6, int sns, long long sstage, int ga,
                       StepArgs<float> none, PlaneSched no_sched) {   // unused: the members carry their arguments
  if ((int)blockIdx.x < ga) {
    batch_w3_cta<NT, R>(pmem, pfirst, np, pns, pstage, blockIdx.x, ga);
  } else {
    step_w6_cta<NT>(none, no_sched, smem6, sfirst, ns6, -1, sns, sstage, (long long)blockIdx.x - ga,
                    (long long)gridDim.x - ga);
  }
}

}  // namespace rt
