// rt_step6.cuh -- the producer side of the warp-specialised binary32 step
// kernels (rt_step7.cuh, rt_step8.cuh, rt_step11.cuh).
//
// Work items are the (z,k) planes of (x,y) at one (l,m) in band order, or
// with the z-march whole z columns of one (k,l,m), walked by persistent CTAs
// (CTA b takes items b, b+G, ...).  Each CTA has NT consumer threads and one
// producer warp:
//
//   producer (one warp): decodes the next items, writes their descriptors
//     (plane offset, left-face velocity bases, face-0 bases, grid constants)
//     into shared memory and issues the 17 bulk copies of E of each item into
//     a ring of `ns` stages (2..4, as many as fit).  Stage s is refilled only
//     after every consumer thread has released it (mbarrier empty[s]);
//     copies complete on full[s]; descriptors are published on dful[s].
//   consumers: the kernels of the files named above.
//
// No CTA-wide barrier runs inside the item loop: warps drift by up to `ns`
// items.  Every mbarrier wait is bounded (status bit 0, no hang).
#pragma once
#include "rt_step3.cuh"

namespace rt {

// work items of the plane schedule: one (z,k,l,m) plane of (x,y) each
__host__ __device__ __forceinline__ long long dense_items(const Dims& d) {
  return (long long)d.n[2] * d.n[3] * d.n[4] * d.n[5];
}

#define RT_WS_MAXSTAGE 4

// per-item values the producer publishes for the consumers
struct WsDesc {
  long long p0;            // offset of cell (0,0) of the plane
  const float* vl[4];      // left-face velocities at (0,0), axes z..m
  const float* b0x;        // face-0 x velocities of the plane (index y)
  const float* b0y;        // face-0 y velocities of the plane (index x)
  float kcfl_r[4], kch_r[4], kcl_r[4], kcfl_l[4];   // dt/(2d) right, dt/d = kch + kcl, dt/(2d) left
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
    float kr = 0.f, kh = 0.f, ko = 0.f, kl = 0.f;
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
        kh = A.t32.chi[a][pidx(c[a] + 1)];
        ko = A.t32.clo[a][pidx(c[a] + 1)];
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
      D.kch_r[lane - 2] = kh;
      D.kcl_r[lane - 2] = ko;
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

}  // namespace rt
