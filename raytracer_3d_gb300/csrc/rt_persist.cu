// rt_persist.cu -- launchers of the persistent binary32 step kernels:
// the two-stage pipelined kernel (rt_step5.cuh, variant RT_VARIANT_PIPE) and
// the warp-specialised multi-stage kernel (rt_step6.cuh, variants
// RT_VARIANT_WS with register look-ahead and RT_VARIANT_WSD without) and
// its 2-wide block form (rt_step7.cuh, RT_VARIANT_W2 / RT_VARIANT_W2D), and
// the form with every operand staged by TMA (rt_step8.cuh, RT_VARIANT_W3),
// the form with the producer folded into warp 0 (rt_step9.cuh,
// RT_VARIANT_W4), and the row-chunk form with consumer groups (rt_step10.cuh,
// RT_VARIANT_W5 with 256-thread groups, RT_VARIANT_W5H with 128), and the
// small-plane form with z slices per item (rt_step11.cuh, RT_VARIANT_W6,
// also for the ensemble class of small planes).
// Kept in a translation unit of their own so the library builds in parallel.
#include <algorithm>

#include "rt_kernels.h"
#include "rt_step11.cuh"

namespace rt {

namespace {

int most_cells(long long nxy, int nt) { return (int)((nxy + nt - 1) / nt); }

template <class K>
cudaError_t set_smem(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

int sm_count() {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return nsm;
}

// one resident wave of persistent CTAs, at most one per item
template <class K>
cudaError_t persistent_grid(K kernel, int block, size_t smem, long long nitems, long long& grid) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  grid = std::min<long long>(nitems, (long long)per_sm * sm_count());
  return cudaSuccess;
}

// ---- two-stage pipelined kernel ----
template <int NT, int MAXC>
cudaError_t launch_pipe_c(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const size_t sm = pipe_smem(A.d);
  cudaError_t e = set_smem(step_pipe_kernel<NT, MAXC>, sm);
  if (e != cudaSuccess) return e;
  const long long nitems = dense_items(A.d);
  long long grid = 0;
  e = persistent_grid(step_pipe_kernel<NT, MAXC>, NT, sm, nitems, grid);
  if (e != cudaSuccess) return e;
  step_pipe_kernel<NT, MAXC><<<(unsigned)grid, NT, sm, st>>>(A, S, nitems);
  return cudaGetLastError();
}

template <int NT>
cudaError_t launch_pipe_nt(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int mc = most_cells((long long)A.d.n[0] * A.d.n[1], NT);
  if (mc <= 1) return launch_pipe_c<NT, 1>(A, S, st);
  if (mc <= 2) return launch_pipe_c<NT, 2>(A, S, st);
  return launch_pipe_c<NT, 4>(A, S, st);
}

bool pipe_ok(const Dims& d, int threads) {
  return tma_ok<float>(d) && pipe_smem(d) <= 220 * 1024 &&
         most_cells((long long)d.n[0] * d.n[1], threads) <= RT_TMA_MAXC && (long long)d.n[0] * d.n[1] <= 4096;
}

// ---- warp-specialised multi-stage kernel ----
// rows per consumer thread: the thread columns are x = t % nx, so NT / nx
// row chunks of R rows must cover ny
int ws_rows(const Dims& d, int nt) {
  const int nyc = nt / d.n[0];
  if (nyc < 1) return 0;
  const int R = (d.n[1] + nyc - 1) / nyc;
  return R <= 1 ? 1 : (R <= 2 ? 2 : (R <= 4 ? 4 : 0));
}
int ws_max_smem() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return v - 1024;
}
int ws_stages(const Dims& d) {
  const long long room = (long long)ws_max_smem() - (long long)ws_head_bytes();
  const long long per = (long long)ws_stage_bytes(d);
  const long long ns = room > 0 ? room / per : 0;
  return (int)std::min<long long>(ns, RT_WS_MAXSTAGE);
}
bool ws_ok(const Dims& d, int threads) {
  if (threads != 128 && threads != 256 && threads != 512) return false;
  return d.n[0] >= 2 && d.n[1] >= 2 && tma_ok<float>(d) && d.n[0] <= threads && ws_rows(d, threads) > 0 &&
         (long long)d.n[0] * d.n[1] <= 4096 && dense_items(d) < (1LL << 31) && ws_stages(d) >= 2;
}

template <int NT, int R, int PF>
cudaError_t launch_ws_r(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int ns = ws_stages(A.d);
  const size_t sm = ws_smem(A.d, ns);
  cudaError_t e = set_smem(step_ws_kernel<NT, R, PF>, sm);
  if (e != cudaSuccess) return e;
  const long long nitems = dense_items(A.d);
  long long grid = 0;
  e = persistent_grid(step_ws_kernel<NT, R, PF>, NT + 32, sm, nitems, grid);
  if (e != cudaSuccess) return e;
  step_ws_kernel<NT, R, PF><<<(unsigned)grid, NT + 32, sm, st>>>(A, S, nitems, ns);
  return cudaGetLastError();
}

template <int NT, int PF>
cudaError_t launch_ws_nt(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int R = ws_rows(A.d, NT);
  if (R == 1) return launch_ws_r<NT, 1, PF>(A, S, st);
  if (R == 2) return launch_ws_r<NT, 2, PF>(A, S, st);
  return launch_ws_r<NT, 4, PF>(A, S, st);
}

template <int PF>
cudaError_t launch_ws_pf(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st) {
  if (threads == 128) return launch_ws_nt<128, PF>(A, S, st);
  if (threads == 256) return launch_ws_nt<256, PF>(A, S, st);
  return launch_ws_nt<512, PF>(A, S, st);
}

// ---- 2-wide block kernel ----
int w2_rows(const Dims& d, int nt) {
  const int nyc = nt / (d.n[0] / 2);
  if (nyc < 1) return 0;
  const int R = (d.n[1] + nyc - 1) / nyc;
  return R <= 1 ? 1 : (R <= 2 ? 2 : (R <= 4 ? 4 : 0));
}
bool w2_ok(const Dims& d, int threads) {
  if (threads != 128 && threads != 256 && threads != 512) return false;
  return d.n[0] >= 2 && d.n[0] % 2 == 0 && d.n[1] >= 2 && tma_ok<float>(d) && d.n[0] / 2 <= threads &&
         w2_rows(d, threads) > 0 && (long long)d.n[0] * d.n[1] <= 4096 && dense_items(d) < (1LL << 31) &&
         ws_stages(d) >= 2;
}

// ZM = 1: z-march, the count is the number of (k,l,m) columns
template <int NT, int R, int PF, int ZM>
cudaError_t launch_w2_r(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int ns = ws_stages(A.d);
  const size_t sm = ws_smem(A.d, ns);
  cudaError_t e = set_smem(step_w2_kernel<NT, R, PF, ZM>, sm);
  if (e != cudaSuccess) return e;
  const long long nitems = ZM ? (long long)A.d.n[3] * A.d.n[4] * A.d.n[5] : dense_items(A.d);
  long long grid = 0;
  e = persistent_grid(step_w2_kernel<NT, R, PF, ZM>, NT + 32, sm, nitems, grid);
  if (e != cudaSuccess) return e;
  step_w2_kernel<NT, R, PF, ZM><<<(unsigned)grid, NT + 32, sm, st>>>(A, S, nitems, ns);
  return cudaGetLastError();
}

template <int NT, int PF, int ZM>
cudaError_t launch_w2_nt(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int R = w2_rows(A.d, NT);
  if (R == 1) return launch_w2_r<NT, 1, PF, ZM>(A, S, st);
  if (R == 2) return launch_w2_r<NT, 2, PF, ZM>(A, S, st);
  return launch_w2_r<NT, 4, PF, ZM>(A, S, st);
}

template <int PF, int ZM = 0>
cudaError_t launch_w2_pf(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st) {
  if (threads == 128) return launch_w2_nt<128, PF, ZM>(A, S, st);
  if (threads == 256) return launch_w2_nt<256, PF, ZM>(A, S, st);
  return launch_w2_nt<512, PF, ZM>(A, S, st);
}

// ---- all operands staged ----
int w3_stages(const Dims& d) {
  const long long room = (long long)ws_max_smem() - (long long)ws_head_bytes();
  const long long per = (long long)(w3_stage_floats(d) * sizeof(float));
  const long long ns = room > 0 ? room / per : 0;
  return (int)std::min<long long>(ns, RT_WS_MAXSTAGE);
}
bool w3_ok(const Dims& d, int threads) {
  return w2_ok(d, threads) && d.n[0] % 4 == 0 && d.n[1] % 4 == 0 && w3_stages(d) >= 2;
}

template <int NT, int R>
cudaError_t launch_w3_r(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int ns = w3_stages(A.d);
  const size_t sm = w3_smem(A.d, ns);
  cudaError_t e = set_smem(step_w3_kernel<NT, R>, sm);
  if (e != cudaSuccess) return e;
  const long long nitems = dense_items(A.d);
  long long grid = 0;
  e = persistent_grid(step_w3_kernel<NT, R>, NT + 32, sm, nitems, grid);
  if (e != cudaSuccess) return e;
  step_w3_kernel<NT, R><<<(unsigned)grid, NT + 32, sm, st>>>(A, S, nitems, ns);
  return cudaGetLastError();
}

template <int NT>
cudaError_t launch_w3_nt(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int R = w2_rows(A.d, NT);
  if (R == 1) return launch_w3_r<NT, 1>(A, S, st);
  if (R == 2) return launch_w3_r<NT, 2>(A, S, st);
  return launch_w3_r<NT, 4>(A, S, st);
}

// ---- producer in warp 0 ----
template <int NT, int R>
cudaError_t launch_w4_r(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int ns = ws_stages(A.d);
  const size_t sm = ws_smem(A.d, ns);
  cudaError_t e = set_smem(step_w4_kernel<NT, R>, sm);
  if (e != cudaSuccess) return e;
  const long long nitems = dense_items(A.d);
  long long grid = 0;
  e = persistent_grid(step_w4_kernel<NT, R>, NT, sm, nitems, grid);
  if (e != cudaSuccess) return e;
  step_w4_kernel<NT, R><<<(unsigned)grid, NT, sm, st>>>(A, S, nitems, ns);
  return cudaGetLastError();
}

template <int NT>
cudaError_t launch_w4_nt(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int R = w2_rows(A.d, NT);
  if (R == 1) return launch_w4_r<NT, 1>(A, S, st);
  if (R == 2) return launch_w4_r<NT, 2>(A, S, st);
  return launch_w4_r<NT, 4>(A, S, st);
}

// ---- row chunks, consumer groups ----
// rows per thread R and rows per chunk hr for groups of gt threads: hr is a
// multiple of 4 (16-byte rows of the face-0 copy), at least 4
struct W5Shape {
  int R = 0, hr = 0, nyc = 0, ns = 0;
};
W5Shape w5_shape(const Dims& d, int gt, int ng) {
  W5Shape w;
  const int nx = d.n[0], ny = d.n[1];
  if (nx < 4 || nx % 4 || ny < 4 || ny % 4 || nx / 2 > gt) return w;
  const int chunks = gt / (nx / 2);
  for (int R = 1; R <= 2; R++) {
    int hr = chunks * R / 4 * 4;
    if (hr > ny) hr = ny;
    if (hr >= 4) {
      w.R = R;
      w.hr = hr;
      break;
    }
  }
  if (!w.R) return w;
  w.nyc = (ny + w.hr - 1) / w.hr;
  W5Layout L{nx, w.hr};
  const long long room = (long long)ws_max_smem() - (long long)w5_head_bytes();
  const long long per = (long long)L.floats() * (long long)sizeof(float);
  w.ns = (int)std::min<long long>(room > 0 ? room / per : 0, RT_WS_MAXSTAGE);
  if (w.ns < ng + 1) w.R = 0;
  return w;
}
bool w5_ok(const Dims& d, int gt, int threads) {
  if (threads % gt || threads / gt < 1 || threads / gt > 4) return false;
  const W5Shape w = w5_shape(d, gt, threads / gt);
  return w.R > 0 && d.n[0] >= 4 && tma_ok<float>(d) && dense_items(d) * w.nyc < (1LL << 31);
}

template <int GT, int NG, int R>
cudaError_t launch_w5_r(const StepArgs<float>& A, const PlaneSched& S, const W5Shape& w, cudaStream_t st) {
  const size_t sm = w5_smem(A.d, w.hr, w.ns);
  cudaError_t e = set_smem(step_w5_kernel<GT, NG, R>, sm);
  if (e != cudaSuccess) return e;
  const long long nitems = dense_items(A.d) * w.nyc;
  long long grid = 0;
  e = persistent_grid(step_w5_kernel<GT, NG, R>, GT * NG + 32, sm, nitems, grid);
  if (e != cudaSuccess) return e;
  step_w5_kernel<GT, NG, R><<<(unsigned)grid, GT * NG + 32, sm, st>>>(A, S, nitems, w.nyc, w.hr, w.ns);
  return cudaGetLastError();
}

template <int GT, int NG>
cudaError_t launch_w5_ng(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const W5Shape w = w5_shape(A.d, GT, NG);
  if (w.R == 1) return launch_w5_r<GT, NG, 1>(A, S, w, st);
  return launch_w5_r<GT, NG, 2>(A, S, w, st);
}

template <int NT, int R>
cudaError_t launch_bw3_r(const void* members, const long long* first, int nmem, int ns, long long stage_floats,
                         int grid, cudaStream_t st) {
  const size_t sm = ws_head_bytes() + (size_t)ns * stage_floats * sizeof(float);
  cudaError_t e = set_smem(batch_w3_kernel<NT, R>, sm);
  if (e != cudaSuccess) return e;
  batch_w3_kernel<NT, R><<<(unsigned)grid, NT + 32, sm, st>>>(
      static_cast<const BatchMember<float>*>(members), first, nmem, ns, stage_floats);
  return cudaGetLastError();
}

template <int NT>
cudaError_t launch_bw3_nt(const void* members, const long long* first, int nmem, int R, int ns,
                          long long stage_floats, int grid, cudaStream_t st) {
  if (R == 1) return launch_bw3_r<NT, 1>(members, first, nmem, ns, stage_floats, grid, st);
  if (R == 2) return launch_bw3_r<NT, 2>(members, first, nmem, ns, stage_floats, grid, st);
  return launch_bw3_r<NT, 4>(members, first, nmem, ns, stage_floats, grid, st);
}

template <int NT>
int bw3_per_sm_nt(int R, size_t smem) {
  int per_sm = 0;
  cudaError_t e;
  if (R == 1) {
    set_smem(batch_w3_kernel<NT, 1>, smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_w3_kernel<NT, 1>, NT + 32, smem);
  } else if (R == 2) {
    set_smem(batch_w3_kernel<NT, 2>, smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_w3_kernel<NT, 2>, NT + 32, smem);
  } else {
    set_smem(batch_w3_kernel<NT, 4>, smem);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_w3_kernel<NT, 4>, NT + 32, smem);
  }
  return e == cudaSuccess ? per_sm : 0;
}

template <int NT>
int w6_per_sm_nt(size_t smem) {
  int per_sm = 0;
  set_smem(step_w6_kernel<NT>, smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, step_w6_kernel<NT>, NT + 32, smem) != cudaSuccess)
    return 0;
  return per_sm;
}

template <int NT>
cudaError_t launch_w6_nt(const StepArgs<float>& A, const PlaneSched& S, const void* members,
                         const long long* first, int nmem, long long nitems, int ns, long long stage_floats,
                         int grid, cudaStream_t st) {
  const size_t sm = w6_head_bytes() + (size_t)ns * stage_floats * sizeof(float);
  cudaError_t e = set_smem(step_w6_kernel<NT>, sm);
  if (e != cudaSuccess) return e;
  step_w6_kernel<NT><<<(unsigned)grid, NT + 32, sm, st>>>(A, S, static_cast<const BatchMember<float>*>(members),
                                                          first, nmem, nitems, ns, stage_floats);
  return cudaGetLastError();
}

}  // namespace

// ---- small-plane staged kernel ----
int w6_slices(const Dims& d, int threads) {
  if (threads != 256 && threads != 512) return 0;
  const int nx = d.n[0], ny = d.n[1];
  if (nx < 4 || nx % 4 || ny < 4 || ny % 4) return 0;
  for (int a = 2; a < 6; a++)
    if (d.n[a] < 2) return 0;
  const long long P = (long long)nx * ny;
  int G = (int)(2LL * threads / P);
  if (G > RT_W6_MAXG) G = RT_W6_MAXG;
  if (G > d.n[2]) G = d.n[2];
  if (G < 1) return 0;
  // at least half of the consumer threads own cells
  if (2 * (G * P / 2) < threads) return 0;
  if (w6_items(d, G) >= (1LL << 31)) return 0;
  return G;
}
long long w6_stage_floats(const Dims& d, int G) { return (long long)w6_layout(d, G).floats(); }
int w6_stages(long long stage_floats) {
  const long long room = (long long)ws_max_smem() - (long long)w6_head_bytes();
  const long long ns = room > 0 ? room / (stage_floats * (long long)sizeof(float)) : 0;
  return (int)std::min<long long>(ns, RT_WS_MAXSTAGE);
}
size_t w6_smem(int ns, long long stage_floats) { return w6_head_bytes() + (size_t)ns * stage_floats * sizeof(float); }
int w6_blocks_per_sm(int threads, size_t smem) {
  return threads == 256 ? w6_per_sm_nt<256>(smem) : w6_per_sm_nt<512>(smem);
}
cudaError_t launch_batch_w6(const void* members, const long long* first, int nmem, int threads, int ns,
                            long long stage_floats, int grid, cudaStream_t st) {
  StepArgs<float> A{};   // unused: the members carry their arguments
  PlaneSched S{};
  if (threads == 256)
    return launch_w6_nt<256>(A, S, members, first, nmem, -1, ns, stage_floats, grid, st);
  return launch_w6_nt<512>(A, S, members, first, nmem, -1, ns, stage_floats, grid, st);
}

// ---- batched form of the fully staged kernel ----
int batch_w3_rows(const Dims& d, int threads, int R_class) {
  if (threads != 128 && threads != 256 && threads != 512) return 0;
  const int nx = d.n[0], ny = d.n[1];
  if (nx < 4 || nx % 4 || ny < 4 || ny % 4 || nx / 2 > threads || !tma_ok<float>(d)) return 0;
  if (dense_items(d) >= (1LL << 31)) return 0;
  const int R = R_class > 0 ? R_class : w2_rows(d, threads);
  if (R <= 0) return 0;
  const int hx = nx / 2, chunks = threads / hx;
  if ((long long)chunks * R < ny) return 0;
  // at least half of the consumer threads own cells of the plane
  const long long busy = (long long)hx * ((ny + R - 1) / R);
  return 2 * busy >= threads ? R : 0;
}
long long batch_w3_stage_floats(const Dims& d) { return (long long)w3_stage_floats(d); }
int batch_w3_stages(long long stage_floats) {
  const long long room = (long long)ws_max_smem() - (long long)ws_head_bytes();
  const long long ns = room > 0 ? room / (stage_floats * (long long)sizeof(float)) : 0;
  return (int)std::min<long long>(ns, RT_WS_MAXSTAGE);
}
size_t batch_w3_smem(int ns, long long stage_floats) {
  return ws_head_bytes() + (size_t)ns * stage_floats * sizeof(float);
}
int batch_w3_blocks_per_sm(int threads, int R, size_t smem) {
  if (threads == 128) return bw3_per_sm_nt<128>(R, smem);
  if (threads == 256) return bw3_per_sm_nt<256>(R, smem);
  return bw3_per_sm_nt<512>(R, smem);
}
cudaError_t launch_batch_w3(const void* members, const long long* first, int nmem, int threads, int R, int ns,
                            long long stage_floats, int grid, cudaStream_t st) {
  if (threads == 128) return launch_bw3_nt<128>(members, first, nmem, R, ns, stage_floats, grid, st);
  if (threads == 256) return launch_bw3_nt<256>(members, first, nmem, R, ns, stage_floats, grid, st);
  return launch_bw3_nt<512>(members, first, nmem, R, ns, stage_floats, grid, st);
}

cudaError_t launch_persist(const StepArgs<float>& A, const StepTuning& tn, cudaStream_t st, bool& done) {
  done = false;
  if (tn.variant == RT_VARIANT_W6 && w6_slices(A.d, tn.threads) > 0) {
    const int G = w6_slices(A.d, tn.threads);
    const long long sf = w6_stage_floats(A.d, G);
    const int ns = w6_stages(sf);
    if (ns >= 2) {
      done = true;
      const PlaneSched S = make_sched(A.d, tn, G);
      const size_t sm = w6_smem(ns, sf);
      const int per_sm = w6_blocks_per_sm(tn.threads, sm);
      if (per_sm < 1) return cudaErrorInvalidConfiguration;
      const long long nitems = w6_items(A.d, G);
      const int grid = (int)std::min<long long>(nitems, (long long)per_sm * sm_count());
      if (tn.threads == 256) return launch_w6_nt<256>(A, S, nullptr, nullptr, 0, nitems, ns, sf, grid, st);
      return launch_w6_nt<512>(A, S, nullptr, nullptr, 0, nitems, ns, sf, grid, st);
    }
  }
  if (tn.variant == RT_VARIANT_W5 && w5_ok(A.d, 256, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.threads == 256) return launch_w5_ng<256, 1>(A, S, st);
    return launch_w5_ng<256, 2>(A, S, st);
  }
  if (tn.variant == RT_VARIANT_W5H && w5_ok(A.d, 128, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.threads == 128) return launch_w5_ng<128, 1>(A, S, st);
    if (tn.threads == 256) return launch_w5_ng<128, 2>(A, S, st);
    return launch_w5_ng<128, 4>(A, S, st);
  }
  if (tn.variant == RT_VARIANT_W4 && w2_ok(A.d, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.threads == 128) return launch_w4_nt<128>(A, S, st);
    if (tn.threads == 256) return launch_w4_nt<256>(A, S, st);
    return launch_w4_nt<512>(A, S, st);
  }
  if (tn.variant == RT_VARIANT_W3 && w3_ok(A.d, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.threads == 128) return launch_w3_nt<128>(A, S, st);
    if (tn.threads == 256) return launch_w3_nt<256>(A, S, st);
    return launch_w3_nt<512>(A, S, st);
  }
  if (tn.variant == RT_VARIANT_W2Z && w2_ok(A.d, tn.threads)) {
    done = true;
    // columns of z in band order over (k,l,m): units are k alone (gz = nz)
    const PlaneSched S = make_sched(A.d, tn, A.d.n[2]);
    return launch_w2_pf<0, 1>(A, S, tn.threads, st);
  }
  if ((tn.variant == RT_VARIANT_W2 || tn.variant == RT_VARIANT_W2D) && w2_ok(A.d, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.variant == RT_VARIANT_W2) return launch_w2_pf<1>(A, S, tn.threads, st);
    return launch_w2_pf<0>(A, S, tn.threads, st);
  }
  if ((tn.variant == RT_VARIANT_WS || tn.variant == RT_VARIANT_WSD) && ws_ok(A.d, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.variant == RT_VARIANT_WS) return launch_ws_pf<1>(A, S, tn.threads, st);
    return launch_ws_pf<0>(A, S, tn.threads, st);
  }
  if (tn.variant == RT_VARIANT_PIPE && pipe_ok(A.d, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.threads == 128) return launch_pipe_nt<128>(A, S, st);
    if (tn.threads == 512) return launch_pipe_nt<512>(A, S, st);
    if (tn.threads == 1024) return launch_pipe_nt<1024>(A, S, st);
    return launch_pipe_nt<256>(A, S, st);
  }
  return cudaSuccess;
}

}  // namespace rt
