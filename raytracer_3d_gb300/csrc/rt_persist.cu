// rt_persist.cu -- launchers of the persistent binary32 step kernels:
// the dispatch over every persistent variant (launch_persist), the form with
// every operand staged by TMA (rt_step8.cuh, RT_VARIANT_W3) single-field and
// batched, and the small-plane form with z slices per item (rt_step11.cuh,
// RT_VARIANT_W6, also the ensemble class of small planes).  The production
// 2-wide z-march kernel is instantiated in rt_persist_w2.cu so the library
// builds in parallel.
#include "rt_persist.cuh"

namespace rt {

namespace {

// ---- all operands staged ----
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

// failure-detection self-test: one CTA of two warps waits on mbarriers that
// nothing completes, through the same bounded-wait helpers the step kernels
// use (a warp wait as the persistent consumers and producer do, a per-thread
// wait as the plane kernels do), with a short poll limit.  Nothing is copied,
// so no transfer is in flight when the waits give up.
#define RT_PROBE_LIMIT (1u << 12)

namespace {
__global__ void __launch_bounds__(64) wait_probe_kernel(int* status, int* completed) {
  __shared__ uint64_t bar[2];
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool a = warp_wait<RT_PROBE_LIMIT>(&bar[0], 0, status);
  const bool b = mbar_wait_bounded<RT_PROBE_LIMIT>(&bar[1], 0, status);
  if (a || b) atomicOr(completed, 1);
}
}  // namespace

cudaError_t launch_wait_probe(int* status, int* completed, cudaStream_t st) {
  wait_probe_kernel<<<1, 64, 0, st>>>(status, completed);
  return cudaGetLastError();
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
  if (tn.variant == RT_VARIANT_W3 && w3_ok(A.d, tn.threads)) {
    done = true;
    const PlaneSched S = make_sched(A.d, tn);
    if (tn.threads == 128) return launch_w3_nt<128>(A, S, st);
    if (tn.threads == 256) return launch_w3_nt<256>(A, S, st);
    return launch_w3_nt<512>(A, S, st);
  }
  if ((tn.variant == RT_VARIANT_W2Z || tn.variant == RT_VARIANT_W2Q) && w2_ok(A.d, tn.threads)) {
    done = true;
    // columns of z in band order over (k,l,m): units are k alone (gz = nz)
    const PlaneSched S = make_sched(A.d, tn, A.d.n[2]);
    return launch_w2z(A, S, tn.threads, tn.variant == RT_VARIANT_W2Q, st);
  }
  return cudaSuccess;
}

}  // namespace rt
