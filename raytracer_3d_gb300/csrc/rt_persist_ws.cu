// rt_persist_ws.cu -- launchers of the earlier persistent binary32 kernels,
// kept as tuning candidates: the two-stage pipelined kernel (rt_step5.cuh,
// RT_VARIANT_PIPE), the warp-specialised one-cell-per-thread kernel
// (rt_step6.cuh, RT_VARIANT_WS with register look-ahead, RT_VARIANT_WSD
// without), the producer folded into warp 0 (rt_step9.cuh, RT_VARIANT_W4)
// and the row-chunk form with consumer groups (rt_step10.cuh, RT_VARIANT_W5
// with 256-thread groups, RT_VARIANT_W5H with 128).
#include "rt_persist.cuh"

namespace rt {

namespace {

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

// ---- warp-specialised multi-stage kernel ----
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

}  // namespace

cudaError_t launch_pipe_family(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st) {
  if (threads == 128) return launch_pipe_nt<128>(A, S, st);
  if (threads == 512) return launch_pipe_nt<512>(A, S, st);
  if (threads == 1024) return launch_pipe_nt<1024>(A, S, st);
  return launch_pipe_nt<256>(A, S, st);
}

cudaError_t launch_ws_family(const StepArgs<float>& A, const PlaneSched& S, int threads, int pf,
                             cudaStream_t st) {
  if (pf) return launch_ws_pf<1>(A, S, threads, st);
  return launch_ws_pf<0>(A, S, threads, st);
}

cudaError_t launch_w4_family(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st) {
  if (threads == 128) return launch_w4_nt<128>(A, S, st);
  if (threads == 256) return launch_w4_nt<256>(A, S, st);
  return launch_w4_nt<512>(A, S, st);
}

cudaError_t launch_w5_family(const StepArgs<float>& A, const PlaneSched& S, int gt, int threads,
                             cudaStream_t st) {
  if (gt == 256) {
    if (threads == 256) return launch_w5_ng<256, 1>(A, S, st);
    return launch_w5_ng<256, 2>(A, S, st);
  }
  if (threads == 128) return launch_w5_ng<128, 1>(A, S, st);
  if (threads == 256) return launch_w5_ng<128, 2>(A, S, st);
  return launch_w5_ng<128, 4>(A, S, st);
}

}  // namespace rt
