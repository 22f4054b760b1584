// rt_persist_w2.cu -- launchers of the 2-wide block warp-specialised kernel
// (rt_step7.cuh): RT_VARIANT_W2 (register look-ahead), RT_VARIANT_W2D
// (without) and RT_VARIANT_W2Z (z-march over (k,l,m) columns, the
// production binary32 kernel).
#include "rt_persist.cuh"

namespace rt {

namespace {

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

template <int PF, int ZM>
cudaError_t launch_w2_pf(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st) {
  if (threads == 128) return launch_w2_nt<128, PF, ZM>(A, S, st);
  if (threads == 256) return launch_w2_nt<256, PF, ZM>(A, S, st);
  return launch_w2_nt<512, PF, ZM>(A, S, st);
}

}  // namespace

cudaError_t launch_w2_family(const StepArgs<float>& A, const PlaneSched& S, int threads, int pf, int zm,
                             cudaStream_t st) {
  if (zm) return launch_w2_pf<0, 1>(A, S, threads, st);
  if (pf) return launch_w2_pf<1, 0>(A, S, threads, st);
  return launch_w2_pf<0, 0>(A, S, threads, st);
}

}  // namespace rt
