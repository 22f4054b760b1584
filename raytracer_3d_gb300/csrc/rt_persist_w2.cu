// rt_persist_w2.cu -- launcher of the production binary32 step kernel
// (rt_step7.cuh: 2-wide blocks, CTAs marching along z over the (k,l,m)
// columns; RT_VARIANT_W2Q with packed pair arithmetic and L2 prefetch of
// the next plane, RT_VARIANT_W2Z the scalar form without prefetch).
#include "rt_persist.cuh"

namespace rt {

namespace {

// the item count is the number of (k,l,m) columns
template <int NT, int R, bool PK, bool PFN>
cudaError_t launch_w2z_r(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int ns = ws_stages(A.d);
  const size_t sm = ws_smem(A.d, ns);
  cudaError_t e = set_smem(step_w2z_kernel<NT, R, PK, PFN>, sm);
  if (e != cudaSuccess) return e;
  const long long nitems = (long long)A.d.n[3] * A.d.n[4] * A.d.n[5];
  long long grid = 0;
  e = persistent_grid(step_w2z_kernel<NT, R, PK, PFN>, NT + 32, sm, nitems, grid);
  if (e != cudaSuccess) return e;
  step_w2z_kernel<NT, R, PK, PFN><<<(unsigned)grid, NT + 32, sm, st>>>(A, S, nitems, ns);
  return cudaGetLastError();
}

template <int NT, bool PK, bool PFN>
cudaError_t launch_w2z_nt(const StepArgs<float>& A, const PlaneSched& S, cudaStream_t st) {
  const int R = w2_rows(A.d, NT);
  if (R == 1) return launch_w2z_r<NT, 1, PK, PFN>(A, S, st);
  if (R == 2) return launch_w2z_r<NT, 2, PK, PFN>(A, S, st);
  return launch_w2z_r<NT, 4, PK, PFN>(A, S, st);
}

template <bool PK, bool PFN>
cudaError_t launch_w2z_pk(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st) {
  if (threads == 128) return launch_w2z_nt<128, PK, PFN>(A, S, st);
  if (threads == 256) return launch_w2z_nt<256, PK, PFN>(A, S, st);
  return launch_w2z_nt<512, PK, PFN>(A, S, st);
}

}  // namespace

cudaError_t launch_w2z(const StepArgs<float>& A, const PlaneSched& S, int threads, bool tuned, cudaStream_t st) {
  return tuned ? launch_w2z_pk<true, true>(A, S, threads, st) : launch_w2z_pk<false, false>(A, S, threads, st);
}

}  // namespace rt
