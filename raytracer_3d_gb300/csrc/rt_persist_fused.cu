// rt_persist_fused.cu -- launcher of the fused batched binary32 step
// (batch_fused_kernel, rt_step11.cuh): the fully staged class and the
// small-plane class of an ensemble in one persistent launch.  Its own
// translation unit so the library builds in parallel.
#include "rt_persist.cuh"

namespace rt {

namespace {

template <int NT, int R>
int fused_per_sm(size_t smem) {
  int per_sm = 0;
  if (set_smem(batch_fused_kernel<NT, R>, smem) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_fused_kernel<NT, R>, NT + 32, smem) !=
      cudaSuccess)
    return 0;
  return per_sm;
}

template <int NT, int R>
cudaError_t fused_launch(const BatchFused& F, int grid, int ga, cudaStream_t st) {
  const size_t sm = batch_fused_smem(F);
  cudaError_t e = set_smem(batch_fused_kernel<NT, R>, sm);
  if (e != cudaSuccess) return e;
  batch_fused_kernel<NT, R><<<(unsigned)grid, NT + 32, sm, st>>>(
      static_cast<const BatchMember<float>*>(F.pmem), F.pfirst, F.np, F.pns, F.pstage,
      static_cast<const BatchMember<float>*>(F.smem6), F.sfirst, F.ns6, F.sns, F.sstage, ga, StepArgs<float>{},
      PlaneSched{});
  return cudaGetLastError();
}

template <int NT>
int per_sm_nt(const BatchFused& F, size_t smem) {
  if (F.pR == 1) return fused_per_sm<NT, 1>(smem);
  if (F.pR == 2) return fused_per_sm<NT, 2>(smem);
  return fused_per_sm<NT, 4>(smem);
}

template <int NT>
cudaError_t launch_nt(const BatchFused& F, int grid, int ga, cudaStream_t st) {
  if (F.pR == 1) return fused_launch<NT, 1>(F, grid, ga, st);
  if (F.pR == 2) return fused_launch<NT, 2>(F, grid, ga, st);
  return fused_launch<NT, 4>(F, grid, ga, st);
}

bool fused_ok(const BatchFused& F) {
  return (F.threads == 256 || F.threads == 512) && (F.pR == 1 || F.pR == 2 || F.pR == 4) && F.np > 0 &&
         F.ns6 > 0;
}

}  // namespace

size_t batch_fused_smem(const BatchFused& F) {
  return std::max(batch_w3_smem(F.pns, F.pstage), w6_smem(F.sns, F.sstage));
}

int batch_fused_blocks_per_sm(const BatchFused& F) {
  if (!fused_ok(F)) return 0;
  const size_t sm = batch_fused_smem(F);
  return F.threads == 256 ? per_sm_nt<256>(F, sm) : per_sm_nt<512>(F, sm);
}

cudaError_t launch_batch_fused(const BatchFused& F, int grid, int ga, cudaStream_t st) {
  if (!fused_ok(F) || ga < 1 || ga >= grid) return cudaErrorInvalidValue;
  return F.threads == 256 ? launch_nt<256>(F, grid, ga, st) : launch_nt<512>(F, grid, ga, st);
}

}  // namespace rt
