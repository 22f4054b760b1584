// rt_persist.cuh -- shared sizing helpers of the persistent binary32 step
// kernels and the launchers of each kernel family, instantiated in two
// translation units so the library builds in parallel:
//   rt_persist.cu     dispatch (launch_persist), the fully staged kernel
//                     (rt_step8.cuh, RT_VARIANT_W3) single-field and batched,
//                     the small-plane z-slice kernel (rt_step11.cuh,
//                     RT_VARIANT_W6) single-field and batched;
//   rt_persist_w2.cu  the production 2-wide block kernel marching along z
//                     (rt_step7.cuh, RT_VARIANT_W2Z).
#pragma once
#include <algorithm>

#include "rt_kernels.h"
#include "rt_step11.cuh"

namespace rt {

inline int most_cells(long long nxy, int nt) { return (int)((nxy + nt - 1) / nt); }

template <class K>
cudaError_t set_smem(K kernel, size_t bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

inline int sm_count() {
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

// ---- stage ring of the warp-specialised kernels ----
inline int ws_max_smem() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return v - 1024;
}
inline int ws_stages(const Dims& d) {
  const long long room = (long long)ws_max_smem() - (long long)ws_head_bytes();
  const long long per = (long long)ws_stage_bytes(d);
  const long long ns = room > 0 ? room / per : 0;
  return (int)std::min<long long>(ns, RT_WS_MAXSTAGE);
}
// ---- 2-wide block kernel ----
inline int w2_rows(const Dims& d, int nt) {
  const int nyc = nt / (d.n[0] / 2);
  if (nyc < 1) return 0;
  const int R = (d.n[1] + nyc - 1) / nyc;
  return R <= 1 ? 1 : (R <= 2 ? 2 : (R <= 4 ? 4 : 0));
}
inline bool w2_ok(const Dims& d, int threads) {
  if (threads != 128 && threads != 256 && threads != 512) return false;
  return d.n[0] >= 2 && d.n[0] % 2 == 0 && d.n[1] >= 2 && tma_ok<float>(d) && d.n[0] / 2 <= threads &&
         w2_rows(d, threads) > 0 && (long long)d.n[0] * d.n[1] <= 4096 && dense_items(d) < (1LL << 31) &&
         ws_stages(d) >= 2;
}

// ---- all operands staged ----
inline int w3_stages(const Dims& d) {
  const long long room = (long long)ws_max_smem() - (long long)ws_head_bytes();
  const long long per = (long long)(w3_stage_floats(d) * sizeof(float));
  const long long ns = room > 0 ? room / per : 0;
  return (int)std::min<long long>(ns, RT_WS_MAXSTAGE);
}
inline bool w3_ok(const Dims& d, int threads) {
  return w2_ok(d, threads) && d.n[0] % 4 == 0 && d.n[1] % 4 == 0 && w3_stages(d) >= 2;
}

// rt_persist_w2.cu (the caller checks w2_ok first)
// packed: the cell-pair arithmetic on the f32x2 instructions (same results)
// tuned: the packed f32x2 arithmetic with the next plane's operands
// prefetched into L2 (RT_VARIANT_W2Q); else the scalar form (RT_VARIANT_W2Z)
cudaError_t launch_w2z(const StepArgs<float>& A, const PlaneSched& S, int threads, bool tuned, cudaStream_t st);

}  // namespace rt
