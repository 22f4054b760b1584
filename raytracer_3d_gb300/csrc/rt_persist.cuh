// rt_persist.cuh -- shared sizing helpers of the persistent binary32 step
// kernels and the launchers of each kernel family.  The families are
// instantiated in three translation units so the library builds in parallel:
//   rt_persist.cu     dispatch (launch_persist), the fully staged kernel
//                     (rt_step8.cuh, RT_VARIANT_W3) single-field and batched,
//                     the small-plane z-slice kernel (rt_step11.cuh,
//                     RT_VARIANT_W6) single-field and batched;
//   rt_persist_w2.cu  the 2-wide block kernel (rt_step7.cuh, RT_VARIANT_W2,
//                     RT_VARIANT_W2D, and RT_VARIANT_W2Z with the z-march);
//   rt_persist_ws.cu  the earlier forms: two-stage pipelined (rt_step5.cuh,
//                     RT_VARIANT_PIPE), warp-specialised one cell per thread
//                     (rt_step6.cuh, RT_VARIANT_WS / RT_VARIANT_WSD),
//                     producer in warp 0 (rt_step9.cuh, RT_VARIANT_W4) and
//                     row chunks with consumer groups (rt_step10.cuh,
//                     RT_VARIANT_W5 / RT_VARIANT_W5H).
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

// ---- two-stage pipelined kernel ----
inline bool pipe_ok(const Dims& d, int threads) {
  return tma_ok<float>(d) && pipe_smem(d) <= 220 * 1024 &&
         most_cells((long long)d.n[0] * d.n[1], threads) <= RT_TMA_MAXC && (long long)d.n[0] * d.n[1] <= 4096;
}

// ---- warp-specialised multi-stage kernel ----
// rows per consumer thread: the thread columns are x = t % nx, so NT / nx
// row chunks of R rows must cover ny
inline int ws_rows(const Dims& d, int nt) {
  const int nyc = nt / d.n[0];
  if (nyc < 1) return 0;
  const int R = (d.n[1] + nyc - 1) / nyc;
  return R <= 1 ? 1 : (R <= 2 ? 2 : (R <= 4 ? 4 : 0));
}
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
inline bool ws_ok(const Dims& d, int threads) {
  if (threads != 128 && threads != 256 && threads != 512) return false;
  return d.n[0] >= 2 && d.n[1] >= 2 && tma_ok<float>(d) && d.n[0] <= threads && ws_rows(d, threads) > 0 &&
         (long long)d.n[0] * d.n[1] <= 4096 && dense_items(d) < (1LL << 31) && ws_stages(d) >= 2;
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

// ---- row chunks, consumer groups ----
// rows per thread R and rows per chunk hr for groups of gt threads: hr is a
// multiple of 4 (16-byte rows of the face-0 copy), at least 4
struct W5Shape {
  int R = 0, hr = 0, nyc = 0, ns = 0;
};
inline W5Shape w5_shape(const Dims& d, int gt, int ng) {
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
inline bool w5_ok(const Dims& d, int gt, int threads) {
  if (threads % gt || threads / gt < 1 || threads / gt > 4) return false;
  const W5Shape w = w5_shape(d, gt, threads / gt);
  return w.R > 0 && d.n[0] >= 4 && tma_ok<float>(d) && dense_items(d) * w.nyc < (1LL << 31);
}

// family launchers; each checks nothing beyond its own template dispatch,
// the callers check the *_ok predicate first
// rt_persist_w2.cu: pf = register look-ahead, zm = z-march over columns
cudaError_t launch_w2_family(const StepArgs<float>& A, const PlaneSched& S, int threads, int pf, int zm,
                             cudaStream_t st);
// rt_persist_ws.cu
cudaError_t launch_pipe_family(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st);
cudaError_t launch_ws_family(const StepArgs<float>& A, const PlaneSched& S, int threads, int pf,
                             cudaStream_t st);
cudaError_t launch_w4_family(const StepArgs<float>& A, const PlaneSched& S, int threads, cudaStream_t st);
// gt = threads per consumer group (256 or 128)
cudaError_t launch_w5_family(const StepArgs<float>& A, const PlaneSched& S, int gt, int threads,
                             cudaStream_t st);

}  // namespace rt
