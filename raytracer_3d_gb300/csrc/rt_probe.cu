// rt_probe.cu -- measured binary64 rate of the GPU, the denominator of the
// roofline of the binary64 step (which is bound by the binary64 pipe, not
// by HBM, on GB300).
//
// Every thread runs 8 or 16 independent fused multiply-add chains
// x = fma(x, a, b); the chains keep the pipe fed without depending on one
// another.  The result is the number of binary64 fma instructions per
// second of the whole GPU, the best of four launch shapes, each timed with
// CUDA events on a second launch (the first warms the clocks and the
// instruction cache).
#include <cuda_runtime.h>

#include "../../include/rt_gb300.h"

namespace rt {

#define RT_PROBE_THREADS 256

template <int CHAINS>
__global__ void __launch_bounds__(RT_PROBE_THREADS) fp64_fma_probe(int iters, double a, double b, double* sink) {
  double x[CHAINS];
#pragma unroll
  for (int c = 0; c < CHAINS; c++) x[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < CHAINS; c++) x[c] = __fma_rn(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CHAINS; c++) s += x[c];
  if (s == 12345.678) sink[0] = s;   // never true for the chosen a, b: keeps the chains live
}

// fma/s of one configuration, timed on its second launch
template <int CHAINS>
static cudaError_t probe_rate(int blocks, int iters, double* sink, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1,
                              double* rate) {
  // a slightly below 1 and b small keep x bounded and normal
  fp64_fma_probe<CHAINS><<<blocks, RT_PROBE_THREADS, 0, st>>>(iters, 0.999999, 1e-6, sink);
  cudaEventRecord(e0, st);
  fp64_fma_probe<CHAINS><<<blocks, RT_PROBE_THREADS, 0, st>>>(iters, 0.999999, 1e-6, sink);
  cudaEventRecord(e1, st);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess && ms > 0.f)
    *rate = (double)blocks * RT_PROBE_THREADS * CHAINS * (double)iters / (ms * 1e-3);
  return e;
}

}  // namespace rt

extern "C" int rt_fp64_rate(double* fma_per_s) {
  using namespace rt;
  if (!fma_per_s) return RT_ERR_ARG;
  *fma_per_s = 0.0;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return RT_ERR_CUDA;
  }
  double* sink = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = RT_OK;
  if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) ||
      cudaEventCreate(&e0) || cudaEventCreate(&e1)) {
    rc = RT_ERR_CUDA;
    goto done;
  }
  // the best of a few shapes: 8 or 16 independent chains per thread, 4 or 8
  // CTAs of 256 threads per SM
  for (int per_sm = 4; per_sm <= 8; per_sm *= 2) {
    double r8 = 0.0, r16 = 0.0;
    if (probe_rate<8>(nsm * per_sm, 1 << 14, sink, st, e0, e1, &r8) != cudaSuccess ||
        probe_rate<16>(nsm * per_sm, 1 << 13, sink, st, e0, e1, &r16) != cudaSuccess) {
      rc = RT_ERR_CUDA;
      goto done;
    }
    if (r8 > *fma_per_s) *fma_per_s = r8;
    if (r16 > *fma_per_s) *fma_per_s = r16;
  }
done:
  cudaGetLastError();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (sink) cudaFree(sink);
  return rc;
}
