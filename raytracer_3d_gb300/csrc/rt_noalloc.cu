// rt_noalloc.cu -- CFL-rate reduction for callers that cannot allocate.
//
// Some callers may not call cudaMalloc at all: code running inside a host
// framework that owns every device allocation through its own pool, a
// process whose allocations are frozen once a CUDA graph or a real-time
// loop has started, or a driver that must not fail on out-of-memory
// halfway through a run.  rt_max_rate_noalloc serves them: it computes the
// same value as rt_max_rate, from device arrays the caller owns, and
// allocates nothing.  Its only scratch is the file-scope array below; every
// GPU that loads this library holds it (256 KiB) until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/rt_gb300.h"
#include "rt_common.cuh"

namespace rt {

// caller-owned device arrays: right-face velocities, face-0 planes and the
// padded grid spacings of the six axes (layout of include/rt_gb300.h)
struct ConstVel {
  const double* vel[6];
  const double* vlo[6];
  const double* d[6];
};

// block partials of the reduction: one double per block
#define RT_NOALLOC_BLOCKS 32768
// cells handled by one block (256 threads x 256 cells each)
#define RT_NOALLOC_THREADS 256
#define RT_NOALLOC_CELLS_PER_BLOCK (256LL * 256LL)
// largest field the scratch can reduce: 32768 x 65536 = 2^31 cells
#define RT_NOALLOC_MAX_CELLS ((long long)RT_NOALLOC_BLOCKS * RT_NOALLOC_CELLS_PER_BLOCK)

static __device__ __align__(256) double g_rate_partials[RT_NOALLOC_BLOCKS];

// per-cell rate: sum over axes with n > 1 of max(|v(F-1)|,|v(F)|)/d(F),
// the same binary64 sequence as the handle-based reduction
__global__ void __launch_bounds__(RT_NOALLOC_THREADS)
    max_rate_noalloc_kernel(Dims d, ConstVel v, double* partial) {
  __shared__ double red[RT_NOALLOC_THREADS];
  const long long first = (long long)blockIdx.x * RT_NOALLOC_CELLS_PER_BLOCK;
  long long last = first + RT_NOALLOC_CELLS_PER_BLOCK;
  if (last > d.ncell) last = d.ncell;
  double best = 0.0;
  for (long long p = first + threadIdx.x; p < last; p += RT_NOALLOC_THREADS) {
    int c[6];
    long long r = p;
    for (int b = 0; b < 6; b++) {
      c[b] = (int)(r % d.n[b]);
      r /= d.n[b];
    }
    double rate = 0.0;
    for (int a = 0; a < 6; a++) {
      if (d.n[a] <= 1) continue;
      const double vr = v.vel[a][p];
      double vl;
      if (c[a] > 0) {
        vl = v.vel[a][p - d.s[a]];
      } else {
        long long q = 0;
        for (int b = 0; b < 6; b++) q += (long long)c[b] * plane_stride(d, a, b);
        vl = v.vlo[a][q];
      }
      rate = dadd(rate, ddiv(fmax2(fabs(vl), fabs(vr)), v.d[a][pidx(c[a] + 1)]));
    }
    best = fmax2(best, rate);
  }
  red[threadIdx.x] = best;
  __syncthreads();
  for (int w = RT_NOALLOC_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax2(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  // every block writes its partial, so nothing has to be cleared between calls
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(RT_NOALLOC_THREADS)
    max_rate_noalloc_finish(const double* partial, int nblocks, double* out) {
  __shared__ double red[RT_NOALLOC_THREADS];
  double best = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += RT_NOALLOC_THREADS) best = fmax2(best, partial[i]);
  red[threadIdx.x] = best;
  __syncthreads();
  for (int w = RT_NOALLOC_THREADS / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax2(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

}  // namespace rt

using namespace rt;

// device address of the scratch array, looked up once per device.  The
// address belongs to the device's primary context: after cudaDeviceReset
// the cached value is stale, so a process that resets a device must not
// call rt_max_rate_noalloc on it again.
#define RT_NOALLOC_MAX_DEVICES 64
static double* g_scratch_ptr[RT_NOALLOC_MAX_DEVICES];
static std::mutex g_scratch_mu;
// message of the calling thread's last failed call (one buffer per thread,
// so concurrent callers neither race on it nor see each other's text)
static thread_local std::string g_noalloc_err;

static int noalloc_fail(int code, const std::string& msg) {
  g_noalloc_err = msg;
  return code;
}

extern "C" {

const char* rt_noalloc_last_error(void) { return g_noalloc_err.c_str(); }

int rt_max_rate_noalloc(const rt_dims* dims, const double* const* vel, const double* const* vlo,
                        const double* const* dgrid, double* out, void* stream) {
  if (!dims || !vel || !vlo || !dgrid || !out)
    return noalloc_fail(RT_ERR_ARG, "rt_max_rate_noalloc: NULL argument");
  // the grid spacings are indexed with the library's halo width
  if (dims->onx != RT_ONX)
    return noalloc_fail(RT_ERR_ARG, "rt_max_rate_noalloc: onx must be " + std::to_string(RT_ONX));
  const int nn[6] = {dims->nx, dims->ny, dims->nz, dims->nk, dims->nl, dims->nm};
  Dims d{};
  long long st = 1;
  for (int a = 0; a < 6; a++) {
    if (nn[a] < 1) return noalloc_fail(RT_ERR_ARG, "rt_max_rate_noalloc: an axis has no points");
    // checked before multiplying, so the running product cannot overflow
    if (st > RT_NOALLOC_MAX_CELLS / nn[a])
      return noalloc_fail(RT_ERR_ARG, "rt_max_rate_noalloc: the field's cells exceed the limit of its fixed "
                                      "scratch (" + std::to_string(RT_NOALLOC_MAX_CELLS) + " cells)");
    d.n[a] = nn[a];
    d.s[a] = st;
    st *= nn[a];
  }
  d.ncell = st;
  fill_plane_strides(d);
  ConstVel v{};
  for (int a = 0; a < 6; a++) {
    if (nn[a] > 1 && (!vel[a] || !vlo[a] || !dgrid[a]))
      return noalloc_fail(RT_ERR_ARG, "rt_max_rate_noalloc: missing array of an active axis");
    v.vel[a] = vel[a];
    v.vlo[a] = vlo[a];
    v.d[a] = dgrid[a];
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(RT_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= RT_NOALLOC_MAX_DEVICES) return noalloc_fail(RT_ERR_CUDA, "device index out of range");
  double* scratch;
  {
    // first call on this device: look up the array's device address (with
    // this device current); later calls reuse it
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_rate_partials);
      if (e != cudaSuccess || !p)
        return noalloc_fail(RT_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = (double*)p;
    }
    scratch = g_scratch_ptr[dev];
  }
  const int nblocks = (int)((d.ncell + RT_NOALLOC_CELLS_PER_BLOCK - 1) / RT_NOALLOC_CELLS_PER_BLOCK);
  cudaStream_t st_ = (cudaStream_t)stream;
  max_rate_noalloc_kernel<<<nblocks, RT_NOALLOC_THREADS, 0, st_>>>(d, v, scratch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(RT_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  max_rate_noalloc_finish<<<1, RT_NOALLOC_THREADS, 0, st_>>>(scratch, nblocks, out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return noalloc_fail(RT_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return RT_OK;
}

}  // extern "C"
