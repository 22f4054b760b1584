// rt_api.cu -- implementation of the C ABI declared in include/rt_gb300.h.
//
// A handle owns, in HBM (unpadded, x fastest):
//   E[2]        ping-pong state                      T
//   vel[6]      right-face velocities                T
//   vlo[6]      face-0 planes                        T
//   lam[3]      growth rates (FP64: x,y,z; FP32: one combined field)
//   grid, tab32 padded 1D grids (binary64) and binary32 tables
//   bg          padded 3D Nsqr, U, V (binary64)
//   scratch     per-block partial sums of the budget reductions
// T is double for RT_FP64 and float for RT_FP32.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rt_gb300.h"
#include "rt_coeff.cuh"
#include "rt_kernels.h"
#include "rt_step.cuh"
#include "rt_step2.cuh"
#include "rt_step3.cuh"

using namespace rt;

struct rt_handle {
  Dims d{};
  rt_params p{};
  cudaStream_t st = nullptr;
  int elem = 8;                 // bytes per state/coefficient element
  double* grid = nullptr;       // 9 padded 1D arrays
  long long goff[9]{};
  float* tab32 = nullptr;       // 24 padded 1D arrays (Tab32)
  long long toff[24]{};
  double* bg = nullptr;         // 3 padded 3D arrays
  long long bglen = 0;
  void* vel[6]{};
  void* vlo[6]{};
  void* lam[3]{};
  double* uc[6]{};              // binary64 form: cached uCFL of the right faces
  double* ucl[6]{};             // and of the face-0 planes
  void* E[2]{};
  int cur = 0;
  int forcing = RT_FORCING_NONE;  // set_forcing before every step (rt_set_forcing)
  double* force = nullptr;      // its interior 5D field (x,y,k,l,m)
  long long force_gen = 0;      // changes with every rt_set_forcing
  double dzt1 = 0.0;            // dzt(1), the bottom cell's spacing
  SplitFluxes split{};          // flux fields of the two-pass binary64 step (allocated on selection)
  double* mu = nullptr;         // fast binary64 step: 1 - dt*lambda per cell (allocated on selection)
  double* tab64 = nullptr;      // and its tables dt/d_a (offsets toff[0..5])
  int uc_holds = 0;             // uc/ucl hold 0: uCFL of the bit-exact kernels, 1: h of the fast step
  double* scratch = nullptr;    // reductions
  long long scratch_len = 0;
  double* vol3 = nullptr;       // 8 x nvol3 wavenumber integrals
  double* result = nullptr;     // DIAG_RESULT_NV doubles
  int* status = nullptr;        // device flag raised by a timed-out wait
  unsigned* seed = nullptr;     // binary32 stochastic-rounding seeds, one per ping-pong buffer
  void* pinned = nullptr;       // host staging of one interior field
  int host_direct = 1;          // 1: the GPU reads / writes host arrays itself when the device can
  int pageable = -1;            // device supports pageable host memory access (-1: not asked yet)
  double rate = 0.0;
  StepTuning tune;
  bool have_grid = false, have_bg = false, have_coeff = false, have_state = false;
  long long steps_since_set = 0;
  long long launches = 0;
  long long bytes = 0;
  cudaEvent_t ev = nullptr;     // orders this handle's stream against a batch stream
  // named phase timers (rt_tic / rt_toc): event pairs on the handle's stream,
  // resolved when rt_timing_secs reads them
  struct Timer {
    double secs = 0.0;
    long long calls = 0;
    cudaEvent_t open = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pairs;
  };
  std::map<std::string, Timer> timers;
  std::string err;
};

static std::string g_create_err;

static int fail(rt_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (h) h->err = buf; else g_create_err = buf;
  return code;
}

#define CUDA_TRY(h, call)                                                              \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(h, RT_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                  __FILE__, __LINE__);                                                 \
  } while (0)

static int dev_alloc(rt_handle* h, void** ptr, size_t n) {
  cudaError_t e = cudaMalloc(ptr, n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return fail(h, RT_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", n, cudaGetErrorString(e));
  }
  h->bytes += (long long)n;
  return RT_OK;
}

// transient device buffer (not counted in the handle's resident bytes),
// stream-ordered on the handle's stream so that allocating and freeing it
// does not synchronise with work running on other streams (a batch)
static int tmp_alloc(rt_handle* h, void** ptr, size_t n) {
  cudaError_t e = cudaMallocAsync(ptr, n, h->st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *ptr = nullptr;
    return fail(h, RT_ERR_NOMEM, "cudaMalloc of %zu bytes (temporary) failed: %s", n,
                cudaGetErrorString(e));
  }
  return RT_OK;
}

static long long padded_len(const Dims& d, int a) { return d.n[a] + 2 * RT_ONX; }

// ---------------------------------------------------------------------------
// host gather/scatter between the padded Fortran layout and the compact
// interior, split over host threads by outer slabs
// ---------------------------------------------------------------------------
template <class F>
static void parallel_slabs(long long nslab, F&& fn) {
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (nslab < 64) nt = 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([&, t] {
      for (long long s = t; s < nslab; s += nt) fn(s);
    });
  for (auto& x : th) x.join();
}

template <class T>
static void gather_interior(const Dims& d, const double* host, T* dst) {
  long long P[6];
  for (int a = 0; a < 6; a++) P[a] = padded_len(d, a);
  const long long nslab = (long long)d.n[2] * d.n[3] * d.n[4] * d.n[5];
  parallel_slabs(nslab, [&](long long s) {
    long long r = s;
    const int k = (int)(r % d.n[2]); r /= d.n[2];
    const int l = (int)(r % d.n[3]); r /= d.n[3];
    const int n = (int)(r % d.n[4]);
    const int m = (int)(r / d.n[4]);
    for (int j = 0; j < d.n[1]; j++) {
      const long long src = RT_ONX + P[0] * ((j + RT_ONX) + P[1] * ((k + RT_ONX) + P[2] *
                            ((l + RT_ONX) + P[3] * ((n + RT_ONX) + P[4] * (long long)(m + RT_ONX)))));
      const long long dst0 = (long long)d.n[0] * (j + (long long)d.n[1] * s);
      for (int i = 0; i < d.n[0]; i++) dst[dst0 + i] = (T)host[src + i];
    }
  });
}

template <class T>
static void scatter_interior(const Dims& d, const T* src, double* host) {
  long long P[6];
  for (int a = 0; a < 6; a++) P[a] = padded_len(d, a);
  const long long nslab = (long long)d.n[2] * d.n[3] * d.n[4] * d.n[5];
  parallel_slabs(nslab, [&](long long s) {
    long long r = s;
    const int k = (int)(r % d.n[2]); r /= d.n[2];
    const int l = (int)(r % d.n[3]); r /= d.n[3];
    const int n = (int)(r % d.n[4]);
    const int m = (int)(r / d.n[4]);
    for (int j = 0; j < d.n[1]; j++) {
      const long long dst = RT_ONX + P[0] * ((j + RT_ONX) + P[1] * ((k + RT_ONX) + P[2] *
                            ((l + RT_ONX) + P[3] * ((n + RT_ONX) + P[4] * (long long)(m + RT_ONX)))));
      const long long src0 = (long long)d.n[0] * (j + (long long)d.n[1] * s);
      for (int i = 0; i < d.n[0]; i++) host[dst + i] = (double)src[src0 + i];
    }
  });
}

// ---------------------------------------------------------------------------
// argument structs for the kernels
// ---------------------------------------------------------------------------
static Grid make_grid(const rt_handle* h) {
  Grid g;
  for (int a = 0; a < 6; a++) g.d[a] = h->grid + h->goff[a];
  g.kt = h->grid + h->goff[6];
  g.lt = h->grid + h->goff[7];
  g.mt = h->grid + h->goff[8];
  return g;
}

template <class T>
static StepArgs<T> make_step_args(const rt_handle* h, int src) {
  StepArgs<T> A;
  A.d = h->d;
  A.g = make_grid(h);
  for (int a = 0; a < 6; a++) {
    A.t32.inv_d[a] = h->tab32 + h->toff[a];
    A.t32.hcfl[a] = h->tab32 + h->toff[6 + a];
    A.t32.chi[a] = h->tab32 + h->toff[12 + a];
    A.t32.clo[a] = h->tab32 + h->toff[18 + a];
    A.vel[a] = (const T*)h->vel[a];
    A.vlo[a] = (const T*)h->vlo[a];
  }
  for (int c = 0; c < 3; c++) A.lam[c] = (const T*)h->lam[c];
  for (int a = 0; a < 6; a++) {
    A.uc[a] = (const T*)h->uc[a];
    A.ucl[a] = (const T*)h->ucl[a];
  }
  A.E = (const T*)h->E[src];
  A.Enew = (T*)h->E[1 - src];
  A.dt = h->p.dt;
  A.dthi = (float)h->p.dt;
  A.dtlo = (float)(h->p.dt - (double)A.dthi);
  A.seed_in = h->seed + src;
  A.seed_out = h->seed + (1 - src);
  A.status = h->status;
  return A;
}

// set_forcing on the state about to be stepped (main.f90:69)
static cudaError_t apply_forcing(rt_handle* h, int buf, cudaStream_t st) {
  const double dzt1 = h->dzt1;
  if (h->p.precision == RT_FP64)
    return launch_forcing<double>((double*)h->E[buf], h->force, (const double*)h->vel[2], h->d, h->p.dt, dzt1,
                                  h->forcing, st);
  return launch_forcing<float>((float*)h->E[buf], h->force, (const float*)h->vel[2], h->d, h->p.dt, dzt1,
                               h->forcing, st);
}

// the per-face values in uc/ucl for the kind of binary64 step about to run:
// uCFL for the bit-exact kernels (kind 0), h, mu and the tables for the fast
// step (kind 1); recomputed only when the kind changes (or dt / the
// coefficients did, which resets uc_holds)
static cudaError_t ensure_uc(rt_handle* h, int kind) {
  if (h->uc_holds == kind) return cudaSuccess;
  const double* vel[6];
  const double* vlo[6];
  for (int a = 0; a < 6; a++) { vel[a] = (const double*)h->vel[a]; vlo[a] = (const double*)h->vlo[a]; }
  cudaError_t e;
  if (kind == 0) {
    e = launch_ucfl(h->d, make_grid(h), h->p.dt, vel, vlo, h->uc, h->ucl, h->st);
    h->launches += 6;
  } else {
    const double* lam[3] = {(const double*)h->lam[0], (const double*)h->lam[1], (const double*)h->lam[2]};
    e = launch_fast_prepare(h->d, make_grid(h), h->p.dt, vel, vlo, lam, h->uc, h->ucl, h->mu, h->tab64, h->toff,
                            h->st);
    h->launches += 7;
  }
  if (e == cudaSuccess) h->uc_holds = kind;
  return e;
}

static bool fast_ready(const rt_handle* h) {
  bool split = false;
  for (int a = 0; a < 6; a++) split = split || h->split.f[a] != nullptr;
  return split && h->mu && h->tab64;
}

// one step of the handle from buffer src into 1 - src; returns the kernels launched
static cudaError_t step_once(rt_handle* h, int src, int* nlaunch) {
  if (h->p.precision == RT_FP64) {
    if (h->tune.variant == RT_VARIANT_FAST && fast_ready(h)) {
      cudaError_t e = ensure_uc(h, 1);
      if (e != cudaSuccess) return e;
      FastTab T;
      for (int a = 0; a < 6; a++) T.c[a] = h->tab64 + h->toff[a];
      *nlaunch = 2;
      return launch_step_fast(make_step_args<double>(h, src), h->split, h->mu, T, h->tune.band, h->st);
    }
    cudaError_t e = ensure_uc(h, 0);
    if (e != cudaSuccess) return e;
    // the two-pass step once its fields exist (rt_set_tuning allocates them;
    // a field with no axis longer than one keeps the fused step)
    bool split = false;
    for (int a = 0; a < 6; a++) split = split || h->split.f[a] != nullptr;
    if (h->tune.variant == RT_VARIANT_SPLIT && split) {
      *nlaunch = 2;
      return launch_step_split(make_step_args<double>(h, src), h->split, h->st);
    }
    *nlaunch = 1;
    return launch_step<double>(make_step_args<double>(h, src), h->tune, h->st);
  }
  *nlaunch = 1;
  return launch_step<float>(make_step_args<float>(h, src), h->tune, h->st);
}

// flux fields of the two-pass binary64 step, for the axes with n > 1
static int ensure_split(rt_handle* h) {
  const Dims& d = h->d;
  for (int a = 0; a < 6; a++) {
    if (d.n[a] <= 1 || h->split.f[a]) continue;
    int rc = dev_alloc(h, (void**)&h->split.f[a], (size_t)d.ncell * sizeof(double));
    if (!rc) rc = dev_alloc(h, (void**)&h->split.f0[a], (size_t)(d.ncell / d.n[a]) * sizeof(double));
    if (rc) return rc;
  }
  return RT_OK;
}

// fast binary64 step: mu and the tables (its flux fields are the two-pass step's)
static int ensure_fast(rt_handle* h) {
  int rc = ensure_split(h);
  if (!rc && !h->mu) rc = dev_alloc(h, (void**)&h->mu, (size_t)h->d.ncell * sizeof(double));
  if (!rc && !h->tab64) rc = dev_alloc(h, (void**)&h->tab64, (size_t)h->toff[6] * sizeof(double));
  return rc;
}

// binary64 form: refresh the cached per-face values (after the coefficients
// or dt change) for the kind of step selected
static int refresh_ucfl(rt_handle* h) {
  if (h->p.precision != RT_FP64 || !h->have_coeff) return RT_OK;
  h->uc_holds = -1;
  const int kind = h->tune.variant == RT_VARIANT_FAST && fast_ready(h) ? 1 : 0;
  cudaError_t e = ensure_uc(h, kind);
  if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "uCFL: %s", cudaGetErrorString(e));
  return RT_OK;
}

// binary32 tables on the padded range: 1/d, dt/(2d), and dt/d as the
// two-term sum chi + clo
static int upload_tab32(rt_handle* h) {
  std::vector<double> hg(h->goff[8] + padded_len(h->d, 5));
  CUDA_TRY(h, cudaMemcpy(hg.data(), h->grid, hg.size() * sizeof(double), cudaMemcpyDeviceToHost));
  std::vector<float> t(h->toff[23] + padded_len(h->d, 5));
  for (int a = 0; a < 6; a++)
    for (long long i = 0; i < padded_len(h->d, a); i++) {
      const double dd = hg[h->goff[a] + i];
      t[h->toff[a] + i] = (float)(1.0 / dd);
      t[h->toff[6 + a] + i] = (float)(0.5 * h->p.dt / dd);
      const double c = h->p.dt / dd;
      const float chi = (float)c;
      t[h->toff[12 + a] + i] = chi;
      t[h->toff[18 + a] + i] = (float)(c - (double)chi);
    }
  CUDA_TRY(h, cudaMemcpy(h->tab32, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice));
  return RT_OK;
}

// after a synchronisation: report a device-side wait that timed out
static int check_status(rt_handle* h) {
  int st = 0;
  CUDA_TRY(h, cudaMemcpy(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (st) return fail(h, RT_ERR_CUDA, "a device-side wait timed out (status %d); results are invalid", st);
  return RT_OK;
}

// ---------------------------------------------------------------------------
// batched ensemble
// ---------------------------------------------------------------------------
struct rt_batch {
  std::vector<rt_handle*> mem;
  std::vector<int> cur0;        // members' ping-pong index when the arrays were built
  std::vector<int> forced;      // members with a forcing, when the arrays were built
  std::vector<long long> fgen;  // and every member's forcing generation then
  int fp64 = 0;
  int parity = 0;               // steps taken since the arrays were built, mod 2
  cudaStream_t st = nullptr;
  void* d_mem[2] = {nullptr, nullptr};   // BatchMember<T> arrays for the two parities
  long long* d_first = nullptr;
  size_t smem = 0;
  bool tma = false;
  bool group = false;           // z-group items (rt_step4.cuh)
  long long max_nxy = 0;
  StepTuning tune;
  int grid = 0;
  int graph_steps = 16;         // steps per captured graph (even)
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // graphs starting at parity 0 / 1
  bool dirty = true;
  long long launches = 0;
  long long cells = 0;
  cudaEvent_t ev = nullptr;
  std::string err;
  // members stepped by the batched fully staged kernel (binary32 form, planes
  // that fill a CTA of pthreads consumer threads); the others use the arrays
  // above (nq members)
  int pthreads = 256;           // 0: every member in the other class
  int np = 0, nq = 0;
  void* d_pmem[2] = {nullptr, nullptr};
  long long* d_pfirst = nullptr;
  int pR = 0, pns = 0, pgrid = 0;
  long long pstage = 0;         // floats per stage
  // members with small planes stepped by the z-slice staged kernel
  int ns6 = 0;
  void* d_smem6[2] = {nullptr, nullptr};
  long long* d_sfirst = nullptr;
  int sns = 0, sgrid = 0, sthreads = 0;
  long long sstage = 0;
  int slice_threads = -1;       // consumer threads of the z-slice class; -1: as pthreads, 0: off
  long long pcells = 0, scells = 0;   // cells of the two persistent classes
  // both persistent classes in one launch (batch_fused_kernel) when they
  // share a thread count: grid and the CTAs of the fully staged class
  int fuse = 0;                 // setting (rt_batch_set_fused)
  int fgrid = 0, fga = 0;       // 0: two launches
};

static int bfail(rt_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf; else g_create_err = buf;
  return code;
}

#define BCUDA_TRY(b, call)                                                             \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return bfail(b, RT_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),    \
                   __FILE__, __LINE__);                                                \
  } while (0)

static void batch_free_graphs(rt_batch* b) {
  for (int k = 0; k < 2; k++)
    if (b->gexec[k]) { cudaGraphExecDestroy(b->gexec[k]); b->gexec[k] = nullptr; }
}

// kernel launches per batch step
static int batch_kernels(const rt_batch* b) {
  const int persistent = b->fgrid > 0 ? 1 : (b->np > 0 ? 1 : 0) + (b->ns6 > 0 ? 1 : 0);
  return (int)b->forced.size() + persistent + (b->nq > 0 ? 1 : 0);
}

static BatchFused batch_fused_args(const rt_batch* b, int par) {
  BatchFused F;
  F.pmem = b->d_pmem[par];
  F.pfirst = b->d_pfirst;
  F.np = b->np;
  F.pR = b->pR;
  F.pns = b->pns;
  F.pstage = b->pstage;
  F.smem6 = b->d_smem6[par];
  F.sfirst = b->d_sfirst;
  F.ns6 = b->ns6;
  F.sns = b->sns;
  F.sstage = b->sstage;
  F.threads = b->pthreads;
  return F;
}

// device time of one class's own launch (0: fully staged, 1: small
// planes) from the members' current states into the other buffers, the
// way a dry step runs (nothing advances); the second of two launches, in
// ms, or a negative value when a launch or an event fails
static float batch_class_ms(rt_batch* b, int cls) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    return -1.f;
  }
  cudaError_t e = cudaSuccess;
  for (int rep = 0; rep < 2 && e == cudaSuccess; rep++) {
    cudaEventRecord(e0, b->st);
    e = cls == 0 ? launch_batch_w3(b->d_pmem[0], b->d_pfirst, b->np, b->pthreads, b->pR, b->pns, b->pstage,
                                   b->pgrid, b->st)
                 : launch_batch_w6(b->d_smem6[0], b->d_sfirst, b->ns6, b->sthreads, b->sns, b->sstage, b->sgrid,
                                   b->st);
    cudaEventRecord(e1, b->st);
  }
  float ms = -1.f;
  if (e == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
    ms = -1.f;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

// one launch for both persistent classes when they run the same thread
// count: the grid of the fused kernel, split between the classes in
// proportion to the device time of each class's own launch (so both
// shares finish together; by their cells if the timing fails), at least
// one CTA each; fgrid = 0 otherwise
static void batch_plan_fused(rt_batch* b) {
  b->fgrid = b->fga = 0;
  if (!b->fuse || b->np == 0 || b->ns6 == 0 || b->sthreads != b->pthreads) return;
  const int per_sm = batch_fused_blocks_per_sm(batch_fused_args(b, 0));
  if (per_sm < 1) return;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int grid = per_sm * nsm;
  if (grid < 2) return;
  double share = (double)b->pcells / (double)(b->pcells + b->scells);
  // the timing launches write the members' other buffers: ordered after
  // everything queued on the members' streams, and before what follows
  bool ordered = true;
  for (rt_handle* h : b->mem)
    ordered = ordered && cudaEventRecord(h->ev, h->st) == cudaSuccess &&
              cudaStreamWaitEvent(b->st, h->ev, 0) == cudaSuccess;
  if (ordered) {
    const float ta = batch_class_ms(b, 0), tb = batch_class_ms(b, 1);
    if (ta > 0.f && tb > 0.f) share = ta / (double)(ta + tb);
    if (cudaEventRecord(b->ev, b->st) == cudaSuccess)
      for (rt_handle* h : b->mem) cudaStreamWaitEvent(h->st, b->ev, 0);
  }
  int ga = (int)(share * grid + 0.5);
  ga = std::max(1, std::min(grid - 1, ga));
  b->fgrid = grid;
  b->fga = ga;
}

// one step of every member, starting from the arrays of parity `par`;
// force = false leaves out the members' forcing (dry steps)
template <class T>
static cudaError_t batch_launch(rt_batch* b, int par, bool force = true) {
  cudaError_t e = cudaSuccess;
  // each member's set_forcing first (main.f90:69), on the state of this parity
  if (force)
    for (int j : b->forced) {
      e = apply_forcing(b->mem[j], b->cur0[j] ^ par, b->st);
      if (e != cudaSuccess) return e;
    }
  if (b->fgrid > 0) {
    e = launch_batch_fused(batch_fused_args(b, par), b->fgrid, b->fga, b->st);
  } else {
    if (b->np)
      e = launch_batch_w3(b->d_pmem[par], b->d_pfirst, b->np, b->pthreads, b->pR, b->pns, b->pstage, b->pgrid,
                          b->st);
    if (e == cudaSuccess && b->ns6)
      e = launch_batch_w6(b->d_smem6[par], b->d_sfirst, b->ns6, b->sthreads, b->sns, b->sstage, b->sgrid, b->st);
  }
  if (e != cudaSuccess || !b->nq) return e;
  const void* mem = b->d_mem[par];
  const int n = b->nq;
  if (b->group) return launch_batch_group<T>(mem, b->d_first, n, b->smem, b->tune.threads, b->grid, b->st);
  if (b->tma)
    return launch_batch_tma<T>(mem, b->d_first, n, b->smem, b->tune.threads, b->grid, b->max_nxy, b->st);
  return launch_batch<T>(mem, b->d_first, n, b->smem, b->tune.threads, b->grid, b->st);
}

// binary32 members whose planes fill the fully staged kernel's CTA form the
// persistent class; its arrays, stage size and grid
template <class T>
static int batch_build_persistent(rt_batch* b, std::vector<int>& rest) {
  const int n = (int)b->mem.size();
  rest.clear();
  b->np = 0;
  std::vector<int> pm;
  if (sizeof(T) == 4 && b->pthreads > 0) {
    int Rc = 0;
    for (int j = 0; j < n; j++) Rc = std::max(Rc, batch_w3_rows(b->mem[j]->d, b->pthreads, 0));
    for (int j = 0; j < n; j++)
      if (Rc > 0 && batch_w3_rows(b->mem[j]->d, b->pthreads, Rc) > 0) pm.push_back(j);
      else rest.push_back(j);
    long long stage = 0;
    for (int j : pm) stage = std::max(stage, batch_w3_stage_floats(b->mem[j]->d));
    const int ns = pm.empty() ? 0 : batch_w3_stages(stage);
    if (ns < 2) {   // no member, or the largest plane leaves no room for two stages
      for (int j : pm) rest.push_back(j);
      std::sort(rest.begin(), rest.end());
      pm.clear();
    } else {
      b->pR = Rc;
      b->pns = ns;
      b->pstage = stage;
    }
  } else {
    for (int j = 0; j < n; j++) rest.push_back(j);
  }
  if (pm.empty()) return RT_OK;
  std::vector<BatchMember<float>> arr[2];
  std::vector<long long> first(pm.size() + 1, 0);
  for (size_t i = 0; i < pm.size(); i++) {
    rt_handle* h = b->mem[pm[i]];
    for (int par = 0; par < 2; par++) {
      BatchMember<float> bm;
      bm.A = make_step_args<float>(h, par == 0 ? h->cur : 1 - h->cur);
      bm.S = make_sched(h->d, b->tune);
      arr[par].push_back(bm);
    }
    first[i + 1] = first[i] + (long long)h->d.n[2] * h->d.n[3] * h->d.n[4] * h->d.n[5];
    b->cur0[pm[i]] = h->cur;
  }
  for (int par = 0; par < 2; par++) {
    if (!b->d_pmem[par]) BCUDA_TRY(b, cudaMalloc(&b->d_pmem[par], (size_t)n * sizeof(BatchMember<float>)));
    BCUDA_TRY(b, cudaMemcpy(b->d_pmem[par], arr[par].data(), pm.size() * sizeof(BatchMember<float>),
                            cudaMemcpyHostToDevice));
  }
  if (!b->d_pfirst) BCUDA_TRY(b, cudaMalloc(&b->d_pfirst, (size_t)(n + 1) * sizeof(long long)));
  BCUDA_TRY(b, cudaMemcpy(b->d_pfirst, first.data(), first.size() * sizeof(long long), cudaMemcpyHostToDevice));
  const int per_sm = batch_w3_blocks_per_sm(b->pthreads, b->pR, batch_w3_smem(b->pns, b->pstage));
  if (per_sm < 1) return bfail(b, RT_ERR_CUDA, "batched staged kernel does not fit on an SM");
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  b->pgrid = (int)std::min<long long>(first.back(), (long long)per_sm * nsm);
  b->np = (int)pm.size();
  b->pcells = 0;
  for (int j : pm) b->pcells += b->mem[j]->d.ncell;
  return RT_OK;
}

// binary32 members left over by the persistent class whose small planes fit
// the z-slice staged kernel; its arrays, stage size and grid
template <class T>
static int batch_build_slices(rt_batch* b, std::vector<int>& rest) {
  const int n = (int)b->mem.size();
  b->ns6 = 0;
  const int want = b->slice_threads >= 0 ? b->slice_threads : b->pthreads;
  if (sizeof(T) != 4 || want <= 0) return RT_OK;
  const int nt = want >= 256 ? want : 256;
  std::vector<int> sm, left;
  std::vector<int> G;
  long long stage = 0;
  for (int j : rest) {
    const int g = w6_slices(b->mem[j]->d, nt);
    if (g > 0) {
      sm.push_back(j);
      G.push_back(g);
      stage = std::max(stage, w6_stage_floats(b->mem[j]->d, g));
    } else {
      left.push_back(j);
    }
  }
  const int ns = sm.empty() ? 0 : w6_stages(stage);
  if (ns < 2) return RT_OK;
  std::vector<BatchMember<float>> arr[2];
  std::vector<long long> first(sm.size() + 1, 0);
  for (size_t i = 0; i < sm.size(); i++) {
    rt_handle* h = b->mem[sm[i]];
    for (int par = 0; par < 2; par++) {
      BatchMember<float> bm;
      bm.A = make_step_args<float>(h, par == 0 ? h->cur : 1 - h->cur);
      bm.S = make_sched(h->d, b->tune, G[i]);
      arr[par].push_back(bm);
    }
    first[i + 1] = first[i] + (long long)((h->d.n[2] + G[i] - 1) / G[i]) * h->d.n[3] * h->d.n[4] * h->d.n[5];
    b->cur0[sm[i]] = h->cur;
  }
  for (int par = 0; par < 2; par++) {
    if (!b->d_smem6[par]) BCUDA_TRY(b, cudaMalloc(&b->d_smem6[par], (size_t)n * sizeof(BatchMember<float>)));
    BCUDA_TRY(b, cudaMemcpy(b->d_smem6[par], arr[par].data(), sm.size() * sizeof(BatchMember<float>),
                            cudaMemcpyHostToDevice));
  }
  if (!b->d_sfirst) BCUDA_TRY(b, cudaMalloc(&b->d_sfirst, (size_t)(n + 1) * sizeof(long long)));
  BCUDA_TRY(b, cudaMemcpy(b->d_sfirst, first.data(), first.size() * sizeof(long long), cudaMemcpyHostToDevice));
  const int per_sm = w6_blocks_per_sm(nt, w6_smem(ns, stage));
  if (per_sm < 1) return bfail(b, RT_ERR_CUDA, "batched z-slice kernel does not fit on an SM");
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  b->sgrid = (int)std::min<long long>(first.back(), (long long)per_sm * nsm);
  b->sns = ns;
  b->sstage = stage;
  b->sthreads = nt;
  b->ns6 = (int)sm.size();
  b->scells = 0;
  for (int j : sm) b->scells += b->mem[j]->d.ncell;
  rest = left;
  return RT_OK;
}

template <class T>
static int batch_build(rt_batch* b) {
  std::vector<int> qm;   // members of the plane / group / TMA class
  int rc = batch_build_persistent<T>(b, qm);
  if (rc) return rc;
  rc = batch_build_slices<T>(b, qm);
  if (rc) return rc;
  batch_plan_fused(b);
  const int n = (int)qm.size();
  b->nq = n;
  std::vector<BatchMember<T>> arr[2];
  std::vector<long long> first(n + 1, 0);
  size_t smem = 0;
  bool tma = true, group = true;
  b->max_nxy = 0;
  std::vector<int> gz(n, 1);
  for (int i = 0; i < n; i++) {
    const int j = qm[i];
    tma = tma && tma_path_ok<T>(b->mem[j]->d);
    gz[i] = group_size<T>(b->mem[j]->d, b->tune);
    group = group && gz[i] > 0;
    b->max_nxy = std::max(b->max_nxy, (long long)b->mem[j]->d.n[0] * b->mem[j]->d.n[1]);
  }
  // z-group items are preferred: they keep the CTA busy on small planes
  if (group) tma = false;
  // the TMA plane kernel covers the largest plane with at most RT_TMA_MAXC cells per thread
  if ((b->max_nxy + b->tune.threads - 1) / b->tune.threads > RT_TMA_MAXC) tma = false;
  // the plain-load batch kernel has no 1024-thread form
  if (!tma && !group && b->tune.threads > 512) b->tune.threads = 512;
  for (int i = 0; i < n; i++) {
    rt_handle* h = b->mem[qm[i]];
    StepTuning tn = b->tune;
    for (int par = 0; par < 2; par++) {
      BatchMember<T> bm;
      bm.A = make_step_args<T>(h, par == 0 ? h->cur : 1 - h->cur);
      bm.S = make_sched(h->d, tn, group ? gz[i] : 1);
      arr[par].push_back(bm);
    }
    first[i + 1] = first[i] + sched_items(h->d, arr[0].back().S);
    smem = std::max(smem, group ? group_path_smem<T>(h->d, gz[i])
                                : (tma ? tma_path_smem<T>(h->d) : plane_smem<T>(h->d)));
    b->cur0[qm[i]] = h->cur;
  }
  if (n > 0) {
    const int nall = (int)b->mem.size();
    for (int par = 0; par < 2; par++) {
      if (!b->d_mem[par]) BCUDA_TRY(b, cudaMalloc(&b->d_mem[par], (size_t)nall * sizeof(BatchMember<T>)));
      BCUDA_TRY(b, cudaMemcpy(b->d_mem[par], arr[par].data(), (size_t)n * sizeof(BatchMember<T>),
                              cudaMemcpyHostToDevice));
    }
    if (!b->d_first) BCUDA_TRY(b, cudaMalloc(&b->d_first, (size_t)(nall + 1) * sizeof(long long)));
    BCUDA_TRY(b, cudaMemcpy(b->d_first, first.data(), (size_t)(n + 1) * sizeof(long long),
                            cudaMemcpyHostToDevice));
    b->smem = smem;
    b->tma = tma;
    b->group = group;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = batch_blocks_per_sm<T>(b->tune.threads, smem, tma, group);
    if (per_sm < 1) return bfail(b, RT_ERR_CUDA, "batch kernel does not fit on an SM");
    const long long items = first[n];
    b->grid = (int)std::min<long long>(items, (long long)per_sm * nsm);
  }
  b->parity = 0;
  b->forced.clear();
  b->fgen.assign(b->mem.size(), 0);
  for (size_t j = 0; j < b->mem.size(); j++) {
    if (b->mem[j]->forcing != RT_FORCING_NONE) b->forced.push_back((int)j);
    b->fgen[j] = b->mem[j]->force_gen;
  }
  // capture graph_steps launches starting at each parity
  batch_free_graphs(b);
  for (int start = 0; start < 2; start++) {
    cudaGraph_t g;
    BCUDA_TRY(b, cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int t = 0; t < b->graph_steps && e == cudaSuccess; t++)
      e = batch_launch<T>(b, (start + t) & 1);
    cudaError_t e2 = cudaStreamEndCapture(b->st, &g);
    if (e != cudaSuccess || e2 != cudaSuccess)
      return bfail(b, RT_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    e = cudaGraphInstantiate(&b->gexec[start], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, RT_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  }
  b->dirty = false;
  return RT_OK;
}

template <class T>
static int batch_run(rt_batch* b, int nsteps) {
  const int n = (int)b->mem.size();
  for (int j = 0; j < n; j++)  // a member stepped on its own, or its forcing changed, since the build
    if (b->mem[j]->cur != (b->cur0[j] ^ b->parity) || b->fgen.size() != (size_t)n ||
        b->mem[j]->force_gen != b->fgen[j])
      b->dirty = true;
  // binary64 members: the batch kernels read uCFL, which a member's own fast
  // steps may have replaced (queued on the member's stream, ordered below)
  for (int j = 0; j < n; j++)
    if (b->mem[j]->p.precision == RT_FP64 && b->mem[j]->uc_holds != 0) {
      cudaError_t e = ensure_uc(b->mem[j], 0);
      if (e != cudaSuccess) return bfail(b, RT_ERR_CUDA, "uCFL: %s", cudaGetErrorString(e));
    }
  // the batch stream runs after everything queued on the members' streams
  for (int j = 0; j < n; j++) {
    BCUDA_TRY(b, cudaEventRecord(b->mem[j]->ev, b->mem[j]->st));
    BCUDA_TRY(b, cudaStreamWaitEvent(b->st, b->mem[j]->ev, 0));
  }
  if (b->dirty) {
    int rc = batch_build<T>(b);
    if (rc) return rc;
  }
  int left = nsteps;
  while (left >= b->graph_steps) {
    BCUDA_TRY(b, cudaGraphLaunch(b->gexec[b->parity], b->st));
    b->launches += (long long)b->graph_steps * batch_kernels(b);
    left -= b->graph_steps;  // graph_steps is even: parity unchanged
  }
  while (left > 0) {
    cudaError_t e = batch_launch<T>(b, b->parity);
    if (e != cudaSuccess) return bfail(b, RT_ERR_CUDA, "batch launch: %s", cudaGetErrorString(e));
    b->launches += batch_kernels(b);
    b->parity ^= 1;
    left -= 1;
  }
  // and later work on a member's own stream runs after the batch
  BCUDA_TRY(b, cudaEventRecord(b->ev, b->st));
  for (int j = 0; j < n; j++) {
    rt_handle* h = b->mem[j];
    BCUDA_TRY(b, cudaStreamWaitEvent(h->st, b->ev, 0));
    h->cur = b->cur0[j] ^ b->parity;
    h->steps_since_set += nsteps;
  }
  return RT_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int rt_batch_create(rt_handle* const* members, int n, rt_batch** out) {
  if (!members || n < 1 || !out) return bfail(nullptr, RT_ERR_ARG, "rt_batch_create: no members");
  *out = nullptr;
  const int prec = members[0]->p.precision;
  for (int j = 0; j < n; j++) {
    rt_handle* h = members[j];
    if (!h) return bfail(nullptr, RT_ERR_ARG, "rt_batch_create: member %d is NULL", j);
    if (h->p.precision != prec) return bfail(nullptr, RT_ERR_ARG, "rt_batch_create: mixed precisions");
    if (!h->have_coeff || !h->have_state)
      return bfail(nullptr, RT_ERR_STATE, "rt_batch_create: member %d needs rt_calc_parameter and rt_set_state", j);
    const bool ok = prec == RT_FP64 ? plane_ok<double>(h->d) : plane_ok<float>(h->d);
    if (!ok) return bfail(nullptr, RT_ERR_ARG, "rt_batch_create: member %d plane nx*ny too large", j);
    for (int k = 0; k < j; k++)
      if (members[k] == h) return bfail(nullptr, RT_ERR_ARG, "rt_batch_create: member %d repeated", j);
  }
  rt_batch* b = new rt_batch();
  b->mem.assign(members, members + n);
  b->cur0.assign(n, 0);
  b->fp64 = prec == RT_FP64;
  for (int j = 0; j < n; j++) b->cells += members[j]->d.ncell;
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming) != cudaSuccess) {
    delete b;
    return bfail(nullptr, RT_ERR_CUDA, "rt_batch_create: stream creation failed");
  }
  // members' own streams may still run setup work: order it before the batch
  for (int j = 0; j < n; j++) cudaStreamSynchronize(members[j]->st);
  *out = b;
  return RT_OK;
}

int rt_batch_destroy(rt_batch* b) {
  if (!b) return RT_OK;
  if (b->st) cudaStreamSynchronize(b->st);
  batch_free_graphs(b);
  for (int k = 0; k < 2; k++) {
    cudaFree(b->d_mem[k]);
    cudaFree(b->d_pmem[k]);
    cudaFree(b->d_smem6[k]);
  }
  cudaFree(b->d_first);
  cudaFree(b->d_pfirst);
  cudaFree(b->d_sfirst);
  if (b->ev) cudaEventDestroy(b->ev);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
  return RT_OK;
}

const char* rt_batch_last_error(const rt_batch* b) { return b ? b->err.c_str() : g_create_err.c_str(); }

int rt_batch_set_tuning(rt_batch* b, int band, int threads, int sweep, int graph_steps) {
  if (!b) return RT_ERR_ARG;
  if (band < 1 || band > 1024) return bfail(b, RT_ERR_ARG, "rt_batch_set_tuning: band %d out of range", band);
  if (threads != 128 && threads != 256 && threads != 512 && threads != 1024)
    return bfail(b, RT_ERR_ARG, "rt_batch_set_tuning: threads must be 128, 256, 512 or 1024");
  if (sweep != 0 && sweep != 1) return bfail(b, RT_ERR_ARG, "rt_batch_set_tuning: sweep must be 0 or 1");
  if (graph_steps < 2 || graph_steps % 2) return bfail(b, RT_ERR_ARG, "rt_batch_set_tuning: graph_steps must be even and >= 2");
  cudaStreamSynchronize(b->st);
  b->tune.band = band;
  b->tune.threads = threads;
  b->tune.sweep = sweep;
  b->graph_steps = graph_steps;
  b->dirty = true;
  return RT_OK;
}

int rt_batch_set_persistent(rt_batch* b, int threads) {
  if (!b) return RT_ERR_ARG;
  if (threads != 0 && threads != 128 && threads != 256 && threads != 512)
    return bfail(b, RT_ERR_ARG, "rt_batch_set_persistent: threads must be 0, 128, 256 or 512");
  cudaStreamSynchronize(b->st);
  b->pthreads = threads;
  b->dirty = true;
  return RT_OK;
}

int rt_batch_set_slices(rt_batch* b, int threads) {
  if (!b) return RT_ERR_ARG;
  if (threads != -1 && threads != 0 && threads != 256 && threads != 512)
    return bfail(b, RT_ERR_ARG, "rt_batch_set_slices: threads must be -1, 0, 256 or 512");
  cudaStreamSynchronize(b->st);
  b->slice_threads = threads;
  b->dirty = true;
  return RT_OK;
}

int rt_batch_set_fused(rt_batch* b, int on) {
  if (!b) return RT_ERR_ARG;
  if (on != 0 && on != 1) return bfail(b, RT_ERR_ARG, "rt_batch_set_fused: on must be 0 or 1");
  cudaStreamSynchronize(b->st);
  b->fuse = on;
  b->dirty = true;
  return RT_OK;
}
int rt_batch_persistent_members(rt_batch* b) {
  if (!b) return RT_ERR_ARG;
  if (b->dirty) {
    const int rc = b->fp64 ? batch_build<double>(b) : batch_build<float>(b);
    if (rc) return rc;
  }
  return b->np + b->ns6;
}

int rt_batch_integrate(rt_batch* b, int nsteps) {
  if (!b) return RT_ERR_ARG;
  if (nsteps < 0) return bfail(b, RT_ERR_ARG, "rt_batch_integrate: nsteps < 0");
  return b->fp64 ? batch_run<double>(b, nsteps) : batch_run<float>(b, nsteps);
}

int rt_batch_dry(rt_batch* b, int nsteps) {
  if (!b) return RT_ERR_ARG;
  const int n = (int)b->mem.size();
  for (int j = 0; j < n; j++) {
    BCUDA_TRY(b, cudaEventRecord(b->mem[j]->ev, b->mem[j]->st));
    BCUDA_TRY(b, cudaStreamWaitEvent(b->st, b->mem[j]->ev, 0));
    if (b->mem[j]->cur != (b->cur0[j] ^ b->parity)) b->dirty = true;
  }
  if (b->dirty) {
    int rc = b->fp64 ? batch_build<double>(b) : batch_build<float>(b);
    if (rc) return rc;
  }
  for (int t = 0; t < nsteps; t++) {
    cudaError_t e =
        b->fp64 ? batch_launch<double>(b, b->parity, false) : batch_launch<float>(b, b->parity, false);
    if (e != cudaSuccess) return bfail(b, RT_ERR_CUDA, "batch launch: %s", cudaGetErrorString(e));
    b->launches += batch_kernels(b) - (long long)b->forced.size();
  }
  BCUDA_TRY(b, cudaEventRecord(b->ev, b->st));
  for (int j = 0; j < n; j++) {
    BCUDA_TRY(b, cudaStreamWaitEvent(b->mem[j]->st, b->ev, 0));
    b->mem[j]->steps_since_set = 0;
  }
  return RT_OK;
}

int rt_batch_sync(rt_batch* b) {
  if (!b) return RT_ERR_ARG;
  BCUDA_TRY(b, cudaStreamSynchronize(b->st));
  for (rt_handle* h : b->mem)
    if (check_status(h)) return bfail(b, RT_ERR_CUDA, "member: %s", h->err.c_str());
  return RT_OK;
}

int rt_batch_stream(rt_batch* b, void** stream) {
  if (!b || !stream) return RT_ERR_ARG;
  *stream = (void*)b->st;
  return RT_OK;
}

long long rt_batch_launch_count(const rt_batch* b) { return b ? b->launches : 0; }
long long rt_batch_cells(const rt_batch* b) { return b ? b->cells : 0; }


int rt_selftest_wait_timeout(int* status, int* completed) {
  if (!status || !completed) return fail(nullptr, RT_ERR_ARG, "rt_selftest_wait_timeout: NULL argument");
  int* dev = nullptr;
  cudaError_t e = cudaMalloc(&dev, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(dev, 0, 2 * sizeof(int));
  if (e == cudaSuccess) e = launch_wait_probe(dev, dev + 1, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int host[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(host, dev, sizeof(host), cudaMemcpyDeviceToHost);
  if (dev) cudaFree(dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(nullptr, RT_ERR_CUDA, "rt_selftest_wait_timeout: %s", cudaGetErrorString(e));
  }
  *status = host[0];
  *completed = host[1];
  return RT_OK;
}

const char* rt_version(void) { return "raytracer_gb300 0.1 (sm_103a)"; }

const char* rt_last_error(const rt_handle* h) { return h ? h->err.c_str() : g_create_err.c_str(); }

int rt_create(const rt_dims* dims, const rt_params* params, rt_handle** out) {
  if (!dims || !params || !out) return fail(nullptr, RT_ERR_ARG, "rt_create: NULL argument");
  *out = nullptr;
  const int nn[6] = {dims->nx, dims->ny, dims->nz, dims->nk, dims->nl, dims->nm};
  for (int a = 0; a < 6; a++)
    if (nn[a] < 1) return fail(nullptr, RT_ERR_ARG, "rt_create: axis %d has %d points", a, nn[a]);
  if (dims->onx != RT_ONX)
    return fail(nullptr, RT_ERR_ARG, "rt_create: onx must be %d (main_module.f90:114), got %d",
                RT_ONX, dims->onx);
  // parallel_mpi.f90:16-25
  if (dims->nk > 1 && dims->nk % 2) return fail(nullptr, RT_ERR_ARG, " nk must be even or one ");
  if (dims->nl > 1 && dims->nl % 2) return fail(nullptr, RT_ERR_ARG, " nl must be even or one ");
  if (dims->nm > 1 && dims->nm % 2) return fail(nullptr, RT_ERR_ARG, " nm must be even or one");
  if (params->precision != RT_FP64 && params->precision != RT_FP32)
    return fail(nullptr, RT_ERR_ARG, "rt_create: unknown precision %d", params->precision);
  if (!(params->dt > 0.0)) return fail(nullptr, RT_ERR_ARG, "rt_create: dt must be > 0");
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    return fail(nullptr, RT_ERR_CUDA, "rt_create: no CUDA device: %s", cudaGetErrorString(ce));
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess || prop.major * 10 + prop.minor < 100) {
    cudaGetLastError();
    return fail(nullptr, RT_ERR_CUDA, "rt_create: device %d is not a Blackwell GPU", dev);
  }

  rt_handle* h = new rt_handle();
  h->p = *params;
  Dims& d = h->d;
  long long st = 1;
  for (int a = 0; a < 6; a++) {
    d.n[a] = nn[a];
    d.s[a] = st;
    st *= nn[a];
  }
  d.ncell = st;
  d.nvol3 = (long long)nn[0] * nn[1] * nn[2];
  d.nspec = (long long)nn[3] * nn[4] * nn[5];
  d.upper_refl = params->enable_upper_reflection ? 1 : 0;
  d.lower_refl = params->enable_lower_reflection ? 1 : 0;
  fill_plane_strides(d);
  h->elem = params->precision == RT_FP64 ? 8 : 4;

  auto bail = [&](int code) {
    g_create_err = h->err;
    rt_destroy(h);
    return code;
  };
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(fail(h, RT_ERR_CUDA, "rt_create: stream creation failed"));

  long long gl = 0;
  for (int a = 0; a < 6; a++) { h->goff[a] = gl; gl += padded_len(d, a); }
  for (int c = 0; c < 3; c++) { h->goff[6 + c] = gl; gl += padded_len(d, 3 + c); }
  long long tl = 0;
  for (int k = 0; k < 24; k++) { h->toff[k] = tl; tl += padded_len(d, k % 6); }
  h->bglen = padded_len(d, 0) * padded_len(d, 1) * padded_len(d, 2);
  int rc;
  if ((rc = dev_alloc(h, (void**)&h->grid, gl * sizeof(double)))) return bail(rc);
  if ((rc = dev_alloc(h, (void**)&h->tab32, tl * sizeof(float)))) return bail(rc);
  if ((rc = dev_alloc(h, (void**)&h->bg, 3 * h->bglen * sizeof(double)))) return bail(rc);
  const size_t fb = (size_t)d.ncell * h->elem;
  for (int k = 0; k < 2; k++)
    if ((rc = dev_alloc(h, &h->E[k], fb))) return bail(rc);
  for (int a = 0; a < 6; a++) {
    if ((rc = dev_alloc(h, &h->vel[a], fb))) return bail(rc);
    if ((rc = dev_alloc(h, &h->vlo[a], (size_t)(d.ncell / d.n[a]) * h->elem))) return bail(rc);
  }
  const int nlam = params->precision == RT_FP64 ? 3 : 1;
  for (int c = 0; c < nlam; c++)
    if ((rc = dev_alloc(h, &h->lam[c], fb))) return bail(rc);
  if (params->precision == RT_FP64)
    for (int a = 0; a < 6; a++) {
      if ((rc = dev_alloc(h, (void**)&h->uc[a], fb))) return bail(rc);
      if ((rc = dev_alloc(h, (void**)&h->ucl[a], (size_t)(d.ncell / d.n[a]) * 8))) return bail(rc);
    }
  const DiagSizes ds = diag_sizes(d);
  h->scratch_len = std::max(ds.scratch_doubles(), max_rate_partials(d)) + 8;
  if ((rc = dev_alloc(h, (void**)&h->scratch, h->scratch_len * sizeof(double)))) return bail(rc);
  if ((rc = dev_alloc(h, (void**)&h->vol3, 8 * d.nvol3 * sizeof(double)))) return bail(rc);
  if ((rc = dev_alloc(h, (void**)&h->result, 32 * sizeof(double)))) return bail(rc);
  if ((rc = dev_alloc(h, (void**)&h->status, sizeof(int)))) return bail(rc);
  if (cudaMemset(h->status, 0, sizeof(int)) != cudaSuccess) return bail(fail(h, RT_ERR_CUDA, "memset"));
  if ((rc = dev_alloc(h, (void**)&h->seed, 2 * sizeof(unsigned)))) return bail(rc);
  if (cudaMemset(h->seed, 0, 2 * sizeof(unsigned)) != cudaSuccess) return bail(fail(h, RT_ERR_CUDA, "memset"));
  *out = h;
  return RT_OK;
}

int rt_destroy(rt_handle* h) {
  if (!h) return RT_OK;
  if (h->st) cudaStreamSynchronize(h->st);
  cudaFree(h->grid);
  cudaFree(h->tab32);
  cudaFree(h->bg);
  for (int k = 0; k < 2; k++) cudaFree(h->E[k]);
  for (int a = 0; a < 6; a++) { cudaFree(h->vel[a]); cudaFree(h->vlo[a]); }
  for (int c = 0; c < 3; c++) cudaFree(h->lam[c]);
  for (int a = 0; a < 6; a++) { cudaFree(h->uc[a]); cudaFree(h->ucl[a]); }
  cudaFree(h->scratch);
  cudaFree(h->vol3);
  cudaFree(h->result);
  cudaFree(h->status);
  cudaFree(h->seed);
  cudaFree(h->force);
  for (int a = 0; a < 6; a++) { cudaFree(h->split.f[a]); cudaFree(h->split.f0[a]); }
  cudaFree(h->mu);
  cudaFree(h->tab64);
  for (auto& kv : h->timers) {
    if (kv.second.open) cudaEventDestroy(kv.second.open);
    for (auto& pr : kv.second.pairs) {
      cudaEventDestroy(pr.first);
      cudaEventDestroy(pr.second);
    }
  }
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->ev) cudaEventDestroy(h->ev);
  if (h->st) cudaStreamDestroy(h->st);
  delete h;
  return RT_OK;
}

int rt_set_grid(rt_handle* h, const double* dxt, const double* dyt, const double* dzt,
                const double* dkt, const double* dlt, const double* dmt, const double* kt,
                const double* lt, const double* mt) {
  if (!h) return RT_ERR_ARG;
  const double* src[9] = {dxt, dyt, dzt, dkt, dlt, dmt, kt, lt, mt};
  for (int k = 0; k < 9; k++) {
    if (!src[k]) return fail(h, RT_ERR_ARG, "rt_set_grid: array %d is NULL", k);
    const int a = k < 6 ? k : k - 3;
    const long long n = padded_len(h->d, a);
    if (k < 6)
      for (long long i = 0; i < n; i++)
        if (!(src[k][i] > 0.0))
          return fail(h, RT_ERR_GRID, "rt_set_grid: spacing %d at padded index %lld is not > 0", k, i);
    CUDA_TRY(h, cudaMemcpy(h->grid + h->goff[k], src[k], n * sizeof(double), cudaMemcpyHostToDevice));
  }
  h->dzt1 = dzt[pidx(1)];
  int rc = upload_tab32(h);
  if (rc) return rc;
  h->have_grid = true;
  h->have_coeff = false;
  return RT_OK;
}

int rt_set_background(rt_handle* h, const double* Nsqr, const double* U, const double* V) {
  if (!h) return RT_ERR_ARG;
  if (!Nsqr || !U || !V) return fail(h, RT_ERR_ARG, "rt_set_background: NULL array");
  const double* src[3] = {Nsqr, U, V};
  for (int k = 0; k < 3; k++)
    CUDA_TRY(h, cudaMemcpy(h->bg + k * h->bglen, src[k], h->bglen * sizeof(double),
                           cudaMemcpyHostToDevice));
  h->have_bg = true;
  h->have_coeff = false;
  return RT_OK;
}

int rt_set_dt(rt_handle* h, double dt) {
  if (!h) return RT_ERR_ARG;
  if (!(dt > 0.0)) return fail(h, RT_ERR_ARG, "rt_set_dt: dt must be > 0");
  h->p.dt = dt;
  if (h->have_grid) {
    int rc = upload_tab32(h);
    if (rc) return rc;
  }
  return refresh_ucfl(h);
}

int rt_calc_parameter(rt_handle* h) {
  if (!h) return RT_ERR_ARG;
  if (!h->have_grid || !h->have_bg)
    return fail(h, RT_ERR_STATE, "rt_calc_parameter: rt_set_grid and rt_set_background first");
  const Dims& d = h->d;
  Background bg;
  bg.Nsqr = h->bg;
  bg.U = h->bg + h->bglen;
  bg.V = h->bg + 2 * h->bglen;
  bg.px = (int)padded_len(d, 0);
  bg.py = (int)padded_len(d, 1);
  Phys ph{h->p.f0, h->p.sign_of_omega_i, h->p.dt};
  const Grid g = make_grid(h);

  CoeffOut64 o64{};
  std::vector<void*> tmp;
  const bool fp64 = h->p.precision == RT_FP64;
  int rc;
  // binary64 destinations: the handle's own fields (FP64) or temporaries
  for (int a = 0; a < 6; a++) {
    if (fp64) {
      o64.vel[a] = (double*)h->vel[a];
      o64.vlo[a] = (double*)h->vlo[a];
    } else {
      void* p1 = nullptr; void* p2 = nullptr;
      if ((rc = tmp_alloc(h, &p1, d.ncell * sizeof(double)))) goto cleanup;
      tmp.push_back(p1);
      if ((rc = tmp_alloc(h, &p2, (d.ncell / d.n[a]) * sizeof(double)))) goto cleanup;
      tmp.push_back(p2);
      o64.vel[a] = (double*)p1;
      o64.vlo[a] = (double*)p2;
    }
  }
  for (int c = 0; c < 3; c++) {
    if (fp64) {
      o64.lam[c] = (double*)h->lam[c];
    } else {
      void* p1 = nullptr;
      if ((rc = tmp_alloc(h, &p1, d.ncell * sizeof(double)))) goto cleanup;
      tmp.push_back(p1);
      o64.lam[c] = (double*)p1;
    }
  }
  {
    cudaError_t e = launch_coeff(d, bg, g, ph, o64, h->st);
    h->launches += 7;
    if (e != cudaSuccess) { rc = fail(h, RT_ERR_CUDA, "coefficients: %s", cudaGetErrorString(e)); goto cleanup; }
    ConstCoeff64 cf;
    for (int a = 0; a < 6; a++) { cf.vel[a] = o64.vel[a]; cf.vlo[a] = o64.vlo[a]; }
    e = launch_max_rate(d, g, cf, h->scratch, h->result, h->st);
    h->launches += 2;
    if (e != cudaSuccess) { rc = fail(h, RT_ERR_CUDA, "max rate: %s", cudaGetErrorString(e)); goto cleanup; }
    if (!fp64) {
      for (int a = 0; a < 6; a++) {
        if ((e = launch_to_fp32(o64.vel[a], (float*)h->vel[a], d.ncell, h->st)) != cudaSuccess) break;
        if ((e = launch_to_fp32(o64.vlo[a], (float*)h->vlo[a], d.ncell / d.n[a], h->st)) != cudaSuccess) break;
        h->launches += 2;
      }
      if (e == cudaSuccess)
        e = launch_lam_combine(o64.lam[0], o64.lam[1], o64.lam[2], d.n[0] > 1, d.n[1] > 1,
                               d.n[2] > 1, (float*)h->lam[0], d.ncell, h->st);
      h->launches += 1;
      if (e != cudaSuccess) { rc = fail(h, RT_ERR_CUDA, "fp32 conversion: %s", cudaGetErrorString(e)); goto cleanup; }
    }
    e = cudaMemcpyAsync(&h->rate, h->result, sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) { rc = fail(h, RT_ERR_CUDA, "calc_parameter: %s", cudaGetErrorString(e)); goto cleanup; }
  }
  h->have_coeff = true;
  rc = refresh_ucfl(h);
cleanup:
  // stream-ordered frees run after the kernels that read the temporaries
  for (void* p : tmp) { cudaFreeAsync(p, h->st); }
  cudaStreamSynchronize(h->st);
  return rc;
}

int rt_max_rate(rt_handle* h, double* rate) {
  if (!h || !rate) return RT_ERR_ARG;
  if (!h->have_coeff) return fail(h, RT_ERR_STATE, "rt_max_rate: rt_calc_parameter first");
  *rate = h->rate;
  return RT_OK;
}

static int ensure_pinned(rt_handle* h) {
  if (h->pinned) return RT_OK;
  cudaError_t e = cudaHostAlloc(&h->pinned, (size_t)h->d.ncell * 8, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    h->pinned = nullptr;
    return fail(h, RT_ERR_NOMEM, "pinned staging allocation failed: %s", cudaGetErrorString(e));
  }
  return RT_OK;
}

int rt_get_field(rt_handle* h, int which, double* out) {
  if (!h || !out) return RT_ERR_ARG;
  if (!h->have_coeff) return fail(h, RT_ERR_STATE, "rt_get_field: rt_calc_parameter first");
  const Dims& d = h->d;
  const bool fp64 = h->p.precision == RT_FP64;
  const void* src = nullptr;
  if (which >= RT_F_XDOT && which <= RT_F_MDOT) src = h->vel[which];
  else if (which >= RT_F_LAMBDA_X && which <= RT_F_LAMBDA_Z && fp64) src = h->lam[which - RT_F_LAMBDA_X];
  else if (which == RT_F_LAMBDA && !fp64) src = h->lam[0];
  else return fail(h, RT_ERR_ARG, "rt_get_field: field %d not available in this precision", which);
  int rc = ensure_pinned(h);
  if (rc) return rc;
  CUDA_TRY(h, cudaMemcpyAsync(h->pinned, src, (size_t)d.ncell * h->elem, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  if (fp64) scatter_interior<double>(d, (const double*)h->pinned, out);
  else scatter_interior<float>(d, (const float*)h->pinned, out);
  if (which <= RT_F_MDOT) {
    // face 0 of the velocity's own axis lives in the plane vlo[a]
    const int a = which;
    const long long np = d.ncell / d.n[a];
    std::vector<double> pl(np);
    if (fp64) {
      CUDA_TRY(h, cudaMemcpy(pl.data(), h->vlo[a], np * 8, cudaMemcpyDeviceToHost));
    } else {
      std::vector<float> pf(np);
      CUDA_TRY(h, cudaMemcpy(pf.data(), h->vlo[a], np * 4, cudaMemcpyDeviceToHost));
      for (long long q = 0; q < np; q++) pl[q] = pf[q];
    }
    long long P[6];
    for (int b = 0; b < 6; b++) P[b] = padded_len(d, b);
    for (long long q = 0; q < np; q++) {
      long long r = q, idx = 0, stp = 1;
      for (int b = 0; b < 6; b++) {
        int f;  // Fortran index
        if (b == a) f = 0;
        else { f = (int)(r % d.n[b]) + 1; r /= d.n[b]; }
        idx += (long long)(f + RT_ONX - 1) * stp;
        stp *= P[b];
      }
      out[idx] = pl[q];
    }
  }
  return RT_OK;
}

// true when host arrays are moved by the GPU through the host's page tables
static bool use_host_direct(rt_handle* h) {
  if (!h->host_direct) return false;
  if (h->pageable < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    h->pageable = (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && v) ? 1 : 0;
  }
  return h->pageable == 1;
}

int rt_set_state(rt_handle* h, const double* E) {
  if (!h || !E) return RT_ERR_ARG;
  const Dims& d = h->d;
  if (use_host_direct(h)) {
    h->cur = 0;
    cudaError_t e = h->p.precision == RT_FP64 ? launch_host_gather<double>(E, (double*)h->E[0], d, h->st)
                                              : launch_host_gather<float>(E, (float*)h->E[0], d, h->st);
    if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "host gather: %s", cudaGetErrorString(e));
    h->launches += 1;
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    h->have_state = true;
    h->steps_since_set = 0;
    return RT_OK;
  }
  int rc = ensure_pinned(h);
  if (rc) return rc;
  if (h->p.precision == RT_FP64) gather_interior<double>(d, E, (double*)h->pinned);
  else gather_interior<float>(d, E, (float*)h->pinned);
  h->cur = 0;
  CUDA_TRY(h, cudaMemcpyAsync(h->E[0], h->pinned, (size_t)d.ncell * h->elem, cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  h->have_state = true;
  h->steps_since_set = 0;
  return RT_OK;
}

int rt_get_state(rt_handle* h, double* E) {
  if (!h || !E) return RT_ERR_ARG;
  if (!h->have_state) return fail(h, RT_ERR_STATE, "rt_get_state: no state (rt_set_state first)");
  const Dims& d = h->d;
  if (use_host_direct(h)) {
    cudaError_t e = h->p.precision == RT_FP64
                        ? launch_host_scatter<double>((const double*)h->E[h->cur], E, d, h->st)
                        : launch_host_scatter<float>((const float*)h->E[h->cur], E, d, h->st);
    if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "host scatter: %s", cudaGetErrorString(e));
    h->launches += 1;
    CUDA_TRY(h, cudaStreamSynchronize(h->st));
    return check_status(h);
  }
  int rc = ensure_pinned(h);
  if (rc) return rc;
  CUDA_TRY(h, cudaMemcpyAsync(h->pinned, h->E[h->cur], (size_t)d.ncell * h->elem, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  if ((rc = check_status(h))) return rc;
  if (h->p.precision == RT_FP64) scatter_interior<double>(d, (const double*)h->pinned, E);
  else scatter_interior<float>(d, (const float*)h->pinned, E);
  return RT_OK;
}

int rt_set_state_interior(rt_handle* h, const void* E) {
  if (!h || !E) return RT_ERR_ARG;
  h->cur = 0;
  CUDA_TRY(h, cudaMemcpyAsync(h->E[0], E, (size_t)h->d.ncell * h->elem, cudaMemcpyHostToDevice, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  h->have_state = true;
  h->steps_since_set = 0;
  return RT_OK;
}

int rt_get_state_interior(rt_handle* h, void* E) {
  if (!h || !E) return RT_ERR_ARG;
  if (!h->have_state) return fail(h, RT_ERR_STATE, "rt_get_state_interior: no state (rt_set_state first)");
  CUDA_TRY(h, cudaMemcpyAsync(E, h->E[h->cur], (size_t)h->d.ncell * h->elem, cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  return check_status(h);
}

int rt_set_host_access(rt_handle* h, int direct) {
  if (!h || (direct != 0 && direct != 1)) return RT_ERR_ARG;
  h->host_direct = direct;
  return RT_OK;
}

int rt_host_direct(rt_handle* h) {
  if (!h) return RT_ERR_ARG;
  return use_host_direct(h) ? 1 : 0;
}

int rt_set_forcing(rt_handle* h, int kind, const double* F) {
  if (!h) return RT_ERR_ARG;
  if (kind != RT_FORCING_NONE && kind != RT_FORCING_FLUX && kind != RT_FORCING_RELAX)
    return fail(h, RT_ERR_ARG, "rt_set_forcing: unknown kind %d", kind);
  if (kind != RT_FORCING_NONE && !F) return fail(h, RT_ERR_ARG, "rt_set_forcing: NULL forcing field");
  const Dims& d = h->d;
  const long long nplane = (long long)d.n[0] * d.n[1] * d.nspec;
  // the work on the stream may still read the old field
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  h->force_gen += 1;
  h->forcing = RT_FORCING_NONE;
  if (kind == RT_FORCING_NONE) return RT_OK;
  if (!h->force) {
    int rc = dev_alloc(h, (void**)&h->force, (size_t)nplane * sizeof(double));
    if (rc) return rc;
  }
  // interior of the padded 5D field (x,y,k,l,m), x fastest
  const long long P0 = padded_len(d, 0), P1 = padded_len(d, 1), P3 = padded_len(d, 3), P4 = padded_len(d, 4);
  std::vector<double> f((size_t)nplane);
  long long q = 0;
  for (int m = 0; m < d.n[5]; m++)
    for (int n = 0; n < d.n[4]; n++)
      for (int l = 0; l < d.n[3]; l++)
        for (int j = 0; j < d.n[1]; j++) {
          const double* row =
              F + RT_ONX + P0 * ((j + RT_ONX) + P1 * ((l + RT_ONX) + P3 * ((n + RT_ONX) + P4 * (long long)(m + RT_ONX))));
          std::memcpy(&f[(size_t)q], row, (size_t)d.n[0] * sizeof(double));
          q += d.n[0];
        }
  CUDA_TRY(h, cudaMemcpy(h->force, f.data(), f.size() * sizeof(double), cudaMemcpyHostToDevice));
  h->forcing = kind;
  return RT_OK;
}

int rt_integrate(rt_handle* h, int nsteps) {
  if (!h) return RT_ERR_ARG;
  if (nsteps < 0) return fail(h, RT_ERR_ARG, "rt_integrate: nsteps < 0");
  if (!h->have_coeff) return fail(h, RT_ERR_STATE, "rt_integrate: rt_calc_parameter first");
  if (!h->have_state) return fail(h, RT_ERR_STATE, "rt_integrate: rt_set_state first");
  for (int t = 0; t < nsteps; t++) {
    cudaError_t e;
    if (h->forcing != RT_FORCING_NONE) {
      e = apply_forcing(h, h->cur, h->st);
      h->launches += 1;
      if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "forcing launch: %s", cudaGetErrorString(e));
    }
    int nl = 1;
    e = step_once(h, h->cur, &nl);
    h->launches += nl;
    if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
    h->cur = 1 - h->cur;
    h->steps_since_set += 1;
  }
  return RT_OK;
}

int rt_step_dry(rt_handle* h, int nsteps) {
  if (!h) return RT_ERR_ARG;
  if (nsteps < 0) return fail(h, RT_ERR_ARG, "rt_step_dry: nsteps < 0");
  if (!h->have_coeff || !h->have_state) return fail(h, RT_ERR_STATE, "rt_step_dry: no state");
  for (int t = 0; t < nsteps; t++) {
    int nl = 1;
    const cudaError_t e = step_once(h, h->cur, &nl);
    h->launches += nl;
    if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "step launch: %s", cudaGetErrorString(e));
  }
  // the other buffer now holds E after one step; the state itself is unchanged,
  // but a following rt_diagnose must not pair it with the old state
  h->steps_since_set = 0;
  return RT_OK;
}

int rt_integrate_host(rt_handle* h, double* E) {
  int rc = rt_set_state(h, E);
  if (rc) return rc;
  if ((rc = rt_integrate(h, 1))) return rc;
  return rt_get_state(h, E);
}

int rt_diagnose(rt_handle* h, rt_budget* o, double* E_int, double* meanfl_int, double* diss_ks,
                double* diss_ke, double* diss_ls, double* diss_le, double* diss_ms,
                double* diss_me) {
  if (!h || !o) return RT_ERR_ARG;
  if (!h->have_state || h->steps_since_set < 1)
    return fail(h, RT_ERR_STATE, "rt_diagnose: needs a step since rt_set_state (diagnose follows integrate, main.f90:70-74)");
  const Dims& d = h->d;
  const int prev = 1 - h->cur;  // state before the last step
  cudaError_t e;
  if (h->p.precision == RT_FP64)
    e = launch_diag<double>(make_step_args<double>(h, prev), (const double*)h->E[h->cur], h->scratch,
                            h->vol3, h->result, h->st);
  else
    e = launch_diag<float>(make_step_args<float>(h, prev), (const float*)h->E[h->cur], h->scratch,
                           h->vol3, h->result, h->st);
  h->launches += 4;
  if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "diagnose launch: %s", cudaGetErrorString(e));
  double r[DIAG_RESULT_NV];
  CUDA_TRY(h, cudaMemcpyAsync(r, h->result, sizeof(r), cudaMemcpyDeviceToHost, h->st));
  std::vector<double> v3((size_t)8 * d.nvol3);
  CUDA_TRY(h, cudaMemcpyAsync(v3.data(), h->vol3, v3.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  {
    int rc = check_status(h);
    if (rc) return rc;
  }
  o->eint = r[0]; o->mflint = r[1]; o->mfl_max = r[2];
  o->umax = r[3]; o->vmax = r[4]; o->wmax = r[5]; o->kmax = r[6]; o->lmax = r[7]; o->mmax = r[8];
  double* b = &o->bfl_xs;
  for (int k = 0; k < 12; k++) b[k] = r[DIAG_CELL_NV + k];
  // CFL, diagnose.f90:295-313
  const double vmx[6] = {o->umax, o->vmax, o->wmax, o->kmax, o->lmax, o->mmax};
  double* cfl = &o->cfl_x;
  std::vector<double> hg(h->goff[8] + padded_len(d, 5));
  CUDA_TRY(h, cudaMemcpy(hg.data(), h->grid, hg.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int a = 0; a < 6; a++) {
    double c = 0;
    for (int i = 1; i <= d.n[a]; i++) {
      const double x = vmx[a] * h->p.dt / hg[h->goff[a] + i + RT_ONX - 1];
      c = c > x ? c : x;
    }
    cfl[a] = c;
  }
  // diagnose.f90:327-328
  o->residual = o->eint + o->mflint + o->bfl_xe + o->bfl_ye + o->bfl_ze + o->bfl_ke + o->bfl_le +
                o->bfl_me - o->bfl_xs - o->bfl_ys - o->bfl_zs - o->bfl_ks - o->bfl_ls - o->bfl_ms;
  double* outs[8] = {E_int, meanfl_int, diss_ks, diss_ke, diss_ls, diss_le, diss_ms, diss_me};
  const long long P0 = padded_len(d, 0), P1 = padded_len(d, 1);
  for (int f = 0; f < 8; f++) {
    if (!outs[f]) continue;
    for (long long q = 0; q < d.nvol3; q++) {
      const int i = (int)(q % d.n[0]), j = (int)((q / d.n[0]) % d.n[1]), k = (int)(q / ((long long)d.n[0] * d.n[1]));
      outs[f][(i + RT_ONX) + P0 * ((j + RT_ONX) + P1 * (long long)(k + RT_ONX))] = v3[(size_t)f * d.nvol3 + q];
    }
  }
  return RT_OK;
}

int rt_get_tendency(rt_handle* h, double* dE, double* meanfl) {
  if (!h) return RT_ERR_ARG;
  if (!dE || !meanfl) return fail(h, RT_ERR_ARG, "rt_get_tendency: NULL array");
  if (!h->have_state || h->steps_since_set < 1)
    return fail(h, RT_ERR_STATE, "rt_get_tendency: needs a step since rt_set_state");
  const Dims& d = h->d;
  const int prev = 1 - h->cur;  // the state the last step started from
  void* dev[2] = {nullptr, nullptr};
  int rc = RT_OK;
  std::vector<double> buf;
  double* outs[2] = {dE, meanfl};
  cudaError_t e;
  for (int k = 0; k < 2 && !rc; k++) rc = tmp_alloc(h, &dev[k], (size_t)d.ncell * sizeof(double));
  if (rc) goto cleanup;
  if (h->p.precision == RT_FP64)
    e = launch_tendency<double>(make_step_args<double>(h, prev), (double*)dev[0], (double*)dev[1], h->st);
  else
    e = launch_tendency<float>(make_step_args<float>(h, prev), (double*)dev[0], (double*)dev[1], h->st);
  h->launches += 1;
  if (e != cudaSuccess) {
    rc = fail(h, RT_ERR_CUDA, "tendency launch: %s", cudaGetErrorString(e));
    goto cleanup;
  }
  buf.resize((size_t)d.ncell);
  for (int k = 0; k < 2; k++) {
    e = cudaMemcpyAsync(buf.data(), dev[k], buf.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) {
      rc = fail(h, RT_ERR_CUDA, "rt_get_tendency: %s", cudaGetErrorString(e));
      goto cleanup;
    }
    scatter_interior(d, buf.data(), outs[k]);
  }
cleanup:
  for (void* p : dev)
    if (p) cudaFreeAsync(p, h->st);
  return rc;
}

int rt_tic(rt_handle* h, const char* name) {
  if (!h) return RT_ERR_ARG;
  if (!name || !*name) return fail(h, RT_ERR_ARG, "rt_tic: empty timer name");
  rt_handle::Timer& t = h->timers[name];
  if (t.open) return fail(h, RT_ERR_STATE, "rt_tic: timer '%s' is already running", name);
  cudaEvent_t e;
  CUDA_TRY(h, cudaEventCreate(&e));
  const cudaError_t r = cudaEventRecord(e, h->st);
  if (r != cudaSuccess) {
    cudaEventDestroy(e);
    return fail(h, RT_ERR_CUDA, "rt_tic: %s", cudaGetErrorString(r));
  }
  t.open = e;
  return RT_OK;
}

int rt_toc(rt_handle* h, const char* name) {
  if (!h) return RT_ERR_ARG;
  if (!name) return fail(h, RT_ERR_ARG, "rt_toc: NULL timer name");
  auto it = h->timers.find(name);
  if (it == h->timers.end() || !it->second.open)
    return fail(h, RT_ERR_STATE, "rt_toc: timer '%s' was not started", name);
  cudaEvent_t e;
  CUDA_TRY(h, cudaEventCreate(&e));
  const cudaError_t r = cudaEventRecord(e, h->st);
  if (r != cudaSuccess) {
    cudaEventDestroy(e);
    return fail(h, RT_ERR_CUDA, "rt_toc: %s", cudaGetErrorString(r));
  }
  it->second.pairs.emplace_back(it->second.open, e);
  it->second.open = nullptr;
  it->second.calls += 1;
  return RT_OK;
}

int rt_timing_secs(rt_handle* h, const char* name, double* secs, long long* calls) {
  if (!h) return RT_ERR_ARG;
  if (!name || !secs) return fail(h, RT_ERR_ARG, "rt_timing_secs: NULL argument");
  auto it = h->timers.find(name);
  if (it == h->timers.end()) {
    *secs = 0.0;
    if (calls) *calls = 0;
    return RT_OK;
  }
  rt_handle::Timer& t = it->second;
  size_t used = 0;  // pairs folded into secs and destroyed
  cudaError_t e = cudaSuccess;
  for (; used < t.pairs.size(); used++) {
    float ms = 0.f;
    e = cudaEventSynchronize(t.pairs[used].second);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t.pairs[used].first, t.pairs[used].second);
    if (e != cudaSuccess) break;
    t.secs += ms * 1e-3;
    cudaEventDestroy(t.pairs[used].first);
    cudaEventDestroy(t.pairs[used].second);
  }
  t.pairs.erase(t.pairs.begin(), t.pairs.begin() + (long)used);
  if (e != cudaSuccess) return fail(h, RT_ERR_CUDA, "rt_timing_secs: %s", cudaGetErrorString(e));
  *secs = t.secs;
  if (calls) *calls = t.calls;
  return RT_OK;
}

int rt_set_tuning(rt_handle* h, int variant, int band, int threads) {
  if (!h) return RT_ERR_ARG;
  if (variant != RT_VARIANT_PLANE && variant != RT_VARIANT_CELL && variant != RT_VARIANT_TMA &&
      variant != RT_VARIANT_GROUP && variant != RT_VARIANT_W3 && variant != RT_VARIANT_W6 &&
      variant != RT_VARIANT_W2Z && variant != RT_VARIANT_W2Q &&
      variant != RT_VARIANT_SPLIT &&
      variant != RT_VARIANT_FAST)
    return fail(h, RT_ERR_ARG, "rt_set_tuning: unknown variant %d", variant);
  if (band < 1 || band > 1024) return fail(h, RT_ERR_ARG, "rt_set_tuning: band %d out of range", band);
  if (threads != 128 && threads != 256 && threads != 512 && threads != 1024)
    return fail(h, RT_ERR_ARG, "rt_set_tuning: threads must be 128, 256, 512 or 1024");
  if (variant == RT_VARIANT_SPLIT && h->p.precision == RT_FP64) {
    const int rc = ensure_split(h);
    if (rc) return rc;
  }
  if (variant == RT_VARIANT_FAST && h->p.precision == RT_FP64) {
    const int rc = ensure_fast(h);
    if (rc) return rc;
  }
  h->tune.variant = variant;
  h->tune.band = band;
  h->tune.threads = threads;
  return RT_OK;
}

int rt_set_schedule_sweep(rt_handle* h, int sweep) {
  if (!h) return RT_ERR_ARG;
  if (sweep != 0 && sweep != 1) return fail(h, RT_ERR_ARG, "rt_set_schedule_sweep: sweep must be 0 or 1");
  h->tune.sweep = sweep;
  return RT_OK;
}

int rt_sync(rt_handle* h) {
  if (!h) return RT_ERR_ARG;
  CUDA_TRY(h, cudaStreamSynchronize(h->st));
  return check_status(h);
}

int rt_stream(rt_handle* h, void** stream) {
  if (!h || !stream) return RT_ERR_ARG;
  *stream = (void*)h->st;
  return RT_OK;
}

long long rt_launch_count(const rt_handle* h) { return h ? h->launches : 0; }
long long rt_cells(const rt_handle* h) { return h ? h->d.ncell : 0; }
long long rt_device_bytes(const rt_handle* h) { return h ? h->bytes : 0; }

}  // extern "C"
