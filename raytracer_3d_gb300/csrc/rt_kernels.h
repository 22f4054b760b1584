// rt_kernels.h -- host-visible launchers of the sm_103a kernels.
#pragma once
#include <cuda_runtime.h>

#include "rt_common.cuh"

namespace rt {

struct Phys;
template <class T> struct StepArgs;

// binary32 literal 1e-12 of diagnose.f90:56, widened to binary64
#define RT_LIT_1EM12 9.9999999600419720e-13

// number of per-block values of the cell reduction: eint, mflint, mfl_max,
// umax, vmax, wmax, kmax, lmax, mmax
#define DIAG_CELL_NV 9
// result vector of launch_diag: DIAG_CELL_NV cell values, then
// bfl_xs, bfl_xe, bfl_ys, bfl_ye, ..., bfl_ms, bfl_me
#define DIAG_RESULT_NV (DIAG_CELL_NV + 12)

struct CoeffOut64 {
  double* vel[6];
  double* vlo[6];
  double* lam[3];
};

struct ConstCoeff64 {
  const double* vel[6];
  const double* vlo[6];
};

struct DiagSizes {
  long long cell_blocks;
  long long plane_blocks;
  long long scratch_doubles() const { return cell_blocks * DIAG_CELL_NV + 6 * plane_blocks * 2; }
};

// grid spacing of 0-based cell c along axis a
__host__ __device__ __forceinline__ double g_d(const Grid& g, int a, int c) { return g.d[a][pidx(c + 1)]; }

cudaError_t launch_coeff(const Dims& d, const Background& bg, const Grid& g, const Phys& ph,
                         const CoeffOut64& out, cudaStream_t st);
long long max_rate_partials(const Dims& d);
cudaError_t launch_max_rate(const Dims& d, const Grid& g, const ConstCoeff64& cf, double* partial,
                            double* out, cudaStream_t st);
cudaError_t launch_to_fp32(const double* src, float* dst, long long n, cudaStream_t st);
// padded host array (pageable, read / written by the GPU directly) <-> the
// unpadded device field
template <class T>
cudaError_t launch_host_gather(const double* host, T* dst, const Dims& d, cudaStream_t st);
template <class T>
cudaError_t launch_host_scatter(const T* src, double* host, const Dims& d, cudaStream_t st);
cudaError_t launch_ucfl(const Dims& d, const Grid& g, double dt, const double* const* vel,
                        const double* const* vlo, double* const* uc, double* const* ucl,
                        cudaStream_t st);
cudaError_t launch_lam_combine(const double* lx, const double* ly, const double* lz, int ux, int uy,
                               int uz, float* dst, long long n, cudaStream_t st);
// step kernel variants (numbers are the rt_set_tuning codes): the
// plane-tiled kernel (rt_step2.cuh), the one-thread-per-cell kernel
// (rt_step.cuh), kept as the fallback for planes that do not fit in shared
// memory, the TMA-staged plane and z-group kernels (rt_step3.cuh,
// rt_step4.cuh) and the persistent binary32 kernels (rt_step7.cuh,
// rt_step8.cuh, rt_step11.cuh).  Codes 4-8 and 10-12 belonged to earlier
// binary32 kernels that were measured slower and removed.
#define RT_VARIANT_PLANE 0
#define RT_VARIANT_CELL 1
#define RT_VARIANT_TMA 2
#define RT_VARIANT_GROUP 3
#define RT_VARIANT_W3 9       // binary32: every operand staged by TMA
#define RT_VARIANT_W6 13      // binary32: small planes, z slices per item
#define RT_VARIANT_W2Z 14     // binary32: 2-wide blocks, z-march
#define RT_VARIANT_W2Q 18     // the same with the cell-pair arithmetic on packed f32x2 instructions and
                              // the next plane's operands prefetched into L2 (the binary32 production step)
#define RT_VARIANT_SPLIT 15   // binary64: every face flux once, two passes (rt_split.cu)
#define RT_VARIANT_FAST 16    // binary64: two passes without divisions (rt_fast.cu), within 1e-12 of the reference
struct StepTuning {
  int variant = RT_VARIANT_TMA;
  int band = 8;       // values per band of the plane schedule
  int threads = 512;  // CTA size of the plane kernels (128, 256, 512)
  int sweep = 0;      // 0: bands over m, 1: bands over l
  int group = 0;      // z planes per item of the group kernel (0: from the CTA size)
};
struct PlaneSched;
PlaneSched make_sched(const Dims& d, const StepTuning& tn);
PlaneSched make_sched(const Dims& d, const StepTuning& tn, int gz);
long long sched_items(const Dims& d, const PlaneSched& S);
template <class T>
bool plane_ok(const Dims& d);
template <class T>
size_t plane_smem(const Dims& d);
// batched ensemble (members: device array of BatchMember<T>)
template <class T>
cudaError_t launch_batch(const void* members, const long long* first, int nmem, size_t smem,
                         int threads, int grid, cudaStream_t st);
template <class T>
int batch_blocks_per_sm(int threads, size_t smem, bool tma, bool group = false);
// group kernel: z planes per item for a CTA of `threads` (0 if the kernel cannot run)
template <class T>
int group_size(const Dims& d, const StepTuning& tn);
template <class T>
size_t group_path_smem(const Dims& d, int G);
template <class T>
cudaError_t launch_batch_group(const void* members, const long long* first, int nmem, size_t smem,
                               int threads, int grid, cudaStream_t st);
template <class T>
bool tma_path_ok(const Dims& d);
template <class T>
size_t tma_path_smem(const Dims& d);
template <class T>
cudaError_t launch_batch_tma(const void* members, const long long* first, int nmem, size_t smem,
                             int threads, int grid, long long max_nxy, cudaStream_t st);
size_t batch_member_bytes(int precision_fp64);
template <class T>
cudaError_t launch_step(const StepArgs<T>& A, const StepTuning& tn, cudaStream_t st);
// batched form of the fully staged persistent kernel (rt_persist.cu):
// rows per consumer thread for a member plane (R_class > 0: the class's
// rows), 0 when the member does not fill at least half of the CTA
int batch_w3_rows(const Dims& d, int threads, int R_class);
long long batch_w3_stage_floats(const Dims& d);
int batch_w3_stages(long long stage_floats);
size_t batch_w3_smem(int ns, long long stage_floats);
int batch_w3_blocks_per_sm(int threads, int R, size_t smem);
cudaError_t launch_batch_w3(const void* members, const long long* first, int nmem, int threads, int R, int ns,
                            long long stage_floats, int grid, cudaStream_t st);
// small-plane staged kernel (rt_persist.cu): z slices per item for a CTA
// of `threads` consumers (0: the field does not fit it), stage size,
// stages, shared memory, residency and the batched launch
int w6_slices(const Dims& d, int threads);
long long w6_stage_floats(const Dims& d, int G);
int w6_stages(long long stage_floats);
size_t w6_smem(int ns, long long stage_floats);
int w6_blocks_per_sm(int threads, size_t smem);
cudaError_t launch_batch_w6(const void* members, const long long* first, int nmem, int threads, int ns,
                            long long stage_floats, int grid, cudaStream_t st);
// both binary32 ensemble classes in one launch (rt_persist_fused.cu):
// the arguments of the two launches above, one thread count for both, the
// grid and the CTAs [0, ga) of the fully staged class
struct BatchFused {
  const void* pmem;
  const long long* pfirst;
  int np, pR, pns;
  long long pstage;
  const void* smem6;
  const long long* sfirst;
  int ns6, sns;
  long long sstage;
  int threads;
};
size_t batch_fused_smem(const BatchFused& F);
int batch_fused_blocks_per_sm(const BatchFused& F);
cudaError_t launch_batch_fused(const BatchFused& F, int grid, int ga, cudaStream_t st);
// persistent binary32 kernels (dispatch in rt_persist.cu; the families in
// rt_persist.cu, rt_persist_w2.cu); done = false when the tuning
// does not select one of them or the shape does not fit them
cudaError_t launch_persist(const StepArgs<float>& A, const StepTuning& tn, cudaStream_t st, bool& done);
// two-pass binary64 step (rt_split.cu): the face fluxes of every axis with
// n > 1 into f[a] (cell shape, the cell's right face) and f0[a] (face-0
// plane, the layout of vlo[a]), then divergence, mean-flow term and update
struct SplitFluxes {
  double* f[6];
  double* f0[6];
};
cudaError_t launch_step_split(const StepArgs<double>& A, const SplitFluxes& F, cudaStream_t st);
// fast binary64 step (rt_fast.cu): the flux fields of the two-pass step,
// h = |v|/2*(1-|v dt/d|) per face (hr: right faces, hl: face-0 planes),
// mu = 1 - dt*lambda per cell and the per-axis tables c[a] = dt/d_a on the
// padded index range
struct FastTab {
  const double* c[6];
};
cudaError_t launch_fast_prepare(const Dims& d, const Grid& g, double dt, const double* const* vel,
                                const double* const* vlo, const double* const* lam, double* const* hr,
                                double* const* hl, double* mu, double* tab, const long long* toff,
                                cudaStream_t st);
// band: m values per band of the spectral-plane order (1: natural order)
cudaError_t launch_step_fast(const StepArgs<double>& A, const SplitFluxes& F, const double* mu, const FastTab& T,
                             int band, cudaStream_t st);
// failure-detection self-test of the bounded waits (rt_persist.cu): one CTA
// whose waits cannot complete; raises *status, leaves *completed at 0
cudaError_t launch_wait_probe(int* status, int* completed, cudaStream_t st);
// set_forcing on the bottom z plane, in place on E (rt_forcing.cu); kind
// RT_FORCING_FLUX or RT_FORCING_RELAX of rt_gb300.h, F the interior 5D
// forcing field (x,y,k,l,m), zdot the z face velocities (RELAX only)
template <class T>
cudaError_t launch_forcing(T* E, const double* F, const T* zdot, const Dims& d, double dt, double dz, int kind,
                           cudaStream_t st);
// dE (after the mean-flow term) and meanfl of every cell of the state A.E,
// as binary64 unpadded fields (rt_kernels.cu)
template <class T>
cudaError_t launch_tendency(const StepArgs<T>& A, double* dE, double* meanfl, cudaStream_t st);
DiagSizes diag_sizes(const Dims& d);
template <class T>
cudaError_t launch_diag(const StepArgs<T>& A, const T* Ecur, double* scratch, double* vol3,
                        double* result, cudaStream_t st);

}  // namespace rt
