/*
 * rt_gb300.h -- C ABI of libraytracer_gb300.so, the GB300 (sm_103a)
 * implementation of raytracer_3D's time-stepping path.
 *
 * The reference path has no plugin or FFI interface: it is a set of
 * argument-free Fortran subroutines working on module state
 * (for_src/main_module.f90:41-77).  Each entry point below replaces one of
 * those subroutines, or the part of one that lies on the path, and is meant
 * to be bound from Fortran with ISO_C_BINDING (bind(C), c_loc of the full
 * padded allocatable arrays).
 *
 * Conventions
 *   - Host arrays use the reference layout: Fortran column-major, x fastest,
 *     every axis padded by onx = 2 ghost cells on both sides
 *     (main_module.f90:114, :135-223).  A 6D array therefore holds
 *     (nx+4)(ny+4)(nz+4)(nk+4)(nl+4)(nm+4) doubles, a 3D array
 *     (nx+4)(ny+4)(nz+4), a 1D grid array n+4.
 *   - Every function returns 0 (RT_OK) or a negative RT_ERR_* code; the
 *     message is available from rt_last_error().  The Fortran side calls
 *     halt_stop (parallel_mpi.f90:223-236) on a nonzero code, the
 *     reference's convention for fatal errors.
 *   - The library copies host arrays on set/get and never keeps a host
 *     pointer.  A handle owns all of its device memory; the model state
 *     stays on the GPU between calls.
 *   - One host thread per handle; several handles may coexist.  Each handle
 *     launches on its own CUDA stream (rt_stream).
 *   - There is no CPU fallback: without a usable sm_103a GPU rt_create fails.
 */
#ifndef RT_GB300_H
#define RT_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define RT_OK 0
#define RT_ERR_ARG (-1)      /* invalid argument or call order          */
#define RT_ERR_NOMEM (-2)    /* device allocation failed                */
#define RT_ERR_CUDA (-3)     /* CUDA runtime error                      */
#define RT_ERR_GRID (-4)     /* grid check failed (calc_grid.f90:260-293) */
#define RT_ERR_STATE (-5)    /* required earlier call missing           */

#define RT_FP64 0            /* plain binary64 form (reference arithmetic) */
#define RT_FP32 1            /* binary32 state/fluxes/velocities, binary64
                                coefficients and budget */

typedef struct rt_handle rt_handle;

/* model sizes, main_module.f90:14-19, :114 */
typedef struct {
  int nx, ny, nz, nk, nl, nm; /* interior points; nk, nl, nm even or 1 */
  int onx;                    /* halo width of the host arrays: must be 2 */
} rt_dims;

/* model parameters, main_module.f90:20-31 */
typedef struct {
  double dt;                  /* time step in s                    */
  double f0;                  /* Coriolis parameter in 1/s         */
  double sign_of_omega_i;     /* +1 or -1                          */
  int enable_upper_reflection;
  int enable_lower_reflection;
  int precision;              /* RT_FP64 or RT_FP32                */
} rt_params;

/* energy budget of diagnose.f90:46-329 (scalars) */
typedef struct {
  double eint, mflint, mfl_max;
  double umax, vmax, wmax, kmax, lmax, mmax;
  double bfl_xs, bfl_xe, bfl_ys, bfl_ye, bfl_zs, bfl_ze;
  double bfl_ks, bfl_ke, bfl_ls, bfl_le, bfl_ms, bfl_me;
  double cfl_x, cfl_y, cfl_z, cfl_k, cfl_l, cfl_m;
  double residual;
} rt_budget;

/* identifiers of rt_get_field */
#define RT_F_XDOT 0
#define RT_F_YDOT 1
#define RT_F_ZDOT 2
#define RT_F_KDOT 3
#define RT_F_LDOT 4
#define RT_F_MDOT 5
#define RT_F_LAMBDA_X 6
#define RT_F_LAMBDA_Y 7
#define RT_F_LAMBDA_Z 8
#define RT_F_LAMBDA 9         /* combined rate used by RT_FP32 */

/* Create a handle: allocate_main_module (main_module.f90:131-238) for the
 * device side.  Validates sizes as pe_decomposition does
 * (parallel_mpi.f90:16-25: nk, nl, nm even or one). */
int rt_create(const rt_dims* dims, const rt_params* params, rt_handle** out);
int rt_destroy(rt_handle* h);
/* message of the last error on h (or of the last failed rt_create for NULL) */
const char* rt_last_error(const rt_handle* h);

/* Grid after calc_grid (calc_grid.f90:4-177): padded 1D arrays of the grid
 * spacings dxt..dmt and wavenumbers kt, lt, mt. */
int rt_set_grid(rt_handle* h, const double* dxt, const double* dyt, const double* dzt,
                const double* dkt, const double* dlt, const double* dmt, const double* kt,
                const double* lt, const double* mt);
/* Background state of set_initial_conditions: padded 3D Nsqr, U, V. */
int rt_set_background(rt_handle* h, const double* Nsqr, const double* U, const double* V);
/* Replaces calc_parameter (calc_parameter.f90:2-264, called at
 * main.f90:47): dispersion relation, face velocities and growth rates,
 * computed on the GPU in binary64 and kept there. */
int rt_calc_parameter(rt_handle* h);
/* Copy a coefficient field to a padded 6D host array.  Velocities: faces
 * 0..n of their own axis and the interior of the others; growth rates:
 * interior.  Other host elements are left untouched. */
int rt_get_field(rt_handle* h, int which, double* out);
/* max over interior cells of sum_a max(|v_a(i-1)|,|v_a(i)|)/d_a(i); a
 * CFL number c gives dt = c / rate */
int rt_max_rate(rt_handle* h, double* rate);
/* change dt after creation (e.g. once rt_max_rate is known) */
int rt_set_dt(rt_handle* h, double dt);

/* Upload / download the wave energy E (padded 6D host array; only the
 * interior is read or written, ghost cells are refilled every step). */
int rt_set_state(rt_handle* h, const double* E);
int rt_get_state(rt_handle* h, double* E);

/* Bottom forcing of the forced configurations (the set_forcing hook,
 * main.f90:69).  From the next rt_integrate on, every step first updates the
 * bottom z plane (Fortran z index 1) of E in place, then integrates:
 *   RT_FORCING_FLUX   E += dt*F/dzt(1)                  lee1.f90:193-212
 *                     (F = flux_lee)
 *   RT_FORCING_RELAX  E -= dt*max(0,zdot)*(E-F)/dzt(1)  critical_gm1.f90:119-139
 *                     (F = E_gm; zdot from rt_calc_parameter)
 * F is a padded 5D host array with axes x,y,k,l,m,
 * (nx+4)(ny+4)(nk+4)(nl+4)(nm+4) doubles like the reference's allocatable;
 * its interior is copied to the device.  RT_FORCING_NONE (F may be NULL)
 * switches the forcing off.  rt_step_dry does not apply it; a batch applies
 * each member's own forcing. */
#define RT_FORCING_NONE 0
#define RT_FORCING_FLUX 1
#define RT_FORCING_RELAX 2
int rt_set_forcing(rt_handle* h, int kind, const double* F);

/* Replaces integrate (integrate.f90:4-271, called at main.f90:70):
 * nsteps forward-Euler steps on the device-resident state. */
int rt_integrate(rt_handle* h, int nsteps);
/* Launch the step nsteps times from the current state WITHOUT advancing it
 * (the spare buffer is overwritten).  For timing schedules (autotuner); the
 * next rt_diagnose needs a real step first. */
int rt_step_dry(rt_handle* h, int nsteps);
/* One integrate on a host array, the literal drop-in for the module-state
 * call: E is uploaded, stepped once and written back (interior). */
int rt_integrate_host(rt_handle* h, double* E);
/* How rt_set_state / rt_get_state / rt_integrate_host move the host's
 * padded array: direct = 1 (default) lets the GPU read and write it in
 * place through the host's page tables when the device supports pageable
 * memory access (cudaDevAttrPageableMemoryAccess, e.g. coherent CPU-GPU
 * systems); direct = 0, or a device without it, gathers the interior on the
 * host into pinned staging and copies.  Results are identical. */
int rt_set_host_access(rt_handle* h, int direct);
/* 1 when the direct path is in use for this handle, 0 otherwise */
int rt_host_direct(rt_handle* h);
/* The state without ghost cells, exactly as the device stores it:
 * nx*ny*nz*nk*nl*nm values, x fastest, binary64 for RT_FP64 handles and
 * binary32 for RT_FP32 handles.  For callers that keep no padded module
 * array (the ensemble and serving layers); no counterpart in the
 * reference, whose state is always the padded module array. */
int rt_set_state_interior(rt_handle* h, const void* E);
int rt_get_state_interior(rt_handle* h, void* E);

/* Budget part of diagnose (diagnose.f90:46-329), for the step taken last.
 * The 3D outputs are padded host arrays (interior written; NULL skips).
 * Requires at least one step since rt_set_state. */
int rt_diagnose(rt_handle* h, rt_budget* out, double* E_int, double* meanfl_int, double* diss_ks,
                double* diss_ke, double* diss_ls, double* diss_le, double* diss_ms,
                double* diss_me);
/* The module arrays dE and meanfl that the last step left behind
 * (integrate.f90:202-262; dE after the mean-flow term), recomputed on the
 * device from the state that step started from: padded 6D host arrays, the
 * interior is written.  With E they form the restart record
 * (restart.f90:15-18).  Needs a step since rt_set_state. */
int rt_get_tendency(rt_handle* h, double* dE, double* meanfl);

/* Schedule of the step kernel.  variant:
 *   2  = plane tiled with bulk-copy (TMA) staging of the E planes (default;
 *        used when a plane of E is a multiple of 16 bytes)
 *   3  = the same with several z planes per work item (small x-y planes)
 *   0  = plane tiled with plain loads,  1 = one thread per cell
 *   9  = binary32: persistent, warp-specialised, every operand staged
 *   13 = binary32: the same for small planes, z slices per work item
 *   14 = binary32: persistent, warp-specialised, 2-wide cell blocks, CTAs
 *        marching along z
 *   18 = 14 with the cell-pair arithmetic on packed f32x2 instructions and
 *        the next plane's operands prefetched into L2 (the production
 *        binary32 step)
 *   15 = binary64 in two passes: every face flux evaluated once into flux
 *        fields (allocated by this call: 48 bytes per cell plus the face-0
 *        planes), then divergence and update
 *   16 = binary64 fast: the two passes of 15 without divisions (limiter
 *        slope selected exactly, update regrouped; 8 more bytes per cell);
 *        within a few units in the last place of the reference's result per
 *        step, NOT bit-identical to it.  band = m values per band of its
 *        spectral-plane order (1: natural order; a width that does not
 *        divide nm is reduced to the largest one that does); fields of
 *        2^31 cells or more are rejected (RT_ERR_CUDA on the step)
 * Every other variant gives the same result: bit-identical to the
 * reference's arithmetic in binary64, and among themselves in binary32.
 * band: values per band of the plane schedule (default 8); threads: CTA
 * size 128, 256, 512 or 1024 (default 512; consumer threads of the
 * persistent variants: 128, 256 or 512).  Codes 4-8, 10-12 and 17 belonged
 * to removed kernels and are rejected.  The binary32 form treats 15 and 16 as
 * 2; shapes a variant cannot run fall back to the next one that can.
 * Chosen by the autotuner (raytracer_3d_gb300.autotune). */
int rt_set_tuning(rt_handle* h, int variant, int band, int threads);
/* Sweep order of the plane schedule: 0 = bands over m (default), 1 = bands
 * over l.  No effect on results. */
int rt_set_schedule_sweep(rt_handle* h, int sweep);
/* number of interior cells of the handle */
long long rt_cells(const rt_handle* h);
/* wait for the handle's stream; fails if a device-side wait timed out */
int rt_sync(rt_handle* h);
/* cudaStream_t of the handle (as void*), for timing with CUDA events */
int rt_stream(rt_handle* h, void** stream);
/* number of kernel launches issued by this handle so far */
long long rt_launch_count(const rt_handle* h);
/* bytes of device memory held by the handle */
long long rt_device_bytes(const rt_handle* h);
/* library version string */
const char* rt_version(void);

/* ---- allocation-free entry point --------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a host framework that owns every device allocation, allocations frozen
 * during graph capture or a real-time loop, no out-of-memory failure
 * allowed mid-run): the CFL rate of rt_max_rate computed from device arrays
 * the caller owns, allocating nothing.
 *   vel[a]   right-face velocities of axis a, cell-shaped, unpadded, x fastest
 *   vlo[a]   face-0 velocities of axis a (cell shape with axis a collapsed)
 *   dgrid[a] padded grid spacing of axis a (n_a + 4 doubles)
 *   out      one device double; receives the rate
 * Inactive axes (n = 1) may pass NULL.  Runs asynchronously on `stream`
 * (a cudaStream_t; NULL = legacy default stream).  Its scratch is a fixed
 * 256 KiB device array inside the library, so fields above 2^31 cells are
 * rejected with RT_ERR_ARG (as is onx != 2).  The first call on a device
 * looks up that array's address and must come before any stream capture;
 * the address is kept for the device's primary context, so after a
 * cudaDeviceReset the entry point must not be called on that device again.
 * All calls share the array: calls that overlap on the GPU race.  Errors
 * are described by rt_noalloc_last_error(), which returns the calling
 * thread's own last message. */
int rt_max_rate_noalloc(const rt_dims* dims, const double* const* vel, const double* const* vlo,
                        const double* const* dgrid, double* out, void* stream);
const char* rt_noalloc_last_error(void);

/* ---- batched ensemble -------------------------------------------------
 * No counterpart in the reference, which advances one field per run: a
 * batch advances many independent fields (members) of possibly different
 * sizes with ONE persistent kernel launch per time step, replayed from
 * captured CUDA graphs.  Members keep ownership of their state and
 * coefficients; each keeps its own dt, grids and parameters.  All members
 * must share one precision and have coefficients and a state.  Work queued
 * on a member's own stream is ordered before the batch, and later member
 * calls (rt_get_state, rt_diagnose, ...) after it.  Results are
 * bit-identical to stepping each member alone. */
typedef struct rt_batch rt_batch;
int rt_batch_create(rt_handle* const* members, int n, rt_batch** out);
int rt_batch_destroy(rt_batch* b);
const char* rt_batch_last_error(const rt_batch* b);
/* band, CTA size (128/256/512/1024), sweep order (0/1) and steps per captured
 * graph (even); chosen by the autotuner (raytracer_3d_gb300.autotune) */
int rt_batch_set_tuning(rt_batch* b, int band, int threads, int sweep, int graph_steps);
/* binary32 members whose x-y planes fill a CTA of `threads` consumer
 * threads (128/256/512; x and y extents multiples of 4) are stepped by the
 * batched warp-specialised kernel with every operand staged by bulk copies;
 * members with smaller planes (every axis z..m longer than one) by its form
 * with several z slices per work item (256 or 512 consumer threads); the
 * others by the z-group / plane kernels.  0 puts every member in the last
 * class.  Default 256.  No effect on results. */
int rt_batch_set_persistent(rt_batch* b, int threads);
/* consumer threads (256 or 512) of the small-plane class alone; 0 turns
 * that class off, -1 (default) follows rt_batch_set_persistent */
int rt_batch_set_slices(rt_batch* b, int threads);
/* 1: when both warp-specialised classes have members and run the same
 * consumer thread count, a batched step is ONE persistent launch whose CTAs
 * are split between the classes in proportion to the device time of each
 * class's own launch, measured when the batch is (re)built -- a build then
 * waits for the work queued before it; 0 (default): one launch per class.
 * No effect on results. */
int rt_batch_set_fused(rt_batch* b, int on);
/* number of members in the two warp-specialised classes (negative: error) */
int rt_batch_persistent_members(rt_batch* b);
/* advance every member by nsteps (asynchronous on the batch stream) */
int rt_batch_integrate(rt_batch* b, int nsteps);
int rt_batch_sync(rt_batch* b);
/* nsteps batch launches that do not advance the members (timing only) */
int rt_batch_dry(rt_batch* b, int nsteps);
int rt_batch_stream(rt_batch* b, void** stream);
long long rt_batch_launch_count(const rt_batch* b);
long long rt_batch_cells(const rt_batch* b);

/* Phase timers, the GPU counterpart of the reference's tic/toc counters
 * (timing_module.f90:34-75, printed at main.f90:86-101): rt_tic / rt_toc
 * record CUDA events on the handle's stream around the named phase (so the
 * device time of the work queued in between is measured, without a
 * synchronisation); rt_timing_secs waits for the recorded events and
 * returns the accumulated seconds and the number of tic/toc pairs.  A toc
 * without its tic, or a second tic, is RT_ERR_STATE; an unknown name reads
 * as 0 s.  The fused step has no separate fluxes / bc exchange / reflection
 * / time tendency phases: they are all inside 'integrate'. */
int rt_tic(rt_handle* h, const char* name);
int rt_toc(rt_handle* h, const char* name);
int rt_timing_secs(rt_handle* h, const char* name, double* secs, long long* calls);

/* Binary64 fused multiply-add instructions per second of the current GPU,
 * measured by a short kernel of independent fma chains timed with CUDA
 * events.  No counterpart in the reference: the denominator of the
 * roofline of the binary64 step, which GB300's binary64 pipe bounds. */
int rt_fp64_rate(double* fma_per_s);

/* Failure-detection self-test of the bounded device waits.  Every wait of
 * the step kernels on an mbarrier gives up after a fixed number of polls,
 * raises a status flag that the next synchronising call turns into
 * RT_ERR_CUDA ("a device-side wait timed out"), lets copies in flight land
 * and returns, so the context stays usable.  This call runs one CTA whose
 * waits can never complete, through the same wait code with a short limit,
 * and reports *status (the raised flag, 1 expected) and *completed (1 if a
 * wait completed, 0 expected).  It touches no handle. */
int rt_selftest_wait_timeout(int* status, int* completed);

#ifdef __cplusplus
}
#endif
#endif
