/*
 * rectv_gb300 -- C ABI of the GB300 (sm_103a) implementation of rectv_gpu's
 * 4D time-resolved tomographic reconstruction (USFFT Radon + temporal basis +
 * 4D total variation, linearised ADMM).
 *
 * Every entry point returns 0 on success and a nonzero RECTV_ERR_* code on
 * failure; rectv_last_error() then returns a message for the calling thread.
 * Pointers are plain addresses; sizes are element counts.  No entry point
 * resets the device.
 *
 * Reference interface replaced (nikitinvv/rectv_gpu):
 *   class rectv, SWIG interface src/cuda/rectv.i:9-28, declared in
 *   src/include/rectv.cuh:7-55, implemented in src/cuda/rectv.cu.
 */
#ifndef RECTV_GB300_H
#define RECTV_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rectv_handle rectv_handle;

enum {
    RECTV_OK = 0,
    RECTV_ERR_ARG = 1,     /* invalid argument or shape */
    RECTV_ERR_CUDA = 2,    /* CUDA runtime error */
    RECTV_ERR_CUFFT = 3,   /* cuFFT error */
    RECTV_ERR_STATE = 4,   /* handle freed / call order */
    RECTV_ERR_NOMEM = 5    /* device memory exhausted */
};

/* Message of the last failing call on this thread ("" if none). */
const char *rectv_last_error(void);

/* Library version string. */
const char *rectv_version(void);

/* ---------------------------------------------------------------------------
 * Reference-compatible object API
 * ------------------------------------------------------------------------- */

/* Replaces rectv::rectv(int n, int ntheta, int m, int nz, int nzp, int ngpus)
 * (src/cuda/rectv.cu:5-59; rectv.i:21).  ngpus is clamped to
 * min(ngpus, nz/nzp) as in rectv.cu:9; all work runs on the current CUDA
 * device.  Device memory is allocated here, as in the reference. */
int rectv_create(int n, int ntheta, int m, int nz, int nzp, int ngpus, rectv_handle **out);

/* Read-only attributes n, ntheta, m, nz of the SWIG class (rectv.i:14-18),
 * plus nzp and the effective ngpus.  Any output pointer may be NULL. */
int rectv_get_dims(const rectv_handle *h, int *n, int *ntheta, int *m, int *nz, int *nzp,
                   int *ngpus);

/* Replaces rectv::run(size_t fres, size_t g, size_t theta, size_t phi, float center,
 * float lambda0, float lambda1, int niter, int titer) (src/cuda/rectv.cu:102-252;
 * rectv.i:23-25).  Host pointers, C-contiguous float32:
 *   fres  [nz][m][n][n]   output (written)
 *   g     [nz][ntheta][n] projection data
 *   theta [ntheta]        angles in radians
 *   phi   [m][2*ntheta]   complex temporal basis, interleaved (re, im)
 * lambda0 is used as given (the Python Solver multiplies it by lambda1 first,
 * src/rectv_gpu/solver.py:76).  Starts from zero, as the reference does.
 * Prints "iter (k/niter), rdiff ||f(k+1)-f(k)||:..." to stderr per outer
 * iteration like rectv.cu:238 unless rectv_set_verbose(h, 0). */
int rectv_run(rectv_handle *h, float *fres, const float *g, const float *theta, const float *phi,
              float center, float lambda0, float lambda1, int niter, int titer);

/* Replaces rectv::check_adjoints(size_t res, size_t g, size_t theta, size_t phi,
 * float lambda1, float center) (src/cuda/rectv.cu:255-290; rectv.i:26).
 * Requires nz == nzp (the reference reads nz+1 gradient planes from a buffer
 * of nzp+1 planes).  res is a host float64 [6] ACCUMULATED into (+=), exactly
 * as in the reference:
 *   res[0] = <R*g, R*g>, res[1] = <g, R R*g>, res[2] = <R R*g, R R*g>,
 *   res[3] = <f, D G f>, res[4] = sum of squares of the first
 *   (n+1)^2 (m+1)(nz+1) floats of the float4 gradient array (rectv.cu:287),
 *   res[5] = <D G f, D G f>,  with f = R* g. */
int rectv_check_adjoints(rectv_handle *h, double *res, const float *g, const float *theta,
                         const float *phi, float lambda1, float center);

/* Replaces rectv::free() (src/cuda/rectv.cu:63-91; rectv.i:27).  Releases all
 * device memory; idempotent; does NOT call cudaDeviceReset.  After it, only
 * rectv_get_dims and rectv_destroy are valid. */
int rectv_free(rectv_handle *h);

/* Replaces rectv::~rectv (src/cuda/rectv.cu:61): frees and deletes the handle. */
void rectv_destroy(rectv_handle *h);

/* Per-iteration log to stderr on (1, default) or off (0). */
int rectv_set_verbose(rectv_handle *h, int verbose);

/* ---------------------------------------------------------------------------
 * Device-resident session API (splits rectv::run, src/cuda/rectv.cu:102-252)
 * All pointers are device pointers; work is queued on the handle's stream.
 * ------------------------------------------------------------------------- */

/* Copies data/angles/basis, builds the angle plan, zeroes f, psi, mu and sets
 * rho = 0.5 (rectv.cu:107-125). */
int rectv_setup_device(rectv_handle *h, const float *d_g, const float *d_theta,
                       const float *d_phi, float center, float lambda0, float lambda1, int titer);

/* Runs niter outer ADMM iterations (rectv.cu:140-246) asynchronously. */
int rectv_iterate(rectv_handle *h, int niter);

/* Copies the current iterate f [nz][m][n][n] to d_f (device pointer). */
int rectv_get_result_device(rectv_handle *h, float *d_f);

/* The CUDA stream (cudaStream_t) all work of this handle is queued on. */
int rectv_get_stream(rectv_handle *h, void **stream);

/* Waits for the handle's stream; returns RECTV_ERR_STATE if a kernel recorded
 * an error on the device since the handle was created (a host/device plan
 * disagreement, or a bounded TMA / tensor-core wait that gave up). */
int rectv_synchronize(rectv_handle *h);

/* Per-outer-iteration statistics of the last run/iterate calls, host arrays of
 * length >= *count on input; *count receives the number of iterations recorded.
 * rdiff = ||f(k+1)-f(k)||^2 (rectv.cu:235-238), rho after the update, and the
 * squared primal/dual residual sums r and s of the rho rule (rectv.cu:223-232). */
int rectv_get_history(rectv_handle *h, double *rdiff, double *rho, double *r, double *s,
                      int *count);

/* Use (1, default) or bypass (0) CUDA-graph replay of the outer iteration. */
int rectv_set_graphs(rectv_handle *h, int enable);

/* ---------------------------------------------------------------------------
 * Instrumentation (no reference counterpart).  Kernel ids:
 *   0 forward USFFT gather, 1 adjoint USFFT scatter, 2 fused gradient-
 *   divergence step, 3 shrink + dual update + residual sums, 4 forward
 *   padded-grid 2D FFT (row and column kernels), 5 inverse padded-grid 2D FFT
 *   (column and row kernels; 4 and 5 exist when 2n is a power of two in
 *   [256, 2048]), 6 fused gradient-divergence step of the first inner
 *   iteration (2 is then the step of the later inner iterations).
 * ------------------------------------------------------------------------- */

/* Enqueue `reps` launches of one kernel over one batch of slices on the
 * handle's stream, on the buffers of the current session (after
 * rectv_setup_device); the caller times them with events on that stream.
 * Kernel 3 overwrites the session's dual variables: use after the last
 * rectv_iterate of a session. */
int rectv_launch_kernel(rectv_handle *h, int which, int reps);

/* Algorithmic DRAM bytes and FP32 flops of one such launch. */
int rectv_kernel_cost(rectv_handle *h, int which, double *bytes, double *flops);

/* Per outer ADMM iteration: launches of this library's kernels and cuFFT
 * executions; and the batch size in slices. */
int rectv_get_launch_counts(rectv_handle *h, int *kernels, int *fft_execs, int *batch_slices);

/* USFFT path of the handle's current geometry (no reference counterpart: the
 * reference interpolates every ray, kernels_radonusfft.cuh:81-144).  *ndir =
 * number of ray directions (theta modulo pi) when the rays of a direction
 * share their sample positions (scans over several half-turns: the
 * interpolation runs once per position, dir_kernels.cu), 0 when every ray is
 * interpolated (tensor-core or FP32 kernels); *nrays = ntheta.  Selected at
 * geometry set-up: directions are used when the rays average at least 2.5
 * per direction (RECTV_DIRS=0 never, RECTV_DIRS=1 whenever possible) and
 * rays are grouped when their samples agree within RECTV_DIR_TOL grid cells
 * (default 2e-3). */
int rectv_get_directions(rectv_handle *h, int *ndir, int *nrays);

/* The same choice for a geometry before any handle exists, on the host alone
 * (no GPU): *ndir = number of directions whose rays would share sample
 * positions, 0 when the rays average fewer than min_group per direction
 * (the per-ray kernels then run); *max_rays = the most rays grouped into one
 * direction.  tol_cells <= 0 and min_group <= 0 take the defaults of geometry
 * set-up (2e-3 grid cells, 2.5 rays); the environment switches are not read,
 * and a handle also needs the tensor-core adjoint (M >= 8) for the path.
 * Measured angles with a calibration factor (a scan that does not return to
 * its angles after each half-turn) are not grouped.  No reference
 * counterpart. */
int rectv_plan_directions(const float *theta, int n, int ntheta, double tol_cells, double min_group, int *ndir,
                          int *max_rays);

/* Self-test of the bounded waits of the tensor-core and TMA kernels: queues
 * on the handle's stream one block that waits on an mbarrier nothing arrives
 * on, first for limit_cycles SM cycles, then nwait - 1 more times with the
 * short limit the kernels use after an expired wait, and records the expiry
 * in the handle's device error counter.  Afterwards rectv_synchronize returns
 * RECTV_ERR_STATE for this handle (the counter is never cleared), and the
 * CUDA context stays usable. */
int rectv_selftest_wait(rectv_handle *h, long long limit_cycles, int nwait);

/* FP32 FMA peak of the current device (the compute roofline of the CUDA-core
 * parts of the USFFT kernels), measured with scalar fma.rn and packed
 * fma.rn.f32x2 chains on every SM, in TFLOP/s. */
int rectv_measure_fp32_peak(double *tflops_fma, double *tflops_fma2);

/* Launch-shape autotuner (no reference counterpart; the reference launches
 * every kernel with fixed 32x32 blocks, rectv.cu:32-33, radonusfft.cu:47-48).
 * On a handle with a set-up session, times the candidate launch shapes of the
 * tensor-core USFFT kernels -- slices per block of the gather (64, 32, 16, 8)
 * and persistent blocks of the scatter (1, 3/4, 1/2 of the SMs) -- applies
 * the fastest and reports them (zper, sc_grid; sc_grid 0 = one block per
 * SM).  Results do not depend on these shapes.  Cached per (device, n,
 * ntheta, m, slices per launch) for the process unless force != 0. */
int rectv_autotune(rectv_handle *h, int force, int *zper, int *sc_grid);

/* Device memory held by the handle (buffers and geometry), in bytes. */
int rectv_get_device_bytes(rectv_handle *h, double *bytes);

/* Estimated device memory of a handle with these dimensions (before creating
 * it), in bytes: the figure the engine admits jobs by. */
int rectv_estimate_bytes(int n, int ntheta, int m, int nz, int nzp, double *bytes);

/* ---------------------------------------------------------------------------
 * Multi-problem engine: the batched form and the serving loop (no reference
 * counterpart: the reference solves one problem per rectv::run and re-zeroes
 * f, fn, psi, mu at its start, rectv.cu:119-122).
 *
 * A job is one reconstruction with its own (n, ntheta, m, nz, nzp) and the
 * arguments of rectv_run; its host buffers (g, theta, phi in; fres out) must
 * stay valid until rectv_engine_run returns (pinned memory lets the copies
 * overlap).  Jobs are admitted in order of arrival when their estimated device
 * memory fits the budget and fewer than max_resident jobs run; an admitted
 * job's state (u, psi, mu, rho, geometry, captured iteration graphs) stays
 * resident until its last iteration, all its iterations are queued on its
 * own stream, and the kernels of all running jobs overlap on the GPU.  A
 * finished job's handle is kept for reuse by a later job of the same
 * dimensions unless RECTV_ENGINE_NO_REUSE, and freed when memory is needed.
 * Each job's result equals what rectv_run computes for it alone.
 * ------------------------------------------------------------------------- */
typedef struct rectv_engine rectv_engine;

enum {
    RECTV_ENGINE_NO_REUSE = 1,      /* free each job's handle when it finishes */
    RECTV_ENGINE_AUTOTUNE = 2,      /* rectv_autotune each job's launch shapes (cached) */
    RECTV_ENGINE_LARGEST_FIRST = 4, /* among equal arrival times, admit the most work first */
    RECTV_ENGINE_AGE_PRIORITY = 8,  /* each job's stream gets a lower priority than every job running
                                       when it was admitted: the oldest runs first, newer jobs fill the
                                       SMs it leaves idle */
    RECTV_ENGINE_SHORTEST_FIRST = 16 /* among the jobs that have arrived, admit the one with the least
                                        work (estimated bytes x iterations) first */
};

/* hbm_budget_bytes <= 0: the free device memory minus 4 GiB; max_resident <= 0:
 * no limit on concurrently running jobs. */
int rectv_engine_create(double hbm_budget_bytes, int max_resident, int flags, rectv_engine **out);

/* Queues a job that arrives arrival_s seconds after rectv_engine_run starts.
 * lambda0 is used as given (as rectv_run).  *job_id receives its index. */
int rectv_engine_submit(rectv_engine *e, int n, int ntheta, int m, int nz, int nzp, const float *g,
                        const float *theta, const float *phi, float center, float lambda0, float lambda1, int niter,
                        int titer, double arrival_s, float *fres, int *job_id);

/* Runs every submitted job to completion (or failure) and returns. */
int rectv_engine_run(rectv_engine *e);

/* Per job: times[3] = (arrival, admission, completion) in seconds after the
 * run started, bytes[2] = (estimated, allocated) device memory,
 * rho_rdiff[2] = last rho and ||f(k+1)-f(k)||^2, tune[2] = (gather slices per
 * block, scatter blocks), *status = 0 waiting, 1 running, 2 done, 3 failed.
 * Any output may be NULL. */
int rectv_engine_job_info(rectv_engine *e, int job_id, double *times, double *bytes, double *rho_rdiff,
                          int *tune, int *status);

/* Failure message of a job ("" unless failed), truncated to len bytes. */
int rectv_engine_job_error(rectv_engine *e, int job_id, char *buf, int len);

/* stats[4] = (makespan s, peak device bytes admitted, budget, peak running jobs). */
int rectv_engine_stats(rectv_engine *e, double *stats);

void rectv_engine_destroy(rectv_engine *e);

/* ---------------------------------------------------------------------------
 * Filtered backprojection and warm start (no counterpart run by the
 * reference: its ramp filter applyfilter and mask circ,
 * kernels_radonusfft.cuh:146-189, and the filter flag of radonusfft::adjR,
 * radonusfft.cu:106, are never used).
 * ------------------------------------------------------------------------- */

/* Static filtered backprojection of every slice: frec [nz][n][n] (host) =
 * circ(pi/4 * R*(applyfilter(g))) with g [nz][ntheta][n], theta [ntheta] host
 * float32 and the rotation centre as in rectv_run.  Uses the handle's buffers
 * (not its reconstruction state). */
int rectv_fbp(rectv_handle *h, float *frec, const float *g, const float *theta, float center);

/* rectv_run starting from finit [nz][m][n][n] (host) instead of zero. */
int rectv_run_init(rectv_handle *h, float *fres, const float *g, const float *theta, const float *phi,
                   const float *finit, float center, float lambda0, float lambda1, int niter, int titer);

/* ---------------------------------------------------------------------------
 * Data ingest: the step before the solver.  Replaces the preprocessing of
 * examples/tao/tao.py:34-41 (flat/dark normalisation, -log, projection ->
 * sinogram transpose):
 *   out[z][theta][x] = -log((data[theta][z][x] - mean_f dark[f][z][x]) /
 *                           (1e-3 + mean_f flat[f][z][x] - mean_f dark[f][z][x]))
 * Host pointers; data [ntheta][nz][n], dark [ndark][nz][n], flat [nflat][nz][n]
 * of element type dtype; out float32 [nz][ntheta][n] (the layout rectv_run
 * takes).  Uses temporary device memory; non-positive ratios give NaN/inf as
 * in the NumPy original.
 * ------------------------------------------------------------------------- */
enum { RECTV_DTYPE_F32 = 0, RECTV_DTYPE_U16 = 1 };

int rectv_preprocess(float *out, const void *data, const void *dark, const void *flat, int dtype, int ntheta,
                     int nz, int n, int ndark, int nflat);

/* ---------------------------------------------------------------------------
 * Allocation-free entry point (no counterpart in the reference).
 *
 * For callers that cannot let a library allocate device memory -- an
 * application that owns the whole device budget through its own pool and
 * passes in only its own buffers, or a processing loop that must not stall,
 * since cudaMalloc/cudaFree can synchronise the device and can fail at run
 * time when memory is fragmented.  It needs no handle and calls no
 * cudaMalloc, cudaFree or allocating library routine.
 *
 * One end-of-iteration ADMM shrink step (solve_reg_ker, the mu update and the
 * two residual norms of admm.cu:101-117, as rectv_iterate runs it) over
 * nchunks chunks of nzp slices, queued on `stream` (a cudaStream_t, or NULL):
 *   d_u_cur, d_u_old  [nchunks*nzp][m][n][n]  iterate after the inner steps,
 *                     and the previous outer iterate (source of the z-halo)
 *   d_psi (out), d_mu (in/out)  [4][nchunks][nzp+1][m+1][n+1][n+1]
 *   d_sums (out)      device double[3]: sum |grad u_cur - psi|^2,
 *                     sum |grad u_old - grad u_cur|^2, sum (u_cur - u_old)^2
 * Its only scratch (FP64 per-block partial sums and the rho value) is a fixed
 * static device array of 1.5 MiB that every GPU loading this library holds
 * until the process exits.  Limit: ceil((n+1)/32)*ceil((n+1)/8)*nchunks*
 * (nzp+1) <= 65536 thread blocks (e.g. n=1024, nzp=8, nchunks=1, any m)
 * and nchunks*(nzp+1) <= 65535; larger problems are rejected with
 * RECTV_ERR_ARG.  `stream` must belong to the current device.  The first
 * call on a device looks up the array's device address, so make that first
 * call before any stream capture; the address is kept for the process's
 * life, so after cudaDeviceReset of a device do not call this entry point on
 * that device again.  All calls share the array, which keeps the last call's
 * contents; each call writes every entry it reads before reading it, so
 * nothing needs clearing.  Calls that can run at the same time on one device
 * (for example on different streams) race on the array. */
int rectv_shrink_noalloc(const float *d_u_cur, const float *d_u_old, float *d_psi, float *d_mu, int n,
                         int m, int nzp, int nchunks, float rho, float lambda0, float lambda1,
                         double *d_sums, void *stream);

/* ---------------------------------------------------------------------------
 * Operator-level entry points (device pointers), the reference's private
 * operators exposed for parity testing.  rectv_op_set_geometry must be called
 * first; it uploads theta/phi and the rotation centre.
 * ------------------------------------------------------------------------- */

/* d_theta [ntheta], d_phi [m][2*ntheta] device pointers; center as in run. */
int rectv_op_set_geometry(rectv_handle *h, const float *d_theta, const float *d_phi, float center);

/* rectv::radonapr (src/cuda/operators.cu:6-32): d_g = tau * R_apr d_f.
 * d_f [nslices][m][n][n], d_g [nslices][ntheta][n]; nslices <= nz. */
int rectv_op_radonapr(rectv_handle *h, float *d_g, const float *d_f, int nslices, float tau);

/* rectv::radonapradj (src/cuda/operators.cu:34-58): d_f += tau * R_apr^T d_g. */
int rectv_op_radonapradj(rectv_handle *h, float *d_f, const float *d_g, int nslices, float tau);

/* rectv::gradient (src/cuda/operators.cu:60-66) on one chunk:
 * d_fm [nzp+2][m][n][n] (slab 0 and nzp+1 are the z-halo), flgl/flgr say
 * whether the halo slabs are used (extendf, kernels_operators.cuh:4-20);
 * d_h2 [nzp+1][m+1][n+1][n+1][4] float (float4 layout of the reference). */
int rectv_op_gradient(rectv_handle *h, float *d_h2, const float *d_fm, float lambda1, int flgl,
                      int flgr);

/* rectv::divergent (src/cuda/operators.cu:68-71): d_fn [nzp][m][n][n] +=
 * tau * div(d_h2) (kernels_operators.cuh:46-73). */
int rectv_op_divergent(rectv_handle *h, float *d_fn, const float *d_h2, float lambda1, float tau);

#ifdef __cplusplus
}
#endif

#endif /* RECTV_GB300_H */
