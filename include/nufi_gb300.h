/*
 * nufi_gb300.h — C ABI of the GB300 (sm_103a) NuFI hot path.
 *
 * The hot path of Numerical Flow Iteration: at time step n every phase-space
 * quadrature point (x, v) is traced backwards through n Störmer–Verlet
 * substeps over the stored B-spline potential coefficients of steps
 * n-1 .. 0, f0 is evaluated at the foot of the characteristic, and
 * rho(x) = -sum_v w f~ is formed.  A periodic Poisson + spline
 * interpolation solve then appends slab n of the coefficient history.
 *
 * Every function returns an int status (NUFI_OK = 0).  On failure a message
 * is kept per handle (nufi_last_error) or per thread for handle-less calls
 * (nufi_last_error(NULL)).  Nothing here throws; the C++ wrappers in
 * include/nufi_gb300/ turn the status codes back into the exception types
 * the reference raises (std::range_error, nufi::cuda::exception,
 * std::invalid_argument).
 *
 * Threading: one handle = one CUDA stream.  Calls on a handle are stream
 * ordered; the download_* calls and nufi_synchronize block.  A handle must
 * not be used from two host threads at once (the reference's cuda_kernel is
 * not thread safe either).
 *
 * Grid conventions (reference nufi/cuda_kernel.cu:37-47, 216-231, 398-418):
 *   x_i = x_min + i*dx      (spatial nodes, dx = (x_max-x_min)/Nx)
 *   v_j = v_min + j*dv + dv/2  (velocity midpoints, dv = (v_max-v_min)/Nv)
 *   flattened quadrature index q = s*Nm + m with s the spatial index
 *   (x fastest, then y, then z) and m the velocity index (u fastest, then
 *   v, then w); Nm = Nu*Nv*Nw.  This is the reference's q order.
 *   rho[s] = -(du*dv*dw) * sum_m f~(s, m)   (no +1 background; the Poisson
 *   solve drops the mean mode).
 * Coefficient history layout (host side, as the reference keeps it):
 *   slab n starts at base + n*stride_t, stride_t = prod_d (N_d + order - 1),
 *   x fastest; each slab is the periodic padding c[i] = c~[i mod N].
 */
#ifndef NUFI_GB300_H
#define NUFI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define NUFI_OK              0
#define NUFI_ERR_INVALID     1  /* bad argument or configuration            */
#define NUFI_ERR_RANGE       2  /* n > Nt, q range outside the grid, sizes  */
#define NUFI_ERR_CUDA        3  /* a CUDA runtime call failed               */
#define NUFI_ERR_UNSUPPORTED 4  /* combination not built (see message)      */
#define NUFI_ERR_DEVICE      5  /* a device-side check raised its flag      */

/* ---- precision modes --------------------------------------------------- */
/* FP64 plain: the whole trace in double, same operation order as the
 * reference's eval_ftilda (nufi/rho.hpp:31-61, 191-232, 318-367).          */
#define NUFI_PREC_FP64        0
/* FP32 split: position = integer cell + FP32 fraction, velocity = exact
 * grid velocity + FP32 kick sum, field tables in FP32, f0 evaluated as a
 * perturbation of its value at the grid velocity; FP64 only in the rho
 * accumulator, the Poisson solve and the spline interpolation solve.
 * f0's phase comes from the cell the foot lands in (the foot wrapped into
 * the domain); when k (x_max - x_min) is not a multiple of 2 pi (to 2.5e-7
 * relative: a single-precision domain length passes) the phase is turned
 * by k (x_max - x_min) per wrap of the foot, which handles with every Nx a
 * power of two do (in 1D up to 256, and not with the split_global_loads or
 * split_plain_kick options; not in batches); NUFI_ERR_UNSUPPORTED for other
 * such handles.  FP64 evaluates f0 at the unwrapped foot, as the
 * reference, for any k.                                                     */
#define NUFI_PREC_FP32_SPLIT  1

/* ---- initial conditions (f0) ------------------------------------------- */
/* params[0] = alpha, params[1] = k (same on every axis)                    */
/* Landau:      (1 + alpha sum_d cos(k x_d)) exp(-|v|^2/2) / (2 pi)^(dim/2)  */
#define NUFI_F0_LANDAU        0
/* Two-stream:  (1 + alpha cos(k x)) v^2 exp(-v^2/2) / sqrt(2 pi)   (1D)    */
#define NUFI_F0_TWO_STREAM    1
/* Bump-on-tail:(1 + alpha cos(k x)) [0.9 N(v;0,1) + 0.1 N(v;u_b,sigma_b)]
 *              params[2] = u_b, params[3] = sigma_b                  (1D)
 *              3D (FP64 only): (1 + alpha sum_d cos(k x_d))
 *              [0.9 N(u;0,1) + 0.1 N(u;u_b,sigma_b)] N(v;0,1) N(w;0,1),
 *              the reference's compiled-in 3D f0 (nufi/config.hpp)         */
#define NUFI_F0_BUMP_ON_TAIL  2

typedef struct nufi_config {
    int32_t dim;          /* 1, 2 or 3                                     */
    int32_t order;        /* B-spline order (4 = cubic)                    */
    int32_t precision;    /* NUFI_PREC_*                                   */
    int32_t f0_kind;      /* NUFI_F0_*                                     */
    int64_t Nx[3];        /* spline nodes per spatial axis (unused: 1)     */
    int64_t Nv[3];        /* quadrature nodes per velocity axis (unused: 1)*/
    int64_t Nt;           /* time steps; slabs 0 .. Nt are kept            */
    double  dt;           /* time-step size                                */
    double  x_min[3], x_max[3];
    double  v_min[3], v_max[3];
    double  f0_params[8];
} nufi_config;

typedef struct nufi_handle nufi_handle;

/* Message of the last failed call on h (or of this thread's last failed
 * handle-less call when h == NULL).  Never NULL. */
const char *nufi_last_error(const nufi_handle *h);

/* ---- lifetime ----------------------------------------------------------
 * Replaces the constructor of nufi::dimN::cuda_kernel<real,order>
 * (nufi/cuda_kernel.hpp:37-38, 82, 124; nufi/cuda_kernel.cu:81-109,
 * 273-286, 468-483): allocates the coefficient history (Nt+1 slabs),
 * rho and the metrics accumulators on `device`.  Checked before any CUDA
 * call: NUFI_ERR_RANGE for Nt > 2^30, more than 2^31 - 1 spatial or
 * velocity nodes, more than 2^20 nodes or 4096 velocity nodes on an axis,
 * or a history above 2^50 bytes; NUFI_ERR_INVALID / NUFI_ERR_UNSUPPORTED
 * for the other configuration errors (among them non-finite domain bounds or
 * f0 parameters, and sigma_b <= 0 for bump-on-tail: NUFI_ERR_INVALID).
 * NUFI_ERR_CUDA (with the CUDA error's
 * name) when no device is usable or an allocation fails. */
int nufi_create(const nufi_config *cfg, int device, nufi_handle **out);
int nufi_destroy(nufi_handle *h);

/* No counterpart in the reference: launch options of a handle or a batch.
 * Every field's 0 is the default (a zeroed struct, or a NULL pointer, is
 * what nufi_create and nufi_batch_create use).  The options choose among
 * kernels and launch shapes of the same computation; none changes what a
 * call computes beyond the rounding of the FP32-split arithmetic, and the
 * GPU tests use them to check one kernel against another.
 *   split_global_loads      1: FP32-split traces read their field tables
 *                           from global memory, not through the
 *                           shared-memory ring
 *   split_plain_kick        1: the 1D FP32-split kick summed in plain,
 *                           uncompensated FP32 (global-load 1D trace; shows
 *                           what the compensation buys)
 *   no_persistent           1: nufi_run as a CUDA graph of per-step
 *                           launches instead of the whole-run kernel
 *   split_ctas_per_sm       0 or 1: one CTA per SM; 2: two smaller CTAs
 *                           per SM (1D staged split trace)
 *   split_threads_per_node  0 or 1: one thread per spatial node; 2: two
 *                           (1D staged split trace)
 *   batch_no_autotune       1: nufi_batch_create keeps the default shapes
 *   batch_adjoint_ppt       0: autotuned; 2 or 4 (FP32-split) or 1, 2, 4
 *                           (FP64): chains per thread of the batch adjoint
 * Other values are NUFI_ERR_INVALID. */
typedef struct nufi_options {
    int32_t split_global_loads;
    int32_t split_plain_kick;
    int32_t no_persistent;
    int32_t split_ctas_per_sm;
    int32_t split_threads_per_node;
    int32_t batch_no_autotune;
    int32_t batch_adjoint_ppt;
    int32_t reserved[9]; /* must be 0 */
} nufi_options;
int nufi_create_ex(const nufi_config *cfg, const nufi_options *opt, int device, nufi_handle **out);

/* ---- reference-facing drop-in calls ------------------------------------ */
/* cuda_kernel::compute_rho (nufi/cuda_kernel.cu:112-132, 289-311, 486-510):
 * rho := -w * sum over q in [q_begin, q_end) of f~(n, q), using slabs
 * 0 .. n-1.  NUFI_ERR_RANGE if n > Nt or q_end > Nq.  Asynchronous. */
int nufi_compute_rho(nufi_handle *h, int64_t n, int64_t q_begin, int64_t q_end);
/* cuda_kernel::download_rho (nufi/cuda_kernel.cu:135-145): rho[s] += the
 * device rho (so the caller zeroes its buffer first).  Blocks. */
int nufi_download_rho(nufi_handle *h, double *rho);
int nufi_download_rho_f32(nufi_handle *h, float *rho);
/* cuda_kernel::upload_phi (nufi/cuda_kernel.cu:147-156): copies slab n from
 * coeffs_base + n*stride_t of the caller's history to the device.  Returns
 * once the caller's values have been read (the buffer may be reused); the
 * transfer is ordered before the handle's later work.  1D FP32-split
 * handles keep the newest uploaded slab staged in pinned host memory: the
 * next compute_rho(n + 1) derives its table inside the trace, and any other
 * call of this library that reads the device history (and nufi_stream, for
 * the caller's own work on the stream) applies it first. */
int nufi_upload_phi(nufi_handle *h, int64_t n, const double *coeffs_base);
int nufi_upload_phi_f32(nufi_handle *h, int64_t n, const float *coeffs_base);
/* cuda_kernel::compute_metrics (nufi/cuda_kernel.cu:158-175, 341-358,
 * 543-560; kernels :53-79, 239-271, 428-466): over q in [q_begin, q_end)
 * of f(n, q) = f0 at the foot of the full backward trace from step n
 * (eval_f, nufi/rho.hpp:63-93: initial half kick with slab n, so slabs
 * 0 .. n must be present), with u0 the point's grid velocity:
 *   m[0] = sum w f            (L1 norm)
 *   m[1] = sum w f^2          (the caller takes the square root)
 *   m[2] = sum w |u0|^2 f / 2 (kinetic energy)
 *   m[3] = sum -w f log f over f > 0 (entropy)
 * w = du dx (1D), dx dy du dv (2D), du dv dw (3D: as the reference, without
 * dx dy dz).  The points lie on the metrics grid: the rho grid, or the grid
 * nufi_set_metrics_grid gave (then q ranges over its Ns * Nm points).
 * Always evaluated in FP64 on the FP64 history, also for FP32-split
 * handles.  An empty range returns without touching the device sums (as the
 * reference); n > Nt is NUFI_ERR_RANGE (the reference does not check).
 * Asynchronous. */
int nufi_compute_metrics(nufi_handle *h, int64_t n, int64_t q_begin, int64_t q_end);
/* The metrics grid of the reference's two-config constructor
 * cuda_kernel(conf, conf_metrics) (nufi/cuda_kernel.cu:96-108, 53-79): point
 * (ix, iu) at x = x_min + ix dx, u = v_min + iu du + du / 2 with dx =
 * (x_max - x_min) / Nx, du = (v_max - v_min) / Nv per axis, weight as in
 * nufi_compute_metrics with these dx, du.  Only dim, Nx, Nv, x_min, x_max,
 * v_min and v_max of `metrics` are read; dim must be the handle's.  f is
 * still evaluated with the handle's own history and splines.  NULL returns
 * to the rho grid.  At most 2^31 - 1 spatial and 2^31 - 1 velocity points
 * (NUFI_ERR_RANGE beyond).  Blocks (one allocation the first time a grid
 * needs more partial sums than the handle holds). */
int nufi_set_metrics_grid(nufi_handle *h, const nufi_config *metrics);
/* cuda_kernel::download_metrics (nufi/cuda_kernel.cu:177-189): m[k] += the
 * device sums.  Blocks. */
int nufi_download_metrics(nufi_handle *h, double *metrics4);

/* ---- device-resident stepping ----------------------------------------- */
/* One full time step on the device: rho(n) from slabs 0..n-1, then the
 * Poisson + interpolation solve (FFT-diagonal kernel) writes slab n and the
 * electric energy W_n = 1/2 int |E|^2 (what poisson::solve returns,
 * nufi/poisson.cpp:66-89).  energy may be NULL; if given, the call blocks. */
int nufi_step(nufi_handle *h, int64_t n, double *energy);
/* Steps n0 .. n1 (inclusive) as one CUDA-graph launch; energy_hist (may be
 * NULL) receives W_n0 .. W_n1.  Blocks when energy_hist != NULL. */
int nufi_run(nufi_handle *h, int64_t n0, int64_t n1, double *energy_hist);
/* Copies slabs n0 .. n1 of the device history into the caller's history
 * (reference layout, slab n at coeffs_base + n*stride_t).  Blocks. */
int nufi_download_history(nufi_handle *h, int64_t n0, int64_t n1, double *coeffs_base);
/* Electric energies W_n0 .. W_n1 recorded by nufi_step / nufi_run. Blocks. */
int nufi_download_energy(nufi_handle *h, int64_t n0, int64_t n1, double *energy);
/* Replaces poisson<double>::solve + dimN::interpolate<double,order>
 * (nufi/poisson.cpp:66-89, 190-219, 328-362; nufi/fields.hpp:63-142,
 * 186-300, 352-490) on host buffers: rho (N values, x fastest) in,
 * padded slab (stride_t values) out, returns W in *energy.  Blocks.
 * When rho is, bit for bit, the rho the last nufi_compute_rho published
 * (a zeroed buffer filled by nufi_download_rho) on a handle whose 1D split
 * trace sums rho itself, the call enables a speculative solve: the
 * following nufi_compute_rho calls also queue the device solve of their own
 * rho behind the trace, and a nufi_field_solve given that same rho returns
 * those results without a launch of its own (identical values: the same
 * kernel on the same input).  Any other input, or a compute_rho whose solve
 * went unused, switches the speculation off again. */
int nufi_field_solve(nufi_handle *h, const double *rho, double *slab_out, double *energy);

/* ---- phase-space sampling and the history on disk ----------------------- */
/* f at arbitrary points, FP64, from the handle's history (slabs 0..n, or
 * 0..n-1 for NUFI_EVAL_FTILDA):
 *   NUFI_EVAL_FTILDA      eval_ftilda (nufi/rho.hpp:31-61, 191-232, 318-367)
 *   NUFI_EVAL_F           eval_f (nufi/rho.hpp:63-96, 234-281, 369-426)
 *   NUFI_EVAL_PHASE_FLOW  1D eval_phase_flow (nufi/rho.hpp:98-131): the
 *                         eval_f trajectory only when n > 1, then
 *                         x - L floor(x / L); f_out unused.
 * pts: npts x (x.., v..) doubles; f_out: npts (may be NULL); feet: npts x
 * (x.., v..) final positions and velocities (may be NULL).  At most 2^36
 * points per call (NUFI_ERR_RANGE above).  Blocks. */
#define NUFI_EVAL_FTILDA     0
#define NUFI_EVAL_F          1
#define NUFI_EVAL_PHASE_FLOW 2
int nufi_eval_points(nufi_handle *h, int64_t n, int mode, int64_t npts, const double *pts, double *f_out,
                     double *feet);
/* The coefficient history as the reference's text files
 * (bin/test_nufi_cpu_3d_isolated.cpp:64-72, 190-211): a header of seven
 * lines (Nt = the configuration's Nt, dt as std::to_string prints it, Nx,
 * Ny, Nz, order, blank) and one coefficient per line, slabs 0..Nt: the
 * computed slabs 0..n1, then zeros for the steps not computed yet (the
 * reference's reader takes Nt + 1 slabs).  nufi_load_history also reads
 * files without the header (bin/test_nufi_gpu_1d.cpp:239, 364-366), uploads
 * the whole slabs found (as upload_phi) and returns their count without
 * trailing all-zero slabs; a header that disagrees with the handle is
 * NUFI_ERR_INVALID.  Resuming a run: load, then nufi_run from step
 * *n_slabs. */
int nufi_save_history(nufi_handle *h, int64_t n1, const char *path);
int nufi_load_history(nufi_handle *h, const char *path, int64_t *n_slabs);

/* ---- gradient of the time-integrated field energy ----------------------
 * No counterpart in the reference.  Objective J = 2 dt sum_{n=0}^{n1} W_n
 * (the time integral of int |E|^2 dx as a rectangle sum over the steps),
 * parameters theta = f0_params[0..3] = (alpha, k, u_b, sigma_b) of the 1D
 * initial conditions (k inside f0 only: the domain stays as configured;
 * u_b, sigma_b only for the bump-on-tail, else their derivatives are 0).
 * nufi_forward: steps 0..n1 (as nufi_run) and J.  nufi_objective: J from
 * the recorded W_n.  nufi_backward: dJ/dtheta (4 doubles) by the adjoint
 * of the whole backward-traced trajectory in FP64: the coefficient history
 * of the forward is the only checkpoint, the characteristics are recomputed
 * and walked back substep by substep (Stormer-Verlet inverted exactly).
 * 1D, orders 4 and 6; NUFI_ERR_RANGE if the forward has not computed slabs
 * 0..n1.  Blocks.  The order of the FP64 additions into the slab adjoints
 * is not fixed: results vary in the last bits between calls. */
int nufi_forward(nufi_handle *h, int64_t n1, double *J);
int nufi_objective(nufi_handle *h, int64_t n1, double *J);
int nufi_backward(nufi_handle *h, int64_t n1, double *grad4);

/* ---- batches of 1D instances --------------------------------------------
 * No counterpart in the reference.  Many 1D1V parameter sets of uneven
 * grid sizes (Nx dividing 256, any Nv, Nt; one precision, order 4) advanced
 * together: each time step is one trace launch over the work units of all
 * instances (256 threads x the tuned chains per thread over one instance's
 * velocity slice), one rho reduction and one field solve for all; the
 * whole run (and the whole adjoint sweep) is one CUDA-graph launch.
 * nufi_batch_create runs the autotuner (launch shapes timed on the device;
 * nufi_options.batch_no_autotune keeps defaults) and reports its choice through
 * nufi_batch_describe.  nufi_batch_forward: J_i = 2 dt sum_n W_n of every
 * instance (count doubles, may be NULL).  nufi_batch_backward: dJ_i/d(alpha,
 * k, u_b, sigma_b) (count x 4 doubles; the FP64 adjoint of nufi_backward).
 * Errors: nufi_batch_last_error(batch) (or NULL after a failed create). */
typedef struct nufi_batch nufi_batch;
int nufi_batch_create(const nufi_config *cfgs, int32_t count, int device, nufi_batch **out);
int nufi_batch_create_ex(const nufi_config *cfgs, int32_t count, const nufi_options *opt, int device,
                         nufi_batch **out);
int nufi_batch_destroy(nufi_batch *b);
const char *nufi_batch_last_error(const nufi_batch *b);
int nufi_batch_forward(nufi_batch *b, double *J);
int nufi_batch_backward(nufi_batch *b, double *grad);
int nufi_batch_energy(nufi_batch *b, int32_t i, double *energy);
int nufi_batch_stream(const nufi_batch *b, void **stream);
int nufi_batch_describe(const nufi_batch *b, char *buf, size_t len);

/* ---- allocation-free rho ------------------------------------------------
 * No counterpart in the reference.  rho of step n over [q_begin, q_end)
 * for callers that must not allocate device memory (no cudaMalloc, no
 * allocating library call): a plugin hosted by a framework that owns all
 * device memory through its own pool and forbids direct allocation, or a
 * real-time loop that reserves its device memory up front because
 * cudaMalloc can synchronise the device and take unbounded time.  FP64
 * plain form only.  The caller
 * passes device buffers: hist (slab k at hist + k*hist_stride doubles,
 * reference layout inside a slab, stride_t <= hist_stride, and
 * (Nt + 1) * hist_stride * 8 <= 2^50 bytes) and rho (Ns
 * doubles, overwritten, not accumulated).  Enqueued on `stream` (a
 * cudaStream_t, NULL = legacy default stream) on the current device;
 * returns without waiting.
 * Scratch: a fixed 8 MiB array inside the library (held by every GPU that
 * loads it until the process exits) for the per-block partial sums; about
 * Nm * Ns / 16 * 8 bytes must fit, larger problems get NUFI_ERR_RANGE.
 * The first call on a device looks up the array's device address (kept
 * for the life of the process, so a cudaDeviceReset between calls is not
 * supported); make that first call before any stream capture.  All calls
 * share the array,
 * so calls that overlap on the GPU (other streams, other threads) race;
 * serialise them.  Device-side range flags are not reported here.
 * Handle-less: errors via nufi_last_error(NULL). */
int nufi_compute_rho_noalloc(const nufi_config *cfg, int64_t n, const double *hist, int64_t hist_stride,
                             int64_t q_begin, int64_t q_end, double *rho, void *stream);

/* ---- information ------------------------------------------------------- */
int nufi_synchronize(nufi_handle *h);
/* stride_t (values per slab), number of spatial nodes, number of points */
int nufi_sizes(const nufi_handle *h, int64_t *stride_t, int64_t *n_spatial, int64_t *n_points);
/* The CUDA stream the handle launches on (cudaStream_t as void*), so that
 * callers can time with events on that stream. */
int nufi_stream(const nufi_handle *h, void **stream);
/* Number of kernels this handle has launched since creation. */
int nufi_launch_count(const nufi_handle *h, int64_t *count);
/* No counterpart in the reference: a JSON object naming the kernels and
 * launch shapes this handle chose (trace, whole-run kernel, field solve),
 * NUL-terminated into buf; NUFI_ERR_RANGE if len is too small (the text is
 * cut). */
int nufi_describe(const nufi_handle *h, char *buf, size_t len);
/* No counterpart in the reference: the plan nufi_create would choose for cfg
 * on a device with `sms` multiprocessors (1..4096), with no CUDA call: the
 * fields of nufi_describe plus "layout" (node counts, slab and table
 * strides, the 2D/3D table row stride and row step, partial-sum rows),
 * "staged_tpn", "solve_smem", "solve_why" and "adjoint" (its grid).  For
 * capacity planning; configuration errors as nufi_create's, via
 * nufi_last_error(NULL). */
int nufi_plan(const nufi_config *cfg, int sms, char *buf, size_t len);
int nufi_plan_ex(const nufi_config *cfg, const nufi_options *opt, int sms, char *buf, size_t len);
/* No counterpart in the reference: the field solve's circulant kernels for
 * cfg, computed on the host with no CUDA call (what nufi_create uploads).
 * Row r of nconv rows of Ns values (x fastest) is G_r; with
 * rho' = rho - mean(rho) the solve is out_r[i] = sum_j G_r[i - j] rho'_j
 * (index differences per axis, periodic):
 *   r = 0: spline coefficients c (unpadded; the slab pads periodically),
 *   r = 1: the potential phi at the nodes (W = prod L / (2 Ns) sum rho' phi),
 *   r = 2, 3, 4 (1D FP32-split only): K A, K B, K C of the per-cell
 *          quadratic of the kick, K = -dt^2 / dx^2.
 * *nconv receives the row count; kernels == NULL queries only.
 * NUFI_ERR_RANGE if len < nconv * Ns, NUFI_ERR_UNSUPPORTED above 16384
 * nodes. */
int nufi_solve_kernels(const nufi_config *cfg, double *kernels, int64_t len, int32_t *nconv);

#ifdef __cplusplus
}
#endif

#endif /* NUFI_GB300_H */
