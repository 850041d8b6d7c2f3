/*
 * chgpu.h -- C ABI of the GB300 channel-flow time step (libchgpu.so).
 *
 * Drop-in replacement for the module procedures that channel.f90 calls on
 * its hot path.  Plain pointers and sizes only; no exit() inside; every
 * entry point returns 0 on success or a negative CHGPU_E* code, with the
 * message in chgpu_last_error().  One handle owns one run's device state
 * (field, RK history, spectra of the products, work buffers, tables) on the
 * current CUDA device and one CUDA stream; call it from one host thread.
 *
 * Field layout at this boundary is the reference's: complex128 interleaved,
 * Fortran order V(iy,iz,ix,ic), iy=-1..ny+1 fastest, then iz=-nz..nz,
 * ix=0..nx, ic=1..3  (dnsdata.f90:132; restart files, dnsdata.f90:821-848).
 *
 * A Fortran 2008 iso_c_binding interface for these entry points ships in
 * channel_gb300/fortran/chgpu_interface.f90.
 */
#ifndef CHGPU_H
#define CHGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHGPU_OK 0
#define CHGPU_E_PARAM -1     /* bad parameters or sizes */
#define CHGPU_E_CUDA -2      /* CUDA runtime error (message has the name) */
#define CHGPU_E_NOMEM -3     /* device allocation failed */
#define CHGPU_E_NONFINITE -4 /* NaN/Inf met in the flow field or CFL */
#define CHGPU_E_STATE -5     /* call out of order (e.g. step before upload) */

#define CHGPU_FP64 0  /* every stage in FP64 */
#define CHGPU_MIXED 1 /* FFTs, products, nonlinear stencils in FP32; solves FP64 */
#define CHGPU_FP64DD 2 /* FFTs, products, nonlinear stencils in double-float (two FP32
                        * numbers, ~48 bits) on the FP32 pipes; everything else FP64 */

/* dns.in after read_dnsin (dnsdata.f90:98-125). `ni` holds 1/Re, the value
 * read_dnsin leaves in `ni`. Logical flags are 0/1. */
typedef struct chgpu_params {
  int nx, ny, nz;
  double alfa0, beta0;
  double ni;
  double a, ymin, ymax;
  int cpi, cpi_type;
  double gamma;
  double meanpx, meanpz;
  double meanflowx, meanflowz;
  double u0, uN;
  double deltat, cflmax, time;
  double dt_field, dt_save, t_max;
  int time_from_restart;
  long long nstep;
  int npy;
  int precision; /* CHGPU_FP64, CHGPU_MIXED or CHGPU_FP64DD */
} chgpu_params;

/* The numbers outstats prints (dnsdata.f90:876-879), plus the scalars the
 * driver needs: line[11] = time, dudy_bot, -dudy_top, dwdy_bot, -dwdy_top,
 * fr_x, meanpx+corrpx, fr_z, meanpz+corrpz, CFL*deltat, deltat. */
typedef struct chgpu_stats {
  double line[11];
  double fr[3];
  double corrpx, corrpz, meanpx, meanpz;
  double cfl;    /* max CFL number measured (runtime_global) */
  double deltat; /* time step for the next step */
  double time;
  long long istep;
} chgpu_stats;

typedef struct chgpu_handle chgpu_handle;

/* init_memory + init_fft + setup_derivatives + setup_boundary_conditions
 * (dnsdata.f90:129-177, ffts.f90:35-76, dnsdata.f90:241-286, 290-308).
 * Allocates everything the step needs on the current device. */
int chgpu_create(const chgpu_params* p, chgpu_handle** out);

/* free_fft + free_memory (ffts.f90:110-115, dnsdata.f90:222-229). */
int chgpu_destroy(chgpu_handle* h);

/* Copy the field in after read_restart_file (dnsdata.f90:677-720) or out
 * before save_restart_file (dnsdata.f90:821-848). `V` holds
 * 3*(nx+1)*(2nz+1)*(ny+3) complex values (twice as many doubles). */
int chgpu_upload_field(chgpu_handle* h, const double* V);
int chgpu_download_field(chgpu_handle* h, double* V);
size_t chgpu_field_doubles(const chgpu_handle* h);

/* The driver's start-up (channel.f90:64-116): sets time and deltat as the
 * driver holds them after re-reading dns.in, runs the initial CFL pass over
 * iy=1..ny-1 (channel.f90:96-99: convolutions with compute_cfl), the flow
 * rate and CPI pressure gradient (channel.f90:101-115), then outstats. */
int chgpu_start(chgpu_handle* h, double time, double deltat, chgpu_stats* st);

/* bc0(0,0)%u=u0; bcn(0,0)%u=uN (channel.f90:122-124). */
int chgpu_set_wall_velocity(chgpu_handle* h, double u0, double uN);

/* buildrhs(ODE, compute_cfl) (dnsdata.f90:611-673): convolutions of every
 * y-plane and the explicit right-hand sides; uses the handle's deltat. */
int chgpu_buildrhs(chgpu_handle* h, const double ode[3], int compute_cfl);

/* linsolve(lambda) (linsolve_blocking.inc:3-107): implicit v and eta solves,
 * wall/ghost values, mean-flow correction, velocity recovery. */
int chgpu_linsolve(chgpu_handle* h, double lambda);

/* outstats (dnsdata.f90:853-880) without file output: CFL max -> deltat
 * (when cflmax>0), wall gradients, the Runtimedata numbers. */
int chgpu_outstats(chgpu_handle* h, chgpu_stats* st);

/* One whole time-loop iteration (channel.f90:118-167): istep+1, three RK
 * substeps (time advance, buildrhs, linsolve) and outstats, all on the
 * device; the step is captured once into a CUDA graph and replayed.
 * `st` may be NULL (then no host synchronisation happens). */
int chgpu_step(chgpu_handle* h, chgpu_stats* st);

/* Read the statistics of the last completed step (synchronises). */
int chgpu_get_stats(chgpu_handle* h, chgpu_stats* st);

/* Wait for all work queued on the handle's stream; reports device-side
 * error flags (non-finite CFL) as CHGPU_E_NONFINITE. */
int chgpu_synchronize(chgpu_handle* h);

/* Ensemble of independent runs (uneven sizes and precisions allowed): every
 * member is an ordinary handle, reached with chgpu_ensemble_member for
 * uploads, chgpu_start, downloads, statistics, tiles or a body force; one
 * chgpu_ensemble_step advances all members by one RK3 step with a single
 * CUDA-graph launch whose branches (one per member, each the member's own
 * step) run concurrently.  The graph is re-captured when a
 * member's launch sequence changes (tiles, body force on/off).  st: NULL, or
 * one record per member (synchronises).  No counterpart in the reference,
 * which runs one channel per MPI job. */
typedef struct chgpu_ensemble chgpu_ensemble;
int chgpu_ensemble_create(const chgpu_params* params, int n, chgpu_ensemble** out);
int chgpu_ensemble_destroy(chgpu_ensemble* e);
int chgpu_ensemble_size(const chgpu_ensemble* e);
chgpu_handle* chgpu_ensemble_member(chgpu_ensemble* e, int i);
int chgpu_ensemble_step(chgpu_ensemble* e, chgpu_stats* st);
int chgpu_ensemble_synchronize(chgpu_ensemble* e);
void* chgpu_ensemble_stream(chgpu_ensemble* e);
/* Message of the ensemble's last failing call (or of a failed create). */
const char* chgpu_ensemble_last_error(const chgpu_ensemble* e);

/* Autotuner of the step's launch shapes on this handle's sizes: the z
 * transforms (1, 2, 4 or 8 columns per block, then 128, 192 or 256 threads
 * per block) and the x-row kernel (1, 2 or 4 rows per block in each of its
 * register-cap variants, then its block size) where the generic transform
 * kernels run, the register cap of the register-blocked x-row kernel where
 * it runs; then the banded solves as one fused kernel (two threads per
 * (kx, +-kz) pair), as factorisation + substitution kernels (four threads
 * per pair), as those two with each substep's factorisation on a side
 * stream, overlapping the substep's transforms (it needs only dt), or with
 * the factorisation ahead and the fused kernel's two threads per pair
 * substituting, or with the factorisation ahead and eight threads per pair
 * substituting (one per system, mode and real / imaginary component); and
 * the step on one stream or in two kx halves, timed as whole steps.  Keeps the fastest; the field, the RK history and the module
 * scalars are saved and put back, and the results of a step do not depend on
 * the tiles.  Optional: without it the handle uses tiles sized from the
 * shared-memory budget, the split solve with the factorisation ahead below
 * 65 536 pairs and the fused solve in two halves from there on.  No
 * counterpart in the reference. */
#define CHGPU_NTILES 7
int chgpu_autotune(chgpu_handle* h);
/* tiles = {z columns per block, x rows per block, x-row variant, z threads
 *          per block, x threads per block, solve form (1: fused, 2: split,
 *          3: split with the factorisation ahead on a side stream, 4: the
 *          factorisation ahead, fused-kernel substitutions, 5: the
 *          factorisation ahead, eight threads per pair), step halves (1 or
 *          2)}.  z columns 0: the
 * register-blocked z kernels (compile-time plans for nzd = 32, 48, 64, 96,
 * 192, 384, 768, 1536); x-row variant 1-3: the generic kernel with its
 * registers capped for that many 256-thread blocks per SM, 4 and 5: the
 * register-blocked x-row kernel (nxd = 32 ... 768) with registers for 3 or
 * 4 resident blocks.  A handle starts with the register-blocked kernels
 * where they measured faster (FP32: z and x; FP64: z); the autotuner keeps
 * that choice and tunes within it, so its tiles do not change the results.
 * Switching between generic and register-blocked kernels with
 * chgpu_set_tiles changes the rounding of the transforms (their
 * factorisations differ), not their accuracy. */
int chgpu_tiles(const chgpu_handle* h, int tiles[CHGPU_NTILES]);
/* Applies tiles found by chgpu_autotune on another handle of the same sizes
 * and precision; CHGPU_E_PARAM when they do not fit this handle. */
int chgpu_set_tiles(chgpu_handle* h, const int tiles[CHGPU_NTILES]);
/* The captured step as one stream (1) or with k_rhs, k_linsolve and the
 * next z-inverse split in two kx halves on two streams (2), which overlaps
 * one half's solve with the other half's work; the default is 2 from 65 536
 * (kx, +-kz) pairs on, else 1.  Results do not depend on it. */
int chgpu_set_step_halves(chgpu_handle* h, int halves);

/* Physical-space export of the field: the reference's exporter
 * out_exporter/out2bin.f90 (convert_outfile :141-203, xz_interpolation
 * :236-275, undersampled_to_fullindex :279-299, filter_vfield :338-347) on
 * the handle's current field.  Planes iy = 0..ny go through the
 * un-dealiased inverse transform on the (2nx+1) x (2nz+1) grid and are
 * sampled on nxtot x nztot points (nint(undersample * (2n+1)), :76-78).
 * `out` (host) receives vec(3, nxtot, 0:ny, nztot) in Fortran order, i.e.
 * the C array out[nztot][ny+1][nxtot][3] -- the body of the .bin file that
 * write_brutal_bin writes (:207-232).  Sample indices past the last grid
 * point (undersample factors whose grid does not divide the period) wrap
 * to the first point of the periodic domain. */
#define CHGPU_EXPORT_ALL 0
#define CHGPU_EXPORT_LARGE 1 /* -l: large scales, modes with |beta0 kz| <= z_threshold kept */
#define CHGPU_EXPORT_SMALL 2 /* -s: small scales, modes with |beta0 kz| > z_threshold kept */
typedef struct chgpu_export_opts {
  int fluct_only;    /* -f: the mean mode (kx, kz) = (0, 0) removed */
  int part;          /* CHGPU_EXPORT_ALL, _LARGE or _SMALL */
  int z_threshold;   /* largesmall_settings.in (an integer, as read there) */
  float undersample; /* -u factor (real*4 in the reference); 1 = full grid */
} chgpu_export_opts;
/* dims = {nxtot, ny+1, nztot} for this factor; CHGPU_E_PARAM when empty. */
int chgpu_export_dims(const chgpu_handle* h, float undersample, int dims[3]);
/* opts NULL = defaults (full field, full grid). */
int chgpu_export_physical(chgpu_handle* h, const chgpu_export_opts* opts, double* out);

/* Body force F(iy,iz,ix,ic) added to the explicit terms of buildrhs: the
 * `bodyforce` hook of the reference (dnsdata.f90:617-659), which
 * set_body_force fills before each buildrhs (channel.f90:129-131).  F has
 * V's restart-file layout and stays in effect until the next call; NULL
 * switches the forcing off.  Its ghost rows are rebuilt as buildrhs does
 * (dnsdata.f90:617-628): F(0) = F(ny) = 0, F(-1) and F(ny+1) such that the
 * compact fourth derivative of F vanishes at iy = 1 and iy = ny-1. */
int chgpu_set_body_force(chgpu_handle* h, const double* F);

/* On-device statistics of the field, the mean and variance profiles of the
 * reference's post-processing (postpro/history/var_history.f90:37-84).
 * chgpu_stats_accumulate adds the current field to compensated running sums
 * (one kernel, in stream order); chgpu_profiles returns for each component
 * ic=1..3 and row iy=-1..ny+1 (arrays of 3*(ny+3), iy fastest)
 *   mean = < Re V(iy,0,0,ic) >,
 *   var  = < sum_{ix,iz} f_ix |V(iy,iz,ix,ic)|^2 > - mean^2, f_ix = 1 (ix=0), 2,
 * over the samples since chgpu_stats_reset (the squared rms profile). */
int chgpu_stats_reset(chgpu_handle* h);
int chgpu_stats_accumulate(chgpu_handle* h);
int chgpu_profiles(chgpu_handle* h, double* mean, double* var, long long* nsamples);

/* Spanwise spectra of the Reynolds-stress budgets, the reference's
 * post-processing program postpro/tke/uiuj_spectra.f90, accumulated on the
 * device from the handle's current field (call chgpu_tke_accumulate between
 * steps, at the statistics cadence).
 *   chgpu_tke_reset(h, mean): the mean profiles removed from each sample,
 *     mean = U, W, P (3 arrays of ny+3, iy = -1..ny+1), as the reference
 *     averages them over the same files first (:135-150); clears the sums.
 *   chgpu_tke_accumulate(h, pressure): one sample.  pressure: NULL, or the
 *     pressure field of this sample in V's restart-file layout (one complex
 *     component); give one with every sample or with none -- without it the
 *     pressure terms (pstrain, ptrsp, PHIptrsp) stay zero.
 *   chgpu_tke_result(h, timestwo, mean7, spectra, profiles, nsamples):
 *     mean7(1:7, iy) = U, W, dU/dy, dW/dy, d2U/dy2, d2W/dy2, P;
 *     spectra(irs, term, iz, iy) and profiles(irs, term, iy) (the sum over
 *     iz), Fortran order with irs fastest, irs = uu, vv, ww, uv, vw, uw,
 *     term = var, prod, psdiss, ttrsp, vdiff, pstrain, ptrsp, PHIttrsp (not
 *     assigned by the reference: zero), PHIvdiff, PHIptrsp; the sums divided
 *     by the number of samples, the flux derivatives taken (:243-259) and,
 *     with timestwo, var doubled (-two, :262) -- the arrays the reference
 *     writes to uiuj_spectra.bin.  Any output may be NULL.
 * All sums are FP64 in every precision path.  The first reset allocates 16
 * field-sized FP64 buffers and the padded-grid work of a chunk of planes
 * (~2 GB). */
int chgpu_tke_reset(chgpu_handle* h, const double* mean);
int chgpu_tke_accumulate(chgpu_handle* h, const double* pressure);
int chgpu_tke_result(chgpu_handle* h, int timestwo, double* mean7, double* spectra, double* profiles,
                     long long* nsamples);

/* Field snapshot for output without stalling the time loop (the dt_field /
 * dt_save writes, dnsdata.f90:882-918).  chgpu_snapshot_async copies V to a
 * device staging buffer in stream order and then, on a side stream while
 * later steps run, to a pinned host buffer owned by the handle.
 * chgpu_snapshot_wait blocks until that copy is complete and points *V at
 * the field (restart-file layout), valid until the next chgpu_snapshot_async.
 * One snapshot may be in flight at a time. */
int chgpu_snapshot_async(chgpu_handle* h);
int chgpu_snapshot_wait(chgpu_handle* h, const double** V);

/* The handle's CUDA stream (cudaStream_t), for callers that order their own
 * work against the solver's. */
void* chgpu_stream(chgpu_handle* h);

/* Per-kernel device timing (the per-step timing of the reference's `chron`
 * flag, channel.f90:119-121,175-178, refined to kernels).  While profiling is
 * on, chgpu_step issues its launches directly on the stream with a CUDA event
 * pair around each kernel instead of replaying the graph.
 * chgpu_kernel_times synchronises and returns, per kernel kind, the summed
 * device milliseconds and launch counts since profiling was switched on. */
#define CHGPU_NKINDS 6 /* z-inverse, x-rows, z-forward, rhs, linsolve, scalars */
int chgpu_set_profiling(chgpu_handle* h, int on);
int chgpu_kernel_times(chgpu_handle* h, double ms[CHGPU_NKINDS], long long launches[CHGPU_NKINDS]);
const char* chgpu_kernel_kind_name(int kind);

/* The device-side waits of the generic z-transform kernels (their bulk
 * copies into shared memory) give up after a bounded number of polls, set the
 * handle's error word and return; the next synchronising call reports
 * CHGPU_E_CUDA ("... did not complete in time").  chgpu_set_wait_limit sets
 * the first wait's poll count (polls >= 0; < 0 restores the default of 2^22,
 * seconds in all), so that the time-out path can be exercised: with 0 the
 * wait gives up at once, then waits (with the full limit) for the copy in
 * flight and returns.  The register-blocked kernels have no such waits.  No
 * counterpart in the reference. */
int chgpu_set_wait_limit(chgpu_handle* h, int polls);

/* Kernel launches issued by the handle since creation (for accounting). */
long long chgpu_launch_count(const chgpu_handle* h);

/* Throughput of the current device, for reporting kernels against the roofs
 * they are bound by: FP64 and FP32 fused multiply-add rates (TFLOP/s, FMA =
 * 2 flops; 8 independent FMA chains per thread, 8 blocks of 256 threads per
 * SM, CUDA events) and a device-to-device copy of 1 GiB (GB/s, read + write
 * bytes).  Any output may be NULL (that measurement is skipped).  Temporarily
 * allocates 2 GiB when copy_gbs is requested.  No counterpart in the
 * reference (its `chron` flag times whole steps only). */
int chgpu_measure_peaks(double* fp64_tflops, double* fp32_tflops, double* copy_gbs, char* err, size_t errlen);

/* y[i] = 1/x[i] as the banded solves form their pivot reciprocals (a
 * Newton-Raphson reciprocal: within half an ulp plus 2^-88 relative of the
 * exact value), for n host values; allocates 16 n bytes of device memory for
 * the call.  No counterpart in the reference (LU5decompStep divides,
 * rbparmat_blocking.f90:41). */
int chgpu_pivot_reciprocal(const double* x, double* y, size_t n, char* err, size_t errlen);

/* The implicit solve of linsolve (linsolve_blocking.inc:3-107) for callers
 * that cannot allocate device memory.  No counterpart in the reference: it
 * exists for hosts that own every byte of device memory themselves (a fixed
 * arena handed out by a framework, memory reserved at start-up, code that may
 * not trigger an allocation between launches) and so cannot let a library
 * call cudaMalloc.  It allocates nothing: no cudaMalloc/cudaFree, no heap.
 *
 *   field   caller's device buffer, complex128 interleaved, plane-major:
 *           [ic=1..3][iy=-1..ny+1][ix=0..nx][iz=-nz..nz] (iz fastest).  On
 *           entry components 1 and 2 hold, for iy=1..ny-1, the eta and v
 *           right-hand sides buildrhs leaves there; on return it holds the
 *           solved u, v, w (all rows), exactly as chgpu_linsolve leaves V.
 *   scalars in/out, host memory, 7 doubles: [0..2] flow rates fr (out),
 *           [3] corrpx and [4] corrpz (in: previous values, out: new),
 *           [5] meanpx (in/out, updated under CPI), [6] meanpz (in).
 *   stream  cudaStream_t to run on (NULL: legacy default stream); the call
 *           copies tables and scalars from host memory on it and returns
 *           after the stream has finished the solve.
 *   err     optional buffer for a message when the call fails.
 * The kernel's scratch (the factors of the two pentadiagonal systems), the
 * wall-normal tables and the scalars live in file-scope device arrays of the
 * library: CHGPU_NOALLOC_SCRATCH_BYTES of factor scratch (enough for
 * 4*(ny-1)*(nx+1)*(nz+1) doubles), ny <= CHGPU_NOALLOC_MAX_NY; larger sizes
 * are rejected with CHGPU_E_PARAM and a message.  Every GPU that loads the
 * library holds these arrays until the process exits.  Each call looks up
 * their device addresses on the current device.  All calls share the
 * arrays: calls that overlap on the GPU race; each call rewrites every word
 * it later reads. */
#define CHGPU_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define CHGPU_NOALLOC_MAX_NY 1024
int chgpu_linsolve_noalloc(const chgpu_params* p, double lambda, double* field, double* scalars, void* stream,
                           char* err, size_t errlen);

/* Message of the last failing call on this handle (or of chgpu_create when
 * h is NULL). Never NULL. */
const char* chgpu_last_error(const chgpu_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* CHGPU_H */
