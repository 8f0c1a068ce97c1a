/*
 * simpois_gpu.h -- C ABI of the GB300 (sm_103a) simpois hole-filling solver.
 *
 * The library fills the NaN pixels of planar float images by Laplace, Poisson
 * (with a data term) or biharmonic interpolation.  Two schedules are offered:
 *
 *  - the reference schedule (params.rtol == 0): the octave pyramid of
 *    imscript's `poisson_rec` (simpois.c:247-285) with `niter` colour-ordered
 *    Gauss-Seidel sweeps per level and the FP64 conjugate-gradient refinement
 *    `-c` selects (cleant_cgpois.c:197-278, minicg.c:24-56);
 *  - the converged schedule (params.rtol > 0): a multigrid-preconditioned
 *    conjugate gradient in FP32 inside an FP64 iterative refinement, run until
 *    the FP64 relative residual ||b - A u|| / ||b|| of the CG operator
 *    (5-point -Laplacian for tstep > 0, 13-point bilaplacian for tstep < 0)
 *    is at most rtol, for every channel of every image independently.
 *
 * It also offers imscript's AMLE interpolator (src/amle.c), simpois_amle*.
 *
 * Images are planar: sample (channel l, row j, column i) of a w x h x pd
 * image is at x[w*h*l + w*j + i], the layout of iio's *_split functions
 * (iio.h:42-43).  NaN marks an unknown pixel; every other value is copied to
 * the output bit for bit.
 *
 * Every entry point returns a status code and never exits the process.  Host
 * buffers are owned by the caller and are not retained after the call
 * returns.  A context is bound to one device and one stream; calls on one
 * context must not overlap (one context per host thread).
 */
#ifndef SIMPOIS_GPU_H
#define SIMPOIS_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SIMPOIS_OK            0
#define SIMPOIS_EINVAL        1  /* invalid argument                          */
#define SIMPOIS_ENOMEM        2  /* device or host allocation failed          */
#define SIMPOIS_NOT_CONVERGED 3  /* rtol not reached within the iteration cap */
#define SIMPOIS_BREAKDOWN     4  /* Krylov breakdown (p.Ap <= 0 or not finite)*/
#define SIMPOIS_ECUDA         5  /* CUDA runtime error                        */
#define SIMPOIS_ENODEV        6  /* no usable CUDA device                     */
#define SIMPOIS_SINGULAR      7  /* a channel has no known pixel: the system
                                    is singular; the reference schedule's
                                    result is returned for it                 */

typedef struct simpois_ctx simpois_ctx;

/* Solver parameters.  The first four are the simpois options -t -n -s -c
 * (simpois.c:357-360) with the reference's defaults; the next three are the
 * environment "smart parameters" PMSFAC, PONLIT, CG_EPS (simpois.c:244-245,
 * cleant_cgpois.c:125).  simpois_default_params() fills the defaults. */
typedef struct {
	float  tstep;     /* -t  0.25; > 0 Laplace/Poisson, < 0 biharmonic,
	                           < -1000 triharmonic (reference schedule only) */
	int    niter;     /* -n  10;  Gauss-Seidel sweeps per level             */
	int    scale;     /* -s  99;  maximum number of octaves                  */
	int    cgit;      /* -c  0;   CG iterations per level, -1 = #unknowns   */
	double pmsfac;    /* PMSFAC 3: data-term factor per octave               */
	double ponlit;    /* PONLIT 0: iterate only at the level of this width   */
	double cg_eps;    /* CG_EPS -1: absolute CG tolerance (< 0 = default)    */
	double rtol;      /* 0 = reference schedule; > 0 converged schedule      */
	int    max_iter;  /* converged schedule: cap on PCG iterations per
	                     channel, summed over refinements (0 = 500)          */
	int    flags;     /* SIMPOIS_FLAG_* bits                                 */
} simpois_params;

/* converged schedule: skip the multigrid preconditioner (plain CG) */
#define SIMPOIS_FLAG_NO_MG       0x1
/* converged schedule: launch the iterations eagerly, without CUDA graphs */
#define SIMPOIS_FLAG_NO_GRAPH    0x2
/* compute rel_residual_out (the FP64 residual of the stored float output) */
#define SIMPOIS_FLAG_OUT_RESID   0x4
/* converged schedule, 5-point operator: run the multigrid cycle with one
 * kernel launch per colour sweep instead of the fused tile kernels (same
 * arithmetic; for testing and comparison) */
#define SIMPOIS_FLAG_UNFUSED     0x8
/* converged schedule: time every launch of the main-loop kernels with a pair
 * of CUDA events on the context's stream (launches are issued eagerly, not
 * from a CUDA graph); see simpois_kernel_stats */
#define SIMPOIS_FLAG_KTIMER      0x10
/* reference schedule: the GS-only variant the ftr viewers use
 * (ftr/minisimpois.c:127-162): the plain clamped Laplacian for every tstep,
 * nearest-neighbour prolongation, no CG branch */
#define SIMPOIS_FLAG_MINI        0x20
/* converged schedule: the fused V-cycle's tile kernels load their regions
 * with the tensor memory accelerator (TMA) instead of vector loads, where a
 * level's rows are multiples of 16 bytes.  Same results bit for bit; measured
 * 1-4 % slower on the workloads here (the tiles are instruction-bound and a
 * TMA load is a wait for the whole box), so it is off by default. */
#define SIMPOIS_FLAG_TMA         0x40

/* Per-channel result record. */
typedef struct {
	int    status;           /* SIMPOIS_* code of this channel               */
	int    unknowns;         /* NaN pixels of this channel                   */
	int    iterations;       /* PCG iterations (converged schedule) or CG
	                            iterations at the finest level (reference)   */
	int    refinements;      /* FP64 refinement steps (converged schedule)   */
	double rel_residual;     /* FP64 relative residual of the solver state   */
	double rel_residual_out; /* same, of the float output (FLAG_OUT_RESID)  */
} simpois_report;

/* One image of a batch: device pointers, planar layout.  dat may be NULL. */
typedef struct {
	const float *in;
	const float *dat;
	float       *out;
	int          w, h, pd;
	float        tstep;   /* per image; overrides params->tstep            */
	double       rtol;    /* per image; overrides params->rtol when > 0    */
} simpois_image;

/* Fill *p with the simpois defaults (-t 0.25 -n 10 -s 99 -c 0, PMSFAC 3,
 * PONLIT 0, CG_EPS -1, rtol 0). */
void simpois_default_params(simpois_params *p);

/* Read PMSFAC, PONLIT, CG_EPS and SIMPOIS_RTOL from the environment into *p,
 * the way the reference's smart parameters do (smapa.h:44-60). */
void simpois_params_from_env(simpois_params *p);

/* Create a context on `device`, issuing work on `stream` (a cudaStream_t,
 * NULL = the legacy default stream). */
int simpois_create(simpois_ctx **ctx, int device, void *stream);
int simpois_destroy(simpois_ctx *ctx);

/* Text for a status code; the last error message recorded on a context. */
const char *simpois_strerror(int status);
const char *simpois_last_error(const simpois_ctx *ctx);

/* Solve one planar w x h x pd image held in HOST memory (the work of
 * poisson_solver_separable, simpois.c:288-302).  dat may be NULL.  reports,
 * if not NULL, receives pd records.  Returns the worst channel status.
 * With rtol > 0, w*h*pd a multiple of 4 and page-locked (cudaHostAlloc /
 * cudaHostRegister), 16-byte aligned out and dat, the call moves only what
 * the converged schedule needs: in whole; dat in the 4-pixel groups holding
 * an unknown, read in place; out back whole while the solve runs (its known
 * pixels are those of in), then its groups holding an unknown, written in
 * place (SIMPOIS_NO_DIRECT_IO=1: whole-buffer copies).  On a failure status
 * out may then hold the input. */
int simpois_solve(simpois_ctx *ctx, float *out, const float *in,
		const float *dat, int w, int h, int pd,
		const simpois_params *params, simpois_report *reports);

/* Same, with every pointer in DEVICE memory; the call returns when the
 * output is written (the context's stream is synchronised). */
int simpois_solve_device(simpois_ctx *ctx, float *out, const float *in,
		const float *dat, int w, int h, int pd,
		const simpois_params *params, simpois_report *reports);

/* Solve n images of possibly different sizes in one batched solve (device
 * pointers).  reports receives sum(pd) records in image order. */
int simpois_solve_batch(simpois_ctx *ctx, const simpois_image *images, int n,
		const simpois_params *params, simpois_report *reports);

/* simpois_solve_batch with every image's in, dat and out in HOST memory (the
 * batched form of poisson_solver_separable, simpois.c:288-302, over many
 * images): the inputs go to the device, the batch is solved, the outputs come
 * back; the call returns when they are written.  Page-locked buffers move at
 * the link's full rate; with rtol > 0 an image whose w*h*pd is a multiple of
 * 4 and whose out and dat are page-locked and 16-byte aligned moves as in
 * simpois_solve: dat only in the 4-pixel groups holding an unknown, out back
 * whole while the solve runs, then its groups holding an unknown. */
int simpois_solve_batch_host(simpois_ctx *ctx, const simpois_image *images,
		int n, const simpois_params *params, simpois_report *reports);

/* FP64 relative residual of a float output `u` (device pointers) for every
 * channel: kind 0 = 5-point -Laplacian, 1 = 13-point bilaplacian; unknowns
 * are the NaN pixels of `in`.  rel and bnorm receive pd values (host). */
int simpois_residual_device(simpois_ctx *ctx, const float *u, const float *in,
		const float *dat, int w, int h, int pd, int kind, double *rel,
		double *bnorm);

/* simpois_residual_device without any memory allocation (no counterpart in
 * the reference).  For callers that may not allocate device memory where
 * they check a result -- a device budget fully reserved up front, a path that
 * must not enter an allocator.  Its scratch is a fixed 1 MiB + 4 KiB array
 * inside the library (held on each GPU that loads the library until exit);
 * at most 16,777,216 pixels per channel and 64 channels, else SIMPOIS_EINVAL.
 * The first call on a device looks up the array's device address and keeps
 * it for the life of the process; a cudaDeviceReset invalidates it, so do not
 * call this entry point on a device after resetting it.  Every call ends by
 * synchronising ctx's stream (the sums come back to the host), so it cannot be
 * called while that stream is being captured.  All calls share the array, so
 * calls that overlap on the GPU race: serialise them. */
int simpois_residual_device_noalloc(simpois_ctx *ctx, const float *u,
		const float *in, const float *dat, int w, int h, int pd, int kind,
		double *rel, double *bnorm);

/* Adjoint of the converged Laplace/Poisson fill (device pointers).  Given
 * grad_out = dL/d(out), solves A lambda = grad_out on the unknowns (A is the
 * symmetric 5-point operator) and writes
 *   grad_in[k]  = grad_out[k] + sum over unknown 5-neighbours p of lambda[p]
 *                 at known pixels k, 0 at unknown pixels;
 *   grad_dat[p] = -lambda[p] at unknown pixels, 0 elsewhere (may be NULL).
 * params->rtol is the tolerance of the adjoint solve (0 = 1e-6). */
int simpois_adjoint_device(simpois_ctx *ctx, const float *grad_out,
		const float *in, int w, int h, int pd, float *grad_in,
		float *grad_dat, const simpois_params *params,
		simpois_report *reports);

/* AMLE fill (absolutely minimizing Lipschitz extension), the work of
 * imscript's amle (src/amle.c:196-246, replaces that function) on every
 * channel of a planar w x h x pd image whose NaN pixels are unknown: nn
 * neighbours of the reference's table (AMLE_NN: 4, 6, 8, 16, 26 or 32; 0..32),
 * niter iterations (AMLE_NITER, the reference's default 100), init (may be
 * NULL, planar like in) the start of the upper iterate at the unknowns (the
 * AMLE_INIT image).  out receives the upper iterate, as the reference's.  The
 * sweeps visit the colour classes (i + k j) mod m in turn instead of raster
 * order: the output is bit for bit the colour-ordered restatement of the
 * reference; with the default 4 neighbours both orders reach the same fixed
 * point.  gap, if not NULL, receives 2 pd values: per channel the max and the
 * mean of |lower - upper| over the unknowns after the last iteration (what
 * the reference prints).  simpois_amle_device takes device pointers,
 * simpois_amle host pointers. */
int simpois_amle_device(simpois_ctx *ctx, float *out, const float *in,
		int w, int h, int pd, int nn, int niter, const float *init,
		double *gap);
int simpois_amle(simpois_ctx *ctx, float *out, const float *in, int w, int h,
		int pd, int nn, int niter, const float *init, double *gap);

/* Autotuner (no counterpart in the reference, which has no launch-shape
 * knobs).  The converged 5-point V-cycle runs the levels wider than a
 * hand-over size in 32 x 32 tile kernels and the rest in one shared-memory
 * block per channel; the hand-over size (8..128) moves work between the two
 * kernels but changes no bit of any result.  Each tile kernel smooths with
 * 1, 2 or 3 red-black sweeps per side over a shared-memory region of the
 * tile plus a halo of 4 (1 or 2 sweeps) or 8 (3 sweeps) pixels; the count
 * is part of the preconditioner, so it changes the iterates (every result
 * still meets its tolerance).
 * simpois_autotune_ex solves the batch like simpois_solve_batch while timing
 * every distinct hand-over among 32, 64 and 128 (plus the default) at 2
 * sweeps, then 1 and 3 sweeps at the best hand-over; it keeps the fastest
 * pair for batches of the same channel shapes and operators on this context
 * (later solves of such batches, and their adjoints, use it), leaves the
 * batch solved with it, and writes it to *coarse_max and *sweeps (either may
 * be NULL; the values of the 5-point channels when the batch mixes
 * operators).  simpois_autotune is simpois_autotune_ex without *sweeps.
 * simpois_set_coarse_max and simpois_set_sweeps fix one choice for every
 * later solve on the context (0 restores tuned-or-default: hand-over 64, 2
 * sweeps); the autotuner then tunes only the other. */
int simpois_autotune_ex(simpois_ctx *ctx, const simpois_image *images, int n,
		const simpois_params *params, simpois_report *reports,
		int *coarse_max, int *sweeps);
int simpois_autotune(simpois_ctx *ctx, const simpois_image *images, int n,
		const simpois_params *params, simpois_report *reports,
		int *coarse_max);
int simpois_set_coarse_max(simpois_ctx *ctx, int coarse_max);
int simpois_set_sweeps(simpois_ctx *ctx, int sweeps);

/* Keeps the autotuner's choices in a text file across processes (NULL or ""
 * stops).  The call reads the choices the file holds for this context's device
 * model (a file written on another model reads as empty; a missing file is
 * fine; a file that is not a tuning file, or holds a malformed choice, gives
 * SIMPOIS_EINVAL and leaves the context without a file).  From then on
 * simpois_autotune_ex solves a batch whose shapes have a known choice with it
 * instead of timing the candidates again, and writes every new choice back
 * (the file is replaced through a temporary file in its directory).
 * SIMPOIS_TUNE_CACHE=path does the same for every new context. */
int simpois_set_tune_cache(simpois_ctx *ctx, const char *path);

/* Device-memory budget of a context (no counterpart in the reference, whose
 * xmalloc exits on an allocation failure, simpois.c:10-19).  A solve whose
 * working set would take the context's device arena above `bytes` returns
 * SIMPOIS_ENOMEM before it allocates, frees or launches anything, leaves the
 * output untouched and the context usable; 0 removes the limit (the default).
 * For services that share one GPU between several contexts. */
int simpois_set_memory_limit(simpois_ctx *ctx, size_t bytes);

/* Instrumentation (no counterpart in the reference): the number of kernel
 * launches this context has issued (a graph replay counts its kernel nodes),
 * and a reset. */
long long simpois_launch_count(const simpois_ctx *ctx);
void simpois_reset_launch_count(simpois_ctx *ctx);

/* Instrumentation (no counterpart in the reference): per-kernel totals of the
 * solves run with SIMPOIS_FLAG_KTIMER, as a JSON object
 *   {"<kernel>": {"launches": n, "ms": t, "bytes": b}, ...}
 * where ms sums the CUDA-event durations of the launches and bytes sums their
 * algorithmic bytes (reads plus writes per active tile pixel).  The string
 * lives until the next call on the context. */
const char *simpois_kernel_stats(simpois_ctx *ctx);
void simpois_reset_kernel_stats(simpois_ctx *ctx);

/* Drop-in replacements with the reference's signatures.  They run on device
 * 0 through a process-wide context and, like the reference, return nothing;
 * a failure is printed to stderr and leaves `out` holding the input.
 *   poisson_solver_separable   simpois.c:288-290
 *   poisson_rec                simpois.c:247-248 (one channel)
 * The smart parameters PMSFAC, PONLIT, CG_EPS and SIMPOIS_RTOL are read from
 * the environment once, as in the reference. */
void poisson_solver_separable(float *out, float *in, float *dat, int w, int h,
		int pd, float tstep, int niter, int scale, float cgrad);
void poisson_rec(float *u, float *g, float *f, int w, int h, float tstep,
		int niter, int scale, int cgit);

/* Drop-in for imscript's amle(y, x, w, h) (src/amle.c:196): one channel on
 * device 0 through the process-wide context, AMLE_NN and AMLE_NITER read from
 * the environment as the reference reads them; AMLE_INIT, an image file, is
 * read by the amle command only. */
void amle(float *y, float *x, int w, int h);

/* Drop-in for poisson_recursive of the ftr viewers (ftr/minisimpois.c:127-149,
 * called in place by ftr/vnav.c:855,893): one channel, the GS-only pyramid of
 * SIMPOIS_FLAG_MINI; u may alias g. */
void poisson_recursive(float *u, float *g, float *f, int w, int h, float tstep,
		int niter, int scale);

#ifdef __cplusplus
}
#endif

#endif /* SIMPOIS_GPU_H */
