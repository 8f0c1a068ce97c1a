/*
 * simpois_oracle.c -- CPU restatement of imscript's `simpois` hole-filling path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it; the product
 * (the CUDA library and the CLI) never links or calls it.
 *
 * Every function restates, with the same floating-point operations in the same
 * order, one step of the reference algorithm (file:line of mnhrdt/imscript
 * given per function), so that in raster order this file reproduces the
 * reference binary bit for bit (pinned by tests/test_oracle_golden.py against
 * fixtures produced by the reference built from its own sources).  It must be
 * compiled with -ffp-contract=off: a fused multiply-add changes the rounding.
 *
 * Two sweep orders are offered for the Gauss-Seidel step:
 *   ORACLE_ORDER_RASTER  the reference's in-place raster sweep (simpois.c:109)
 *   ORACLE_ORDER_COLOUR  the colour-ordered sweep the GPU runs: colour classes
 *                        (i+j)&1 for the 5-point operator, (i+3j)%5 for the
 *                        13-point bilaplacian, (i+5j)%13 for the 25-point
 *                        triharmonic operator, each class swept in turn.
 *                        Within a class no pixel reads another of its class,
 *                        so the result does not depend on the order inside a
 *                        class and is the exact CPU image of the GPU sweep.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_ORDER_RASTER 0
#define ORACLE_ORDER_COLOUR 1

typedef struct {
	double pmsfac;   /* data-term factor per octave   (simpois.c:244,262)     */
	double ponlit;   /* only iterate at this width     (simpois.c:245,272)     */
	double cg_eps;   /* <0: per-branch default, else absolute CG tolerance
	                    (cleant_cgpois.c:125,245)                              */
	int order;       /* ORACLE_ORDER_RASTER or ORACLE_ORDER_COLOUR            */
	int cg_log;      /* 1: print the per-iteration trace of minicg.c:46       */
} oracle_opts;

typedef struct {        /* statistics of the last CG call (for tests)       */
	int iterations;
	double rr_final;
} oracle_cg_stats;

static oracle_cg_stats g_last_cg;

static void *ora_alloc(size_t n)
{
	void *p = malloc(n ? n : 1);
	if (!p) { fprintf(stderr, "oracle: out of memory (%zu bytes)\n", n); abort(); }
	return p;
}

/* ---- stencils on float images (simpois.c:25-90) ------------------------- */

/* clamp-to-edge fetch; same clamp order as simpois.c:25-32 */
static float fetch(const float *u, int w, int h, int i, int j)
{
	if (i < 0) i = 0;
	if (j < 0) j = 0;
	if (i >= w) i = w - 1;
	if (j >= h) j = h - 1;
	return u[i + j * w];
}

/* 5-point Laplacian, clamped; float, left-to-right (simpois.c:35-46) */
static float lap5(const float *u, int w, int h, int i, int j)
{
	float r = -4 * fetch(u, w, h, i, j)
		+ fetch(u, w, h, i + 1, j)
		+ fetch(u, w, h, i, j + 1)
		+ fetch(u, w, h, i - 1, j)
		+ fetch(u, w, h, i, j - 1);
	return r;
}

/* composed Laplacian of Laplacian (simpois.c:48-57) */
static float lap_lap(const float *u, int w, int h, int i, int j)
{
	float r = -4 * lap5(u, w, h, i, j)
		+ lap5(u, w, h, i + 1, j)
		+ lap5(u, w, h, i, j + 1)
		+ lap5(u, w, h, i - 1, j)
		+ lap5(u, w, h, i, j - 1);
	return r;
}

/* composed Laplacian of bilaplacian (simpois.c:59-68) */
static float lap_lap_lap(const float *u, int w, int h, int i, int j)
{
	float r = -4 * lap_lap(u, w, h, i, j)
		+ lap_lap(u, w, h, i + 1, j)
		+ lap_lap(u, w, h, i, j + 1)
		+ lap_lap(u, w, h, i - 1, j)
		+ lap_lap(u, w, h, i, j - 1);
	return r;
}

/* Laplacian over the finite neighbours only (simpois.c:72-90) */
static float lap_finite(const float *u, int w, int h, int i, int j)
{
	float x = fetch(u, w, h, i, j);
	float a = fetch(u, w, h, i + 1, j);
	float b = fetch(u, w, h, i, j + 1);
	float c = fetch(u, w, h, i - 1, j);
	float d = fetch(u, w, h, i, j - 1);
	float r = 0;
	if (isfinite(a)) r += a - x;
	if (isfinite(b)) r += b - x;
	if (isfinite(c)) r += c - x;
	if (isfinite(d)) r += d - x;
	return r;
}

/* ---- Gauss-Seidel (simpois.c:93-119) -------------------------------------- */

typedef float (*stencil_fn)(const float *, int, int, int, int);

/* operator and effective time step for a given tstep (simpois.c:96-106) */
static stencil_fn pick_operator(float *tstep, int *ncolours, int *ci, int *cj)
{
	if (*tstep < 0) {
		if (*tstep < -1000) {
			*tstep += 1000;
			*tstep *= -1;
			*ncolours = 13; *ci = 1; *cj = 5;
			return lap_lap_lap;
		}
		*ncolours = 5; *ci = 1; *cj = 3;
		return lap_lap;
	}
	*ncolours = 2; *ci = 1; *cj = 1;
	return lap_finite;
}

/* one sweep over the unknown list; raster or colour order */
static void gs_sweep(float *u, const float *f, int w, int h,
		const int *omega, int n_omega, float tstep, int order)
{
	int ncol, ci, cj;
	stencil_fn op = pick_operator(&tstep, &ncol, &ci, &cj);
	if (order == ORACLE_ORDER_RASTER) {
		for (int p = 0; p < n_omega; p++) {
			int ij = omega[p];
			int i = ij % w, j = ij / w;
			float l = op(u, w, h, i, j);
			float d = f ? f[ij] : 0;
			u[ij] = u[ij] + tstep * (l - d);
		}
		return;
	}
	for (int c = 0; c < ncol; c++)
		for (int p = 0; p < n_omega; p++) {
			int ij = omega[p];
			int i = ij % w, j = ij / w;
			if ((ci * i + cj * j) % ncol != c) continue;
			float l = op(u, w, h, i, j);
			float d = f ? f[ij] : 0;
			u[ij] = u[ij] + tstep * (l - d);
		}
}

/* raster list of the NaN pixels (simpois.c:123-141) */
static int *nan_list(int *n_out, const float *g, int w, int h)
{
	int n = 0;
	for (int k = 0; k < w * h; k++)
		if (isnan(g[k])) n++;
	int *lst = ora_alloc(sizeof(int) * (size_t)(n ? n : 1));
	int c = 0;
	for (int k = 0; k < w * h; k++)
		if (isnan(g[k])) lst[c++] = k;
	*n_out = n;
	return lst;
}

/* u = finite(g) ? g : init, then niter sweeps (simpois.c:144-168) */
static void gs_with_init(float *u, const float *f, const float *g, int w,
		int h, float tstep, int niter, const float *init, int order)
{
	int n;
	int *omega = nan_list(&n, g, w, h);
	for (int k = 0; k < w * h; k++)
		u[k] = isfinite(g[k]) ? g[k] : init[k];
	for (int it = 0; it < niter; it++)
		gs_sweep(u, f, w, h, omega, n, tstep, order);
	free(omega);
}

/* ---- pyramid (simpois.c:172-239) ------------------------------------------ */

/* 2x2 mean of the finite samples, NaN if none (simpois.c:172-196) */
static void restrict2(float *out, int ow, int oh, const float *in, int iw, int ih)
{
	if (!out || !in) return;
	for (int j = 0; j < oh; j++)
	for (int i = 0; i < ow; i++) {
		float a[4], m = 0;
		a[0] = fetch(in, iw, ih, 2 * i, 2 * j);
		a[1] = fetch(in, iw, ih, 2 * i + 1, 2 * j);
		a[2] = fetch(in, iw, ih, 2 * i, 2 * j + 1);
		a[3] = fetch(in, iw, ih, 2 * i + 1, 2 * j + 1);
		int cnt = 0;
		for (int k = 0; k < 4; k++)
			if (isfinite(a[k])) { m += a[k]; cnt += 1; }
		out[ow * j + i] = cnt ? m / cnt : NAN;
	}
}

/* bilinear cell (simpois.c:199-208) */
static float bilin_cell(float a, float b, float c, float d, float x, float y)
{
	float r = 0;
	r += a * (1 - x) * (1 - y);
	r += b * (x) * (1 - y);
	r += c * (1 - x) * (y);
	r += d * (x) * (y);
	return r;
}

/* cell-centred bilinear prolongation (simpois.c:211-239) */
static void prolong2(float *out, int ow, int oh, const float *in, int iw, int ih)
{
	if (!out || !in) return;
	for (int j = 0; j < oh; j++)
	for (int i = 0; i < ow; i++) {
		float p = (i - 0.5) / 2;
		float q = (j - 0.5) / 2;
		int ip = floor(p);
		int iq = floor(q);
		float a = fetch(in, iw, ih, ip, iq);
		float b = fetch(in, iw, ih, ip + 1, iq);
		float c = fetch(in, iw, ih, ip, iq + 1);
		float d = fetch(in, iw, ih, ip + 1, iq + 1);
		out[ow * j + i] = bilin_cell(a, b, c, d, p - ip, q - iq);
	}
}

/* ---- CG on the unknowns (cleant_cgpois.c:1-278, minicg.c:1-56) ------------ */

typedef struct {
	int w, h, n;
	const int *idx;      /* unknown -> pixel index (raster)        */
	const int *inv;      /* pixel -> unknown index, or -1          */
	const float *bd;     /* boundary data at knowns (0 after RHS)  */
} cg_state;

/* gather: the unknown's value rounded to float, else the boundary datum
 * (cleant_cgpois.c:48-65) */
static float cg_fetch(const double *x, const cg_state *e, int i, int j)
{
	if (i < 0) i = 0;
	if (j < 0) j = 0;
	if (i >= e->w) i = e->w - 1;
	if (j >= e->h) j = e->h - 1;
	int k = j * e->w + i;
	int q = e->inv[k];
	if (q < 0) return e->bd[k];
	return x[q];
}

/* y = -Lap x restricted to the unknowns; the stencil is evaluated in float
 * (cleant_cgpois.c:67-89) */
static void op_minus_lap(double *y, const double *x, int n, const cg_state *e)
{
	for (int p = 0; p < n; p++) {
		int i = e->idx[p] % e->w, j = e->idx[p] / e->w;
		double r = -4 * cg_fetch(x, e, i, j)
			+ cg_fetch(x, e, i + 1, j)
			+ cg_fetch(x, e, i, j + 1)
			+ cg_fetch(x, e, i - 1, j)
			+ cg_fetch(x, e, i, j - 1);
		y[p] = -r;
	}
}

/* y = 13-point bilaplacian with a single clamp (cleant_cgpois.c:91-121) */
static void op_bilap13(double *y, const double *x, int n, const cg_state *e)
{
	for (int p = 0; p < n; p++) {
		int i = e->idx[p] % e->w, j = e->idx[p] / e->w;
		double r = 20 * cg_fetch(x, e, i, j)
			- 8 * cg_fetch(x, e, i + 1, j)
			- 8 * cg_fetch(x, e, i, j + 1)
			- 8 * cg_fetch(x, e, i - 1, j)
			- 8 * cg_fetch(x, e, i, j - 1)
			+ 2 * cg_fetch(x, e, i + 1, j + 1)
			+ 2 * cg_fetch(x, e, i + 1, j - 1)
			+ 2 * cg_fetch(x, e, i - 1, j + 1)
			+ 2 * cg_fetch(x, e, i - 1, j - 1)
			+ cg_fetch(x, e, i + 2, j)
			+ cg_fetch(x, e, i, j + 2)
			+ cg_fetch(x, e, i - 2, j)
			+ cg_fetch(x, e, i, j - 2);
		y[p] = r;
	}
}

typedef void (*cg_op)(double *, const double *, int, const cg_state *);

static double dot(const double *a, const double *b, int n)
{
	double r = 0;
	for (int k = 0; k < n; k++) r += a[k] * b[k];
	return r;
}

/* plain CG, absolute stop sqrt(r.r) < eps, no breakdown guard (minicg.c:24-56) */
static void cg_solve(double *x, cg_op A, const double *b, int n,
		const cg_state *e, const double *x0, int max_iter, double eps, int log)
{
	double *r = ora_alloc(sizeof(double) * n);
	double *p = ora_alloc(sizeof(double) * n);
	double *Ap = ora_alloc(sizeof(double) * n);
	A(Ap, x0, n, e);
	for (int k = 0; k < n; k++) x[k] = x0[k];
	for (int k = 0; k < n; k++) r[k] = b[k] - Ap[k];
	for (int k = 0; k < n; k++) p[k] = r[k];
	int it = 0;
	double rr_new = NAN;
	for (it = 0; it < max_iter; it++) {
		A(Ap, p, n, e);
		double App = dot(Ap, p, n);
		double rr_old = dot(r, r, n);
		double alpha = rr_old / App;
		for (int k = 0; k < n; k++) x[k] = x[k] + alpha * p[k];
		for (int k = 0; k < n; k++) r[k] = r[k] - alpha * Ap[k];
		rr_new = dot(r, r, n);
		if (log) fprintf(stderr, "n=%d iter=%d, rr_new=%g\n", n, it, rr_new);
		if (sqrt(rr_new) < eps) { it++; break; }
		double beta = rr_new / rr_old;
		for (int k = 0; k < n; k++) p[k] = r[k] + beta * p[k];
	}
	g_last_cg.iterations = it;
	g_last_cg.rr_final = rr_new;
	free(r); free(p); free(Ap);
}

/* build b, run CG from init, scatter (cleant_cgpois.c:197-264) */
static void cg_extension(float *out, cg_op A, const float *in, const float *dat,
		int w, int h, const float *init, int maxit, float eps,
		const oracle_opts *o)
{
	int n;
	int *idx = nan_list(&n, in, w, h);
	if (!n) {
		for (int k = 0; k < w * h; k++)
			out[k] = isfinite(in[k]) ? in[k] : init[k];
		free(idx);
		g_last_cg.iterations = 0;
		g_last_cg.rr_final = 0;
		return;
	}
	int *inv = ora_alloc(sizeof(int) * (size_t)w * h);
	for (int k = 0; k < w * h; k++) inv[k] = -1;
	for (int p = 0; p < n; p++) inv[idx[p]] = p;
	float *bd = ora_alloc(sizeof(float) * (size_t)w * h);
	for (int k = 0; k < w * h; k++) bd[k] = in[k];
	cg_state e = { w, h, n, idx, inv, bd };

	double *b = ora_alloc(sizeof(double) * n);
	double *zero = ora_alloc(sizeof(double) * n);
	for (int p = 0; p < n; p++) zero[p] = 0;
	A(b, zero, n, &e);
	free(zero);
	for (int p = 0; p < n; p++)
		b[p] = (dat ? -dat[idx[p]] : 0) - b[p];
	for (int k = 0; k < w * h; k++)
		if (inv[k] < 0) bd[k] = 0;

	double *sol = ora_alloc(sizeof(double) * n);
	double *x0 = ora_alloc(sizeof(double) * n);
	for (int p = 0; p < n; p++) x0[p] = init[idx[p]];
	float cg_eps = o->cg_eps >= 0 ? o->cg_eps : eps;
	float cg_maxit = maxit == -1 ? n : maxit;
	cg_solve(sol, A, b, n, &e, x0, cg_maxit, cg_eps, o->cg_log);

	for (int k = 0; k < w * h; k++) out[k] = in[k];
	for (int p = 0; p < n; p++) out[idx[p]] = sol[p];

	free(bd); free(sol); free(x0); free(idx); free(inv); free(b);
}

/* ---- the GS-only variant of ftr/minisimpois.c ------------------------------
 * poisson_recursive (ftr/minisimpois.c:127-149): the same octave pyramid, with
 * the plain clamped Laplacian for every tstep (ftr/minisimpois.c:17-41), the
 * nearest-neighbour prolongation (ftr/minisimpois.c:117-124), fs *= 3 and no
 * CG branch.  In place (u == g) works: g is read before u is written.        */

static void gs_sweep_plain(float *u, const float *f, int w, int h, const int *omega, int n_omega,
		float tstep, int order)
{
	for (int c = 0; c < (order == ORACLE_ORDER_RASTER ? 1 : 2); c++)
		for (int p = 0; p < n_omega; p++) {
			int ij = omega[p];
			int i = ij % w, j = ij / w;
			if (order != ORACLE_ORDER_RASTER && ((i + j) & 1) != c) continue;
			float l = lap5(u, w, h, i, j);
			float d = f ? f[ij] : 0;
			u[ij] = u[ij] + tstep * (l - d);
		}
}

static void prolong_nearest(float *out, int ow, int oh, const float *in, int iw, int ih)
{
	for (int j = 0; j < oh; j++)
	for (int i = 0; i < ow; i++)
		out[ow * j + i] = fetch(in, iw, ih, i / 2, j / 2);
}

static void mini_level(float *u, const float *g, const float *f, int w, int h, float tstep,
		int niter, int scale, int order)
{
	float *init = ora_alloc(sizeof(float) * (size_t)w * h);
	for (int k = 0; k < w * h; k++) init[k] = 0;
	if (scale > 1 && (w > 1 || h > 1)) {
		int ws = ceil(w / 2.0);
		int hs = ceil(h / 2.0);
		float *gs = ora_alloc(sizeof(float) * (size_t)ws * hs);
		float *fs = f ? ora_alloc(sizeof(float) * (size_t)ws * hs) : NULL;
		float *us = ora_alloc(sizeof(float) * (size_t)ws * hs);
		restrict2(gs, ws, hs, g, w, h);
		restrict2(fs, ws, hs, f, w, h);
		if (f) for (int k = 0; k < ws * hs; k++) fs[k] *= 3;
		mini_level(us, gs, fs, ws, hs, tstep, niter, scale - 1, order);
		prolong_nearest(init, w, h, us, ws, hs);
		free(gs); free(fs); free(us);
	}
	int n;
	int *omega = nan_list(&n, g, w, h);
	for (int k = 0; k < w * h; k++)
		u[k] = isfinite(g[k]) ? g[k] : init[k];
	for (int it = 0; it < niter; it++)
		gs_sweep_plain(u, f, w, h, omega, n, tstep, order);
	free(omega);
	free(init);
}

void oracle_poisson_recursive(float *u, const float *g, const float *f, int w, int h,
		float tstep, int niter, int scale, int order)
{
	mini_level(u, g, f, w, h, tstep, niter, scale, order);
}

/* ---- recursion and channel loop (simpois.c:247-302) ----------------------- */

static void rec_level(float *u, const float *g, const float *f, int w, int h,
		float tstep, int niter, int scale, int cgit, const oracle_opts *o)
{
	float *init = ora_alloc(sizeof(float) * (size_t)w * h);
	if (scale > 1 && (w > 1 || h > 1)) {
		int ws = ceil(w / 2.0);
		int hs = ceil(h / 2.0);
		float *gs = ora_alloc(sizeof(float) * (size_t)ws * hs);
		float *fs = f ? ora_alloc(sizeof(float) * (size_t)ws * hs) : NULL;
		float *us = ora_alloc(sizeof(float) * (size_t)ws * hs);
		restrict2(gs, ws, hs, g, w, h);
		restrict2(fs, ws, hs, f, w, h);
		if (f) for (int k = 0; k < ws * hs; k++) fs[k] *= o->pmsfac;
		rec_level(us, gs, fs, ws, hs, tstep, niter, scale - 1, cgit, o);
		prolong2(init, w, h, us, ws, hs);
		free(gs); free(fs); free(us);
	} else {
		for (int k = 0; k < w * h; k++) init[k] = 0;
	}
	if (o->ponlit && o->ponlit != w)
		niter = cgit = 0;
	gs_with_init(u, f, g, w, h, tstep, niter, init, o->order);
	free(init);
	if (cgit && tstep > 0) {
		float cg_eps = 1e-6;
		cg_extension(u, op_minus_lap, g, f, w, h, u, cgit, cg_eps, o);
	} else {
		float cg_eps = 1e-9;
		cg_extension(u, op_bilap13, g, f, w, h, u, cgit, cg_eps, o);
	}
}

/* ---- exported entry points (ctypes) -------------------------------------- */

void oracle_default_opts(oracle_opts *o)
{
	o->pmsfac = 3;
	o->ponlit = 0;
	o->cg_eps = -1;
	o->order = ORACLE_ORDER_RASTER;
	o->cg_log = 0;
}

/* poisson_rec (simpois.c:247) */
void oracle_poisson_rec(float *u, const float *g, const float *f, int w, int h,
		float tstep, int niter, int scale, int cgit, const oracle_opts *o)
{
	rec_level(u, g, f, w, h, tstep, niter, scale, cgit, o);
}

/* poisson_solver_separable (simpois.c:288); channels are planar */
void oracle_poisson_solver_separable(float *out, const float *in,
		const float *dat, int w, int h, int pd, float tstep, int niter,
		int scale, float cgrad, const oracle_opts *o)
{
	for (int l = 0; l < pd; l++) {
		size_t off = (size_t)w * h * l;
		rec_level(out + off, in + off, dat ? dat + off : NULL, w, h,
				tstep, niter, scale, cgrad, o);
	}
}

/* the main_simpois mask rule: NaN where mask > 0, every channel
 * (simpois.c:421-424) */
void oracle_apply_mask(float *img, const float *mask, int w, int h, int pd)
{
	for (long k = 0; k < (long)w * h * pd; k++)
		if (mask[k % ((long)w * h)] > 0) img[k] = NAN;
}

/* single building blocks, exposed for kernel-level parity tests */
void oracle_restrict(float *out, int ow, int oh, const float *in, int iw, int ih)
{
	restrict2(out, ow, oh, in, iw, ih);
}

void oracle_prolong(float *out, int ow, int oh, const float *in, int iw, int ih)
{
	prolong2(out, ow, oh, in, iw, ih);
}

void oracle_gs(float *u, const float *f, const float *g, int w, int h,
		float tstep, int niter, const float *init, int order)
{
	gs_with_init(u, f, g, w, h, tstep, niter, init, order);
}

/* the CG branch alone: kind 0 = -Lap (eps 1e-6), 1 = 13-pt bilaplacian
 * (eps 1e-9); returns the iteration count */
int oracle_cg_extension(float *out, const float *in, const float *dat, int w,
		int h, const float *init, int maxit, int kind, const oracle_opts *o,
		double *rr_final)
{
	cg_extension(out, kind ? op_bilap13 : op_minus_lap, in, dat, w, h, init,
			maxit, kind ? 1e-9f : 1e-6f, o);
	if (rr_final) *rr_final = g_last_cg.rr_final;
	return g_last_cg.iterations;
}

/* ---- FP64 residual of the CG operators ------------------------------------
 * The relative residual ||b - A u_U|| / ||b|| over the unknowns (NaN pixels of
 * g), evaluated in double on the float output u.  kind 0: A = -Lap (5-point,
 * clamped), b = -f_U + Lap_UK g_K; kind 1: A = 13-point clamped bilaplacian,
 * b = -f_U - A_UK g_K (cleant_cgpois.c:67-121, 226-233).  Pixels of u that are
 * not unknowns are read from g.  Returns ||b|| in *bnorm; 0 when there is no
 * unknown.                                                                    */

static double fetch64(const float *v, const float *g, const unsigned char *unk,
		int w, int h, int i, int j, int zero_unknowns)
{
	if (i < 0) i = 0;
	if (j < 0) j = 0;
	if (i >= w) i = w - 1;
	if (j >= h) j = h - 1;
	int k = j * w + i;
	if (unk[k]) return zero_unknowns ? 0.0 : (double)v[k];
	return (double)g[k];
}

static double apply64(int kind, const float *v, const float *g,
		const unsigned char *unk, int w, int h, int i, int j, int zu)
{
#define F(di, dj) fetch64(v, g, unk, w, h, i + (di), j + (dj), zu)
	if (kind == 0)
		return 4 * F(0, 0) - F(1, 0) - F(0, 1) - F(-1, 0) - F(0, -1);
	return 20 * F(0, 0) - 8 * (F(1, 0) + F(0, 1) + F(-1, 0) + F(0, -1))
		+ 2 * (F(1, 1) + F(1, -1) + F(-1, 1) + F(-1, -1))
		+ F(2, 0) + F(0, 2) + F(-2, 0) + F(0, -2);
#undef F
}

double oracle_rel_residual(const float *u, const float *g, const float *f,
		int w, int h, int kind, double *bnorm)
{
	unsigned char *unk = ora_alloc((size_t)w * h);
	for (long k = 0; k < (long)w * h; k++) unk[k] = isnan(g[k]) ? 1 : 0;
	double rr = 0, bb = 0;
	for (int j = 0; j < h; j++)
	for (int i = 0; i < w; i++) {
		long k = (long)j * w + i;
		if (!unk[k]) continue;
		/* b = -f - A(0 at unknowns, g at knowns);
		 * b - A_UU u_U = -f - A(u at unknowns, g at knowns) */
		double fk = f ? -(double)f[k] : 0.0;
		double bk = fk - apply64(kind, u, g, unk, w, h, i, j, 1);
		double rk = fk - apply64(kind, u, g, unk, w, h, i, j, 0);
		rr += rk * rk;
		bb += bk * bk;
	}
	free(unk);
	if (bnorm) *bnorm = sqrt(bb);
	if (bb == 0) return rr == 0 ? 0.0 : INFINITY;
	return sqrt(rr / bb);
}

/* ||b||_2 of the CG system, for the CG_EPS = rtol * ||b|| recipe */
double oracle_rhs_norm(const float *g, const float *f, int w, int h, int kind)
{
	double bn = 0;
	oracle_rel_residual(g, g, f, w, h, kind, &bn);
	return bn;
}
