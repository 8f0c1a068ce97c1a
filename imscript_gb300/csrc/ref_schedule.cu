// ref_schedule.cu -- the reference schedule of simpois on the GPU.
//
// This is the octave pyramid of `poisson_rec` (simpois.c:247-285) as the
// simpois command runs it by default: restrict the data (simpois.c:172-196),
// recurse, prolong bilinearly (simpois.c:199-239), run `niter` Gauss-Seidel
// sweeps (simpois.c:93-119), then the CG branch (cleant_cgpois.c:197-278,
// minicg.c:24-56).  Every float operation is issued in the reference's order
// with explicit round-to-nearest intrinsics (no FMA contraction), so the only
// difference from the reference is the sweep order: the unknowns are swept in
// colour classes, (i+j)&1 for the 5-point operator, (i+3j)%5 for the 13-point
// bilaplacian, (i+5j)%13 for the 25-point triharmonic operator.  No pixel
// reads another pixel of its own class, so a class is updated in parallel and
// the result is independent of the order inside a class.
//
// The CG keeps the reference's arithmetic: FP64 vectors, the stencil evaluated
// in float on the float-rounded iterate (cleant_cgpois.c:48-65,77-81), FP64
// dot products (deterministic two-stage reductions), the absolute stopping
// test sqrt(r.r) < eps.  One deliberate difference: a breakdown (p.Ap == 0 or
// a non-finite step) stops the iteration with SIMPOIS_BREAKDOWN and keeps the
// last iterate, where the reference divides 0/0 and fills the image with NaN.
#include <math.h>

#include "common.cuh"
#include "solvers.h"

namespace {

// ------------------------------------------------------------ exact stencils

__device__ __forceinline__ float fetchc(const float *__restrict__ u, int w, int h, int i, int j)
{
	return u[clampi(j, h) * w + clampi(i, w)];
}

// 5-point Laplacian with clamp, float, left to right (simpois.c:35-46)
__device__ __forceinline__ float lap5(const float *u, int w, int h, int i, int j)
{
	float r = __fmul_rn(-4.f, fetchc(u, w, h, i, j));
	r = __fadd_rn(r, fetchc(u, w, h, i + 1, j));
	r = __fadd_rn(r, fetchc(u, w, h, i, j + 1));
	r = __fadd_rn(r, fetchc(u, w, h, i - 1, j));
	r = __fadd_rn(r, fetchc(u, w, h, i, j - 1));
	return r;
}

// Laplacian of the Laplacian (simpois.c:48-57)
__device__ __forceinline__ float lap_lap(const float *u, int w, int h, int i, int j)
{
	float r = __fmul_rn(-4.f, lap5(u, w, h, i, j));
	r = __fadd_rn(r, lap5(u, w, h, i + 1, j));
	r = __fadd_rn(r, lap5(u, w, h, i, j + 1));
	r = __fadd_rn(r, lap5(u, w, h, i - 1, j));
	r = __fadd_rn(r, lap5(u, w, h, i, j - 1));
	return r;
}

// Laplacian of the bilaplacian (simpois.c:59-68)
__device__ float lap_lap_lap(const float *u, int w, int h, int i, int j)
{
	float r = __fmul_rn(-4.f, lap_lap(u, w, h, i, j));
	r = __fadd_rn(r, lap_lap(u, w, h, i + 1, j));
	r = __fadd_rn(r, lap_lap(u, w, h, i, j + 1));
	r = __fadd_rn(r, lap_lap(u, w, h, i - 1, j));
	r = __fadd_rn(r, lap_lap(u, w, h, i, j - 1));
	return r;
}

// Laplacian over the finite neighbours (simpois.c:72-90)
__device__ __forceinline__ float lap_finite(const float *u, int w, int h, int i, int j)
{
	float x = fetchc(u, w, h, i, j);
	float a = fetchc(u, w, h, i + 1, j);
	float b = fetchc(u, w, h, i, j + 1);
	float c = fetchc(u, w, h, i - 1, j);
	float d = fetchc(u, w, h, i, j - 1);
	float r = 0.f;
	if (isfinite(a)) r = __fadd_rn(r, __fsub_rn(a, x));
	if (isfinite(b)) r = __fadd_rn(r, __fsub_rn(b, x));
	if (isfinite(c)) r = __fadd_rn(r, __fsub_rn(c, x));
	if (isfinite(d)) r = __fadd_rn(r, __fsub_rn(d, x));
	return r;
}

// ------------------------------------------------------------ pyramid kernels

// 2x2 mean of the finite samples, NaN if none (simpois.c:172-196); when
// `scaled`, the result is multiplied by pmsfac in double and rounded to float
// as `fs[i] *= PMSFAC()` does (simpois.c:262).
__global__ void k_restrict(float *__restrict__ out, int ow, int oh,
		const float *__restrict__ in, int iw, int ih, int scaled, double pmsfac)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	int j = blockIdx.y * blockDim.y + threadIdx.y;
	int l = blockIdx.z;
	if (i >= ow || j >= oh) return;
	const float *src = in + (size_t)iw * ih * l;
	float a[4];
	a[0] = fetchc(src, iw, ih, 2 * i, 2 * j);
	a[1] = fetchc(src, iw, ih, 2 * i + 1, 2 * j);
	a[2] = fetchc(src, iw, ih, 2 * i, 2 * j + 1);
	a[3] = fetchc(src, iw, ih, 2 * i + 1, 2 * j + 1);
	float m = 0.f;
	int cnt = 0;
#pragma unroll
	for (int k = 0; k < 4; k++)
		if (isfinite(a[k])) { m = __fadd_rn(m, a[k]); cnt++; }
	float r = cnt ? __fdiv_rn(m, (float)cnt) : __int_as_float(0x7fc00000);
	if (scaled) r = __double2float_rn(__dmul_rn((double)r, pmsfac));
	out[(size_t)ow * oh * l + (size_t)ow * j + i] = r;
}

// init = bilinear prolongation of the coarse solution (simpois.c:225-239), or
// the nearest-neighbour one of ftr/minisimpois.c:117-124 when `nearest`, or 0
// at the coarsest level; then u = finite(g) ? g : init (simpois.c:159-160).
__global__ void k_prolong_init(float *__restrict__ u, const float *__restrict__ g,
		int ow, int oh, const float *__restrict__ uc, int iw, int ih, int nearest)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	int j = blockIdx.y * blockDim.y + threadIdx.y;
	int l = blockIdx.z;
	if (i >= ow || j >= oh) return;
	size_t k = (size_t)ow * oh * l + (size_t)ow * j + i;
	float init = 0.f;
	if (uc && nearest) {
		init = fetchc(uc + (size_t)iw * ih * l, iw, ih, i / 2, j / 2);
	} else if (uc) {
		const float *src = uc + (size_t)iw * ih * l;
		float p = __double2float_rn(((double)i - 0.5) / 2);
		float q = __double2float_rn(((double)j - 0.5) / 2);
		int ip = (int)floor((double)p);
		int iq = (int)floor((double)q);
		float a = fetchc(src, iw, ih, ip, iq);
		float b = fetchc(src, iw, ih, ip + 1, iq);
		float c = fetchc(src, iw, ih, ip, iq + 1);
		float d = fetchc(src, iw, ih, ip + 1, iq + 1);
		float x = __fsub_rn(p, (float)ip);
		float y = __fsub_rn(q, (float)iq);
		float x1 = __fsub_rn(1.f, x), y1 = __fsub_rn(1.f, y);
		float r = 0.f;
		r = __fadd_rn(r, __fmul_rn(__fmul_rn(a, x1), y1));
		r = __fadd_rn(r, __fmul_rn(__fmul_rn(b, x), y1));
		r = __fadd_rn(r, __fmul_rn(__fmul_rn(c, x1), y));
		r = __fadd_rn(r, __fmul_rn(__fmul_rn(d, x), y));
		init = r;
	}
	float gv = g[k];
	u[k] = isfinite(gv) ? gv : init;
}

// One colour class of a Gauss-Seidel sweep, in place (simpois.c:109-118):
// u[p] += tstep * (op(u)[p] - f[p]) for the NaN pixels p of g in the class.
// op: 0 = lap_finite, 1 = lap_lap, 2 = lap_lap_lap, 3 = lap5 (the plain
// clamped Laplacian of ftr/minisimpois.c:17-41).
__global__ void k_gs_class(float *__restrict__ u, const float *__restrict__ g,
		const float *__restrict__ f, int w, int h, float tstep, int op,
		int ncol, int cj, int colour)
{
	int i = blockIdx.x * blockDim.x + threadIdx.x;
	int j = blockIdx.y * blockDim.y + threadIdx.y;
	int l = blockIdx.z;
	if (i >= w || j >= h) return;
	if ((i + cj * j) % ncol != colour) return;
	size_t off = (size_t)w * h * l;
	size_t ij = (size_t)w * j + i;
	if (!isnan(g[off + ij])) return;
	float *ul = u + off;
	float lv = op == 0 ? lap_finite(ul, w, h, i, j)
		: op == 1 ? lap_lap(ul, w, h, i, j)
		: op == 2 ? lap_lap_lap(ul, w, h, i, j) : lap5(ul, w, h, i, j);
	float d = f ? f[off + ij] : 0.f;
	ul[ij] = __fadd_rn(ul[ij], __fmul_rn(tstep, __fsub_rn(lv, d)));
}

// has_nan[l] = 1 when channel l of g holds a NaN pixel
__global__ void k_nan_any(const float *__restrict__ g, size_t cs, int *__restrict__ has_nan)
{
	size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	int l = blockIdx.y;
	bool is = k < cs && isnan(g[cs * l + k]);
	if (__any_sync(0xffffffffu, is) && (threadIdx.x & 31) == 0) atomicOr(has_nan + l, 1);
}

// The CG branch when it runs no iteration (cleant_cgpois.c:202-256): with no
// unknown it leaves u as it is; otherwise `out = in` followed by the scatter
// of the unchanged solution, i.e. u = g at every non-NaN pixel.
__global__ void k_restore_known(float *__restrict__ u, const float *__restrict__ g, size_t cs,
		const int *__restrict__ has_nan)
{
	size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	int l = blockIdx.y;
	if (k >= cs || !has_nan[l]) return;
	float gv = g[cs * l + k];
	if (!isnan(gv)) u[cs * l + k] = gv;
}

// ------------------------------------------------------------ CG compaction

// Per block of 1024 pixels: number of NaN pixels.
__global__ void k_nan_count(const float *__restrict__ g, int n, int *__restrict__ bcount)
{
	__shared__ int sh[32];
	int k = blockIdx.x * 1024 + threadIdx.x;
	int c = 0;
	for (int t = 0; t < 4; t++) {
		int kk = k + t * 256;
		if (kk < n && isnan(g[kk])) c++;
	}
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x == 0) {
		int s = 0;
		for (int q = 0; q < 8; q++) s += sh[q];
		bcount[blockIdx.x] = s;
	}
}

// Exclusive scan of the block counts (single block), total in boff[nb].
__global__ void k_scan_counts(int *__restrict__ bcount, int nb, int *__restrict__ boff)
{
	__shared__ int sh[1024];
	__shared__ int carry;
	if (threadIdx.x == 0) carry = 0;
	__syncthreads();
	for (int base = 0; base < nb; base += 1024) {
		int k = base + threadIdx.x;
		int v = k < nb ? bcount[k] : 0;
		sh[threadIdx.x] = v;
		__syncthreads();
		for (int o = 1; o < 1024; o <<= 1) {
			int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
			__syncthreads();
			sh[threadIdx.x] += t;
			__syncthreads();
		}
		if (k < nb) boff[k] = carry + sh[threadIdx.x] - v;
		__syncthreads();
		if (threadIdx.x == 1023) carry += sh[1023];
		__syncthreads();
	}
	if (threadIdx.x == 0) boff[nb] = carry;
}

// Raster-ordered unknown list idx[] and inverse map inv[] (-1 at knowns),
// the build_mask3 / invert_mask3 pair (cleant_cgpois.c:6-38).
__global__ void k_nan_fill(const float *__restrict__ g, int n, const int *__restrict__ boff,
		int *__restrict__ idx, int *__restrict__ inv)
{
	__shared__ int wsum[32];
	int base = blockIdx.x * 1024;
	int pos = boff[blockIdx.x];
	for (int t = 0; t < 4; t++) {
		int k = base + t * 256 + threadIdx.x;
		bool is = k < n && isnan(g[k]);
		unsigned bal = __ballot_sync(0xffffffffu, is);
		int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
		int before = __popc(bal & ((1u << lane) - 1));
		if (lane == 0) wsum[warp] = __popc(bal);
		__syncthreads();
		int woff = 0;
		for (int q = 0; q < warp; q++) woff += wsum[q];
		int tot = 0;
		for (int q = 0; q < 8; q++) tot += wsum[q];
		if (k < n) {
			if (is) {
				idx[pos + woff + before] = k;
				inv[k] = pos + woff + before;
			} else {
				inv[k] = -1;
			}
		}
		pos += tot;
		__syncthreads();
	}
}

// ------------------------------------------------------------ reference CG

struct CgState {
	double rr_old, app, alpha, beta, rr_new;
	int iter, done, status, maxit;
	unsigned int cnt;
	double eps;
};

// masked gather (cleant_cgpois.c:48-65): the unknown's value rounded to float,
// else the boundary datum (g before the RHS is built, 0 after)
__device__ __forceinline__ float cg_fetch(const double *__restrict__ x, const int *__restrict__ inv,
		const float *__restrict__ g, int w, int h, int i, int j, bool boundary)
{
	int k = clampi(j, h) * w + clampi(i, w);
	int q = inv[k];
	if (q < 0) return boundary ? g[k] : 0.f;
	return (float)x[q];
}

__device__ __forceinline__ double cg_apply(int kind, const double *x, const int *inv, const float *g,
		int w, int h, int i, int j, bool bd)
{
#define G(di, dj) cg_fetch(x, inv, g, w, h, i + (di), j + (dj), bd)
	if (kind == 0) {  // -(-4c + E + S + W + N)  (cleant_cgpois.c:77-88)
		float r = __fmul_rn(-4.f, G(0, 0));
		r = __fadd_rn(r, G(1, 0));
		r = __fadd_rn(r, G(0, 1));
		r = __fadd_rn(r, G(-1, 0));
		r = __fadd_rn(r, G(0, -1));
		return -(double)r;
	}
	// 20c - 8(E,S,W,N) + 2(diagonals) + (distance 2)  (cleant_cgpois.c:101-113)
	float r = __fmul_rn(20.f, G(0, 0));
	r = __fsub_rn(r, __fmul_rn(8.f, G(1, 0)));
	r = __fsub_rn(r, __fmul_rn(8.f, G(0, 1)));
	r = __fsub_rn(r, __fmul_rn(8.f, G(-1, 0)));
	r = __fsub_rn(r, __fmul_rn(8.f, G(0, -1)));
	r = __fadd_rn(r, __fmul_rn(2.f, G(1, 1)));
	r = __fadd_rn(r, __fmul_rn(2.f, G(1, -1)));
	r = __fadd_rn(r, __fmul_rn(2.f, G(-1, 1)));
	r = __fadd_rn(r, __fmul_rn(2.f, G(-1, -1)));
	r = __fadd_rn(r, G(2, 0));
	r = __fadd_rn(r, G(0, 2));
	r = __fadd_rn(r, G(-2, 0));
	r = __fadd_rn(r, G(0, -2));
	return (double)r;
#undef G
}

// Last block of a grid: every block adds its partial, the last one to arrive
// sums the partials in block order (deterministic) and returns true.
__device__ bool last_block_sum(double v, double *partial, unsigned int *cnt, double *total, double *sh)
{
	__shared__ bool am_last;
	double s = block_sum<256>(v, sh);
	if (threadIdx.x == 0) {
		partial[blockIdx.x] = s;
		__threadfence();
		unsigned prev = atomicAdd(cnt, 1u);
		am_last = prev == gridDim.x - 1;
	}
	__syncthreads();
	if (!am_last) return false;
	__threadfence();
	double acc = 0;
	for (int k = threadIdx.x; k < (int)gridDim.x; k += 256) acc += __ldcg(partial + k);
	acc = block_sum<256>(acc, sh);
	if (threadIdx.x == 0) { *total = acc; *cnt = 0; }
	__syncthreads();
	return true;
}

// b = (dat ? -dat : 0) - A(0 at unknowns | g at knowns); x = x0 = (double)init
__global__ void k_cg_rhs(int kind, const int *__restrict__ idx, const int *__restrict__ inv,
		const float *__restrict__ g, const float *__restrict__ f, const float *__restrict__ init,
		int w, int h, int n, double *__restrict__ b, double *__restrict__ x, const double *__restrict__ zero)
{
	int p = blockIdx.x * 256 + threadIdx.x;
	if (p >= n) return;
	int k = idx[p];
	int i = k % w, j = k / w;
	double a0 = cg_apply(kind, zero, inv, g, w, h, i, j, true);
	float mf = f ? -f[k] : 0.f;
	b[p] = __dsub_rn((double)mf, a0);
	x[p] = (double)init[k];
}

// Ap = A x0; r = b - Ap; p = r; rr_old = r.r  (minicg.c:32-36 and the first
// rr_old of minicg.c:41)
__global__ void k_cg_start(int kind, const int *__restrict__ idx, const int *__restrict__ inv,
		const float *__restrict__ g, int w, int h, int n, const double *__restrict__ b,
		const double *__restrict__ x, double *__restrict__ r, double *__restrict__ pv,
		double *partial, CgState *st)
{
	__shared__ double sh[32];
	int p = blockIdx.x * 256 + threadIdx.x;
	double rr = 0;
	if (p < n) {
		int k = idx[p];
		double ap = cg_apply(kind, x, inv, g, w, h, k % w, k / w, false);
		double rv = __dsub_rn(b[p], ap);
		r[p] = rv;
		pv[p] = rv;
		rr = __dmul_rn(rv, rv);
	}
	double tot;
	if (last_block_sum(rr, partial, &st->cnt, &tot, sh) && threadIdx.x == 0) {
		st->rr_old = tot;
		st->iter = 0;
		st->done = st->maxit <= 0;
		st->status = SIMPOIS_OK;
	}
}

// Ap = A p; App = Ap.p; alpha = rr_old / App  (minicg.c:39-42)
__global__ void k_cg_spmv(int kind, const int *__restrict__ idx, const int *__restrict__ inv,
		const float *__restrict__ g, int w, int h, int n, const double *__restrict__ pv,
		double *__restrict__ ap, double *partial, CgState *st)
{
	__shared__ double sh[32];
	if (st->done) return;
	int p = blockIdx.x * 256 + threadIdx.x;
	double s = 0;
	if (p < n) {
		int k = idx[p];
		double a = cg_apply(kind, pv, inv, g, w, h, k % w, k / w, false);
		ap[p] = a;
		s = __dmul_rn(a, pv[p]);
	}
	double tot;
	if (last_block_sum(s, partial, &st->cnt, &tot, sh) && threadIdx.x == 0) {
		st->app = tot;
		double alpha = st->rr_old / tot;
		if (tot == 0 || !isfinite(alpha)) {
			st->status = SIMPOIS_BREAKDOWN;
			st->done = 1;
		}
		st->alpha = alpha;
	}
}

// x += alpha p; r -= alpha Ap; rr_new = r.r; stop test; beta (minicg.c:43-49)
__global__ void k_cg_update(int n, double *__restrict__ x, double *__restrict__ r,
		const double *__restrict__ pv, const double *__restrict__ ap, double *partial, CgState *st)
{
	__shared__ double sh[32];
	if (st->done) return;
	double alpha = st->alpha;
	int p = blockIdx.x * 256 + threadIdx.x;
	double s = 0;
	if (p < n) {
		x[p] = __dadd_rn(x[p], __dmul_rn(alpha, pv[p]));
		double rv = __dsub_rn(r[p], __dmul_rn(alpha, ap[p]));
		r[p] = rv;
		s = __dmul_rn(rv, rv);
	}
	double tot;
	if (last_block_sum(s, partial, &st->cnt, &tot, sh) && threadIdx.x == 0) {
		st->rr_new = tot;
		st->iter += 1;
		if (sqrt(tot) < st->eps || st->iter >= st->maxit) {
			st->done = 1;
		} else {
			st->beta = tot / st->rr_old;
			st->rr_old = tot;
		}
	}
}

// p = r + beta p  (minicg.c:50)
__global__ void k_cg_pupdate(int n, const double *__restrict__ r, double *__restrict__ pv, const CgState *st)
{
	if (st->done) return;
	int p = blockIdx.x * 256 + threadIdx.x;
	if (p < n) pv[p] = __dadd_rn(r[p], __dmul_rn(st->beta, pv[p]));
}

// out = in; out[unknowns] = (float)x  (cleant_cgpois.c:251-256)
__global__ void k_cg_scatter(float *__restrict__ u, const float *__restrict__ g,
		const int *__restrict__ inv, const double *__restrict__ x, int n)
{
	int k = blockIdx.x * 256 + threadIdx.x;
	if (k >= n) return;
	int q = inv[k];
	u[k] = q < 0 ? g[k] : (float)x[q];
}

inline unsigned nblk(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }

struct RefLevel {
	int w, h;
	float *g, *f, *u;
};

}  // namespace

// CG branch of one level of one channel (cleant_cgpois.c:197-264).
static int ref_cg_channel(simpois_ctx *ctx, int kind, float *u, const float *g, const float *f,
		int w, int h, int maxit_param, float eps_default, const simpois_params *prm, char *ws,
		int *iters_out, int *status_out)
{
	cudaStream_t s = ctx->stream;
	int n_px = w * h;
	int nb = (n_px + 1023) / 1024;
	Layout L;
	size_t o_bcount = L.take(sizeof(int) * (nb + 1));
	size_t o_boff = L.take(sizeof(int) * (nb + 1));
	size_t o_inv = L.take(sizeof(int) * (size_t)n_px);
	size_t o_state = L.take(sizeof(CgState));
	size_t o_part = L.take(sizeof(double) * (size_t)(n_px / 256 + 2));
	size_t o_idx = L.take(sizeof(int) * (size_t)n_px);
	int *bcount = (int *)(ws + o_bcount), *boff = (int *)(ws + o_boff);
	int *inv = (int *)(ws + o_inv), *idx = (int *)(ws + o_idx);
	CgState *st = (CgState *)(ws + o_state);
	double *partial = (double *)(ws + o_part);

	k_nan_count<<<nb, 256, 0, s>>>(g, n_px, bcount); ctx->launches++;
	k_scan_counts<<<1, 1024, 0, s>>>(bcount, nb, boff); ctx->launches++;
	k_nan_fill<<<nb, 256, 0, s>>>(g, n_px, boff, idx, inv); ctx->launches++;
	SP_LAUNCH_CHECK(ctx);
	int n = 0;
	SP_CUDA(ctx, cudaMemcpyAsync(&n, boff + nb, sizeof(int), cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	*iters_out = 0;
	*status_out = SIMPOIS_OK;
	if (n == 0) return SIMPOIS_OK;  // nothing to fill: out = finite(in) ? in : init == u

	size_t o_b = L.take(sizeof(double) * n), o_x = L.take(sizeof(double) * n);
	size_t o_r = L.take(sizeof(double) * n), o_p = L.take(sizeof(double) * n);
	size_t o_ap = L.take(sizeof(double) * n), o_zero = L.take(sizeof(double) * n);
	double *b = (double *)(ws + o_b), *x = (double *)(ws + o_x), *r = (double *)(ws + o_r);
	double *pv = (double *)(ws + o_p), *ap = (double *)(ws + o_ap), *zero = (double *)(ws + o_zero);

	float cg_eps = prm->cg_eps >= 0 ? (float)prm->cg_eps : eps_default;
	float cg_maxit_f = maxit_param == -1 ? (float)n : (float)maxit_param;
	CgState h0 = {};
	h0.maxit = (int)cg_maxit_f;
	h0.eps = (double)cg_eps;
	SP_CUDA(ctx, cudaMemcpyAsync(st, &h0, sizeof(h0), cudaMemcpyHostToDevice, s));
	SP_CUDA(ctx, cudaMemsetAsync(zero, 0, sizeof(double) * n, s));
	unsigned nbn = nblk(n, 256);
	k_cg_rhs<<<nbn, 256, 0, s>>>(kind, idx, inv, g, f, u, w, h, n, b, x, zero); ctx->launches++;
	k_cg_start<<<nbn, 256, 0, s>>>(kind, idx, inv, g, w, h, n, b, x, r, pv, partial, st); ctx->launches++;
	SP_LAUNCH_CHECK(ctx);
	CgState hs = h0;
	const int chunk = 16;
	for (;;) {
		for (int c = 0; c < chunk; c++) {
			k_cg_spmv<<<nbn, 256, 0, s>>>(kind, idx, inv, g, w, h, n, pv, ap, partial, st); ctx->launches++;
			k_cg_update<<<nbn, 256, 0, s>>>(n, x, r, pv, ap, partial, st); ctx->launches++;
			k_cg_pupdate<<<nbn, 256, 0, s>>>(n, r, pv, st); ctx->launches++;
		}
		SP_LAUNCH_CHECK(ctx);
		SP_CUDA(ctx, cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, s));
		SP_CUDA(ctx, cudaStreamSynchronize(s));
		if (hs.done) break;
	}
	k_cg_scatter<<<nblk(n_px, 256), 256, 0, s>>>(u, g, inv, x, n_px); ctx->launches++;
	SP_LAUNCH_CHECK(ctx);
	*iters_out = hs.iter;
	*status_out = hs.status;
	return SIMPOIS_OK;
}

size_t ref_workspace_bytes(int w, int h, int pd, bool has_f)
{
	size_t px = (size_t)w * h;
	size_t total = 0;
	int lw = w, lh = h;
	// pyramid levels >= 1: g, f, u per channel; level 0: u
	total += px * pd * 4 + 256;
	for (int k = 0; k < 64 && (lw > 1 || lh > 1); k++) {
		lw = (lw + 1) / 2;
		lh = (lh + 1) / 2;
		total += (size_t)lw * lh * pd * 4 * (has_f ? 3 : 2) + 768;
	}
	// CG workspace at the finest level (all pixels unknown in the worst case)
	total += px * (4 + 4 + 6 * 8) + ((px + 1023) / 1024 + 2) * 8 + (px / 256 + 2) * 8 + 4096;
	return total;
}

int ref_solve(simpois_ctx *ctx, float *out, const float *in, const float *dat, int w, int h,
		int pd, const simpois_params *prm, simpois_report *rep, char *ws)
{
	cudaStream_t s = ctx->stream;
	// level dims: poisson_rec recurses while scale > 1 and the image is not 1x1
	std::vector<RefLevel> lv;
	Layout L;
	{
		int lw = w, lh = h, sc = prm->scale;
		std::vector<size_t> og, of, ou;
		for (;;) {
			RefLevel r = {lw, lh, nullptr, nullptr, nullptr};
			lv.push_back(r);
			size_t n = (size_t)lw * lh * pd * sizeof(float);
			if (lv.size() == 1) {
				og.push_back(0); of.push_back(0);
			} else {
				og.push_back(L.take(n));
				of.push_back(dat ? L.take(n) : 0);
			}
			ou.push_back(L.take(n));
			if (!(sc > 1 && (lw > 1 || lh > 1))) break;
			lw = (int)ceil(lw / 2.0);
			lh = (int)ceil(lh / 2.0);
			sc -= 1;
		}
		for (size_t k = 0; k < lv.size(); k++) {
			lv[k].g = k ? (float *)(ws + og[k]) : (float *)in;
			lv[k].f = dat ? (k ? (float *)(ws + of[k]) : (float *)dat) : nullptr;
			lv[k].u = (float *)(ws + ou[k]);
		}
	}
	char *cg_ws = ws + ((L.off + 255) / 256) * 256;
	const dim3 B2(32, 8);
	int nl = (int)lv.size();
	for (int k = 0; k + 1 < nl; k++) {
		dim3 G(nblk(lv[k + 1].w, 32), nblk(lv[k + 1].h, 8), pd);
		k_restrict<<<G, B2, 0, s>>>(lv[k + 1].g, lv[k + 1].w, lv[k + 1].h, lv[k].g, lv[k].w,
				lv[k].h, 0, 1.0); ctx->launches++;
		if (dat) {
			k_restrict<<<G, B2, 0, s>>>(lv[k + 1].f, lv[k + 1].w, lv[k + 1].h, lv[k].f,
					lv[k].w, lv[k].h, 1, prm->pmsfac); ctx->launches++;
		}
	}
	SP_LAUNCH_CHECK(ctx);

	// operator of the sweeps (simpois.c:96-106)
	float t = prm->tstep;
	int op = 0, ncol = 2, cj = 1;
	// the ftr/minisimpois.c variant: plain Laplacian whatever the sign of t,
	// nearest-neighbour prolongation, no CG branch
	const bool mini = (prm->flags & SIMPOIS_FLAG_MINI) != 0;
	if (mini) {
		op = 3;
	} else if (t < 0) {
		op = 1; ncol = 5; cj = 3;
		if (t < -1000) {
			t += 1000;
			t *= -1;
			op = 2; ncol = 13; cj = 5;
		}
	}
	for (int l = 0; l < pd; l++) {
		rep[l].iterations = 0;
		rep[l].status = SIMPOIS_OK;
	}
	for (int k = nl - 1; k >= 0; k--) {
		RefLevel &c = lv[k];
		dim3 G(nblk(c.w, 32), nblk(c.h, 8), pd);
		k_prolong_init<<<G, B2, 0, s>>>(c.u, c.g, c.w, c.h, k + 1 < nl ? lv[k + 1].u : nullptr,
				k + 1 < nl ? lv[k + 1].w : 0, k + 1 < nl ? lv[k + 1].h : 0, mini); ctx->launches++;
		int niter = prm->niter, cgit = prm->cgit;
		if (!mini && prm->ponlit != 0 && prm->ponlit != (double)c.w) niter = cgit = 0;
		for (int it = 0; it < niter; it++)
			for (int col = 0; col < ncol; col++) {
				k_gs_class<<<G, B2, 0, s>>>(c.u, c.g, c.f, c.w, c.h, t, op, ncol, cj, col); ctx->launches++;
			}
		SP_LAUNCH_CHECK(ctx);
		if (mini) continue;
		bool poisson = cgit && prm->tstep > 0;
		int maxit = cgit;
		// float cg_maxit = maxit == -1 ? nmask : maxit; a non-positive cap runs
		// no iteration, and then the branch only restores the known pixels
		if (maxit == 0 || maxit < -1) {
			size_t cs = (size_t)c.w * c.h;
			int *has_nan = (int *)cg_ws;
			SP_CUDA(ctx, cudaMemsetAsync(has_nan, 0, sizeof(int) * pd, s));
			dim3 G1(nblk(cs, 256), pd);
			k_nan_any<<<G1, 256, 0, s>>>(c.g, cs, has_nan); ctx->launches++;
			k_restore_known<<<G1, 256, 0, s>>>(c.u, c.g, cs, has_nan); ctx->launches++;
			SP_LAUNCH_CHECK(ctx);
		} else {
			size_t cs = (size_t)c.w * c.h;
			for (int l = 0; l < pd; l++) {
				int iters = 0, st = SIMPOIS_OK;
				int r = ref_cg_channel(ctx, poisson ? 0 : 1, c.u + cs * l, c.g + cs * l,
						c.f ? c.f + cs * l : nullptr, c.w, c.h, maxit,
						poisson ? 1e-6f : 1e-9f, prm, cg_ws, &iters, &st);
				if (r) return r;
				if (k == 0) rep[l].iterations = iters;
				if (st != SIMPOIS_OK) rep[l].status = st;
			}
		}
	}
	SP_CUDA(ctx, cudaMemcpyAsync(out, lv[0].u, sizeof(float) * (size_t)w * h * pd,
			cudaMemcpyDeviceToDevice, s));
	return SIMPOIS_OK;
}
