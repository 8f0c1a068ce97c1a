// mg_solver.cu -- the converged schedule: batched multigrid-preconditioned
// conjugate gradient in FP32 inside an FP64 iterative refinement.
//
// Problem.  For every channel of every image, the unknowns U are the NaN
// pixels of g.  The system is the one the reference's CG solves
// (cleant_cgpois.c:197-264): A = -Laplacian (5-point, clamp-to-edge, kind 0,
// cleant_cgpois.c:67-89) or the 13-point bilaplacian with a single clamp
// (kind 1, cleant_cgpois.c:91-121), restricted to U, and b = -f_U - A_UK g_K.
//
// Refinement (FP64).  The solution lives in an FP64 image Ufull (g at the
// known pixels).  Each refinement step computes r = b - A Ufull in FP64 and
// its norm (the FP64 relative residual reported to the caller), stops when it
// is <= rtol, otherwise solves A d = (float)r in FP32 and adds d in FP64.
//
// Inner solve (FP32 vectors, FP64 reductions).  Preconditioned CG, the
// preconditioner one V(2,2)-cycle of geometric multigrid on the masked grid:
//   * level l+1 is ceil(w/2) x ceil(h/2); a coarse pixel is unknown iff all
//     its (existing) children are unknown, so that every coarse level keeps
//     the known pixels that make it non-singular;
//   * the coarse operators are the same clamped stencils on the coarse masks;
//   * smoothing is colour-ordered Gauss-Seidel (2 colours and 2 sweeps for 5
//     points, 5 colours and 4 sweeps for 13 points), forward before the coarse correction and backward after it,
//     so the cycle is a symmetric operator when A is;
//   * restriction sums the children's residuals (times 2 for the 13-point
//     operator), prolongation injects the coarse correction into the unknown
//     children; the coarsest level (<= 4 x 4) gets 10 symmetric sweeps.
//
// Batching.  All problems of a call share every launch: each level keeps one
// list of 32 x 32 tiles that contain unknowns, over all problems.  Every
// reduction is per problem and deterministic: each tile writes its partial
// sum, the last tile of a problem to finish (an atomic counter) sums the
// problem's partials in tile order and updates the problem's scalars.  A
// problem whose inner solve has converged skips every later launch (early
// retirement).  One PCG iteration is captured once into a CUDA graph and
// replayed; the host reads one counter every few iterations.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "solvers.h"

namespace {

constexpr int MAXLEV = 16;
constexpr int COARSE_MAX = 4;       // coarsest level: max(w, h) <= 4
constexpr int COARSE_SWEEPS = 10;   // symmetric sweeps on the coarsest level
constexpr int NU5 = 2;              // pre- and post-smoothing sweeps, 5-point
constexpr int NU13 = 4;             // pre- and post-smoothing sweeps, 13-point
constexpr int MAX_OUTER = 8;        // FP64 refinement steps
constexpr int INNER_MAX = 60;       // PCG iterations per refinement step
constexpr double TAU_MIN = 2e-6;    // FP32 inner solve: smallest relative decrease

struct LevelDev {
	int w, h;
	uint8_t *mask;   // 1 = unknown
	float *b;        // right-hand side (level 0: the PCG residual r)
	float *z;        // correction (level 0: the preconditioned residual)
};

struct ProbDev {
	int nlev, kind, w, h;
	const float *g;      // input channel
	const float *rhs;    // fill: f (sign -1) ; adjoint: grad_out (sign +1)
	float rhs_sign;
	float *out;
	double *U;           // FP64 solution image (g or 0 at the known pixels)
	float *x, *p, *q;    // level-0 PCG vectors
	double rtol;
	LevelDev lv[MAXLEV];
};

struct ProbState {
	double bnorm2, rho, alpha, beta, rr, tau2, rel, rel_first;
	int iter, total_iter, outer, inner_active, outer_active, status;
	unsigned int cnt;
	int max_iter;
	int nknown, nunknown;   // pixel counts of the channel
};

struct Globals {
	int inner_count;   // problems whose inner solve is running
	int pad[31];
};

// ------------------------------------------------------------------ stencils

__constant__ int8_t c_di13[12] = {1, 0, -1, 0, 1, 1, -1, -1, 2, 0, -2, 0};
__constant__ int8_t c_dj13[12] = {0, 1, 0, -1, 1, -1, 1, -1, 0, 2, 0, -2};
__constant__ float c_cf13[12] = {-8, -8, -8, -8, 2, 2, 2, 2, 1, 1, 1, 1};

// Split the masked operator at unknown (i, j) of a level into its diagonal
// (coefficients of the stencil points that clamp onto the pixel itself) and
// the off-diagonal sum over the unknown pixels (known pixels hold 0).
template <int K>
__device__ __forceinline__ void split(const LevelDev &L, const float *__restrict__ z, int i, int j,
		float &diag, float &off)
{
	const int w = L.w, h = L.h;
	if (K == 0) {
		diag = 4.f;
		off = 0.f;
		const int k = j * w + i;
		if (i + 1 < w) { if (L.mask[k + 1]) off -= z[k + 1]; } else diag -= 1.f;
		if (i > 0)     { if (L.mask[k - 1]) off -= z[k - 1]; } else diag -= 1.f;
		if (j + 1 < h) { if (L.mask[k + w]) off -= z[k + w]; } else diag -= 1.f;
		if (j > 0)     { if (L.mask[k - w]) off -= z[k - w]; } else diag -= 1.f;
	} else {
		diag = 20.f;
		off = 0.f;
#pragma unroll
		for (int s = 0; s < 12; s++) {
			int qi = clampi(i + c_di13[s], w), qj = clampi(j + c_dj13[s], h);
			if (qi == i && qj == j) {
				diag += c_cf13[s];
			} else {
				int q = qj * w + qi;
				if (L.mask[q]) off += c_cf13[s] * z[q];
			}
		}
	}
}

// A ufull at (i, j) in FP64 on a full image (known pixels included); when
// `zero_unknown`, unknown pixels read as 0 (this gives A_UK g_K).
template <int K>
__device__ __forceinline__ double apply64(const double *__restrict__ U, const uint8_t *__restrict__ m,
		int w, int h, int i, int j, bool zero_unknown)
{
	auto at = [&](int a, int b) -> double {
		int q = clampi(b, h) * w + clampi(a, w);
		return (zero_unknown && m[q]) ? 0.0 : U[q];
	};
	if (K == 0) return 4.0 * at(i, j) - at(i + 1, j) - at(i, j + 1) - at(i - 1, j) - at(i, j - 1);
	double r = 20.0 * at(i, j);
#pragma unroll
	for (int s = 0; s < 12; s++) r += (double)c_cf13[s] * at(i + c_di13[s], j + c_dj13[s]);
	return r;
}

__device__ __forceinline__ int colour_of(int K, int i, int j) { return K == 0 ? ((i + j) & 1) : (i + 3 * j) % 5; }

// ------------------------------------------------------------------ tile helpers

__device__ __forceinline__ int tile_i(int4 t) { return t.y * SP_TILE + (threadIdx.x & 31); }
__device__ __forceinline__ int tile_j(int4 t, int r) { return t.z * SP_TILE + (threadIdx.x >> 5) + SP_BLOCK_Y * r; }

// Per-problem deterministic reduction of up to two values over the level-0
// tiles of the problem.  Returns true in the last tile's block (all threads);
// the sums are then in tot[0..1] (thread 0).
__device__ bool problem_sum2(double v0, double v1, int prob, const int *__restrict__ tbeg,
		const int *__restrict__ tcnt, double *partial, ProbState *st, double *tot, double *sh)
{
	__shared__ bool am_last;
	double s0 = block_sum<SP_THREADS>(v0, sh);
	double s1 = block_sum<SP_THREADS>(v1, sh);
	if (threadIdx.x == 0) {
		partial[2 * blockIdx.x] = s0;
		partial[2 * blockIdx.x + 1] = s1;
		__threadfence();
		unsigned prev = atomicAdd(&st[prob].cnt, 1u);
		am_last = prev == (unsigned)tcnt[prob] - 1;
	}
	__syncthreads();
	if (!am_last) return false;
	__threadfence();
	double a0 = 0, a1 = 0;
	const int b0 = tbeg[prob], n = tcnt[prob];
	for (int k = threadIdx.x; k < n; k += SP_THREADS) {
		a0 += __ldcg(partial + 2 * (b0 + k));
		a1 += __ldcg(partial + 2 * (b0 + k) + 1);
	}
	a0 = block_sum<SP_THREADS>(a0, sh);
	a1 = block_sum<SP_THREADS>(a1, sh);
	if (threadIdx.x == 0) {
		tot[0] = a0;
		tot[1] = a1;
		st[prob].cnt = 0;
	}
	return true;
}

// ------------------------------------------------------------------ setup kernels

// Level 0 over all tiles: mask = isnan(g); U = g at the knowns (fill) or 0
// (adjoint), 0 at the unknowns; flag = tile holds an unknown; per-problem
// pixel counts.
__global__ void k_setup0(const ProbDev *__restrict__ P, ProbState *st, const int4 *__restrict__ all,
		int *__restrict__ flag, int adjoint)
{
	__shared__ int cnt[2];
	int4 t = all[blockIdx.x];
	const ProbDev &pr = P[t.x];
	if (threadIdx.x < 2) cnt[threadIdx.x] = 0;
	__syncthreads();
	int i = tile_i(t);
	int nu = 0, nk = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			float gv = pr.g[k];
			bool u = isnan(gv);
			pr.lv[0].mask[k] = u;
			pr.U[k] = (u || adjoint) ? 0.0 : (double)gv;
			nu += u;
			nk += !u;
		}
	}
	for (int o = 16; o > 0; o >>= 1) {
		nu += __shfl_down_sync(0xffffffffu, nu, o);
		nk += __shfl_down_sync(0xffffffffu, nk, o);
	}
	if ((threadIdx.x & 31) == 0) {
		atomicAdd(&cnt[0], nu);
		atomicAdd(&cnt[1], nk);
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		flag[blockIdx.x] = cnt[0] > 0;
		if (cnt[0]) atomicAdd(&st[t.x].nunknown, cnt[0]);
		if (cnt[1]) atomicAdd(&st[t.x].nknown, cnt[1]);
	}
}

// Level l >= 1 over all tiles: unknown iff every existing child is unknown.
__global__ void k_mask_down(const ProbDev *__restrict__ P, const int4 *__restrict__ all, int l, int *__restrict__ flag)
{
	__shared__ int any;
	int4 t = all[blockIdx.x];
	const ProbDev &pr = P[t.x];
	const LevelDev &C = pr.lv[l], &F = pr.lv[l - 1];
	if (threadIdx.x == 0) any = 0;
	__syncthreads();
	int i = tile_i(t);
	int mine = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < C.w && j < C.h) {
			bool u = true;
			for (int b = 0; b < 2; b++)
				for (int a = 0; a < 2; a++) {
					int fi = 2 * i + a, fj = 2 * j + b;
					if (fi < F.w && fj < F.h) u = u && F.mask[(size_t)fj * F.w + fi];
				}
			C.mask[(size_t)j * C.w + i] = u;
			mine |= u;
		}
	}
	if (__any_sync(0xffffffffu, mine) && (threadIdx.x & 31) == 0) atomicOr(&any, 1);
	__syncthreads();
	if (threadIdx.x == 0) flag[blockIdx.x] = any;
}

// One block per level: ordered compaction of the level's tile list by flag.
// For level 0 also the per-problem tile ranges (tbeg, tcnt).
__global__ void k_compact(const int4 *const *__restrict__ all, const int *const *__restrict__ flag,
		const int *__restrict__ nall, int4 *const *__restrict__ act, int *__restrict__ nact,
		int *__restrict__ tbeg, int *__restrict__ tcnt)
{
	__shared__ int wsum[32];
	__shared__ int carry;
	const int l = blockIdx.x;
	const int n = nall[l];
	if (threadIdx.x == 0) carry = 0;
	__syncthreads();
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int base = 0; base < n; base += 1024) {
		int k = base + threadIdx.x;
		bool on = k < n && flag[l][k];
		unsigned bal = __ballot_sync(0xffffffffu, on);
		if (lane == 0) wsum[warp] = __popc(bal);
		__syncthreads();
		int off = carry;
		for (int q = 0; q < warp; q++) off += wsum[q];
		off += __popc(bal & ((1u << lane) - 1));
		if (on) {
			int4 t = all[l][k];
			act[l][off] = t;
			if (l == 0) {
				atomicMin(tbeg + t.x, off);
				atomicAdd(tcnt + t.x, 1);
			}
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			int s = 0;
			for (int q = 0; q < 32; q++) s += wsum[q];
			carry += s;
		}
		__syncthreads();
	}
	if (threadIdx.x == 0) nact[l] = carry;
}

// ------------------------------------------------------------------ refinement kernels

// r = rhs_sign*rhs - A U (FP64) at the unknowns; b0 = (float)r; x = 0.
// The last tile of a problem decides: converged, or start an inner solve.
template <int K>
__global__ void k_resid64(const ProbDev *__restrict__ P, ProbState *st, const int4 *__restrict__ tl,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial,
		Globals *gl, int first)
{
	__shared__ double sh[32];
	int4 t = tl[blockIdx.x];
	const int prob = t.x;
	if (!st[prob].outer_active) return;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	int i = tile_i(t);
	double rr = 0, bb = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			if (L.mask[k]) {
				double s = pr.rhs ? (double)pr.rhs_sign * (double)pr.rhs[k] : 0.0;
				double rk = s - apply64<K>(pr.U, L.mask, pr.w, pr.h, i, j, false);
				L.b[k] = (float)rk;
				pr.x[k] = 0.f;
				rr += rk * rk;
				if (first) {
					double bk = s - apply64<K>(pr.U, L.mask, pr.w, pr.h, i, j, true);
					bb += bk * bk;
				}
			}
		}
	}
	double tot[2];
	if (problem_sum2(rr, bb, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		if (first) s.bnorm2 = tot[1];
		if (first && s.nknown == 0) s.status = SIMPOIS_SINGULAR;
		double rel = s.bnorm2 > 0 ? sqrt(tot[0] / s.bnorm2) : 0.0;
		if (first) s.rel_first = rel;
		s.rel = rel;
		bool ok = rel <= pr.rtol;
		if (ok || !isfinite(rel) || s.outer >= MAX_OUTER || s.total_iter >= s.max_iter ||
				s.status != SIMPOIS_OK) {
			s.outer_active = 0;
			s.inner_active = 0;
			if (s.status == SIMPOIS_OK && !ok) s.status = SIMPOIS_NOT_CONVERGED;
		} else {
			s.outer += 1;
			s.iter = 0;
			s.inner_active = 1;
			double tau = fmax(0.3 * pr.rtol / rel, TAU_MIN);
			s.tau2 = tau * tau * tot[0];
			s.rho = 0;
			s.beta = 0;
			atomicAdd(&gl->inner_count, 1);
		}
	}
}

// U += x at the unknowns (end of an inner solve)
__global__ void k_uadd(const ProbDev *__restrict__ P, const ProbState *__restrict__ st, const int4 *__restrict__ tl)
{
	int4 t = tl[blockIdx.x];
	if (!st[t.x].outer_active) return;
	const ProbDev &pr = P[t.x];
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			if (pr.lv[0].mask[k]) pr.U[k] += (double)pr.x[k];
		}
	}
}

// ------------------------------------------------------------------ PCG kernels

// p = z + beta p at the unknowns
__global__ void k_pupdate(const ProbDev *__restrict__ P, const ProbState *__restrict__ st, const int4 *__restrict__ tl)
{
	int4 t = tl[blockIdx.x];
	if (!st[t.x].inner_active) return;
	const ProbDev &pr = P[t.x];
	const float beta = (float)st[t.x].beta;
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			if (pr.lv[0].mask[k])
				pr.p[k] = beta != 0.f ? pr.lv[0].z[k] + beta * pr.p[k] : pr.lv[0].z[k];
		}
	}
}

// q = A p, alpha = rho / (p.q)
template <int K>
__global__ void k_spmv(const ProbDev *__restrict__ P, ProbState *st, const int4 *__restrict__ tl,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial, Globals *gl)
{
	__shared__ double sh[32];
	int4 t = tl[blockIdx.x];
	const int prob = t.x;
	if (!st[prob].inner_active) return;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	int i = tile_i(t);
	double pq = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			if (L.mask[k]) {
				float d, o;
				split<K>(L, pr.p, i, j, d, o);
				float pk = pr.p[k];
				float qk = d * pk + o;
				pr.q[k] = qk;
				pq += (double)pk * (double)qk;
			}
		}
	}
	double tot[2];
	if (problem_sum2(pq, 0.0, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		double a = s.rho / tot[0];
		if (!(tot[0] > 0) || !isfinite(a)) {
			s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			s.alpha = 0;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.alpha = a;
		}
	}
}

// x += alpha p; r -= alpha q; r.r; the inner stopping test
__global__ void k_xr(const ProbDev *__restrict__ P, ProbState *st, const int4 *__restrict__ tl,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial, Globals *gl)
{
	__shared__ double sh[32];
	int4 t = tl[blockIdx.x];
	const int prob = t.x;
	if (!st[prob].inner_active) return;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	const float a = (float)st[prob].alpha;
	int i = tile_i(t);
	double rr = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			if (L.mask[k]) {
				pr.x[k] += a * pr.p[k];
				float rk = L.b[k] - a * pr.q[k];
				L.b[k] = rk;
				rr += (double)rk * rk;
			}
		}
	}
	double tot[2];
	if (problem_sum2(rr, 0.0, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		s.rr = tot[0];
		s.iter += 1;
		s.total_iter += 1;
		if (tot[0] <= s.tau2 || s.iter >= INNER_MAX || s.total_iter >= s.max_iter) {
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		}
	}
}

// rho_new = r.z; beta = rho_new / rho (0 on the first iteration)
__global__ void k_rz(const ProbDev *__restrict__ P, ProbState *st, const int4 *__restrict__ tl,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial, Globals *gl)
{
	__shared__ double sh[32];
	int4 t = tl[blockIdx.x];
	const int prob = t.x;
	if (!st[prob].inner_active) return;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	int i = tile_i(t);
	double rz = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			if (L.mask[k]) rz += (double)L.b[k] * (double)L.z[k];
		}
	}
	double tot[2];
	if (problem_sum2(rz, 0.0, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		if (!(tot[0] > 0) || !isfinite(tot[0])) {
			// r = 0 exactly, or a preconditioner that is not positive here
			if (tot[0] != 0) s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.beta = s.rho > 0 ? tot[0] / s.rho : 0.0;
			s.rho = tot[0];
		}
	}
}

// z = r (no preconditioner)
__global__ void k_copy_rz(const ProbDev *__restrict__ P, const ProbState *__restrict__ st, const int4 *__restrict__ tl)
{
	int4 t = tl[blockIdx.x];
	if (!st[t.x].inner_active) return;
	const ProbDev &pr = P[t.x];
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			pr.lv[0].z[k] = pr.lv[0].b[k];
		}
	}
}

// ------------------------------------------------------------------ V-cycle kernels

// z = 0 on level l (problems for which l is not the coarsest level)
__global__ void k_zero(const ProbDev *__restrict__ P, const ProbState *__restrict__ st, const int4 *__restrict__ tl, int l)
{
	int4 t = tl[blockIdx.x];
	const ProbDev &pr = P[t.x];
	if (!st[t.x].inner_active || l >= pr.nlev - 1) return;
	const LevelDev &L = pr.lv[l];
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < L.w && j < L.h) L.z[(size_t)j * L.w + i] = 0.f;
	}
}

// one colour class of Gauss-Seidel on A z = b at level l
template <int K>
__global__ void k_smooth(const ProbDev *__restrict__ P, const ProbState *__restrict__ st, const int4 *__restrict__ tl,
		int l, int colour)
{
	int4 t = tl[blockIdx.x];
	const ProbDev &pr = P[t.x];
	if (!st[t.x].inner_active || l >= pr.nlev - 1) return;
	const LevelDev &L = pr.lv[l];
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < L.w && j < L.h && colour_of(K, i, j) == colour) {
			size_t k = (size_t)j * L.w + i;
			if (L.mask[k]) {
				float d, o;
				split<K>(L, L.z, i, j, d, o);
				L.z[k] = (L.b[k] - o) / d;
			}
		}
	}
}

// b_{l} = rscale * sum over the unknown children of (b - A z)_{l-1}
template <int K>
__global__ void k_restrict_res(const ProbDev *__restrict__ P, const ProbState *__restrict__ st,
		const int4 *__restrict__ tl, int l, float rscale)
{
	int4 t = tl[blockIdx.x];
	const ProbDev &pr = P[t.x];
	if (!st[t.x].inner_active || l >= pr.nlev) return;
	const LevelDev &C = pr.lv[l], &F = pr.lv[l - 1];
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < C.w && j < C.h) {
			size_t kc = (size_t)j * C.w + i;
			if (!C.mask[kc]) continue;
			float s = 0.f;
			for (int b = 0; b < 2; b++)
				for (int a = 0; a < 2; a++) {
					int fi = 2 * i + a, fj = 2 * j + b;
					if (fi < F.w && fj < F.h) {
						size_t kf = (size_t)fj * F.w + fi;
						float d, o;
						split<K>(F, F.z, fi, fj, d, o);
						s += F.b[kf] - (d * F.z[kf] + o);
					}
				}
			C.b[kc] = rscale * s;
		}
	}
}

// z_l += z_{l+1}(parent) at the unknowns whose parent is unknown
__global__ void k_prolong_add(const ProbDev *__restrict__ P, const ProbState *__restrict__ st,
		const int4 *__restrict__ tl, int l)
{
	int4 t = tl[blockIdx.x];
	const ProbDev &pr = P[t.x];
	if (!st[t.x].inner_active || l >= pr.nlev - 1) return;
	const LevelDev &F = pr.lv[l], &C = pr.lv[l + 1];
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < F.w && j < F.h) {
			size_t kf = (size_t)j * F.w + i;
			size_t kc = (size_t)(j >> 1) * C.w + (i >> 1);
			if (F.mask[kf] && C.mask[kc]) F.z[kf] += C.z[kc];
		}
	}
}

// Coarsest level of every problem, one block each: symmetric colour sweeps
// in shared memory.
template <int K>
__global__ void k_coarsest(const ProbDev *__restrict__ P, const ProbState *__restrict__ st)
{
	constexpr int NC = K == 0 ? 2 : 5;
	__shared__ float z[64], b[64];
	__shared__ uint8_t m[64];
	const int prob = blockIdx.x;
	if (!st[prob].inner_active) return;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[pr.nlev - 1];
	const int n = L.w * L.h;
	const int k = threadIdx.x;
	if (k < n) {
		m[k] = L.mask[k];
		b[k] = L.b[k];
		z[k] = 0.f;
	}
	__syncthreads();
	LevelDev Ls = L;
	Ls.mask = m;
	const int i = k % max(L.w, 1), j = k / max(L.w, 1);
	for (int s = 0; s < COARSE_SWEEPS; s++)
		for (int dir = 0; dir < 2; dir++)
			for (int cc = 0; cc < NC; cc++) {
				int c = dir ? NC - 1 - cc : cc;
				if (k < n && m[k] && colour_of(K, i, j) == c) {
					float d, o;
					split<K>(Ls, z, i, j, d, o);
					z[k] = (b[k] - o) / d;
				}
				__syncthreads();
			}
	if (k < n) L.z[k] = m[k] ? z[k] : 0.f;
}

// out = unknown ? (float)U : g over all tiles (fill)
__global__ void k_finalize(const ProbDev *__restrict__ P, const int4 *__restrict__ all)
{
	int4 t = all[blockIdx.x];
	const ProbDev &pr = P[t.x];
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < pr.w && j < pr.h) {
			size_t k = (size_t)j * pr.w + i;
			pr.out[k] = pr.lv[0].mask[k] ? (float)pr.U[k] : pr.g[k];
		}
	}
}

// Adjoint scatter (5-point): grad_in = grad_out + sum of lambda over the
// unknown 5-neighbours at the known pixels, 0 at the unknowns; grad_dat =
// -lambda at the unknowns, 0 elsewhere.
__global__ void k_adjoint_scatter(const ProbDev *__restrict__ P, const int4 *__restrict__ all,
		const float *const *__restrict__ gout, float *const *__restrict__ gin, float *const *__restrict__ gdat)
{
	int4 t = all[blockIdx.x];
	const ProbDev &pr = P[t.x];
	const uint8_t *m = pr.lv[0].mask;
	const int w = pr.w, h = pr.h;
	int i = tile_i(t);
	for (int r = 0; r < SP_ROWS; r++) {
		int j = tile_j(t, r);
		if (i < w && j < h) {
			size_t k = (size_t)j * w + i;
			if (m[k]) {
				gin[t.x][k] = 0.f;
				if (gdat[t.x]) gdat[t.x][k] = -(float)pr.U[k];
			} else {
				double s = gout[t.x][k];
				if (i + 1 < w && m[k + 1]) s += pr.U[k + 1];
				if (i > 0 && m[k - 1]) s += pr.U[k - 1];
				if (j + 1 < h && m[k + w]) s += pr.U[k + w];
				if (j > 0 && m[k - w]) s += pr.U[k - w];
				gin[t.x][k] = (float)s;
				if (gdat[t.x]) gdat[t.x][k] = 0.f;
			}
		}
	}
}

// FP64 residual of a float output, dense per problem (one launch per problem)
template <int K>
__global__ void k_dense_resid(const float *__restrict__ u, const float *__restrict__ g, const float *__restrict__ f,
		int w, int h, double *partial, unsigned int *cnt, double *res)
{
	__shared__ double sh[32];
	__shared__ bool am_last;
	size_t k = (size_t)blockIdx.x * 256 + threadIdx.x;
	double rr = 0, bb = 0;
	if (k < (size_t)w * h && isnan(g[k])) {
		int i = (int)(k % w), j = (int)(k / w);
		auto at = [&](int a, int b, bool zu) -> double {
			int q = clampi(b, h) * w + clampi(a, w);
			float gv = g[q];
			if (isnan(gv)) return zu ? 0.0 : (double)u[q];
			return (double)gv;
		};
		auto A = [&](bool zu) -> double {
			if (K == 0) return 4.0 * at(i, j, zu) - at(i + 1, j, zu) - at(i, j + 1, zu) - at(i - 1, j, zu) - at(i, j - 1, zu);
			double r = 20.0 * at(i, j, zu);
			for (int s = 0; s < 12; s++) r += (double)c_cf13[s] * at(i + c_di13[s], j + c_dj13[s], zu);
			return r;
		};
		double fk = f ? -(double)f[k] : 0.0;
		double rk = fk - A(false), bk = fk - A(true);
		rr = rk * rk;
		bb = bk * bk;
	}
	double s0 = block_sum<256>(rr, sh), s1 = block_sum<256>(bb, sh);
	if (threadIdx.x == 0) {
		partial[2 * blockIdx.x] = s0;
		partial[2 * blockIdx.x + 1] = s1;
		__threadfence();
		am_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
	}
	__syncthreads();
	if (!am_last) return;
	__threadfence();
	double a0 = 0, a1 = 0;
	for (int q = threadIdx.x; q < (int)gridDim.x; q += 256) {
		a0 += __ldcg(partial + 2 * q);
		a1 += __ldcg(partial + 2 * q + 1);
	}
	a0 = block_sum<256>(a0, sh);
	a1 = block_sum<256>(a1, sh);
	if (threadIdx.x == 0) {
		res[0] = a0;
		res[1] = a1;
		*cnt = 0;
	}
}

// ------------------------------------------------------------------ host plan

struct Plan {
	int n = 0, nlev_max = 0, kind_mask = 0;
	std::vector<ProbDev> hp;
	ProbDev *dp = nullptr;
	ProbState *dst = nullptr;
	Globals *gl = nullptr;
	int4 *all[MAXLEV] = {}, *act[MAXLEV] = {};
	int *flag[MAXLEV] = {};
	int nall[MAXLEV] = {}, nact[MAXLEV] = {};
	int *dnall = nullptr, *dnact = nullptr;
	int4 **dall = nullptr, **dact = nullptr;
	int **dflag = nullptr;
	int *tbeg = nullptr, *tcnt = nullptr;
	double *partial = nullptr;
	const float **gout = nullptr;
	float **gin = nullptr, **gdat = nullptr;
	long long *nl = nullptr;   // the context's launch counter
};

inline int ntiles(int v) { return (v + SP_TILE - 1) / SP_TILE; }

// Level dims of a problem: halve (ceil) while max(w, h) > COARSE_MAX.
int level_dims(int w, int h, int *lw, int *lh)
{
	int n = 0;
	lw[0] = w;
	lh[0] = h;
	while (n + 1 < MAXLEV && std::max(lw[n], lh[n]) > COARSE_MAX) {
		lw[n + 1] = (lw[n] + 1) / 2;
		lh[n + 1] = (lh[n] + 1) / 2;
		n++;
	}
	return n + 1;
}

template <int K>
void launch_vcycle(const Plan &pl, cudaStream_t s)
{
	constexpr int NC = K == 0 ? 2 : 5;
	constexpr int NU = K == 0 ? NU5 : NU13;
	const float rscale = K == 0 ? 1.f : 2.f;
	const int L = pl.nlev_max;
	for (int l = 0; l + 1 < L; l++) {
		if (!pl.nact[l]) continue;
		k_zero<<<pl.nact[l], SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[l], l); ++*pl.nl;
		for (int sw = 0; sw < NU; sw++)
			for (int c = 0; c < NC; c++) {
				k_smooth<K><<<pl.nact[l], SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[l], l, c); ++*pl.nl;
			}
		if (pl.nact[l + 1]) {
			k_restrict_res<K><<<pl.nact[l + 1], SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[l + 1], l + 1, rscale); ++*pl.nl;
		}
	}
	k_coarsest<K><<<pl.n, 64, 0, s>>>(pl.dp, pl.dst); ++*pl.nl;
	for (int l = L - 2; l >= 0; l--) {
		if (!pl.nact[l]) continue;
		k_prolong_add<<<pl.nact[l], SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[l], l); ++*pl.nl;
		for (int sw = 0; sw < NU; sw++)
			for (int c = NC - 1; c >= 0; c--) {
				k_smooth<K><<<pl.nact[l], SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[l], l, c); ++*pl.nl;
			}
	}
}

template <int K>
void launch_precond(const Plan &pl, const MgOptions &opt, cudaStream_t s)
{
	if (opt.use_mg)
		launch_vcycle<K>(pl, s);
	else {
		k_copy_rz<<<pl.nact[0], SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0]); ++*pl.nl;
	}
}

template <int K>
void launch_iteration(const Plan &pl, const MgOptions &opt, cudaStream_t s)
{
	const int nt = pl.nact[0];
	k_pupdate<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0]); ++*pl.nl;
	k_spmv<K><<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
	k_xr<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
	launch_precond<K>(pl, opt, s);
	k_rz<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
}

template <int K>
int run_kind(simpois_ctx *ctx, Plan &pl, const MgOptions &opt)
{
	cudaStream_t s = ctx->stream;
	int *hcount = (int *)ctx->pinned;
	const int nt = pl.nact[0];
	if (nt == 0) return SIMPOIS_OK;
	cudaGraphExec_t gexec = nullptr;
	long long per_iter = 0;   // kernel nodes of one captured iteration
	if (opt.use_graph) {
		cudaGraph_t graph;
		long long before = *pl.nl;
		SP_CUDA(ctx, cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal));
		launch_iteration<K>(pl, opt, ctx->capture_stream);
		SP_CUDA(ctx, cudaStreamEndCapture(ctx->capture_stream, &graph));
		per_iter = *pl.nl - before;
		*pl.nl = before;
		cudaError_t e = cudaGraphInstantiate(&gexec, graph, 0);
		cudaGraphDestroy(graph);
		if (e != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
	}
	int rc = SIMPOIS_OK;
	for (int outer = 0; outer <= MAX_OUTER; outer++) {
		k_resid64<K><<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl,
				outer == 0); ++*pl.nl;
		launch_precond<K>(pl, opt, s);
		k_rz<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
		cudaError_t e = cudaMemcpyAsync(hcount, &pl.gl->inner_count, sizeof(int), cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess) e = cudaStreamSynchronize(s);
		if (e != cudaSuccess) { rc = ctx_fail(ctx, SIMPOIS_ECUDA, "refinement: %s", cudaGetErrorString(e)); break; }
		if (*hcount == 0) break;
		int chunk = 4;
		for (int guard = 0; guard < 4 * INNER_MAX; guard++) {
			for (int c = 0; c < chunk; c++) {
				if (gexec) {
					e = cudaGraphLaunch(gexec, s);
					*pl.nl += per_iter;
				} else
					launch_iteration<K>(pl, opt, s), e = cudaGetLastError();
				if (e != cudaSuccess) break;
			}
			if (e == cudaSuccess)
				e = cudaMemcpyAsync(hcount, &pl.gl->inner_count, sizeof(int), cudaMemcpyDeviceToHost, s);
			if (e == cudaSuccess) e = cudaStreamSynchronize(s);
			if (e != cudaSuccess) break;
			if (*hcount == 0) break;
			chunk = 2;
		}
		if (e != cudaSuccess) { rc = ctx_fail(ctx, SIMPOIS_ECUDA, "inner solve: %s", cudaGetErrorString(e)); break; }
		k_uadd<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0]); ++*pl.nl;
	}
	if (gexec) cudaGraphExecDestroy(gexec);
	return rc;
}

}  // namespace

int mg_solve(simpois_ctx *ctx, const MgProblem *probs, int n, const MgOptions &opt, simpois_report *rep)
{
	if (n <= 0) return SIMPOIS_OK;
	cudaStream_t s = ctx->stream;
	Plan pl;
	pl.nl = &ctx->launches;
	pl.n = n;
	pl.hp.resize(n);
	int kinds = 0;
	Layout Lo;
	std::vector<size_t> off_mask[MAXLEV], off_b[MAXLEV], off_z[MAXLEV];
	std::vector<size_t> off_U(n), off_x(n), off_p(n), off_q(n);
	std::vector<std::vector<int4>> lists(MAXLEV);
	for (int k = 0; k < n; k++) {
		const MgProblem &q = probs[k];
		int lw[MAXLEV], lh[MAXLEV];
		int nl = level_dims(q.w, q.h, lw, lh);
		ProbDev &d = pl.hp[k];
		memset(&d, 0, sizeof(d));
		d.nlev = nl;
		d.kind = q.kind;
		d.w = q.w;
		d.h = q.h;
		d.rtol = q.rtol;
		kinds |= 1 << q.kind;
		pl.nlev_max = std::max(pl.nlev_max, nl);
		for (int l = 0; l < nl; l++) {
			size_t px = (size_t)lw[l] * lh[l];
			d.lv[l].w = lw[l];
			d.lv[l].h = lh[l];
			off_mask[l].push_back(Lo.take(px));
			off_b[l].push_back(Lo.take(px * 4));
			off_z[l].push_back(Lo.take(px * 4));
			for (int ty = 0; ty < ntiles(lh[l]); ty++)
				for (int tx = 0; tx < ntiles(lw[l]); tx++) lists[l].push_back(make_int4(k, tx, ty, 0));
		}
		for (int l = nl; l < MAXLEV; l++) {
			off_mask[l].push_back(0);
			off_b[l].push_back(0);
			off_z[l].push_back(0);
		}
		size_t px = (size_t)q.w * q.h;
		off_U[k] = Lo.take(px * 8);
		off_x[k] = Lo.take(px * 4);
		off_p[k] = Lo.take(px * 4);
		off_q[k] = Lo.take(px * 4);
	}
	if (kinds == 3) return ctx_fail(ctx, SIMPOIS_EINVAL, "a batch mixes 5-point and 13-point problems");
	const int K = kinds == 2 ? 1 : 0;
	size_t o_dp = Lo.take(sizeof(ProbDev) * n);
	size_t o_st = Lo.take(sizeof(ProbState) * n);
	size_t o_gl = Lo.take(sizeof(Globals));
	size_t o_all[MAXLEV], o_act[MAXLEV], o_flag[MAXLEV];
	for (int l = 0; l < pl.nlev_max; l++) {
		pl.nall[l] = (int)lists[l].size();
		o_all[l] = Lo.take(sizeof(int4) * lists[l].size());
		o_act[l] = Lo.take(sizeof(int4) * lists[l].size());
		o_flag[l] = Lo.take(sizeof(int) * lists[l].size());
	}
	size_t o_dnall = Lo.take(sizeof(int) * MAXLEV), o_dnact = Lo.take(sizeof(int) * MAXLEV);
	size_t o_dall = Lo.take(sizeof(int4 *) * MAXLEV), o_dact = Lo.take(sizeof(int4 *) * MAXLEV);
	size_t o_dflag = Lo.take(sizeof(int *) * MAXLEV);
	size_t o_tbeg = Lo.take(sizeof(int) * n), o_tcnt = Lo.take(sizeof(int) * n);
	size_t o_part = Lo.take(sizeof(double) * 2 * std::max<size_t>(1, lists[0].size()));
	size_t o_gptr = Lo.take(sizeof(void *) * 3 * n);
	size_t total = Lo.off;
	int rc = ctx_arena_reserve(ctx, total);
	if (rc) return rc;
	char *A = ctx->arena;

	// host images of the device tables, staged in pinned memory
	size_t stage_bytes = sizeof(ProbDev) * n + sizeof(ProbState) * n + sizeof(Globals);
	for (int l = 0; l < pl.nlev_max; l++) stage_bytes += sizeof(int4) * lists[l].size();
	stage_bytes += 64 * MAXLEV + sizeof(void *) * 3 * n + sizeof(int) * n + 16 * (MAXLEV + 16) + 4096;
	rc = ctx_pinned_reserve(ctx, stage_bytes + 256);
	if (rc) return rc;
	char *stage = ctx->pinned + 256;  // the first 256 bytes hold read-back scalars

	for (int k = 0; k < n; k++) {
		ProbDev &d = pl.hp[k];
		const MgProblem &q = probs[k];
		d.g = q.g;
		d.out = q.out;
		if (opt.mode == MG_ADJOINT) {
			d.rhs = opt.grad_out[k];
			d.rhs_sign = 1.f;
		} else {
			d.rhs = q.f;
			d.rhs_sign = -1.f;
		}
		d.U = (double *)(A + off_U[k]);
		d.x = (float *)(A + off_x[k]);
		d.p = (float *)(A + off_p[k]);
		d.q = (float *)(A + off_q[k]);
		for (int l = 0; l < d.nlev; l++) {
			d.lv[l].mask = (uint8_t *)(A + off_mask[l][k]);
			d.lv[l].b = (float *)(A + off_b[l][k]);
			d.lv[l].z = (float *)(A + off_z[l][k]);
		}
	}
	pl.dp = (ProbDev *)(A + o_dp);
	pl.dst = (ProbState *)(A + o_st);
	pl.gl = (Globals *)(A + o_gl);
	pl.tbeg = (int *)(A + o_tbeg);
	pl.tcnt = (int *)(A + o_tcnt);
	pl.partial = (double *)(A + o_part);
	pl.dnall = (int *)(A + o_dnall);
	pl.dnact = (int *)(A + o_dnact);
	pl.dall = (int4 **)(A + o_dall);
	pl.dact = (int4 **)(A + o_dact);
	pl.dflag = (int **)(A + o_dflag);
	for (int l = 0; l < pl.nlev_max; l++) {
		pl.all[l] = (int4 *)(A + o_all[l]);
		pl.act[l] = (int4 *)(A + o_act[l]);
		pl.flag[l] = (int *)(A + o_flag[l]);
	}

	// stage and upload: problem table, states, tile lists, pointer tables
	size_t so = 0;
	auto put = [&](void *dst, const void *src, size_t bytes) -> cudaError_t {
		so = (so + 15) / 16 * 16;
		memcpy(stage + so, src, bytes);
		cudaError_t e = cudaMemcpyAsync(dst, stage + so, bytes, cudaMemcpyHostToDevice, s);
		so += bytes;
		return e;
	};
	std::vector<ProbState> hst(n);
	for (int k = 0; k < n; k++) {
		memset(&hst[k], 0, sizeof(ProbState));
		hst[k].outer_active = 1;
		hst[k].status = SIMPOIS_OK;
		hst[k].max_iter = opt.max_iter > 0 ? opt.max_iter : 500;
	}
	Globals hg;
	memset(&hg, 0, sizeof(hg));
	SP_CUDA(ctx, put(pl.dp, pl.hp.data(), sizeof(ProbDev) * n));
	SP_CUDA(ctx, put(pl.dst, hst.data(), sizeof(ProbState) * n));
	SP_CUDA(ctx, put(pl.gl, &hg, sizeof(hg)));
	for (int l = 0; l < pl.nlev_max; l++)
		SP_CUDA(ctx, put(pl.all[l], lists[l].data(), sizeof(int4) * lists[l].size()));
	SP_CUDA(ctx, put(pl.dnall, pl.nall, sizeof(int) * MAXLEV));
	SP_CUDA(ctx, put(pl.dall, pl.all, sizeof(int4 *) * MAXLEV));
	SP_CUDA(ctx, put(pl.dact, pl.act, sizeof(int4 *) * MAXLEV));
	SP_CUDA(ctx, put(pl.dflag, pl.flag, sizeof(int *) * MAXLEV));
	std::vector<int> init_beg(n, INT_MAX);
	SP_CUDA(ctx, put(pl.tbeg, init_beg.data(), sizeof(int) * n));
	SP_CUDA(ctx, cudaMemsetAsync(pl.tcnt, 0, sizeof(int) * n, s));
	if (opt.mode == MG_ADJOINT) {
		pl.gout = (const float **)(A + o_gptr);
		pl.gin = (float **)(A + o_gptr) + n;
		pl.gdat = (float **)(A + o_gptr) + 2 * n;
		SP_CUDA(ctx, put(pl.gout, opt.grad_out, sizeof(void *) * n));
		SP_CUDA(ctx, put(pl.gin, opt.grad_in, sizeof(void *) * n));
		SP_CUDA(ctx, put(pl.gdat, opt.grad_dat, sizeof(void *) * n));
	}

	// masks, tile flags, compacted lists
	k_setup0<<<pl.nall[0], SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.all[0], pl.flag[0], opt.mode == MG_ADJOINT); ++*pl.nl;
	for (int l = 1; l < pl.nlev_max; l++) {
		k_mask_down<<<pl.nall[l], SP_THREADS, 0, s>>>(pl.dp, pl.all[l], l, pl.flag[l]); ++*pl.nl;
	}
	k_compact<<<pl.nlev_max, 1024, 0, s>>>(pl.dall, pl.dflag, pl.dnall, pl.dact, pl.dnact, pl.tbeg, pl.tcnt); ++*pl.nl;
	SP_LAUNCH_CHECK(ctx);
	int *hn = (int *)ctx->pinned;
	SP_CUDA(ctx, cudaMemcpyAsync(hn, pl.dnact, sizeof(int) * MAXLEV, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	for (int l = 0; l < pl.nlev_max; l++) pl.nact[l] = hn[l];

	rc = K == 0 ? run_kind<0>(ctx, pl, opt) : run_kind<1>(ctx, pl, opt);
	if (rc) return rc;

	if (opt.mode == MG_ADJOINT) {
		k_adjoint_scatter<<<pl.nall[0], SP_THREADS, 0, s>>>(pl.dp, pl.all[0], pl.gout, pl.gin, pl.gdat); ++*pl.nl;
	}
	else {
		k_finalize<<<pl.nall[0], SP_THREADS, 0, s>>>(pl.dp, pl.all[0]); ++*pl.nl;
	}
	SP_LAUNCH_CHECK(ctx);
	ProbState *hs = (ProbState *)stage;
	SP_CUDA(ctx, cudaMemcpyAsync(hs, pl.dst, sizeof(ProbState) * n, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	for (int k = 0; k < n; k++) {
		rep[k].status = hs[k].status;
		rep[k].unknowns = hs[k].nunknown;
		rep[k].iterations = hs[k].total_iter;
		rep[k].refinements = hs[k].outer;
		rep[k].rel_residual = hs[k].rel;
		rep[k].rel_residual_out = -1;
	}
	if (opt.out_resid && opt.mode == MG_FILL) {
		std::vector<const float *> u(n);
		std::vector<double> rel(n), bn(n);
		for (int k = 0; k < n; k++) u[k] = probs[k].out;
		rc = mg_residual(ctx, probs, u.data(), n, rel.data(), bn.data());
		if (rc) return rc;
		for (int k = 0; k < n; k++) rep[k].rel_residual_out = rel[k];
	}
	return SIMPOIS_OK;
}

int mg_residual(simpois_ctx *ctx, const MgProblem *probs, const float *const *u, int n, double *rel,
		double *bnorm)
{
	cudaStream_t s = ctx->stream;
	size_t maxblk = 1;
	for (int k = 0; k < n; k++) maxblk = std::max(maxblk, ((size_t)probs[k].w * probs[k].h + 255) / 256);
	// a private slice at the top of the pinned buffer is not needed: use a
	// small device scratch taken from cudaMallocAsync's pool
	double *scratch = nullptr;
	size_t bytes = sizeof(double) * (2 * maxblk + 2 * n) + 64;
	SP_CUDA(ctx, cudaMallocAsync((void **)&scratch, bytes, s));
	unsigned int *cnt = (unsigned int *)(scratch + 2 * maxblk + 2 * n);
	SP_CUDA(ctx, cudaMemsetAsync(cnt, 0, 16, s));
	for (int k = 0; k < n; k++) {
		const MgProblem &q = probs[k];
		unsigned nb = (unsigned)(((size_t)q.w * q.h + 255) / 256);
		if (q.kind == 0) {
			k_dense_resid<0><<<nb, 256, 0, s>>>(u[k], q.g, q.f, q.w, q.h, scratch, cnt, scratch + 2 * maxblk + 2 * k); ctx->launches++;
		}
		else {
			k_dense_resid<1><<<nb, 256, 0, s>>>(u[k], q.g, q.f, q.w, q.h, scratch, cnt, scratch + 2 * maxblk + 2 * k); ctx->launches++;
		}
	}
	SP_LAUNCH_CHECK(ctx);
	std::vector<double> h(2 * n);
	SP_CUDA(ctx, cudaMemcpyAsync(h.data(), scratch + 2 * maxblk, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaFreeAsync(scratch, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	for (int k = 0; k < n; k++) {
		bnorm[k] = sqrt(h[2 * k + 1]);
		rel[k] = h[2 * k + 1] > 0 ? sqrt(h[2 * k] / h[2 * k + 1]) : (h[2 * k] > 0 ? INFINITY : 0.0);
	}
	return SIMPOIS_OK;
}
