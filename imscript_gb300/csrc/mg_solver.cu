// mg_solver.cu -- the converged schedule: batched multigrid-preconditioned
// conjugate gradient in FP32 inside an iterative refinement carried in
// float-float (5-point) or FP64 (13-point).
//
// Problem.  For every channel of every image, the unknowns U are the NaN
// pixels of g.  The system is the one the reference's CG solves
// (cleant_cgpois.c:197-264): A = -Laplacian (5-point, clamp-to-edge, kind 0,
// cleant_cgpois.c:67-89) or the 13-point bilaplacian with a single clamp
// (kind 1, cleant_cgpois.c:91-121), restricted to U, and b = -f_U - A_UK g_K.
//
// Refinement.  The solution of the unknowns lives in U (known pixels are read
// from g): float-float pairs (~48 bits) for the 5-point operator, FP64 for the
// 13-point one.  Each refinement step computes r = b - A u in that precision
// (the 5-point one in difference form) and its norm (the relative residual
// reported to the caller), stops when it is <= rtol, otherwise solves
// A d = (float)r and adds d.  FP64 issues at a small fraction of the FP32
// rate on this GPU, so it is spent only where float-float is not enough: the
// FP32 PCG's dot products sum their per-pixel terms as float-float pairs and
// go to double once per block; the first step (U = 0) needs no FP64 at all.
//
// Inner solve, 5-point (FP32).  Preconditioned CG; the preconditioner is one
// V(2,2)-cycle of geometric multigrid on the masked grid:
//   * level l+1 is ceil(w/2) x ceil(h/2); a coarse pixel is unknown iff all
//     its (existing) children are unknown, so that every coarse level keeps
//     the known pixels that make it non-singular;
//   * the coarse operators are the same clamped stencils on the coarse masks,
//     read through per-level cell codes (which neighbours are unknown, how
//     many sides are clamped);
//   * smoothing is red-black Gauss-Seidel, forward before the coarse
//     correction and backward after it, so the cycle is symmetric;
//   * restriction sums the children's residuals, prolongation injects the
//     coarse correction into the unknown children; the coarsest level
//     (<= 4 x 4) gets 4 symmetric sweeps.
// The fused cycle: k_pre5 / k_post5 take one 32 x 32 tile per block with a
// halo of 4 in shared memory (all sweeps of a level in one launch, the
// restriction or the injection fused in), k_coarse5 takes every level below
// the hand-over size of a problem in one block.  k_pre5 at level 0 also takes
// the PCG step (x, r), so an iteration is k_spmv5 and one V-cycle.  The SpMV
// is evaluated in difference form and the iterate carried as float-float, so
// that the FP32 recurrence's residual stays close to the true one.
//
// Inner solve, 13-point.  PCG with FP64 vectors and A p (an FP32 recurrence
// cannot resolve the biharmonic's smoothest modes), preconditioned by two
// fused 5-point V-cycles, with the flexible (Polak-Ribiere) beta since the
// FP32 preconditioner is only approximately symmetric.  Without the fused
// kernels (SIMPOIS_FLAG_UNFUSED), the one-launch-per-sweep cycle and FP32
// PCG serve both operators (5 colours and 4 sweeps for 13 points).
//
// Batching.  Each level keeps one list of 32 x 32 tiles that contain
// unknowns, over all problems of a call, problem after problem.  Every
// reduction is per problem and deterministic: each tile writes its partial
// sum, the last tile of a problem to finish (an atomic counter) sums the
// problem's partials in tile order and updates the problem's scalars.  A
// problem whose inner solve has converged skips every later launch (early
// retirement).  The problems are split into groups (contiguous ranges with
// about equal work); the solve is one CUDA graph in which every group is an
// independent branch with its own two nested device-driven WHILE loops
// (refinement steps, PCG iterations) over its slices of the tile lists, so
// one group's latency-bound coarse levels overlap another's fine ones.  The
// graph is captured once per plan (a new plan of the same topology updates it
// in place) and replayed; the small tables go up in one copy, and the tile
// lists of every level are written on the device from per-problem offsets.
//
// Launches.  The V-cycle kernels use programmatic dependent launch: each
// waits (griddepcontrol.wait) before its first dependent access and any early
// return, then releases the next kernel.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include <cudaTypedefs.h>   // CUtensorMap and the cuTensorMapEncodeTiled prototype

#include "common.cuh"
#include "solvers.h"

namespace {

constexpr int MAXLEV = 16;
constexpr int GMAX = 16;              // problem groups of a solve graph (the context's node tables)
constexpr int COARSE_MAX = 4;       // coarsest level: max(w, h) <= 4
constexpr int COARSE_SWEEPS = 4;    // symmetric sweeps on the coarsest level (<= 4 x 4)
constexpr int NU5 = 2;              // pre- and post-smoothing sweeps, 5-point
constexpr int NU13 = 4;             // pre- and post-smoothing sweeps, 13-point
constexpr int MAX_OUTER = 8;        // FP64 refinement steps
constexpr int INNER_MAX = 60;       // PCG iterations per refinement step (5-point)
constexpr int INNER_MAX13 = 600;    // the same for the FP64 13-point PCG
constexpr double TAU_MIN = 5e-7;    // FP32 inner solve: smallest relative decrease (measured: one refinement step fewer than 2e-6 on 2048^2 x 3)

struct LevelDev {
	int w, h;
	uint8_t *mask;   // 1 = unknown
	uint8_t *code;   // 5-point cell code (cell_code), levels below the coarsest
	// TMA tile maps of b (40 x 40 floats) and code (64 x 40 bytes) for the
	// tile kernels' region loads; null where the level's layout allows none
	const CUtensorMap *tmb, *tmc;
	float *b;        // right-hand side (level 0: the PCG residual r)
	float *z;        // correction (level 0: the preconditioned residual);
	                 // fused path: the pre-smoothed correction
	float *z2;       // fused path: the correction after the coarse
	                 // correction and post-smoothing (level 0: the PCG z)
};

struct ProbDev {
	int nlev, kind, w, h;
	int nfine;           // fused path: levels below this one use the tile
	                     // kernels; levels nfine.. are solved by k_coarse5
	const float *g;      // input channel
	const float *rhs;    // fill: f (sign -1) ; adjoint: grad_out (sign +1)
	float rhs_sign;
	int known_zero;      // adjoint: the known pixels hold 0 (fill: g)
	int vec4;            // w % 4 == 0 and g, out 16-byte aligned: setup and
	                     // finalize move 4-pixel groups with vector accesses
	float *out;
	double *U;           // the solution at the unknown pixels (the known ones
	                     // are read from g): FP64 for the 13-point operator,
	                     // float-float pairs (hi, lo) for the 5-point one (uff)
	float *x, *p, *q;    // level-0 PCG vectors
	float *xlo;          // x is carried as x + xlo (float-float): an FP32 x
	                     // alone cannot hold a solution much larger than the
	                     // right-hand side to the accuracy the residual needs
	float *p2;           // fused path: second search-direction buffer
	float *b_alt;        // fused path: the other level-0 residual buffer (k_pre5
	                     // writes the updated r there, k_rr5 swaps it with lv[0].b)
	const CUtensorMap *tmb_alt;   // the TMA map of b_alt (swapped with lv[0].tmb)
	double *r64, *p64, *p64b, *q64;   // 13-point: FP64 Krylov vectors (else null); p64 and p64b
	                                 // hold p_new of even and odd iterations
	double tau_min;            // FP32 inner solve: smallest relative decrease
	double rtol;
	LevelDev lv[MAXLEV];
	// k_coarse5's shared-memory layout of levels nfine.. (byte offsets of b,
	// z and the cell codes), planned on the host
	int coff_b[MAXLEV], coff_z[MAXLEV], coff_m[MAXLEV];
};

// The 5-point solution as float-float pairs: its refinement residual, the
// iterate update and the output then take no FP64 operation, which issues at
// a small fraction of the FP32 rate on this GPU; 48 bits hold the solution
// far below any residual the refinement is asked for.
__device__ __forceinline__ float2 *uff(const ProbDev &pr) { return reinterpret_cast<float2 *>(pr.U); }

// a - b for float-float values: the high parts' difference exact (TwoSum),
// the low parts' rounded once
__device__ __forceinline__ FF ff_sub(FF a, FF b)
{
	const FF s = ff_two_sum(a.hi, -b.hi);
	return ff_norm(s.hi, __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo)));
}

struct ProbState {
	double bnorm2, rho, alpha, beta, rr, tau2, rel, rel_first;
	float alpha_f, beta_f;   // (float)alpha and (float)beta, rounded once where they are set
	double cross;   // FP64 biharmonic PCG: r_new . z_old (flexible beta)
	int iter, total_iter, outer, inner_active, outer_active, status;
	int pending;    // fused 5-point PCG: alpha is set, x and r await their update
	unsigned int cnt;
	int max_iter;
	int nknown, nunknown;   // pixel counts of the channel
};

struct Globals {
	int inner_count;    // problems whose inner solve is running
	int outer_count;    // problems whose refinement is running
	int guard_inner;    // inner-loop bodies run since the loop started
	int guard_outer;    // refinement bodies run
	int n_inner;        // inner-loop bodies run in total (launch accounting)
	int n_outer;        // refinement bodies run in total
	int tma_timeout;    // a TMA region load did not complete in time
	int pad[25];
};
// read back into the first 256 bytes of the pinned staging, ahead of the
// states that follow them
static_assert(sizeof(Globals) <= 256, "Globals must fit the pinned read-back slot");

// ------------------------------------------------------------------ stencils

__constant__ int8_t c_di13[12] = {1, 0, -1, 0, 1, 1, -1, -1, 2, 0, -2, 0};
__constant__ int8_t c_dj13[12] = {0, 1, 0, -1, 1, -1, 1, -1, 0, 2, 0, -2};
__constant__ float c_cf13[12] = {-8, -8, -8, -8, 2, 2, 2, 2, 1, 1, 1, 1};

// num / diag for a Gauss-Seidel update.  The 5-point diagonals 4, 2 and 1 are
// powers of two: multiplying by their reciprocal is exact and gives the same
// float as the division, at a fraction of the instructions.
__device__ __forceinline__ float gs_div(float num, float diag)
{
	if (diag == 4.f) return num * 0.25f;
	if (diag == 2.f) return num * 0.5f;
	if (diag == 1.f) return num;
	return num / diag;
}

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

// The FP64 solution image at pixel q: U at the unknowns, the known value
// (g, or 0 for the adjoint) elsewhere.
__device__ __forceinline__ double known_at(const double *__restrict__ U, const uint8_t *__restrict__ m,
		const float *__restrict__ g, int known_zero, size_t q)
{
	return m[q] ? U[q] : (known_zero ? 0.0 : (double)g[q]);
}

// A u at (i, j) in FP64 on the full image (known pixels included, with the
// clamp-to-edge extension).
template <int K>
__device__ __forceinline__ double apply64(const double *__restrict__ U, const uint8_t *__restrict__ m,
		const float *__restrict__ g, int known_zero, int w, int h, int i, int j)
{
	auto at = [&](int a, int b) -> double {
		return known_at(U, m, g, known_zero, (size_t)clampi(b, h) * w + clampi(a, w));
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

// The 4-pixel row group a thread takes in the level-0 PCG updates (k_xr,
// k_rz and the fused kernels' PCG work): row tid / 8 of the tile, columns
// 4 (tid % 8) + 0..3; a thread adds its terms left to right.  Level-0 arrays
// live in the arena (256-byte aligned), so a full group of a level whose
// width is a multiple of 4 moves as one 16-byte access.
struct Grp {
	size_t k;   // first pixel
	int n;      // pixels of the group in the image (0..4)
	bool vec;   // one aligned 16-byte access
};

__device__ __forceinline__ Grp grp_of(int4 t, int w, int h)
{
	const int i = t.y * SP_TILE + 4 * (threadIdx.x & 7), j = t.z * SP_TILE + (threadIdx.x >> 3);
	Grp g;
	g.n = (i < w && j < h) ? min(4, w - i) : 0;
	g.k = g.n ? (size_t)j * w + i : 0;
	g.vec = g.n == 4 && (w & 3) == 0;
	return g;
}

__device__ __forceinline__ void ld4(const float *p, const Grp &g, float v[4])
{
	if (g.vec) {
		const float4 q = *(const float4 *)(p + g.k);
		v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
	} else {
#pragma unroll
		for (int e = 0; e < 4; e++) v[e] = e < g.n ? p[g.k + e] : 0.f;
	}
}

__device__ __forceinline__ void ldm4(const uint8_t *p, const Grp &g, uint8_t v[4])
{
	if (g.vec) {
		const uchar4 q = *(const uchar4 *)(p + g.k);
		v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
	} else {
#pragma unroll
		for (int e = 0; e < 4; e++) v[e] = e < g.n ? p[g.k + e] : 0;
	}
}

__device__ __forceinline__ void st4(float *p, const Grp &g, const float v[4])
{
	if (g.vec) {
		*(float4 *)(p + g.k) = make_float4(v[0], v[1], v[2], v[3]);
	} else {
#pragma unroll
		for (int e = 0; e < 4; e++)
			if (e < g.n) p[g.k + e] = v[e];
	}
}

// A 4-cell row group of a shared-memory region (first column gi a multiple of
// 4): the number of its cells inside the w x h level (0..4) and the loads of
// its cells -- one 16-byte (4-byte) access when the level's rows keep that
// alignment (vec: w a multiple of 4, where a group is wholly in or out), else
// one access per cell in the image.  Cells outside read 0.
__device__ __forceinline__ int group_cells(int gi, int gj, int w, int h)
{
	return (gi >= 0 && gi < w && gj >= 0 && gj < h) ? min(4, w - gi) : 0;
}

__device__ __forceinline__ float4 gload4(const float *p, size_t k, int n, bool vec)
{
	float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
	if (vec) {
		if (n) v = *(const float4 *)(p + k);
	} else {
		if (n > 0) v.x = p[k];
		if (n > 1) v.y = p[k + 1];
		if (n > 2) v.z = p[k + 2];
		if (n > 3) v.w = p[k + 3];
	}
	return v;
}

__device__ __forceinline__ uint32_t gload4u8(const uint8_t *p, size_t k, int n, bool vec)
{
	if (vec) return n ? *(const uint32_t *)(p + k) : 0u;
	uint32_t v = 0;
	if (n > 0) v |= p[k];
	if (n > 1) v |= (uint32_t)p[k + 1] << 8;
	if (n > 2) v |= (uint32_t)p[k + 2] << 16;
	if (n > 3) v |= (uint32_t)p[k + 3] << 24;
	return v;
}

__device__ __forceinline__ void gstore4(float *p, size_t k, int n, bool vec, float4 v)
{
	if (vec) {
		if (n) *(float4 *)(p + k) = v;
	} else {
		if (n > 0) p[k] = v.x;
		if (n > 1) p[k + 1] = v.y;
		if (n > 2) p[k + 2] = v.z;
		if (n > 3) p[k + 3] = v.w;
	}
}

// Per-problem deterministic reduction of two float-float values over the
// level-0 tiles of the problem.  Returns true in the last tile's block (all
// threads); the sums are then in tot[0..1] (thread 0).
__device__ bool problem_sum2_ff(FF v0, FF v1, int prob, const int *__restrict__ tbeg,
		const int *__restrict__ tcnt, double *partial, ProbState *st, double *tot, double *sh)
{
	__shared__ bool am_last;
	double s0 = block_sum_ff<SP_THREADS>(v0, sh);
	double s1 = block_sum_ff<SP_THREADS>(v1, sh);
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

// problem_sum2_ff for a single value whose block sum s0 thread 0 holds.
__device__ bool problem_sum1_block(double s0, int prob, const int *__restrict__ tbeg, const int *__restrict__ tcnt,
		double *partial, ProbState *st, double *tot, double *sh)
{
	__shared__ bool am_last;
	if (threadIdx.x == 0) {
		partial[2 * blockIdx.x] = s0;
		__threadfence();
		unsigned prev = atomicAdd(&st[prob].cnt, 1u);
		am_last = prev == (unsigned)tcnt[prob] - 1;
	}
	__syncthreads();
	if (!am_last) return false;
	__threadfence();
	double a0 = 0;
	const int b0 = tbeg[prob], n = tcnt[prob];
	for (int k = threadIdx.x; k < n; k += SP_THREADS) a0 += __ldcg(partial + 2 * (b0 + k));
	a0 = block_sum<SP_THREADS>(a0, sh);
	if (threadIdx.x == 0) {
		tot[0] = a0;
		tot[1] = 0;
		st[prob].cnt = 0;
	}
	return true;
}

__device__ bool problem_sum1(double v0, int prob, const int *__restrict__ tbeg, const int *__restrict__ tcnt,
		double *partial, ProbState *st, double *tot, double *sh)
{
	return problem_sum1_block(block_sum<SP_THREADS>(v0, sh), prob, tbeg, tcnt, partial, st, tot, sh);
}

// problem_sum1 of float-float per-thread terms (the FP32 PCG's dot products)
__device__ bool problem_sum1_ff(FF v0, int prob, const int *__restrict__ tbeg, const int *__restrict__ tcnt,
		double *partial, ProbState *st, double *tot, double *sh)
{
	return problem_sum1_block(block_sum_ff<SP_THREADS>(v0, sh), prob, tbeg, tcnt, partial, st, tot, sh);
}

// ------------------------------------------------------------------ setup kernels

// Tiles per block of the passes over every tile (setup, finalize): each
// thread takes a 4-pixel row group of each of its block's tiles, and every
// load is issued before the first store.
constexpr int TPB = 4;

// The row group of tile t a thread covers: first pixel k and its pixel count
// (0 when the group lies outside the image).
__device__ __forceinline__ int group_of(const ProbDev &pr, int4 t, size_t &k)
{
	const int i = t.y * SP_TILE + 4 * (threadIdx.x & 7), j = t.z * SP_TILE + (threadIdx.x >> 3);
	if (i >= pr.w || j >= pr.h) return 0;
	k = (size_t)j * pr.w + i;
	return min(4, pr.w - i);
}

// The tile lists of every level, problem after problem, tiles in row order:
// entry e of level l (lbeg[l] <= e < lbeg[l + 1]) is tile e - lbeg[l] - off[k]
// of the last problem k whose first entry off[k] (loff, n + 1 per level) is at
// or below it (problems without the level share the next one's offset).
__global__ void k_fill_lists(const ProbDev *__restrict__ P, int n, int nlev, const int *__restrict__ lbeg,
		const int *__restrict__ loff, int4 *__restrict__ lists)
{
	const int total = lbeg[nlev];
	for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
		int l = 0;
		while (lbeg[l + 1] <= e) l++;
		const int *o = loff + (size_t)l * (n + 1);
		const int r = e - lbeg[l];
		int lo = 0, hi = n - 1;
		while (lo < hi) {
			const int mid = (lo + hi + 1) >> 1;
			if (o[mid] <= r) lo = mid;
			else hi = mid - 1;
		}
		const int t = r - o[lo], tw = (P[lo].lv[l].w + SP_TILE - 1) / SP_TILE;
		lists[e] = make_int4(lo, t % tw, t / tw, 0);
	}
}

// Level 0 over all tiles: mask = isnan(g); U = 0 at the unknowns; flag =
// tile holds an unknown; per-problem pixel counts.
__global__ void __launch_bounds__(SP_THREADS) k_setup0(const ProbDev *__restrict__ P, ProbState *st,
		const int4 *__restrict__ all, int nall, int *__restrict__ flag)
{
	__shared__ int cnt[TPB][2];
	if (threadIdx.x < 2 * TPB) cnt[threadIdx.x >> 1][threadIdx.x & 1] = 0;
	int4 tt[TPB];
	size_t kk[TPB];
	int nv[TPB];
	float gv[TPB][4];
#pragma unroll
	for (int q = 0; q < TPB; q++) {
		const int b = blockIdx.x * TPB + q;
		tt[q] = b < nall ? all[b] : make_int4(-1, 0, 0, 0);
	}
#pragma unroll
	for (int q = 0; q < TPB; q++) {
		nv[q] = 0;
		kk[q] = 0;
		if (tt[q].x < 0) continue;
		const ProbDev &pr = P[tt[q].x];
		nv[q] = group_of(pr, tt[q], kk[q]);
		if (nv[q] == 4 && pr.vec4) {
			const float4 v = *(const float4 *)(pr.g + kk[q]);
			gv[q][0] = v.x; gv[q][1] = v.y; gv[q][2] = v.z; gv[q][3] = v.w;
		} else {
#pragma unroll
			for (int e = 0; e < 4; e++) gv[q][e] = e < nv[q] ? pr.g[kk[q] + e] : 0.f;
		}
	}
	__syncthreads();   // cnt is zeroed
#pragma unroll
	for (int q = 0; q < TPB; q++) {
		int nu = 0, nk = 0;
		if (nv[q]) {
			const ProbDev &pr = P[tt[q].x];
			uint32_t mw = 0;
#pragma unroll
			for (int e = 0; e < 4; e++) {
				if (e >= nv[q]) break;
				const bool u = isnan(gv[q][e]);
				nu += u;
				nk += !u;
				if (u) pr.U[kk[q] + e] = 0.0;   // known pixels: read from g when needed
				mw |= (uint32_t)u << (8 * e);
			}
			if (nv[q] == 4 && (pr.w & 3) == 0) {   // the mask lives in the arena
				*(uint32_t *)(pr.lv[0].mask + kk[q]) = mw;
			} else {
				for (int e = 0; e < nv[q]; e++) pr.lv[0].mask[kk[q] + e] = (mw >> (8 * e)) & 1u;
			}
		}
		for (int o = 16; o > 0; o >>= 1) {
			nu += __shfl_down_sync(0xffffffffu, nu, o);
			nk += __shfl_down_sync(0xffffffffu, nk, o);
		}
		if ((threadIdx.x & 31) == 0 && (nu || nk)) {
			atomicAdd(&cnt[q][0], nu);
			atomicAdd(&cnt[q][1], nk);
		}
	}
	__syncthreads();
	if (threadIdx.x < TPB) {
		const int q = threadIdx.x, b = blockIdx.x * TPB + q;
		if (b < nall) {
			flag[b] = cnt[q][0] > 0;
			if (cnt[q][0]) atomicAdd(&st[tt[q].x].nunknown, cnt[q][0]);
			if (cnt[q][1]) atomicAdd(&st[tt[q].x].nknown, cnt[q][1]);
		}
	}
}

// Cell code of a 5-point cell: bit 0 unknown; bits 1-4 the E, W, S, N
// neighbour is in the image and unknown; bits 5-7 the number of clamped sides
// (the diagonal is 4 minus it).  0 for a known cell.
__device__ __forceinline__ uint8_t cell_code(const uint8_t *m, int i, int j, int w, int h)
{
	const size_t k = (size_t)j * w + i;
	if (!m[k]) return 0;
	int code = 1, nd = 0;
	if (i + 1 < w) { if (m[k + 1]) code |= 2; } else nd++;
	if (i > 0)     { if (m[k - 1]) code |= 4; } else nd++;
	if (j + 1 < h) { if (m[k + w]) code |= 8; } else nd++;
	if (j > 0)     { if (m[k - w]) code |= 16; } else nd++;
	return (uint8_t)(code | (nd << 5));
}

// Cell codes of the 4 cells (fi..fi+3, fj) of a level whose width is a
// multiple of 4: 3 word loads and 2 byte loads for 4 codes.
__device__ __forceinline__ void codes4(const LevelDev &F, int fi, int fj)
{
	const size_t k = (size_t)fj * F.w + fi;
	const uint32_t mc = *(const uint32_t *)(F.mask + k);
	const uint32_t mn = fj > 0 ? *(const uint32_t *)(F.mask + k - F.w) : 0u;
	const uint32_t ms = fj + 1 < F.h ? *(const uint32_t *)(F.mask + k + F.w) : 0u;
	const uint32_t ml = fi > 0 ? F.mask[k - 1] : 0u, mr = fi + 4 < F.w ? F.mask[k + 4] : 0u;
	uint32_t out = 0;
#pragma unroll
	for (int e = 0; e < 4; e++) {
		if (!((mc >> (8 * e)) & 1u)) continue;
		uint32_t code = 1, nd = 0;
		if (e < 3) { if ((mc >> (8 * e + 8)) & 1u) code |= 2; }
		else if (fi + 4 < F.w) { if (mr) code |= 2; }
		else nd++;
		if (e > 0) { if ((mc >> (8 * e - 8)) & 1u) code |= 4; }
		else if (fi > 0) { if (ml) code |= 4; }
		else nd++;
		if (fj + 1 < F.h) { if ((ms >> (8 * e)) & 1u) code |= 8; } else nd++;
		if (fj > 0) { if ((mn >> (8 * e)) & 1u) code |= 16; } else nd++;
		out |= (code | (nd << 5)) << (8 * e);
	}
	*(uint32_t *)(F.code + k) = out;
}

// The PCG operator A p at a cell in difference form: p_c per known in-image
// neighbour plus (p_c - p_n) per unknown in-image neighbour, in the order E,
// W, S, N.  Mathematically diag * p_c + off; the differences of neighbouring
// values are exact, so there is no cancellation of 4 p_c against its
// neighbours where p is much larger than A p (smooth iterates of large holes),
// which keeps the FP32 recurrence's residual close to the true one.
__device__ __forceinline__ float a5_diff(float pc, float pe, float pw, float ps, float pn, int code)
{
	const int nunk = ((code >> 1) & 1) + ((code >> 2) & 1) + ((code >> 3) & 1) + ((code >> 4) & 1);
	float q = __fmul_rn((float)(4 - (code >> 5) - nunk), pc);
	if (code & 2) q = __fadd_rn(q, __fsub_rn(pc, pe));
	if (code & 4) q = __fadd_rn(q, __fsub_rn(pc, pw));
	if (code & 8) q = __fadd_rn(q, __fsub_rn(pc, ps));
	if (code & 16) q = __fadd_rn(q, __fsub_rn(pc, pn));
	return q;
}

// Level l >= 1 over all tiles: unknown iff every existing child is unknown;
// also the cell codes of level l-1 (when l-1 >= 1).
__global__ void k_mask_down(const ProbDev *__restrict__ P, const int4 *__restrict__ all, int l, int *__restrict__ flag)
{
	__shared__ int any;
	int4 t = all[blockIdx.x];
	const ProbDev &pr = P[t.x];
	const LevelDev &C = pr.lv[l], &F = pr.lv[l - 1];
	if (threadIdx.x == 0) any = 0;
	__syncthreads();
	int mine = 0;
	if ((F.w & 7) == 0) {
		// a row group of 4 coarse cells: its children are 8 bytes of each of
		// two fine rows (aligned: F.w and 2 i are multiples of 8)
		const Grp g = grp_of(t, C.w, C.h);
		if (g.n) {
			const int i = t.y * SP_TILE + 4 * (threadIdx.x & 7), j = t.z * SP_TILE + (threadIdx.x >> 3);
			const uint8_t *f0 = F.mask + (size_t)(2 * j) * F.w + 2 * i;
			const unsigned long long r0 = *(const unsigned long long *)f0;
			const unsigned long long r1 = 2 * j + 1 < F.h ? *(const unsigned long long *)(f0 + F.w) : r0;
			const unsigned long long both = r0 & r1;   // masks are 0 or 1
			uint32_t out = 0;
#pragma unroll
			for (int e = 0; e < 4; e++) {
				const uint32_t u = (uint32_t)((both >> (16 * e)) & (both >> (16 * e + 8)) & 1ull);
				out |= u << (8 * e);
			}
			*(uint32_t *)(C.mask + g.k) = out;
			mine = out != 0;
		}
	} else {
		int i = tile_i(t);
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
	}
	if (__any_sync(0xffffffffu, mine) && (threadIdx.x & 31) == 0) atomicOr(&any, 1);
	__syncthreads();
	if (threadIdx.x == 0) flag[blockIdx.x] = any;
	// the mask of level l-1 >= 1 is complete: its cell codes under this tile
	// (level 0 has its own pass, k_codes0)
	if (l - 1 < 1) return;
	if ((F.w & 3) == 0) {
		for (int q = threadIdx.x; q < SP_TILE * SP_TILE; q += SP_THREADS) {
			const int fi = 2 * SP_TILE * t.y + 4 * (q & (SP_TILE / 2 - 1)), fj = 2 * SP_TILE * t.z + q / (SP_TILE / 2);
			if (fi < F.w && fj < F.h) codes4(F, fi, fj);
		}
	} else {
		for (int q = threadIdx.x; q < 4 * SP_TILE * SP_TILE; q += SP_THREADS) {
			const int fi = 2 * SP_TILE * t.y + (q & (2 * SP_TILE - 1)), fj = 2 * SP_TILE * t.z + q / (2 * SP_TILE);
			if (fi < F.w && fj < F.h) F.code[(size_t)fj * F.w + fi] = cell_code(F.mask, fi, fj, F.w, F.h);
		}
	}
}

// Cell codes of level 0 over all tiles (TPB per block), once its mask is
// complete: every problem has them, even one of a single level.
__global__ void __launch_bounds__(SP_THREADS) k_codes0(const ProbDev *__restrict__ P, const int4 *__restrict__ all,
		int nall)
{
#pragma unroll
	for (int q = 0; q < TPB; q++) {
		const int b = blockIdx.x * TPB + q;
		if (b >= nall) return;
		const int4 t = all[b];
		const LevelDev &F = P[t.x].lv[0];
		if ((F.w & 3) == 0) {
			const int fi = t.y * SP_TILE + 4 * (threadIdx.x & 7), fj = t.z * SP_TILE + (threadIdx.x >> 3);
			if (fi < F.w && fj < F.h) codes4(F, fi, fj);
		} else {
			const int fi = t.y * SP_TILE + (threadIdx.x & 31);
			for (int r = 0; r < SP_ROWS; r++) {
				const int fj = t.z * SP_TILE + (threadIdx.x >> 5) + SP_BLOCK_Y * r;
				if (fi < F.w && fj < F.h) F.code[(size_t)fj * F.w + fi] = cell_code(F.mask, fi, fj, F.w, F.h);
			}
		}
	}
}

// One block per level: ordered compaction of the level's tile list by flag.
// For level 0 also the per-problem tile ranges (tbeg, tcnt).
__global__ void k_compact(const int4 *const *__restrict__ all, const int *const *__restrict__ flag,
		const int *__restrict__ nall, int4 *const *__restrict__ act, int *__restrict__ nact,
		int *__restrict__ tbeg, int *__restrict__ tcnt, int *__restrict__ pcnt, int nprob)
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
			atomicAdd(pcnt + (size_t)l * nprob + t.x, 1);   // active tiles per level and problem
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

// The end of a refinement residual pass: |r|^2 summed over the problem's
// tiles; the problem's last tile decides: converged, or start an inner solve.
__device__ void resid_finish(FF rr, bool first, const ProbDev &pr, int prob, ProbState *st,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial, Globals *gl, double *sh)
{
	double tot[2];
	if (problem_sum1_ff(rr, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		if (first) s.bnorm2 = tot[0];
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
			atomicSub(&gl->outer_count, 1);
		} else {
			s.outer += 1;
			s.iter = 0;
			s.inner_active = 1;
			// an FP32 inner solve stalls near TAU_MIN; the FP64 one goes to rtol
			double tau = pr.r64 ? 0.5 * pr.rtol / rel : fmax(0.3 * pr.rtol / rel, pr.tau_min);
			s.tau2 = tau * tau * tot[0];
			s.rho = 0;
			s.beta = 0;
			s.beta_f = (float)s.beta;
			s.pending = 0;
			atomicAdd(&gl->inner_count, 1);
		}
	}
}

// The 5-point refinement residual, one tile per block: the solution's values on
// the tile and a 1-pixel halo go to shared memory first, as float-float pairs
// (U at the unknowns -- 0 on the first step, before any solve --, the known
// value, or 0 for the adjoint; nothing outside the image), so each pixel reads
// its neighbours there instead of testing and loading each from global
// memory.  Per unknown, in difference form: r = s + sum over the in-image
// neighbours (E, S, W, N) of (u_n - u_c); b0 = (float) r, x = xlo = 0.
__global__ void __launch_bounds__(SP_THREADS, 8) k_resid5(const ProbDev *__restrict__ P, ProbState *st,
		const int4 *__restrict__ tl, const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial,
		Globals *gl)
{
	constexpr int RW = SP_TILE + 2, RN = RW * RW;   // region: 34 x 34
	constexpr int NIT = (RN + SP_THREADS - 1) / SP_THREADS;
	__shared__ float2 sv[RN];
	__shared__ uint8_t sm[RN];
	__shared__ double sh[32];
	const int4 t = tl[blockIdx.x];
	const int prob = t.x;
	if (!st[prob].outer_active) return;
	// the first refinement step also forms ||b||; every block of the problem
	// reads `outer` before the problem's last block changes it
	const bool first = st[prob].outer == 0;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	const int w = pr.w, h = pr.h, x0 = t.y * SP_TILE - 1, y0 = t.z * SP_TILE - 1;
	const float2 *U2 = uff(pr);
	// every mask byte of the thread's region cells first, then every value:
	// two round trips to memory, not two per cell
	size_t qv[NIT];
	uint8_t mv[NIT];
#pragma unroll
	for (int it = 0; it < NIT; it++) {
		const int c = threadIdx.x + it * SP_THREADS;
		const int ry = c / RW, rx = c - ry * RW, gi = x0 + rx, gj = y0 + ry;
		const bool in = c < RN && gi >= 0 && gi < w && gj >= 0 && gj < h;
		qv[it] = in ? (size_t)gj * w + gi : 0;
		mv[it] = in ? (uint8_t)(L.mask[qv[it]] ? 1 : 2) : 0;   // 1 unknown, 2 known, 0 outside
	}
#pragma unroll
	for (int it = 0; it < NIT; it++) {
		const int c = threadIdx.x + it * SP_THREADS;
		float2 v = make_float2(0.f, 0.f);
		if (mv[it] == 1 && !first) v = U2[qv[it]];
		else if (mv[it] == 2 && !pr.known_zero) v.x = pr.g[qv[it]];
		if (c < RN) {
			sv[c] = v;
			sm[c] = mv[it] == 1;
		}
	}
	__syncthreads();
	const int i = tile_i(t);
	FF rr = {0.f, 0.f};   // |r|^2 from the float r
#pragma unroll
	for (int r = 0; r < SP_ROWS; r++) {
		const int j = tile_j(t, r);
		if (i >= w || j >= h) continue;
		const size_t k = (size_t)j * w + i;
		const int c = (j - y0) * RW + (i - x0);
		if (!sm[c]) continue;
		const FF uc = {sv[c].x, sv[c].y};
		FF acc = {0.f, 0.f};
		if (i + 1 < w) acc = ff_add(acc, ff_sub(FF{sv[c + 1].x, sv[c + 1].y}, uc));
		if (j + 1 < h) acc = ff_add(acc, ff_sub(FF{sv[c + RW].x, sv[c + RW].y}, uc));
		if (i > 0) acc = ff_add(acc, ff_sub(FF{sv[c - 1].x, sv[c - 1].y}, uc));
		if (j > 0) acc = ff_add(acc, ff_sub(FF{sv[c - RW].x, sv[c - RW].y}, uc));
		const FF rv = ff_add(FF{pr.rhs ? pr.rhs_sign * pr.rhs[k] : 0.f, 0.f}, acc);   // exact sign flip
		const float rf = rv.hi;   // normalised: hi is the float nearest hi + lo
		L.b[k] = rf;
		pr.x[k] = 0.f;
		pr.xlo[k] = 0.f;
		ff_add_prod(rr, rf, rf);
	}
	resid_finish(rr, first, pr, prob, st, tbeg, tcnt, partial, gl, sh);
}

// r = rhs_sign*rhs - A U (FP64) at the unknowns; b0 = (float)r; x = 0 (the
// biharmonic PCG: r64 = r and b0).
// The last tile of a problem decides: converged, or start an inner solve.
template <int K>
__global__ void k_resid64(const ProbDev *__restrict__ P, ProbState *st, const int4 *__restrict__ tl,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial,
		Globals *gl)
{
	__shared__ double sh[32];
	int4 t = tl[blockIdx.x];
	const int prob = t.x;
	if (!st[prob].outer_active) return;
	// the first refinement step also forms ||b||; every block of the problem
	// reads `outer` before the problem's last block changes it
	const bool first = st[prob].outer == 0;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	const int i = tile_i(t), w = pr.w, h = pr.h;
	FF rr = {0.f, 0.f};   // |r|^2 from the float r (FP64 issues at 1/70 rate)
	// U is 0 at every unknown until the first refinement step adds to it, so
	// there b = rhs - A_UK g_K is exactly this residual: ||b|| = ||r||.
#pragma unroll
	for (int r = 0; r < SP_ROWS; r++) {
		const int j = tile_j(t, r);
		const bool in = i < w && j < h;
		const size_t k = in ? (size_t)j * w + i : 0;
		const uint8_t m = in ? L.mask[k] : 0;
		double rk = 0;
		if (first) {
			// U is 0 at every unknown: r = rhs_sign*rhs - A_UK g_K, the known
			// neighbours' weighted values (exact products of small integer
			// weights and floats) summed in float-float -- no FP64 operation,
			// which issues at a small fraction of the FP32 rate on this GPU,
			// until U holds a solution
			if (m) {
				FF acc = {pr.rhs ? pr.rhs_sign * pr.rhs[k] : 0.f, 0.f};   // exact sign flip
				if (!pr.known_zero) {
					if (K == 0) {
						const int qi[4] = {i + 1 < w ? i + 1 : i, i, i > 0 ? i - 1 : i, i};
						const int qj[4] = {j, j + 1 < h ? j + 1 : j, j, j > 0 ? j - 1 : j};
#pragma unroll
						for (int e = 0; e < 4; e++) {
							const size_t q = (size_t)qj[e] * w + qi[e];
							if (!L.mask[q]) acc = ff_add(acc, FF{pr.g[q], 0.f});
						}
					} else {
#pragma unroll
						for (int e = 0; e < 12; e++) {
							const size_t q = (size_t)clampi(j + c_dj13[e], h) * w + clampi(i + c_di13[e], w);
							if (!L.mask[q]) ff_add_prod(acc, -c_cf13[e], pr.g[q]);
						}
					}
				}
				const float rf = acc.hi;   // acc is normalised: hi is the float nearest hi + lo
				if (pr.r64) {
					pr.r64[k] = (double)acc.hi + (double)acc.lo;
					L.b[k] = rf;
					pr.x[k] = rf;
				} else {
					L.b[k] = rf;
					pr.x[k] = 0.f;
					pr.xlo[k] = 0.f;
				}
				ff_add_prod(rr, rf, rf);
			}
			continue;
		}
		if (K == 0 && m) {
			// float-float, in difference form: r = s + sum over the in-image
			// neighbours of (u_n - u_c) (a neighbour clamped onto the pixel
			// adds 0), u_n the solution or the known value
			const float2 *U2 = uff(pr);
			const FF uc = {U2[k].x, U2[k].y};
			const int qi[4] = {i + 1 < w ? i + 1 : i, i, i > 0 ? i - 1 : i, i};
			const int qj[4] = {j, j + 1 < h ? j + 1 : j, j, j > 0 ? j - 1 : j};
			FF acc = {0.f, 0.f};
#pragma unroll
			for (int e = 0; e < 4; e++) {
				const size_t q = (size_t)qj[e] * w + qi[e];
				if (q == k) continue;
				FF un = {0.f, 0.f};
				if (L.mask[q]) {
					const float2 v = U2[q];
					un = FF{v.x, v.y};
				} else if (!pr.known_zero) {
					un = FF{pr.g[q], 0.f};
				}
				acc = ff_add(acc, ff_sub(un, uc));
			}
			const FF r = ff_add(FF{pr.rhs ? pr.rhs_sign * pr.rhs[k] : 0.f, 0.f}, acc);   // exact sign flip
			const float rf = r.hi;
			L.b[k] = rf;
			pr.x[k] = 0.f;
			pr.xlo[k] = 0.f;
			ff_add_prod(rr, rf, rf);
			continue;
		} else if (m) {
			const double s = pr.rhs ? (double)(pr.rhs_sign * pr.rhs[k]) : 0.0;
			rk = s - apply64<K>(pr.U, L.mask, pr.g, pr.known_zero, w, h, i, j);
		}
		if (m) {
			const float rf = (float)rk;
			if (pr.r64) {
				pr.r64[k] = rk;     // the FP64 PCG starts from this residual
				L.b[k] = rf;        // and the first V-cycle from its float copy,
				pr.x[k] = rf;       // which r . z reads from x (unused by this PCG)
			} else {
				L.b[k] = rf;
				pr.x[k] = 0.f;
				pr.xlo[k] = 0.f;
			}
			ff_add_prod(rr, rf, rf);
		}
	}
	resid_finish(rr, first, pr, prob, st, tbeg, tcnt, partial, gl, sh);
}

// After compaction: a problem without unknowns is finished before it starts;
// outer_count = the problems that have an unknown.
__global__ void k_init_counts(ProbState *st, const int *__restrict__ tcnt, int n, Globals *gl)
{
	__shared__ int cnt;
	if (threadIdx.x == 0) cnt = 0;
	__syncthreads();
	for (int p = threadIdx.x; p < n; p += blockDim.x) {
		if (tcnt[p] > 0)
			atomicAdd(&cnt, 1);
		else
			st[p].outer_active = 0;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		gl->outer_count = cnt;
		gl->inner_count = 0;
		gl->guard_outer = 0;
		gl->guard_inner = 0;
		gl->n_inner = 0;
		gl->n_outer = 0;
	}
}

// Condition of a device-side WHILE loop: continue while problems are still
// running (count > 0) and the loop has run fewer than gmax bodies.  `reset`
// marks the evaluation before the loop's first body.
__global__ void k_setcond(cudaGraphConditionalHandle h, Globals *gl, int outer, int reset, int gmax)
{
	if (threadIdx.x != 0) return;
	int *guard = outer ? &gl->guard_outer : &gl->guard_inner;
	const int count = outer ? gl->outer_count : gl->inner_count;
	if (reset) {
		*guard = 0;
	} else {
		*guard += 1;
		if (outer) gl->n_outer += 1; else gl->n_inner += 1;
	}
	cudaGraphSetConditional(h, (count > 0 && *guard < gmax) ? 1u : 0u);
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
			if (!pr.lv[0].mask[k]) continue;
			if (pr.kind == 0) {
				float2 &u = uff(pr)[k];
				const FF v = ff_add(FF{u.x, u.y}, FF{pr.x[k], pr.xlo[k]});
				u = make_float2(v.hi, v.lo);
			} else {
				pr.U[k] += (double)pr.x[k] + (double)pr.xlo[k];
			}
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
	const float beta = st[t.x].beta_f;
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
	FF pq = {0.f, 0.f};
	if (K == 0) {
		// k_spmv5's order: the 4 cells of a row group per thread, in row order
		const Grp g = grp_of(t, pr.w, pr.h);
		for (int e = 0; e < g.n; e++) {
			const size_t k = g.k + e;
			if (L.mask[k]) {
				const int code = L.code[k];
				const float *p = pr.p;
				const float pk = p[k];
				const float qk = a5_diff(pk, (code & 2) ? p[k + 1] : 0.f, (code & 4) ? p[k - 1] : 0.f,
						(code & 8) ? p[k + pr.w] : 0.f, (code & 16) ? p[k - pr.w] : 0.f, code);
				pr.q[k] = qk;
				ff_add_prod(pq, pk, qk);
			}
		}
	} else {
		int i = tile_i(t);
		for (int r = 0; r < SP_ROWS; r++) {
			int j = tile_j(t, r);
			if (i < pr.w && j < pr.h) {
				size_t k = (size_t)j * pr.w + i;
				if (L.mask[k]) {
					float pk = pr.p[k], qk;
					if (K == 0) {
						const int code = L.code[k];
						const float *p = pr.p;
						qk = a5_diff(pk, (code & 2) ? p[k + 1] : 0.f, (code & 4) ? p[k - 1] : 0.f,
								(code & 8) ? p[k + pr.w] : 0.f, (code & 16) ? p[k - pr.w] : 0.f, code);
					} else {
						float d, o;
						split<K>(L, pr.p, i, j, d, o);
						qk = d * pk + o;
					}
					pr.q[k] = qk;
					ff_add_prod(pq, pk, qk);
				}
			}
		}
	}
	double tot[2];
	if (problem_sum1_ff(pq, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		double a = s.rho / tot[0];
		if (!(tot[0] > 0) || !isfinite(a)) {
			s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			s.alpha = 0;
			s.alpha_f = (float)s.alpha;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.alpha = a;
			s.alpha_f = (float)s.alpha;
		}
	}
}

// x += alpha p; r -= alpha q; r.r; the inner stopping test
__global__ void __launch_bounds__(SP_THREADS) k_xr(const ProbDev *__restrict__ P, ProbState *st, const int4 *__restrict__ tl,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial, Globals *gl,
		int use_p2)
{
	__shared__ double sh[32];
	int4 t = tl[blockIdx.x];
	const int prob = t.x;
	if (!st[prob].inner_active) return;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	const float a = st[prob].alpha_f;
	const float *pv = use_p2 ? pr.p2 : pr.p;
	FF rr = {0.f, 0.f};
	const Grp g = grp_of(t, pr.w, pr.h);
	if (g.n) {
		uint8_t m[4];
		float xv[4], xl[4], pk[4], bk[4], qk[4];
		ldm4(L.mask, g, m);
		ld4(pr.x, g, xv);
		ld4(pr.xlo, g, xl);
		ld4(pv, g, pk);
		ld4(L.b, g, bk);
		ld4(pr.q, g, qk);
#pragma unroll
		for (int e = 0; e < 4; e++) {
			if (!m[e]) continue;   // known pixels are written back unchanged
			FF xn = {xv[e], xl[e]};
			ff_add_prod(xn, a, pk[e]);
			xv[e] = xn.hi;
			xl[e] = xn.lo;
			bk[e] = __fmaf_rn(-a, qk[e], bk[e]);
			ff_add_prod(rr, bk[e], bk[e]);
		}
		st4(pr.x, g, xv);
		st4(pr.xlo, g, xl);
		st4(L.b, g, bk);
	}
	double tot[2];
	if (problem_sum1_ff(rr, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
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
	FF rz = {0.f, 0.f};
	const Grp g = grp_of(t, pr.w, pr.h);
	if (g.n) {
		uint8_t m[4];
		float bv[4], zv[4];
		ldm4(L.mask, g, m);
		ld4(L.b, g, bv);
		ld4(L.z, g, zv);
#pragma unroll
		for (int e = 0; e < 4; e++)
			if (m[e]) ff_add_prod(rz, bv[e], zv[e]);
	}
	double tot[2];
	if (problem_sum1_ff(rz, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		if (!(tot[0] > 0) || !isfinite(tot[0])) {
			// r = 0 exactly, or a preconditioner that is not positive here
			if (tot[0] != 0) s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.beta = s.rho > 0 ? tot[0] / s.rho : 0.0;
			s.beta_f = (float)s.beta;
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
				L.z[k] = gs_div(L.b[k] - o, d);
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
					z[k] = gs_div(b[k] - o, d);
				}
				__syncthreads();
			}
	if (k < n) L.z[k] = m[k] ? z[k] : 0.f;
}

// ------------------------------------------------------------------ fused 5-point V-cycle
//
// Overlapped tiling: a block loads its 32 x 32 tile plus a halo of FH pixels
// into shared memory and runs the colour sweeps on shrinking regions, so each
// level costs two launches (pre, post) instead of eleven.  A pixel of the halo
// is updated from exactly the values the block that owns it uses, so the
// fused cycle computes what the per-sweep kernels compute, bit for bit (the
// float operations are issued in the same order as in split<0>).

// Region geometry of the tile kernels for NU sweeps per side (2 NU
// half-sweeps): the halo FH needs one pixel per half-sweep and stays a
// multiple of 4 (the region loads move aligned groups of 4 cells: the region's
// first column, tile x - FH, and its width must be multiples of 4), so NU = 1
// and 2 use a halo of 4, NU = 3 one of 8.  The pre-smoothing's first
// half-sweep starts on ring R0 = FH - 2 NU of the region.
template <int NU>
struct Geo {
	static constexpr int FH = NU <= 2 ? 4 : 8;
	static constexpr int FR = SP_TILE + 2 * FH;   // side of the shared region
	static constexpr int FN = FR * FR;
	static constexpr int H = 2 * NU;              // half-sweeps per side
	static constexpr int R0 = FH - H;
	static constexpr int KC = (FN / 2 + SP_THREADS - 1) / SP_THREADS;   // cells of a colour per thread
	static constexpr int NV = (FN / 4 + SP_THREADS - 1) / SP_THREADS;   // 4-cell groups per thread
	static_assert(FH % 4 == 0 && FR % 4 == 0 && R0 >= 0, "region columns must stay 4-aligned");
	static_assert(KC * H <= 32, "the sweep masks fit 32 bits");
};
// the sweeps-per-side values the fused kernels are built for
constexpr int NU_MIN = 1, NU_MAX = 3;
// FP32 inner solves stop at this relative decrease at the latest (the FP32
// recurrence drifts below it); SIMPOIS_TAU_MIN overrides it for tuning.
double tau_min()
{
	static double v = [] {
		const char *e = getenv("SIMPOIS_TAU_MIN");
		double x = e ? atof(e) : TAU_MIN;
		return x > 0 ? x : TAU_MIN;
	}();
	return v;
}

// SIMPOIS_VERBOSE=1: print each refinement step's residual to stderr
bool verbose()
{
	static bool v = [] {
		const char *e = getenv("SIMPOIS_VERBOSE");
		return e && atoi(e) > 0;
	}();
	return v;
}

// Problem groups of a batched fused 5-point solve, run as concurrent graph
// branches (SIMPOIS_GROUPS, default 8 -- measured best against 4 and 16 on
// 256 uneven instances and on 32 images of 1024^2; 1 keeps the whole batch
// in one).  Results are the same.
int groups_max()
{
	static int v = [] {
		const char *e = getenv("SIMPOIS_GROUPS");
		const int g = e ? atoi(e) : 8;
		return g < 1 ? 1 : (g > GMAX ? GMAX : g);
	}();
	return v;
}

// Programmatic dependent launches between the fused V-cycle kernels (on by
// default; SIMPOIS_NO_PDL=1 launches them plainly).  Results are the same.
bool pdl_enabled()
{
	static bool v = [] {
		const char *e = getenv("SIMPOIS_NO_PDL");
		return !(e && atoi(e) > 0);
	}();
	return v;
}

// Hand-over size of the fused V-cycle: levels with max(w, h) <= it run in
// k_coarse5 (one block per problem), wider levels in the tile kernels.
// Level 0 of a problem of at most SMALL_MAX x SMALL_MAX always runs in
// k_coarse5 and level 0 of a larger problem always in the tile kernels, so
// the hand-over size (8..128) moves work between kernels but changes no bit
// of a result (both compute the same sweeps, restrictions and injections).
// Default 64; SIMPOIS_COARSE_MAX overrides the default.
constexpr int SMALL_MAX = 64;

int clamp_coarse_max(int x) { return x < 8 ? 8 : (x > 128 ? 128 : x); }

int default_coarse_max()
{
	static int v = [] {
		const char *e = getenv("SIMPOIS_COARSE_MAX");
		return clamp_coarse_max(e ? atoi(e) : 64);
	}();
	return v;
}

// Levels of a problem that run in the tile kernels (the level nfine and the
// coarser ones run in k_coarse5).
int handover_level(const int *lw, const int *lh, int nl, int cmax)
{
	if (std::max(lw[0], lh[0]) <= SMALL_MAX) return 0;
	int nf = 1;
	while (nf < nl - 1 && std::max(lw[nf], lh[nf]) > cmax) nf++;
	return nf;
}

// ------------------------------------------------------------------ TMA
// Region loads of the tile kernels through the tensor memory accelerator: one
// thread arms an mbarrier with the byte count and issues the 2-D tile copies;
// every thread waits on the barrier's phase.  The wait is bounded: after
// TMA_SPIN unsuccessful probes it records the failure in Globals::tma_timeout
// and keeps waiting (bounded again) for the copies it started, so that no
// copy lands in shared memory after the block has moved on.
constexpr int TMA_SPIN = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
	return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
			: "memory");
}

// 2-D tile copy of the box at element coordinates (x, y) of map into dst;
// x * element size is a multiple of 16 bytes, dst is 128-byte aligned
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
	asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
			" [%0], [%1, {%2, %3}], [%4];"
			::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
			: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(ok)
			: "r"(smem_u32(bar)), "r"(parity)
			: "memory");
	return ok != 0;
}

// wait for phase 0 of bar; false (and the failure recorded) if it did not
// complete within the bound
__device__ __forceinline__ bool mbar_wait0(uint64_t *bar, int *timeout_flag)
{
	for (int it = 0; it < TMA_SPIN; it++)
		if (mbar_try_wait(bar, 0)) return true;
	atomicExch(timeout_flag, 1);
	for (int it = 0; it < TMA_SPIN; it++)
		if (mbar_try_wait(bar, 0)) return false;
	return false;
}

// Region code of a shared region cell: the level's cell code (cell_code) with
// the neighbour bits that point out of the region cleared (those cells are
// not in shared memory), for a group of 4 cells of a row (x the lowest byte).
template <int FR>
__device__ __forceinline__ uint32_t region_codes4(uint32_t cd, int rx, int ry)
{
	if (rx == 0) cd &= ~0x00000004u;        // W of the first column
	if (rx == FR - 4) cd &= ~0x02000000u;   // E of the last column
	if (ry == 0) cd &= ~0x10101010u;        // N of the first row
	if (ry == FR - 1) cd &= ~0x08080808u;   // S of the last row
	return cd;
}

// The off-diagonal sum of split<0> from a cell code (same operations, same
// order: E, W, S, N).
__device__ __forceinline__ float off_code(const float *z, int c, int R, int code)
{
	float off = 0.f;
	if (code & 2) off -= z[c + 1];
	if (code & 4) off -= z[c - 1];
	if (code & 8) off -= z[c + R];
	if (code & 16) off -= z[c - R];
	return off;
}

__device__ __forceinline__ float diag_code(int code) { return 4.f - (float)(code >> 5); }

// The colour cells of the FR x FR region a thread owns: for colour col, cell
// q = tid + 256 k (k < KC, q < FN / 2) of the compacted class, packed as
// (region index) | (ring << 12); ring = distance to the region's edge.
// x0 + y0 is even for every tile (both are multiples of 32 minus FH), so
// the cells depend on the thread alone: a table built at compile time.
template <int FR>
struct CellTable {
	static constexpr int KC = (FR * FR / 2 + SP_THREADS - 1) / SP_THREADS;
	int v[2][KC][SP_THREADS];
};

template <int FR>
constexpr CellTable<FR> make_cell_table()
{
	CellTable<FR> t{};
	for (int col = 0; col < 2; col++)
		for (int k = 0; k < CellTable<FR>::KC; k++)
			for (int tid = 0; tid < SP_THREADS; tid++) {
				const int q = tid + SP_THREADS * k;
				if (q >= FR * FR / 2) {
					t.v[col][k][tid] = -1;
					continue;
				}
				const int ry = q / (FR / 2);
				const int rx = 2 * (q - ry * (FR / 2)) + ((col ^ ry) & 1);
				const int a = rx < ry ? rx : ry, b = FR - 1 - rx < FR - 1 - ry ? FR - 1 - rx : FR - 1 - ry;
				t.v[col][k][tid] = (ry * FR + rx) | ((a < b ? a : b) << 12);
			}
	return t;
}

__device__ const CellTable<Geo<2>::FR> g_cells40 = make_cell_table<Geo<2>::FR>();
__device__ const CellTable<Geo<3>::FR> g_cells48 = make_cell_table<Geo<3>::FR>();
static_assert(Geo<1>::FR == Geo<2>::FR, "NU = 1 and 2 share the region");
constexpr int CELL_MASK = 4095;   // region index of a cell-table entry

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialisation may be scheduled while the kernel before it drains; it calls
// grid_wait() before its first access to anything an earlier kernel wrote
// (and before any early return, so that its own completion still implies the
// completion of every kernel before it), and grid_release() to let the next
// kernel be scheduled.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void grid_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <int NU>
__device__ __forceinline__ void own_cells(int cells[2][Geo<NU>::KC])
{
	constexpr int KC = Geo<NU>::KC;
#pragma unroll
	for (int col = 0; col < 2; col++)
#pragma unroll
		for (int k = 0; k < KC; k++) {
			if constexpr (Geo<NU>::FR == 40)
				cells[col][k] = g_cells40.v[col][k][threadIdx.x];
			else
				cells[col][k] = g_cells48.v[col][k][threadIdx.x];
		}
}

// The smoothing sweeps of a tile kernel: half-sweep s (0 .. H - 1) updates
// colour s & 1 on the cells of ring >= R0 + s in the pre-smoothing (k_pre5),
// colour 1 - (s & 1) on the cells of ring >= R0 + s + 1 in the
// post-smoothing (k_post5): every cell whose value reaches the tile (ring >=
// FH) through the remaining half-sweeps, so the tile's values are exact (and
// after the pre-smoothing ring FH - 1 too, which the restriction's residual
// reads).  Which of a thread's KC cells of that colour take part is decided
// once per tile: bit KC s + k of the masks is set when cell k is unknown and
// on a deep enough ring.
template <int NU, bool post>
__device__ __forceinline__ uint32_t sweep_masks(const uint8_t *sc, const int cells[2][Geo<NU>::KC])
{
	using G = Geo<NU>;
	constexpr int KC = G::KC;
	uint32_t unk = 0;   // bit KC col + k: the cell is unknown
#pragma unroll
	for (int col = 0; col < 2; col++)
#pragma unroll
		for (int k = 0; k < KC; k++) {
			const int e = cells[col][k];
			if (e >= 0 && (sc[e & CELL_MASK] & 1)) unk |= 1u << (KC * col + k);
		}
	uint32_t m = 0;
#pragma unroll
	for (int s = 0; s < G::H; s++) {
		const int col = post ? 1 - (s & 1) : (s & 1), lo = G::R0 + (post ? s + 1 : s);
#pragma unroll
		for (int k = 0; k < KC; k++)
			if (((unk >> (KC * col + k)) & 1u) && (cells[col][k] >> 12) >= lo) m |= 1u << (KC * s + k);
	}
	return m;
}

// Half-sweep of colour col over the cells of mask m (KC bits).  In the first
// half-sweep from z = 0 (zero set) every neighbour is 0: the off-diagonal sum
// is +0 and b - (+0) is b, so z = b / diag gives the same float.  In the
// others every neighbour of an updated cell lies in the region, and every
// neighbour off_code skips -- a known cell or one outside the image -- holds
// +0 in the region and is never written; x - (+0) is x for every float (-0
// and NaN included), so the four neighbours are subtracted without tests, in
// off_code's order, with the same result.  plain4: no cell of the region has
// a clamped side (every diagonal is 4), and num * 0.25 is gs_div(num, 4).
template <int NU, bool zero, bool plain4>
__device__ __forceinline__ void sweep_masked(float *sz, const float *sb, const uint8_t *sc,
		const int cells[2][Geo<NU>::KC], int col, uint32_t m)
{
	constexpr int FR = Geo<NU>::FR;
#pragma unroll
	for (int k = 0; k < Geo<NU>::KC; k++) {
		if (!((m >> k) & 1u)) continue;
		const int c = cells[col][k] & CELL_MASK;
		const float num = zero ? sb[c] : sb[c] - ((((0.f - sz[c + 1]) - sz[c - 1]) - sz[c + FR]) - sz[c - FR]);
		sz[c] = plain4 ? num * 0.25f : gs_div(num, diag_code(sc[c]));
	}
}

// The H half-sweeps of k_pre5 (post = false: the first from z = 0) or
// k_post5, each followed by a block barrier.
template <int NU, bool post, bool plain4>
__device__ __forceinline__ void run_sweeps(float *sz, const float *sb, const uint8_t *sc,
		const int cells[2][Geo<NU>::KC], uint32_t ms)
{
	constexpr int KC = Geo<NU>::KC;
#pragma unroll
	for (int s = 0; s < Geo<NU>::H; s++) {
		const int col = post ? 1 - (s & 1) : (s & 1);
		const uint32_t m = (ms >> (KC * s)) & ((1u << KC) - 1u);
		if (!post && s == 0)
			sweep_masked<NU, true, plain4>(sz, sb, sc, cells, col, m);
		else
			sweep_masked<NU, false, plain4>(sz, sb, sc, cells, col, m);
		__syncthreads();
	}
}

// Clamp-count bits of 4 packed cell codes: nonzero when a cell of the group
// lies on the image border (its diagonal is below 4).
constexpr uint32_t CLAMP_BITS4 = 0xE0E0E0E0u;

// Pre-smoothing from z = 0 (NU5 forward red-black sweeps), residual, and its
// restriction (sum over the children) into b of level l+1.  Writes z of level
// l (the pre-smoothed correction).
// At level 0 with a PCG step pending (alpha set by k_spmv5) it first takes
// that step, as k_xr would: x += alpha p and r -= alpha q on the tile (the
// new r goes to b_alt, which k_rr5 then swaps with lv[0].b,
// as neighbouring tiles still read the old r of this tile's cells), with r
// recomputed on the whole region as the right-hand side of the sweeps, and
// |r|^2 summed and tested as in k_xr (same operations, same order).
template <int NU>
__global__ void __launch_bounds__(SP_THREADS, 8) k_pre5(ProbDev *P, ProbState *st, const int4 *__restrict__ tl,
		int l, const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial, Globals *gl,
		int use_p2)
{
	constexpr int FH = Geo<NU>::FH, FR = Geo<NU>::FR, FN = Geo<NU>::FN;
	__shared__ __align__(128) float sb[FN];
	__shared__ __align__(128) uint8_t stc[FR * 64];   // TMA: the code box (64 bytes a row)
	__shared__ __align__(16) float sz[FN];
	__shared__ __align__(16) uint8_t sc[FN];
	__shared__ double sh[32];
	__shared__ uint64_t bar;
	// Before the dependency wait, what no kernel of the solve's loop writes:
	// the tile, the level tables of levels l and l + 1 (the last level-0 tile
	// of this kernel swaps lv[0].b with b_alt, and the kernel before a level-0
	// launch is k_spmv5 or k_resid64, which write no table), the cell codes
	// and the coarse mask.  The kernel before this one writes b of this level
	// (the restriction) and the problem's state: those come after the wait.
	const int4 t = tl[blockIdx.x];
	const int prob = t.x;
	const ProbDev &pr = P[prob];
	const int nf = pr.nfine;
	const LevelDev L = pr.lv[l], C = pr.lv[l + 1];
	const bool fine = l < nf;
	const int x0 = t.y * SP_TILE - FH, y0 = t.z * SP_TILE - FH;
	// the coarse cell this thread restricts to (16 x 16 per tile)
	const int ci = t.y * (SP_TILE / 2) + (threadIdx.x & 15), cj = t.z * (SP_TILE / 2) + (threadIdx.x >> 4);
	const bool cun = fine && ci < C.w && cj < C.h && C.mask[(size_t)cj * C.w + ci];
	constexpr int NV = (FN / 4 + SP_THREADS - 1) / SP_THREADS;   // 4-cell groups per thread
	const bool vec = (L.w & 3) == 0;
	const bool tma = NU == 2 && L.tmb;   // the TMA boxes are laid out for a halo of 4
	uint32_t cdv[NV];   // the region codes of the thread's groups
	if (fine && !tma) {
#pragma unroll
		for (int it = 0; it < NV; it++) {
			const int f = threadIdx.x + it * SP_THREADS;
			cdv[it] = 0;
			if (f < FN / 4) {
				const int ry = f / (FR / 4), rx = 4 * (f - ry * (FR / 4)), gi = x0 + rx, gj = y0 + ry;
				const int n = group_cells(gi, gj, L.w, L.h);
				const size_t k = n ? (size_t)gj * L.w + gi : 0;
				const uint32_t cd = region_codes4<FR>(gload4u8(L.code, k, n, vec), rx, ry);
				cdv[it] = cd;
				const int c = ry * FR + rx;
				*(uint32_t *)(sc + c) = cd;
				*(float4 *)(sz + c) = make_float4(0.f, 0.f, 0.f, 0.f);
			}
		}
	}
	uint32_t clampbits = 0;   // any clamp bits in the thread's groups
#pragma unroll
	for (int it = 0; it < NV; it++) clampbits |= (fine && !tma) ? cdv[it] : 0u;
	grid_wait();
	grid_release();
	const int active = st[prob].inner_active, pending = st[prob].pending;
	const float alpha_f = st[prob].alpha_f;
	const bool upd = l == 0 && pending;
	const float a = upd ? alpha_f : 0.f;
	const float *qv = pr.q;
	// b (and at level 0 q) of the region: issued with the state's loads, before
	// the early-return test, so that one round trip follows the wait
	if (fine && !tma) {
#pragma unroll
		for (int it = 0; it < NV; it++) {
			const int f = threadIdx.x + it * SP_THREADS;
			if (f < FN / 4) {
				const int ry = f / (FR / 4), rx = 4 * (f - ry * (FR / 4)), gi = x0 + rx, gj = y0 + ry;
				const uint32_t cd = cdv[it];
				float4 bv = make_float4(0.f, 0.f, 0.f, 0.f);
				if (cd) {   // a group holding an unknown lies (partly) in the image
					const int n = min(4, L.w - gi);
					const size_t k = (size_t)gj * L.w + gi;
					bv = gload4(L.b, k, n, vec);
					if (l == 0) {
						const float4 qq = gload4(qv, k, n, vec);
						if (upd) {
							bv.x = __fmaf_rn(-a, qq.x, bv.x);
							bv.y = __fmaf_rn(-a, qq.y, bv.y);
							bv.z = __fmaf_rn(-a, qq.z, bv.z);
							bv.w = __fmaf_rn(-a, qq.w, bv.w);
						}
					}
				}
				*(float4 *)(sb + ry * FR + rx) = make_float4((cd & 1u) ? bv.x : 0.f, (cd & 0x100u) ? bv.y : 0.f,
						(cd & 0x10000u) ? bv.z : 0.f, (cd & 0x1000000u) ? bv.w : 0.f);
			}
		}
	}
	if (!active || !fine) return;
	if (tma) {
		// TMA: b as a 40 x 40 box at (x0, y0) straight into sb, the codes as a
		// 64 x 40 box from x0 - 12 (a 16-byte boundary); out of the image both
		// read 0 (a known cell).  b stays unmasked: it is read at unknown cells
		// only (sweeps, restriction of unknown children, the PCG step).
		if (threadIdx.x == 0) {
			mbar_init(&bar, 1);
			mbar_expect_tx(&bar, (uint32_t)(FN * sizeof(float) + FR * 64));
			tma_load_2d(sb, L.tmb, x0, y0, &bar);
			tma_load_2d(stc, L.tmc, x0 - 12, y0, &bar);
		}
		for (int c = threadIdx.x; c < FN; c += SP_THREADS) sz[c] = 0.f;
		__syncthreads();   // the barrier is initialised
		mbar_wait0(&bar, &gl->tma_timeout);
#pragma unroll
		for (int it = 0; it < NV; it++) {
			const int f = threadIdx.x + it * SP_THREADS;
			if (f < FN / 4) {
				const int ry = f / (FR / 4), rx = 4 * (f - ry * (FR / 4));
				const uint32_t cd = region_codes4<FR>(*(const uint32_t *)(stc + ry * 64 + rx + 12), rx, ry);
				*(uint32_t *)(sc + ry * FR + rx) = cd;
				clampbits |= cd;
				if (upd && cd) {
					const int gi = x0 + rx, gj = y0 + ry;   // a group with an unknown is in the image
					const float4 qq = *(const float4 *)(qv + (size_t)gj * L.w + gi);
					float *b4 = sb + ry * FR + rx;
					b4[0] = __fmaf_rn(-a, qq.x, b4[0]);
					b4[1] = __fmaf_rn(-a, qq.y, b4[1]);
					b4[2] = __fmaf_rn(-a, qq.z, b4[2]);
					b4[3] = __fmaf_rn(-a, qq.w, b4[3]);
				}
			}
		}
	}
	// the PCG step on the tile: the pixel -> thread map and the order of the
	// |r|^2 terms are those of k_xr
	FF rr = {0.f, 0.f};
	if (upd) {
		const float *pv = use_p2 ? pr.p2 : pr.p;
		const Grp g = grp_of(t, L.w, L.h);
		float xv[4], xl[4], pk[4];
		uint8_t mk[4];
		if (g.n) {
			ldm4(L.mask, g, mk);
			ld4(pr.x, g, xv);
			ld4(pr.xlo, g, xl);
			ld4(pv, g, pk);
		}
		__syncthreads();   // sb holds the new r
		if (g.n) {
			const float *rb = sb + ((threadIdx.x >> 3) + FH) * FR + 4 * (threadIdx.x & 7) + FH;
			float rk[4];
#pragma unroll
			for (int e = 0; e < 4; e++) {
				rk[e] = rb[e];
				if (!mk[e]) continue;
				FF xn = {xv[e], xl[e]};
				ff_add_prod(xn, a, pk[e]);
				xv[e] = xn.hi;
				xl[e] = xn.lo;
				ff_add_prod(rr, rk[e], rk[e]);
			}
			st4(pr.x, g, xv);
			st4(pr.xlo, g, xl);
			st4(pr.b_alt, g, rk);
		}
	}
	int cells[2][Geo<NU>::KC];
	own_cells<NU>(cells);
	// the region holds the b and codes of every cell now; half-sweep s updates
	// colour s&1 on the cells of ring >= R0 + s; at s = 0 every neighbour is
	// 0, so the outermost ring needs no outside value
	const bool plain4 = !__syncthreads_or((clampbits & CLAMP_BITS4) != 0);
	const uint32_t ms = sweep_masks<NU, false>(sc, cells);
	if (plain4)
		run_sweeps<NU, false, true>(sz, sb, sc, cells, ms);
	else
		run_sweeps<NU, false, false>(sz, sb, sc, cells, ms);
	// write the pre-smoothed correction of the tile
	{
		const Grp g = grp_of(t, L.w, L.h);
		if (g.n) st4(L.z, g, sz + ((threadIdx.x >> 3) + FH) * FR + 4 * (threadIdx.x & 7) + FH);
	}
	// restriction: one coarse cell per thread.  A known child adds +0 to a sum
	// that starts at +0 and so is never -0: it is skipped; an unknown one's
	// neighbours are subtracted without tests (see sweep_masked)
	if (cun) {
		float acc = 0.f;
		for (int bb = 0; bb < 2; bb++)
			for (int aa = 0; aa < 2; aa++) {
				const int fi = 2 * ci + aa, fj = 2 * cj + bb;
				if (fi < L.w && fj < L.h) {
					const int c = (fj - y0) * FR + (fi - x0);
					const int code = sc[c];
					if (code & 1) {
						const float off = (((0.f - sz[c + 1]) - sz[c - 1]) - sz[c + FR]) - sz[c - FR];
						acc += sb[c] - (diag_code(code) * sz[c] + off);
					}
				}
			}
		C.b[(size_t)cj * C.w + ci] = 1.f * acc;
	}
	if (!upd) return;
	// the tile's |r|^2; k_rr5 sums the problem's tiles and ends the step
	const double s0 = block_sum_ff<SP_THREADS>(rr, sh);
	if (threadIdx.x == 0) partial[2 * blockIdx.x] = s0;
}

// The sum of per-tile partials of one problem, in tile order: the order and
// tree of problem_sum1's last block (the per-sweep kernels' reductions), so
// the fused path's scalars carry the same bits.
__device__ __forceinline__ double tiles_sum(const double *partial, int b0, int n, double *sh)
{
	double a0 = 0;
	for (int k = threadIdx.x; k < n; k += SP_THREADS) a0 += __ldcg(partial + 2 * (b0 + k));
	return block_sum<SP_THREADS>(a0, sh);
}

// The end of k_pre5's PCG step at level 0, one block per problem of the group
// (the problems p0 ..) that took it in the tile kernel: |r|^2 from the tiles'
// partials, the iteration counts, the swap of the residual buffers (every tile
// is done with the old r), the stop test.  In its own launch, so that the
// tile kernel's blocks exit without waiting for an atomic to learn which is
// the last.
__global__ void __launch_bounds__(SP_THREADS) k_rr5(ProbDev *P, ProbState *st, const int *__restrict__ tbeg,
		const int *__restrict__ tcnt, const double *partial, Globals *gl, int p0)
{
	__shared__ double sh[32];
	const int prob = p0 + blockIdx.x;
	grid_wait();
	grid_release();
	if (!st[prob].inner_active || !st[prob].pending || P[prob].nfine == 0) return;
	const double tot = tiles_sum(partial, tbeg[prob], tcnt[prob], sh);
	if (threadIdx.x == 0) {
		ProbState &s = st[prob];
		s.rr = tot;
		s.iter += 1;
		s.total_iter += 1;
		s.pending = 0;
		ProbDev &w = P[prob];
		float *nb = w.b_alt;
		w.b_alt = w.lv[0].b;
		w.lv[0].b = nb;
		const CUtensorMap *nm = w.tmb_alt;   // and its TMA map
		w.tmb_alt = w.lv[0].tmb;
		w.lv[0].tmb = nm;
		if (tot <= s.tau2 || s.iter >= INNER_MAX || s.total_iter >= s.max_iter) {
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		}
	}
}

// Coarse correction (injection from z2 of level l+1) and post-smoothing
// (NU5 backward sweeps); writes z2 of level l.  At level 0 also the tile's r.z
// partial (k_beta5 forms the PCG scalars beta, rho).
template <int NU>
__global__ void __launch_bounds__(SP_THREADS, 8) k_post5(const ProbDev *__restrict__ P, ProbState *st,
		const int4 *__restrict__ tl, int l, const int *__restrict__ tbeg, const int *__restrict__ tcnt,
		double *partial, Globals *gl, int pcg)
{
	constexpr int FH = Geo<NU>::FH, FR = Geo<NU>::FR, FN = Geo<NU>::FN;
	__shared__ __align__(16) float sb[FN], sz[FN];
	__shared__ __align__(16) uint8_t sc[FN];
	__shared__ double sh[32];
	// Before the dependency wait: the kernel before this one (k_post5 of level
	// l + 1 or k_coarse5) writes only z2 of level l + 1, so the tile, the level
	// tables, the problem's inner_active (k_coarse5 changes it only for
	// problems without tile levels, which return here), the cell codes, b and z
	// of this level and the coarse mask are loaded first; the coarse
	// correction after the wait.
	const int4 t = tl[blockIdx.x];
	const int prob = t.x;
	const ProbDev &pr = P[prob];
	const int active = st[prob].inner_active, nf = pr.nfine;
	const LevelDev L = pr.lv[l], C = pr.lv[l + 1];
	const bool fine = active && l < nf;
	const int x0 = t.y * SP_TILE - FH, y0 = t.z * SP_TILE - FH;
	constexpr int NV = (FN / 4 + SP_THREADS - 1) / SP_THREADS;
	const bool vec = (L.w & 3) == 0;
	uint32_t addm = 0;   // per group (4 bits each) the cells that take the correction
	uint32_t clampbits = 0;   // any clamp bits in the thread's groups
	if (fine) {
		// groups of 4 cells of a row (with w % 4 == 0 wholly inside or outside
		// the image, every access aligned)
#pragma unroll
		for (int it = 0; it < NV; it++) {
			const int f = threadIdx.x + it * SP_THREADS;
			if (f < FN / 4) {
				const int ry = f / (FR / 4), rx = 4 * (f - ry * (FR / 4)), gi = x0 + rx, gj = y0 + ry;
				const int n = group_cells(gi, gj, L.w, L.h);
				const size_t k = n ? (size_t)gj * L.w + gi : 0;
				const size_t kc = n ? (size_t)(gj >> 1) * C.w + (gi >> 1) : 0;
				const uint32_t cd = region_codes4<FR>(gload4u8(L.code, k, n, vec), rx, ry);
				clampbits |= cd;
				float4 bv = make_float4(0.f, 0.f, 0.f, 0.f), zv = bv;
				uint8_t cm0 = 0, cm1 = 0;
				if (cd) {
					bv = gload4(L.b, k, n, vec);
					zv = gload4(L.z, k, n, vec);
					cm0 = C.mask[kc];
					if (n > 2) cm1 = C.mask[kc + 1];
				}
				const int c = ry * FR + rx;
				*(uint32_t *)(sc + c) = cd;
				const bool m0 = cd & 1u, m1 = cd & 0x100u, m2 = cd & 0x10000u, m3 = cd & 0x1000000u;
				*(float4 *)(sb + c) = make_float4(m0 ? bv.x : 0.f, m1 ? bv.y : 0.f, m2 ? bv.z : 0.f,
						m3 ? bv.w : 0.f);
				*(float4 *)(sz + c) = make_float4(m0 ? zv.x : 0.f, m1 ? zv.y : 0.f, m2 ? zv.z : 0.f,
						m3 ? zv.w : 0.f);
				const uint32_t am = (m0 && cm0 ? 1u : 0u) | (m1 && cm0 ? 2u : 0u) | (m2 && cm1 ? 4u : 0u) |
						(m3 && cm1 ? 8u : 0u);
				addm |= am << (4 * it);
			}
		}
	}
	grid_wait();
	grid_release();
	if (!fine) return;
	// the coarse correction: z + z2 of the coarse cell at the unknown cells
	// whose coarse cell is unknown (the same sum as before, z + cz)
#pragma unroll
	for (int it = 0; it < NV; it++) {
		const uint32_t am = (addm >> (4 * it)) & 15u;
		const int f = threadIdx.x + it * SP_THREADS;
		if (am) {
			const int ry = f / (FR / 4), rx = 4 * (f - ry * (FR / 4)), gi = x0 + rx, gj = y0 + ry;
			const float *zc = C.z2 + (size_t)(gj >> 1) * C.w + (gi >> 1);
			float2 cz;
			if (vec) {   // C.w is even and gi / 2 too: an aligned pair
				cz = *(const float2 *)zc;
			} else {
				cz.x = (am & 3u) ? zc[0] : 0.f;
				cz.y = (am & 12u) ? zc[1] : 0.f;
			}
			float *z4 = sz + ry * FR + rx;
			if (am & 1u) z4[0] = z4[0] + cz.x;
			if (am & 2u) z4[1] = z4[1] + cz.x;
			if (am & 4u) z4[2] = z4[2] + cz.y;
			if (am & 8u) z4[3] = z4[3] + cz.y;
		}
	}
	int cells[2][Geo<NU>::KC];
	own_cells<NU>(cells);
	// half-sweep s updates colour 1 - (s&1) on the cells of ring >= R0 + s + 1
	const bool plain4 = !__syncthreads_or((clampbits & CLAMP_BITS4) != 0);
	const uint32_t ms = sweep_masks<NU, true>(sc, cells);
	if (plain4)
		run_sweeps<NU, true, true>(sz, sb, sc, cells, ms);
	else
		run_sweeps<NU, true, false>(sz, sb, sc, cells, ms);
	// z2 of the tile and, in k_rz's order, r.z
	FF rz = {0.f, 0.f};
	{
		const Grp g = grp_of(t, L.w, L.h);
		if (g.n) {
			const int rc = ((threadIdx.x >> 3) + FH) * FR + 4 * (threadIdx.x & 7) + FH;
			st4(L.z2, g, sz + rc);
#pragma unroll
			for (int e = 0; e < 4; e++)
				if (e < g.n && (sc[rc + e] & 1)) ff_add_prod(rz, sb[rc + e], sz[rc + e]);
		}
	}
	if (l != 0 || !pcg) return;
	// the tile's r.z; k_beta5 sums the problem's tiles
	const double s0 = block_sum_ff<SP_THREADS>(rz, sh);
	if (threadIdx.x == 0) partial[2 * blockIdx.x] = s0;
}

// beta and rho from the level-0 tiles' r.z partials of k_post5, one block per
// problem of the group (the problems p0 .. whose level 0 runs in the tile
// kernels; k_coarse5 ends the others' iterations itself).
__global__ void __launch_bounds__(SP_THREADS) k_beta5(const ProbDev *__restrict__ P, ProbState *st,
		const int *__restrict__ tbeg, const int *__restrict__ tcnt, const double *partial, Globals *gl, int p0)
{
	__shared__ double sh[32];
	const int prob = p0 + blockIdx.x;
	grid_wait();
	grid_release();
	if (!st[prob].inner_active || P[prob].nfine == 0) return;
	const double tot = tiles_sum(partial, tbeg[prob], tcnt[prob], sh);
	if (threadIdx.x == 0) {
		ProbState &s = st[prob];
		if (!(tot > 0) || !isfinite(tot)) {
			// r = 0 exactly, or a preconditioner that is not positive here
			if (tot != 0) s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.beta = s.rho > 0 ? tot / s.rho : 0.0;
			s.beta_f = (float)s.beta;
			s.rho = tot;
		}
	}
}

// Shared-memory layout of the coarse levels of one problem.
struct CoarseLayout {
	int off_m[MAXLEV], off_b[MAXLEV], off_z[MAXLEV];   // byte offsets
	int bytes;
};

__device__ __host__ inline CoarseLayout coarse_layout(const int *lw, const int *lh, int c, int L)
{
	CoarseLayout cl;
	int o = 0;
	for (int l = c; l < L; l++) {
		const int n = lw[l] * lh[l];
		cl.off_b[l] = o;
		o += 4 * n;
		cl.off_z[l] = o;
		o += 4 * n;
	}
	for (int l = c; l < L; l++) {
		cl.off_m[l] = o;
		o += lw[l] * lh[l];
	}
	cl.bytes = (o + 15) / 16 * 16;
	return cl;
}

// One red-black half-sweep (colour) over a whole level held in shared memory;
// the 1024 threads map to 32 x 32 (half-columns, rows) of the colour's cells.
// The Gauss-Seidel update and A z of a cell from its cell code (the same
// operations, in the same order, as split<0>: E, W, S, N).
__device__ __forceinline__ void gs5_code(float *z, const float *b, int code, int c, int w)
{
	z[c] = gs_div(b[c] - off_code(z, c, w, code), diag_code(code));
}

__device__ __forceinline__ float az5_code(const float *z, int code, int c, int w)
{
	return diag_code(code) * z[c] + off_code(z, c, w, code);
}

// m holds cell codes (0 at known cells)
__device__ __forceinline__ void smem_sweep5(float *z, const float *b, const uint8_t *m, int w, int h, int colour)
{
	const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const int hw = (w + 1) >> 1;
	for (int j = ty; j < h; j += nw)
		for (int k = tx; k < hw; k += 32) {
			const int i = 2 * k + ((colour ^ j) & 1);
			const int c = j * w + i;
			if (i < w && m[c]) gs5_code(z, b, m[c], c, w);
		}
	__syncthreads();
}

// The same half-sweep done by one warp (levels of at most 256 cells).
__device__ __forceinline__ void warp_sweep5(float *z, const float *b, const uint8_t *m, int w, int h, int colour)
{
	const int lane = threadIdx.x & 31, hw = (w + 1) >> 1;
	if (w <= 16) {
		// 8 half-columns x 4 rows of lanes: no division in the loop
		const int i = 2 * (lane & 7);
		for (int j = lane >> 3; j < h; j += 4) {
			const int ic = i + ((colour ^ j) & 1);
			const int c = j * w + ic;
			if (ic < w && m[c]) gs5_code(z, b, m[c], c, w);
		}
	} else {
		for (int q = lane; q < hw * h; q += 32) {
			const int j = q / hw, i = 2 * (q - j * hw) + ((colour ^ j) & 1);
			const int c = j * w + i;
			if (i < w && m[c]) gs5_code(z, b, m[c], c, w);
		}
	}
	__syncwarp();
}

// Levels l0 .. L-1 of the cycle by warp 0 alone (all of them hold at most 256
// cells): the same sweeps, restriction and injection as the block-wide code,
// synchronised with __syncwarp instead of block barriers.
__device__ void warp_vcycle5(float *const *Z, float *const *B, const uint8_t *const *M, const int *lw,
		const int *lh, int l0, int L, int nu)
{
	const int lane = threadIdx.x & 31;
	for (int l = l0; l + 1 < L; l++) {
		for (int s = 0; s < nu; s++) {
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 0);
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 1);
		}
		const int wc = lw[l + 1], hc = lh[l + 1];
		for (int c = lane; c < wc * hc; c += 32) {
			const int cj = c / wc, ci = c - cj * wc;
			if (!M[l + 1][c]) continue;
			float acc = 0.f;
			for (int bb = 0; bb < 2; bb++)
				for (int aa = 0; aa < 2; aa++) {
					const int fi = 2 * ci + aa, fj = 2 * cj + bb;
					if (fi < lw[l] && fj < lh[l]) {
						const int f = fj * lw[l] + fi;
						acc += B[l][f] - az5_code(Z[l], M[l][f], f, lw[l]);
					}
				}
			B[l + 1][c] = 1.f * acc;
		}
		__syncwarp();
	}
	{
		const int l = L - 1;
		for (int s = 0; s < COARSE_SWEEPS; s++) {
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 0);
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 1);
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 1);
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 0);
		}
	}
	for (int l = L - 2; l >= l0; l--) {
		const int wc = lw[l + 1];
		for (int c = lane; c < lw[l] * lh[l]; c += 32) {
			const int j = c / lw[l], i = c - j * lw[l];
			const int kc = (j >> 1) * wc + (i >> 1);
			if (M[l][c] && M[l + 1][kc]) Z[l][c] += Z[l + 1][kc];
		}
		__syncwarp();
		for (int s = 0; s < nu; s++) {
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 1);
			warp_sweep5(Z[l], B[l], M[l], lw[l], lh[l], 0);
		}
	}
}

// The V-cycle below level nfine of every problem, one block per problem, all
// in shared memory: the same sweeps, restriction and injection as the tile
// kernels, with the coarsest level (<= 4 x 4) getting COARSE_SWEEPS symmetric
// sweeps.  Reads b of level nfine, writes z2 of level nfine.  When nfine == 0
// (a problem of at most SMALL_MAX x SMALL_MAX) it also takes a pending PCG
// step first (x += alpha p, r -= alpha q in place, |r|^2 and the convergence
// test of k_xr, summed in another order) and forms r.z and the PCG scalars.
__global__ void __launch_bounds__(1024, 1) k_coarse5(const ProbDev *__restrict__ P, ProbState *st, Globals *gl,
		int pcg, int use_p2, int p0, int nu)
{
	extern __shared__ __align__(16) unsigned char smem[];
	__shared__ double sh[32];
	__shared__ int stopped;
	// the level table in shared memory (no per-thread copies)
	__shared__ int s_w[MAXLEV], s_h[MAXLEV], s_pre[MAXLEV + 1];
	__shared__ float *s_Z[MAXLEV], *s_B[MAXLEV];
	__shared__ uint8_t *s_M[MAXLEV];
	__shared__ const uint8_t *s_gm[MAXLEV];
	const int prob = p0 + blockIdx.x;   // the launch covers problems p0 ..
	grid_wait();
	grid_release();
	if (!st[prob].inner_active) return;
	const ProbDev &pr = P[prob];
	const int c0 = pr.nfine, L = pr.nlev;
	const bool upd = c0 == 0 && pcg && st[prob].pending;
	const float a = upd ? st[prob].alpha_f : 0.f;
	const float *pv = use_p2 ? pr.p2 : pr.p;
	FF rr = {0.f, 0.f};
	if (threadIdx.x < L) {
		const int l = threadIdx.x;
		s_w[l] = pr.lv[l].w;
		s_h[l] = pr.lv[l].h;
		// cell codes (the coarsest level has none: its code is formed below)
		s_gm[l] = l + 1 < L ? pr.lv[l].code : pr.lv[l].mask;
		if (l >= c0) {
			s_Z[l] = (float *)(smem + pr.coff_z[l]);
			s_B[l] = (float *)(smem + pr.coff_b[l]);
			s_M[l] = (uint8_t *)(smem + pr.coff_m[l]);
		}
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		int pre = 0;
		for (int l = c0; l < L; l++) {
			s_pre[l] = pre;
			pre += s_w[l] * s_h[l];
		}
		s_pre[L] = pre;
		stopped = 0;
	}
	__syncthreads();
	// every level's cell codes (and b of level c0) in one flat loop: the
	// loads of successive iterations do not depend on each other
	const int total = s_pre[L];
	const float *gb = pr.lv[c0].b;
#pragma unroll 4
	for (int q = threadIdx.x; q < total; q += blockDim.x) {
		int l = c0;
		while (q >= s_pre[l + 1]) l++;
		const int c = q - s_pre[l];
		uint8_t mv = s_gm[l][c];
		if (l + 1 == L && mv) {   // the coarsest level: its code from its mask
			const int w = s_w[l], h = s_h[l], j = c / w;
			mv = cell_code(s_gm[l], c - j * w, j, w, h);
		}
		s_M[l][c] = mv;
		s_Z[l][c] = 0.f;
		if (l == c0) {
			float bv = mv ? gb[c] : 0.f;
			if (upd && mv) {
				FF xn = {pr.x[c], pr.xlo[c]};
				ff_add_prod(xn, a, pv[c]);
				pr.x[c] = xn.hi;
				pr.xlo[c] = xn.lo;
				bv = __fmaf_rn(-a, pr.q[c], bv);
				pr.lv[0].b[c] = bv;
				ff_add_prod(rr, bv, bv);
			}
			s_B[l][c] = bv;
		}
	}
	if (upd) {
		const double rrs = block_sum_ff<1024>(rr, sh);
		if (threadIdx.x == 0) {
			ProbState &s = st[prob];
			s.rr = rrs;
			s.iter += 1;
			s.total_iter += 1;
			s.pending = 0;
			if (rrs <= s.tau2 || s.iter >= INNER_MAX || s.total_iter >= s.max_iter) {
				s.inner_active = 0;
				atomicSub(&gl->inner_count, 1);
				stopped = 1;
			}
		}
	}
	__syncthreads();
	// levels ls.. hold at most 64 cells: warp 0 runs them alone
	int ls = c0;
	while (ls < L - 1 && s_w[ls] * s_h[ls] > 64) ls++;
	const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5, nw = blockDim.x >> 5;
	// down (block-wide levels)
	for (int l = c0; l < ls; l++) {
		float *z = s_Z[l], *b = s_B[l];
		const uint8_t *m = s_M[l];
		const int w = s_w[l], h = s_h[l];
		for (int s = 0; s < nu; s++) {
			smem_sweep5(z, b, m, w, h, 0);
			smem_sweep5(z, b, m, w, h, 1);
		}
		float *bc = s_B[l + 1];
		const uint8_t *mc = s_M[l + 1];
		const int wc = s_w[l + 1], hc = s_h[l + 1];
		for (int cj = ty; cj < hc; cj += nw)
			for (int ci = tx; ci < wc; ci += 32) {
				const int c = cj * wc + ci;
				if (!mc[c]) continue;
				float acc = 0.f;
				for (int bb = 0; bb < 2; bb++)
					for (int aa = 0; aa < 2; aa++) {
						const int fi = 2 * ci + aa, fj = 2 * cj + bb;
						if (fi < w && fj < h) {
							const int f = fj * w + fi;
							acc += b[f] - az5_code(z, m[f], f, w);
						}
					}
				bc[c] = 1.f * acc;
			}
		__syncthreads();
	}
	if (threadIdx.x < 32) warp_vcycle5(s_Z, s_B, s_M, s_w, s_h, ls, L, nu);
	__syncthreads();
	// up (block-wide levels)
	for (int l = ls - 1; l >= c0; l--) {
		float *z = s_Z[l], *b = s_B[l];
		const uint8_t *m = s_M[l];
		const float *zc = s_Z[l + 1];
		const uint8_t *mc = s_M[l + 1];
		const int w = s_w[l], h = s_h[l], wc = s_w[l + 1];
		for (int j = ty; j < h; j += nw)
			for (int i = tx; i < w; i += 32) {
				const int c = j * w + i, kc = (j >> 1) * wc + (i >> 1);
				if (m[c] && mc[kc]) z[c] += zc[kc];
			}
		__syncthreads();
		for (int s = 0; s < nu; s++) {
			smem_sweep5(z, b, m, w, h, 1);
			smem_sweep5(z, b, m, w, h, 0);
		}
	}
	const float *z = s_Z[c0], *b = s_B[c0];
	const uint8_t *m = s_M[c0];
	float *gz2 = pr.lv[c0].z2;
	FF rzf = {0.f, 0.f};
	for (int c = threadIdx.x; c < s_w[c0] * s_h[c0]; c += blockDim.x) {
		gz2[c] = m[c] ? z[c] : 0.f;
		if (m[c]) ff_add_prod(rzf, b[c], z[c]);
	}
	if (c0 != 0 || !pcg) return;
	const double rz = block_sum_ff<1024>(rzf, sh);
	if (threadIdx.x == 0 && !stopped) {
		ProbState &s = st[prob];
		if (!(rz > 0) || !isfinite(rz)) {
			if (rz != 0) s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.beta = s.rho > 0 ? rz / s.rho : 0.0;
			s.beta_f = (float)s.beta;
			s.rho = rz;
		}
	}
}

// p_new = z + beta p_old on the tile and a 1-pixel halo (as k_pupdate), then
// q = A p_new and alpha = rho / (p_new . q) (as k_spmv<0>).  p_old and p_new
// are different buffers (the halo of a neighbour must still see p_old).
// The region is 40 x 34 (4-aligned columns) and moves in groups of 4 cells
// (16-byte accesses when the level width is a multiple of 4), each thread then
// applying A to 4 cells of a row; the products p.q are summed in k_spmv<0>'s
// order.
__global__ void __launch_bounds__(SP_THREADS, 8) k_spmv5(const ProbDev *__restrict__ P, ProbState *st,
		const int4 *__restrict__ tl, const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial,
		Globals *gl, int new_is_p2)
{
	constexpr int RW = SP_TILE + 8, RH = SP_TILE + 2;    // region: 40 x 34
	__shared__ __align__(16) float sp[RW * RH];
	__shared__ __align__(16) uint8_t sc[RW * RH];
	__shared__ double sh[32];
	// Before the dependency wait: the tile, the level table, the cell codes and
	// p_old (the previous SpMV's p_new); the kernel before this one (k_post5
	// at level 0) writes z2 and the PCG scalars, loaded after it.
	const int4 t = tl[blockIdx.x];
	const int prob = t.x;
	const ProbDev &pr = P[prob];
	const LevelDev L = pr.lv[0];
	const float *pold = new_is_p2 ? pr.p : pr.p2;
	float *pnew = new_is_p2 ? pr.p2 : pr.p;
	FF pq = {0.f, 0.f};
	const bool vec = (L.w & 3) == 0;
	const int x0 = t.y * SP_TILE - 4, y0 = t.z * SP_TILE - 1;
	constexpr int NV = (RW * RH / 4 + SP_THREADS - 1) / SP_THREADS;
	// p_old of the region in sp, the codes in sc (p_old is read whatever beta
	// is: it is only used when beta != 0); groups of 4 cells of a row
#pragma unroll
	for (int it = 0; it < NV; it++) {
		const int f = threadIdx.x + it * SP_THREADS;
		if (f < RW * RH / 4) {
			const int ry = f / (RW / 4), rx = 4 * (f - ry * (RW / 4)), gi = x0 + rx, gj = y0 + ry;
			const int n = group_cells(gi, gj, L.w, L.h);
			const size_t k = n ? (size_t)gj * L.w + gi : 0;
			const uint32_t cd = gload4u8(L.code, k, n, vec);
			const float4 po = cd ? gload4(pold, k, n, vec) : make_float4(0.f, 0.f, 0.f, 0.f);
			const int c = ry * RW + rx;
			*(uint32_t *)(sc + c) = cd;
			*(float4 *)(sp + c) = po;
		}
	}
	grid_wait();
	grid_release();
	const int active = st[prob].inner_active;
	const float beta = st[prob].beta_f;
	// z2 of the region, issued with the state's loads
	float4 zr[NV];
#pragma unroll
	for (int it = 0; it < NV; it++) {
		const int f = threadIdx.x + it * SP_THREADS;
		zr[it] = make_float4(0.f, 0.f, 0.f, 0.f);
		if (f < RW * RH / 4) {
			const int ry = f / (RW / 4), rx = 4 * (f - ry * (RW / 4)), gi = x0 + rx, gj = y0 + ry;
			const uint32_t cd = *(const uint32_t *)(sc + ry * RW + rx);
			if (cd) zr[it] = gload4(L.z2, (size_t)gj * L.w + gi, min(4, L.w - gi), vec);   // in the image
		}
	}
	if (!active) return;
#pragma unroll
	for (int it = 0; it < NV; it++) {
		const int f = threadIdx.x + it * SP_THREADS;
		if (f < RW * RH / 4) {
			const int ry = f / (RW / 4), rx = 4 * (f - ry * (RW / 4));
			const int c = ry * RW + rx;
			const uint32_t cd = *(const uint32_t *)(sc + c);
			const float4 zv = zr[it], po = *(const float4 *)(sp + c);
			*(float4 *)(sp + c) = make_float4((cd & 1u) ? (beta != 0.f ? zv.x + beta * po.x : zv.x) : 0.f,
					(cd & 0x100u) ? (beta != 0.f ? zv.y + beta * po.y : zv.y) : 0.f,
					(cd & 0x10000u) ? (beta != 0.f ? zv.z + beta * po.z : zv.z) : 0.f,
					(cd & 0x1000000u) ? (beta != 0.f ? zv.w + beta * po.w : zv.w) : 0.f);
		}
	}
	__syncthreads();
	// 4 cells of a row per thread (every neighbour is in the region); p.q
	// summed over them in row order, as k_spmv does
	{
		const int ty = threadIdx.x >> 3, tx = 4 * (threadIdx.x & 7);
		const int gi = t.y * SP_TILE + tx, gj = t.z * SP_TILE + ty;
		const int c = (ty + 1) * RW + tx + 4;
		float pk[4], qk[4];
#pragma unroll
		for (int e = 0; e < 4; e++) {
			const int code = sc[c + e];
			pk[e] = sp[c + e];
			qk[e] = 0.f;
			if (code & 1) {
				const int ce = c + e;
				qk[e] = a5_diff(pk[e], sp[ce + 1], sp[ce - 1], sp[ce + RW], sp[ce - RW], code);
				ff_add_prod(pq, pk[e], qk[e]);
			}
		}
		const int n = group_cells(gi, gj, L.w, L.h);
		if (n) {
			const size_t k = (size_t)gj * L.w + gi;
			gstore4(pnew, k, n, vec, make_float4(pk[0], pk[1], pk[2], pk[3]));
			gstore4(pr.q, k, n, vec, make_float4(qk[0], qk[1], qk[2], qk[3]));
		}
	}
	// the tile's p.q; k_alpha5 sums the problem's tiles (a block here does not
	// wait for an atomic to learn whether it is the problem's last)
	const double s0 = block_sum_ff<SP_THREADS>(pq, sh);
	if (threadIdx.x == 0) partial[2 * blockIdx.x] = s0;
}

// alpha = rho / (p.q) per problem, p.q summed over the problem's level-0 tile
// partials of k_spmv5 in tile order -- the order and tree of problem_sum1's
// last block, so the bits are those of the per-sweep path's k_spmv.  One
// block per problem of the group (the problems p0 ..).
__global__ void __launch_bounds__(SP_THREADS) k_alpha5(ProbState *st, const int *__restrict__ tbeg,
		const int *__restrict__ tcnt, const double *partial, Globals *gl, int p0)
{
	__shared__ double sh[32];
	const int prob = p0 + blockIdx.x;
	grid_wait();
	grid_release();
	if (!st[prob].inner_active) return;
	const double a0 = tiles_sum(partial, tbeg[prob], tcnt[prob], sh);
	if (threadIdx.x == 0) {
		ProbState &s = st[prob];
		const double a = s.rho / a0;
		if (!(a0 > 0) || !isfinite(a)) {
			s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			s.alpha = 0;
			s.alpha_f = (float)s.alpha;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.alpha = a;
			s.alpha_f = (float)s.alpha;
			s.pending = 1;   // k_pre5 (or k_coarse5) at level 0 takes the step
		}
	}
}

// ------------------------------------------------------------------ 13-point PCG in FP64
//
// The biharmonic system needs FP64 Krylov vectors: for a hole d pixels wide
// the smoothest mode has eigenvalue ~(pi/d)^4 (1e-10 for d = 1024), far below
// the FP32 rounding of the 13-point sum (~64 * 6e-8), so an FP32 A p cannot
// see the components that converge last.  The preconditioner stays in FP32:
// away from the image border the masked 13-point operator is L^2 + B B^T, with
// L the masked 5-point -Laplacian and B B^T >= 0 the coupling through known
// pixels, so two symmetric 5-point V-cycles (V V ~ L^-2) precondition it;
// the coarse grids resolve the smooth modes that FP32 cannot see on the fine
// one.

// Every kernel of the loop takes one level-0 tile per block, each thread a
// 4-pixel row group of it (grp_of), and follows the programmatic-dependent-
// launch protocol of the tile kernels: what an earlier kernel than the one
// just before it wrote may be loaded before grid_wait() (every kernel of the
// chain waits before it releases, so those have completed), the rest after.

__device__ __forceinline__ void ld4d(const double *p, const Grp &g, double v[4])
{
	if (g.vec) {
		const double2 a = *(const double2 *)(p + g.k), b = *(const double2 *)(p + g.k + 2);
		v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
	} else {
#pragma unroll
		for (int e = 0; e < 4; e++) v[e] = e < g.n ? p[g.k + e] : 0.0;
	}
}

__device__ __forceinline__ void st4d(double *p, const Grp &g, const double v[4])
{
	if (g.vec) {
		*(double2 *)(p + g.k) = make_double2(v[0], v[1]);
		*(double2 *)(p + g.k + 2) = make_double2(v[2], v[3]);
	} else {
#pragma unroll
		for (int e = 0; e < 4; e++)
			if (e < g.n) p[g.k + e] = v[e];
	}
}

// b0 = z2_0: the second V-cycle's right-hand side, on the row groups that
// hold an unknown (b0 is read at the unknowns only)
__global__ void __launch_bounds__(SP_THREADS) k_z2b(const ProbDev *__restrict__ P, const ProbState *__restrict__ st,
		const int4 *__restrict__ tl)
{
	const int4 t = tl[blockIdx.x];
	const ProbDev &pr = P[t.x];
	const Grp g = grp_of(t, pr.w, pr.h);
	uint8_t m[4] = {0, 0, 0, 0};
	if (g.n) ldm4(pr.lv[0].mask, g, m);
	grid_wait();
	grid_release();
	if (!st[t.x].inner_active || !(m[0] | m[1] | m[2] | m[3])) return;
	float z[4];
	ld4(pr.lv[0].z2, g, z);
	st4(pr.lv[0].b, g, z);
}

// rho = r . z (the float r, kept in x, against the float z, summed in
// float-float: the scalars need ~1e-7, not FP64); flexible beta = (rho - r . z_old) / rho_old
// (0 on the first iteration of an inner solve).
__global__ void __launch_bounds__(SP_THREADS) k_rz13(const ProbDev *__restrict__ P, ProbState *st,
		const int4 *__restrict__ tl, const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial,
		Globals *gl)
{
	__shared__ double sh[32];
	const int4 t = tl[blockIdx.x];
	const int prob = t.x;
	const ProbDev &pr = P[prob];
	const Grp g = grp_of(t, pr.w, pr.h);
	uint8_t m[4] = {0, 0, 0, 0};
	float r[4];
	if (g.n) ldm4(pr.lv[0].mask, g, m);
	const bool any = m[0] | m[1] | m[2] | m[3];
	if (any) ld4(pr.x, g, r);   // (float) r, written by k_xr13 or k_resid64 two kernels back or more
	grid_wait();
	grid_release();
	if (!st[prob].inner_active) return;
	FF rz = {0.f, 0.f};
	if (any) {
		float z[4];
		ld4(pr.lv[0].z2, g, z);
#pragma unroll
		for (int e = 0; e < 4; e++)
			if (m[e]) ff_add_prod(rz, r[e], z[e]);
	}
	double tot[2];
	if (problem_sum1_ff(rz, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		if (!(tot[0] > 0) || !isfinite(tot[0])) {
			if (tot[0] != 0) s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		} else {
			// flexible (Polak-Ribiere) beta = r_new . (z_new - z_old) / rho_old:
			// the FP32 preconditioner is only approximately symmetric, and this
			// form keeps the FP64 recurrence converging where the classical
			// r.z / rho_old stalls (small images with holes at the border)
			s.beta = s.rho > 0 ? (tot[0] - s.cross) / s.rho : 0.0;
			s.beta_f = (float)s.beta;
			s.rho = tot[0];
		}
	}
}

// Exclusive prefix sum of one count per thread over the block (thread order);
// returns the thread's offset, the total in *total.
__device__ __forceinline__ int block_scan(int v, int *sw, int *total)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	int x = v;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const int y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= o) x += y;
	}
	if (lane == 31) sw[warp] = x;
	__syncthreads();
	int base = 0, all = 0;
#pragma unroll
	for (int k = 0; k < SP_THREADS / 32; k++) {
		const int c = sw[k];
		base += k < warp ? c : 0;
		all += c;
	}
	__syncthreads();   // sw may be reused
	*total = all;
	return base + x - v;
}

// p_new = z + beta p_old (z alone on the first iteration of an inner solve);
// q = A p_new with the 13-point single-clamp operator (cleant_cgpois.c:91-121)
// in FP64; alpha = rho / (p.q).  Iteration parity par writes p_new into
// p64 (par 0) or p64b (par 1) and reads p_old from the other: neighbouring
// tiles still read p_old in their halo.  The region is the tile with 2 rows and
// 4 columns of halo (40 x 36, 4-aligned column groups), loaded in row groups
// (p_old, z and 0 at the known pixels).  An FP64 instruction occupies this
// GPU's FP64 pipe for a whole warp whatever its active lanes, so the FP64 work
// runs over compacted lists instead of the pixel grid: the unknown cells of the
// region (p_new) and of the tile (A p_new, p.q), in row order.  A neighbour
// outside the image is the clamped pixel, which lies in the region (the single
// clamp of the reference's 13-point operator); tiles 2 or more pixels from
// every image side take the constant offsets instead.
__global__ void __launch_bounds__(SP_THREADS) k_pspmv13(const ProbDev *__restrict__ P, ProbState *st,
		const int4 *__restrict__ tl, const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial,
		Globals *gl, int par)
{
	constexpr int RW = SP_TILE + 8, RH = SP_TILE + 4;   // region: 40 x 36
	constexpr int NG = RW * RH / 4;                      // 4-cell groups
	constexpr int NV = (NG + SP_THREADS - 1) / SP_THREADS;
	__shared__ __align__(16) double sp[RW * RH];
	__shared__ __align__(16) float sz[RW * RH];
	__shared__ __align__(16) uint8_t sc[RW * RH];
	__shared__ uint16_t lreg[RW * RH], lown[SP_TILE * SP_TILE], lnb[RW * RH];
	__shared__ __align__(16) double sy[RW * RH];   // inner tiles: y = L p at the cells in lnb
	__shared__ __align__(16) uint8_t fnb[RW * RH];
	__shared__ double sh[32];
	__shared__ int sw[SP_THREADS / 32];
	const int4 t = tl[blockIdx.x];
	const int prob = t.x;
	const ProbDev &pr = P[prob];
	const LevelDev &L = pr.lv[0];
	const int w = pr.w, h = pr.h;
	const double *pold = par ? pr.p64 : pr.p64b;
	double *pnew = par ? pr.p64b : pr.p64;
	const bool vec = (w & 3) == 0;
	const int x0 = t.y * SP_TILE - 4, y0 = t.z * SP_TILE - 2;
	// before the dependency wait: the codes, z (written by the last V-cycle's
	// level-0 kernel, two launches back) and p_old (the previous SpMV's), into
	// the region with 0 at the known pixels
	int nreg = 0;
#pragma unroll
	for (int it = 0; it < NV; it++) {
		const int f = threadIdx.x + it * SP_THREADS;
		if (f < NG) {
			const int ry = f / (RW / 4), rx = 4 * (f - ry * (RW / 4)), gi = x0 + rx, gj = y0 + ry;
			const int n = group_cells(gi, gj, w, h);
			const size_t k = n ? (size_t)gj * w + gi : 0;
			const uint32_t cd = gload4u8(L.code, k, n, vec) & 0x01010101u;   // the unknown bits
			const int c = ry * RW + rx;
			*(uint32_t *)(sc + c) = cd;
			float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
			double2 pa = make_double2(0.0, 0.0), pb = make_double2(0.0, 0.0);
			if (cd) {
				z = gload4(L.z2, k, n, vec);
				if (vec) {
					pa = *(const double2 *)(pold + k);
					pb = *(const double2 *)(pold + k + 2);
				} else {
					pa.x = pold[k];
					if (n > 1) pa.y = pold[k + 1];
					if (n > 2) pb.x = pold[k + 2];
					if (n > 3) pb.y = pold[k + 3];
				}
				nreg += __popc(cd);
			}
			*(float4 *)(sz + c) = make_float4((cd & 1u) ? z.x : 0.f, (cd & 0x100u) ? z.y : 0.f,
					(cd & 0x10000u) ? z.z : 0.f, (cd & 0x1000000u) ? z.w : 0.f);
			*(double2 *)(sp + c) = make_double2((cd & 1u) ? pa.x : 0.0, (cd & 0x100u) ? pa.y : 0.0);
			*(double2 *)(sp + c + 2) = make_double2((cd & 0x10000u) ? pb.x : 0.0, (cd & 0x1000000u) ? pb.y : 0.0);
		}
	}
	// the lists: unknown region cells in group order, unknown tile cells in row order
	const int ty = threadIdx.x >> 3, tx = 4 * (threadIdx.x & 7);
	const int cown = (ty + 2) * RW + tx + 4;   // the thread's 4 tile cells
	__syncthreads();   // sc
	const uint32_t mown = *(const uint32_t *)(sc + cown);
	int nr = 0, no = 0;
	int offr = block_scan(nreg, sw, &nr);
#pragma unroll
	for (int it = 0; it < NV; it++) {
		const int f = threadIdx.x + it * SP_THREADS;
		if (f < NG) {
			const int ry = f / (RW / 4), rx = 4 * (f - ry * (RW / 4)), c = ry * RW + rx;
			const uint32_t cd = *(const uint32_t *)(sc + c);
#pragma unroll
			for (int e = 0; e < 4; e++)
				if ((cd >> (8 * e)) & 1u) lreg[offr++] = (uint16_t)(c + e);
		}
	}
	int offo = block_scan(__popc(mown), sw, &no);
#pragma unroll
	for (int e = 0; e < 4; e++)
		if ((mown >> (8 * e)) & 1u) lown[offo++] = (uint16_t)(cown + e);
	// A tile 2 or more pixels from every image side applies the 13-point
	// operator as L L (L = 4 - the 4 neighbours: L^2 has the weights 20, -8,
	// 2, 1 of the 13 points): y = L p on the tile's unknowns and their 4
	// neighbours (p is 0 at the known pixels, so y there is what the 13-point
	// sum reads through them), then q = L y -- 8 FP64 operations an unknown
	// and 4 a ring cell instead of 13.  Near a side the single clamp of the
	// 13-point operator differs from composing clamped 5-point ones, so those
	// tiles take the 13 points.
	const bool inner = t.y * SP_TILE >= 2 && t.y * SP_TILE + SP_TILE + 2 <= w && t.z * SP_TILE >= 2 &&
			t.z * SP_TILE + SP_TILE + 2 <= h;
	int nn = 0;
	if (inner) {
#pragma unroll
		for (int it = 0; it < NV; it++) {
			const int f = threadIdx.x + it * SP_THREADS;
			if (f < NG) *(uint32_t *)(fnb + 4 * f) = 0u;
		}
		__syncthreads();
#pragma unroll
		for (int e = 0; e < 4; e++)
			if ((mown >> (8 * e)) & 1u) {
				const int c = cown + e;
				fnb[c] = fnb[c + 1] = fnb[c - 1] = fnb[c + RW] = fnb[c - RW] = 1;
			}
		__syncthreads();
		int cnt = 0;
#pragma unroll
		for (int it = 0; it < NV; it++) {
			const int f = threadIdx.x + it * SP_THREADS;
			if (f < NG) cnt += __popc(*(const uint32_t *)(fnb + 4 * f));
		}
		int offn = block_scan(cnt, sw, &nn);
#pragma unroll
		for (int it = 0; it < NV; it++) {
			const int f = threadIdx.x + it * SP_THREADS;
			if (f < NG) {
				const uint32_t m = *(const uint32_t *)(fnb + 4 * f);
#pragma unroll
				for (int e = 0; e < 4; e++)
					if ((m >> (8 * e)) & 1u) lnb[offn++] = (uint16_t)(4 * f + e);
			}
		}
	}
	grid_wait();
	grid_release();
	if (!st[prob].inner_active) return;
	const double beta = st[prob].beta;
	__syncthreads();   // lreg, lown
	for (int k = threadIdx.x; k < nr; k += SP_THREADS) {
		const int c = lreg[k];
		sp[c] = beta != 0 ? fma(beta, sp[c], (double)sz[c]) : (double)sz[c];
	}
	__syncthreads();
	if (inner) {
		for (int k = threadIdx.x; k < nn; k += SP_THREADS) {
			const int c = lnb[k];
			sy[c] = fma(4.0, sp[c], -(((sp[c + 1] + sp[c - 1]) + sp[c + RW]) + sp[c - RW]));
		}
		__syncthreads();
	}
	constexpr int DI[12] = {1, 0, -1, 0, 1, 1, -1, -1, 2, 0, -2, 0};
	constexpr int DJ[12] = {0, 1, 0, -1, 1, -1, 1, -1, 0, 2, 0, -2};
	constexpr double CF[12] = {-8, -8, -8, -8, 2, 2, 2, 2, 1, 1, 1, 1};
	double pq = 0.0;
	for (int k = threadIdx.x; k < no; k += SP_THREADS) {
		const int c = lown[k];
		const int ry = c / RW, rx = c - ry * RW, i = x0 + rx, j = y0 + ry;
		const double pk = sp[c];
		double qk;
		if (inner) {
			qk = fma(4.0, sy[c], -(((sy[c + 1] + sy[c - 1]) + sy[c + RW]) + sy[c - RW]));
		} else {
			double off = 0.0;
#pragma unroll
			for (int s2 = 0; s2 < 12; s2++) {
				const int qi = clampi(i + DI[s2], w), qj = clampi(j + DJ[s2], h);
				off = fma(CF[s2], sp[(qj - y0) * RW + (qi - x0)], off);
			}
			qk = fma(20.0, pk, off);
		}
		pq = fma(pk, qk, pq);
		const size_t g = (size_t)j * w + i;   // p and q are read at the unknowns only
		pnew[g] = pk;
		pr.q64[g] = qk;
	}
	double tot[2];
	if (problem_sum1(pq, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		const double a = s.rho / tot[0];
		if (!(tot[0] > 0) || !isfinite(a)) {
			s.status = SIMPOIS_BREAKDOWN;
			s.inner_active = 0;
			s.alpha = 0;
			s.alpha_f = (float)s.alpha;
			atomicSub(&gl->inner_count, 1);
		} else {
			s.alpha = a;
			s.alpha_f = (float)s.alpha;
		}
	}
}

// U += alpha p_new (the FP64 solution itself); r -= alpha q; b0 = (float) r,
// the first V-cycle's right-hand side (and a copy in x for k_rz13); |r|^2 and
// r . z_old (flexible beta)
// from the float r in float-float (the stop test and the scalars need ~1e-7);
// the stop test.
__global__ void __launch_bounds__(SP_THREADS) k_xr13(const ProbDev *__restrict__ P, ProbState *st,
		const int4 *__restrict__ tl, const int *__restrict__ tbeg, const int *__restrict__ tcnt, double *partial,
		Globals *gl, int par)
{
	__shared__ double sh[32];
	const int4 t = tl[blockIdx.x];
	const int prob = t.x;
	const ProbDev &pr = P[prob];
	const Grp g = grp_of(t, pr.w, pr.h);
	uint8_t m[4] = {0, 0, 0, 0};
	double u[4], r[4];
	float zo[4];
	if (g.n) ldm4(pr.lv[0].mask, g, m);
	const bool any = m[0] | m[1] | m[2] | m[3];   // row groups without an unknown move nothing
	if (any) {   // written two or more launches back
		ld4d(pr.U, g, u);
		ld4d(pr.r64, g, r);
		ld4(pr.lv[0].z2, g, zo);
	}
	grid_wait();
	grid_release();
	if (!st[prob].inner_active) return;
	const double a = st[prob].alpha;
	FF rr = {0.f, 0.f}, cross = {0.f, 0.f};
	if (any) {
		double pv[4], qv[4];
		ld4d(par ? pr.p64b : pr.p64, g, pv);
		ld4d(pr.q64, g, qv);
		float rf[4];
#pragma unroll
		for (int e = 0; e < 4; e++) {
			rf[e] = 0.f;
			if (!m[e]) continue;
			u[e] = fma(a, pv[e], u[e]);
			r[e] = fma(-a, qv[e], r[e]);
			rf[e] = (float)r[e];
			ff_add_prod(rr, rf[e], rf[e]);
			ff_add_prod(cross, rf[e], zo[e]);
		}
		st4d(pr.U, g, u);
		st4d(pr.r64, g, r);
		st4(pr.lv[0].b, g, rf);
		st4(pr.x, g, rf);   // for r . z (k_rz13): x is not used by this PCG
	}
	double tot[2];
	if (problem_sum2_ff(rr, cross, prob, tbeg, tcnt, partial, st, tot, sh) && threadIdx.x == 0) {
		ProbState &s = st[prob];
		s.rr = tot[0];
		s.cross = tot[1];
		s.iter += 1;
		s.total_iter += 1;
		if (tot[0] <= s.tau2 || s.iter >= INNER_MAX13 || s.total_iter >= s.max_iter) {
			s.inner_active = 0;
			atomicSub(&gl->inner_count, 1);
		}
	}
}

// out = unknown ? (float)U : g over all tiles (fill)
__global__ void __launch_bounds__(SP_THREADS) k_finalize(const ProbDev *__restrict__ P,
		const int4 *__restrict__ all, int nall)
{
	int4 tt[TPB];
	size_t kk[TPB];
	int nv[TPB];
	float gv[TPB][4];
	uint32_t mw[TPB];
#pragma unroll
	for (int q = 0; q < TPB; q++) {
		const int b = blockIdx.x * TPB + q;
		tt[q] = b < nall ? all[b] : make_int4(-1, 0, 0, 0);
	}
#pragma unroll
	for (int q = 0; q < TPB; q++) {
		nv[q] = 0;
		kk[q] = 0;
		mw[q] = 0;
		if (tt[q].x < 0) continue;
		const ProbDev &pr = P[tt[q].x];
		nv[q] = group_of(pr, tt[q], kk[q]);
		if (nv[q] == 4 && pr.vec4) {
			const float4 v = *(const float4 *)(pr.g + kk[q]);
			gv[q][0] = v.x; gv[q][1] = v.y; gv[q][2] = v.z; gv[q][3] = v.w;
			mw[q] = *(const uint32_t *)(pr.lv[0].mask + kk[q]);
		} else {
#pragma unroll
			for (int e = 0; e < 4; e++) {
				gv[q][e] = e < nv[q] ? pr.g[kk[q] + e] : 0.f;
				mw[q] |= (e < nv[q] ? (uint32_t)pr.lv[0].mask[kk[q] + e] : 0u) << (8 * e);
			}
		}
	}
#pragma unroll
	for (int q = 0; q < TPB; q++) {
		if (!nv[q]) continue;
		const ProbDev &pr = P[tt[q].x];
		float v[4];
#pragma unroll
		for (int e = 0; e < 4; e++)   // U is read (and rounded) at the unknowns only
			v[e] = ((mw[q] >> (8 * e)) & 1u) ? (pr.kind == 0 ? uff(pr)[kk[q] + e].x : (float)pr.U[kk[q] + e])
					: gv[q][e];
		if (nv[q] == 4 && pr.vec4)
			*(float4 *)(pr.out + kk[q]) = make_float4(v[0], v[1], v[2], v[3]);
		else
			for (int e = 0; e < nv[q]; e++) pr.out[kk[q] + e] = v[e];
	}
}

// Adjoint scatter (5-point): grad_in = grad_out + sum of lambda over the
// unknown 5-neighbours at the known pixels, 0 at the unknowns; grad_dat =
// -lambda at the unknowns, 0 elsewhere.
__global__ void k_adjoint_scatter(const ProbDev *__restrict__ P, const int4 *__restrict__ all, int nall,
		const float *const *__restrict__ gout, float *const *__restrict__ gin, float *const *__restrict__ gdat)
{
	for (int q = 0; q < TPB; q++) {   // TPB tiles per block
		const int b = blockIdx.x * TPB + q;
		if (b >= nall) return;
		const int4 t = all[b];
		const ProbDev &pr = P[t.x];
		const uint8_t *m = pr.lv[0].mask;
		const int w = pr.w, h = pr.h;
		const int i = tile_i(t);
		for (int r = 0; r < SP_ROWS; r++) {
			const int j = tile_j(t, r);
			if (i >= w || j >= h) continue;
			const size_t k = (size_t)j * w + i;
			const float2 *U2 = uff(pr);   // the adjoint is of the 5-point fill
			if (m[k]) {
				gin[t.x][k] = 0.f;
				if (gdat[t.x]) gdat[t.x][k] = -U2[k].x;
				continue;
			}
			const bool e = i + 1 < w && m[k + 1], wn = i > 0 && m[k - 1];
			const bool sn = j + 1 < h && m[k + w], nn = j > 0 && m[k - w];
			if (e || wn || sn || nn) {   // float-float sums only next to an unknown
				FF s = {gout[t.x][k], 0.f};
				if (e) s = ff_add(s, FF{U2[k + 1].x, U2[k + 1].y});
				if (wn) s = ff_add(s, FF{U2[k - 1].x, U2[k - 1].y});
				if (sn) s = ff_add(s, FF{U2[k + w].x, U2[k + w].y});
				if (nn) s = ff_add(s, FF{U2[k - w].x, U2[k - w].y});
				gin[t.x][k] = s.hi;
			} else {
				gin[t.x][k] = gout[t.x][k];   // (float)(double)v == v
			}
			if (gdat[t.x]) gdat[t.x][k] = 0.f;
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
	int fused = 0;             // 5-point fused V-cycle (k_pre5/k_coarse5/k_post5)
	int nfine_max = 0;         // largest nfine over the problems
	int coarse_smem = 0;       // dynamic shared memory of k_coarse5
	struct KTimer *kt = nullptr;   // kernel timer, or null
	// device-driven solve: the loop counters are read back with the final
	// states (one synchronisation); the launch count is completed then
	const Globals *hg = nullptr;
	int pdl = 0;   // programmatic dependent launches between the V-cycle kernels
	int nu = NU5;  // 5-point smoothing sweeps per side of the V-cycle
	// problem groups: contiguous problem ranges solved as concurrent branches
	// of the solve graph, each with its own loop counters (gls[g]) and its
	// slice of every level's active tile list (stable compaction keeps a
	// problem's tiles together); a view of one group is a Plan itself
	int p0 = 0;                  // first problem of this view
	int ngroups = 1;
	int gp0[GMAX] = {}, gpn[GMAX] = {}, gnfine[GMAX] = {};
	// k_coarse5's threads per block, for the view (for each group): 1024 when a
	// problem runs level 0 in it (its PCG step and r.z are laid out for 1024
	// threads) or when the call has at most one problem per SM (each block's
	// levels then go faster on more warps); else 256, four blocks to an SM
	int coarse_nt = 1024, gcoarse_nt[GMAX] = {};
	int gbeg[GMAX][MAXLEV] = {}, gcnt[GMAX][MAXLEV] = {};
	Globals *gls = nullptr;      // GMAX loop-counter blocks (gl == gls: group 0)
	int *tbeg_rel = nullptr;     // level-0 tile offsets relative to the group's first tile
	int *pcnt = nullptr;         // active tiles per (level, problem)
};

// The view of problem group g: its problems, its tile-list slices, its loop
// counters, its slice of the reduction partials.
Plan group_view(const Plan &pl, int g)
{
	Plan v = pl;
	v.n = pl.gpn[g];
	v.p0 = pl.gp0[g];
	v.nfine_max = pl.gnfine[g];
	v.coarse_nt = pl.gcoarse_nt[g];
	for (int l = 0; l < MAXLEV; l++) {
		v.act[l] = pl.act[l] ? pl.act[l] + pl.gbeg[g][l] : nullptr;
		v.nact[l] = pl.gcnt[g][l];
	}
	v.gl = pl.gls + g;
	v.partial = pl.partial + 2 * (size_t)pl.gbeg[g][0];
	v.tbeg = pl.tbeg_rel;
	v.ngroups = 1;
	return v;
}

// Launch with programmatic stream serialisation when pdl is set (the kernel
// must call grid_wait() before its dependent accesses), else a plain launch.
template <typename... P, typename... A>
void launch_k(int pdl, void (*k)(P...), int grid, int block, size_t smem, cudaStream_t s, A... args)
{
	if (!pdl) {
		k<<<grid, block, smem, s>>>(args...);
		return;
	}
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(grid);
	cfg.blockDim = dim3(block);
	cfg.dynamicSmemBytes = smem;
	cfg.stream = s;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	cudaLaunchKernelEx(&cfg, k, args...);
}

// Kernel timer: an event pair around each launch of the main-loop kernels,
// with the launch's algorithmic bytes counted over the active tiles of the
// problems still iterating (read back before each launch group).
struct KTimer {
	struct Rec {
		const char *name;
		cudaEvent_t a, b;
		double bytes;
	};
	simpois_ctx *ctx;
	std::vector<Rec> recs;
	std::vector<int> tiles;         // tiles[l * n + p]: active tiles of problem p at level l
	std::vector<int> coarse_cells;  // cells of the k_coarse5 top level per problem
	std::vector<char> active;       // inner_active per problem (host copy)
	size_t next_ev = 0;
	int n = 0;
	cudaEvent_t ev()
	{
		if (next_ev == ctx->evpool.size()) {
			cudaEvent_t e;
			cudaEventCreate(&e);
			ctx->evpool.push_back(e);
		}
		return ctx->evpool[next_ev++];
	}
	double px(int l) const
	{
		double s = 0;
		for (int p = 0; p < n; p++)
			if (active[p]) s += (double)tiles[l * n + p] * SP_TILE * SP_TILE;
		return s;
	}
	double cells() const
	{
		double s = 0;
		for (int p = 0; p < n; p++)
			if (active[p]) s += coarse_cells[p];
		return s;
	}
};

// algorithmic bytes per tile pixel of each timed kernel (reads + writes)
constexpr double BPX_PRE5 = 1 + 4 + 4 + 0.25 + 1;         // mask, b, z; coarse mask, coarse b
constexpr double BPX_POST5 = 1 + 4 + 4 + 1 + 0.25 + 4;    // mask, b, z, coarse z2, coarse mask; z2
constexpr double BPX_SPMV5 = 1 + 4 + 4 + 4 + 4;           // mask, z2, p_old; p_new, q
constexpr double BPX_STEP = 4 + 4 + 4 + 4 + 1 + 4 + 4 + 4; // k_pre5's PCG step: q, x, xlo, p, mask; x, xlo, r
constexpr double BPX_RESID64 = 1 + 8 + 4 + 4 + 4 + 4;     // mask, U, rhs; b, x, xlo
constexpr double BPX_UADD = 1 + 8 + 4 + 4 + 8;            // mask, U, x, xlo; U
constexpr double BPX_PSPMV13 = 1 + 4 + 8 + 8 + 8;        // mask, z2, p_old; p_new, q (FP64)
constexpr double BPX_XR13 = 1 + 8 + 8 + 4 + 8 + 8 + 8 + 8 + 4 + 4; // mask, U, r, z2, p, q; U, r, b, x
constexpr double BPX_Z2B = 4 + 4;                         // z2; b
constexpr double BPX_RZ13 = 1 + 4 + 4;                    // mask, (float) r, z2
constexpr double BPC_COARSE5 = 1 + 4 + 4 + 0.34;          // per top coarse cell: mask, b; z2; coarser masks

#define KT_BEGIN(pl, s)                                            \
	cudaEvent_t kt_a_ = nullptr;                               \
	if ((pl).kt) {                                             \
		kt_a_ = (pl).kt->ev();                             \
		cudaEventRecord(kt_a_, s);                         \
	}
#define KT_END(pl, s, nm, by)                                      \
	if ((pl).kt) {                                             \
		cudaEvent_t kt_b_ = (pl).kt->ev();                 \
		cudaEventRecord(kt_b_, s);                         \
		(pl).kt->recs.push_back({nm, kt_a_, kt_b_, (by)}); \
	}

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
	const int NU = K == 0 ? pl.nu : NU13;
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
	k_xr<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl, 0); ++*pl.nl;
	launch_precond<K>(pl, opt, s);
	k_rz<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
}

// Fused 5-point V-cycle: k_pre5 down the fine levels, k_coarse5 for the rest,
// k_post5 back up; r.z and beta come out of k_post5 at level 0 (or k_coarse5
// for problems without fine levels).
// Kernel timer: refresh the host copy of which problems are still iterating.
void kt_refresh(const Plan &pl, cudaStream_t s)
{
	if (!pl.kt) return;
	std::vector<ProbState> h(pl.n);
	cudaMemcpyAsync(h.data(), pl.dst, sizeof(ProbState) * pl.n, cudaMemcpyDeviceToHost, s);
	cudaStreamSynchronize(s);
	for (int p = 0; p < pl.n; p++) pl.kt->active[p] = h[p].inner_active != 0;
}

// The refinement residual: the region-staged 5-point kernel, or the 13-point
// one (FP64).
template <int K>
void launch_resid(const Plan &pl, int nt, cudaStream_t s)
{
	if constexpr (K == 0)
		k_resid5<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl);
	else
		k_resid64<K><<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl);
	++*pl.nl;
}

// pcg = 0: the cycle is half of the biharmonic preconditioner and leaves the
// 5-point PCG scalars alone.  step: the cycle follows k_spmv5 (whose search
// direction is p2 when use_p2), so level 0 first takes the pending PCG step;
// it only changes the kernel timer's byte count (the kernels read `pending`).
void launch_vcycle_fused(const Plan &pl, cudaStream_t s, int pcg = 1, int use_p2 = 0, int step = 0)
{
	kt_refresh(pl, s);
	auto pre = pl.nu == 1 ? k_pre5<1> : pl.nu == 3 ? k_pre5<3> : k_pre5<2>;
	auto post = pl.nu == 1 ? k_post5<1> : pl.nu == 3 ? k_post5<3> : k_post5<2>;
	for (int l = 0; l < pl.nfine_max; l++) {
		if (!pl.nact[l]) continue;
		KT_BEGIN(pl, s);
		launch_k(pl.pdl, pre, pl.nact[l], SP_THREADS, 0, s, pl.dp, pl.dst, (const int4 *)pl.act[l], l,
				(const int *)pl.tbeg, (const int *)pl.tcnt, pl.partial, pl.gl, use_p2); ++*pl.nl;
		KT_END(pl, s, "k_pre5", pl.kt->px(l) * (BPX_PRE5 + (l == 0 && step ? BPX_STEP : 0.0)));
		if (l == 0 && pcg && step) {
			KT_BEGIN(pl, s);
			launch_k(pl.pdl, k_rr5, pl.n, SP_THREADS, 0, s, pl.dp, pl.dst, (const int *)pl.tbeg,
					(const int *)pl.tcnt, (const double *)pl.partial, pl.gl, pl.p0); ++*pl.nl;
			KT_END(pl, s, "k_rr5", 0.0);
		}
	}
	{
		KT_BEGIN(pl, s);
		// (the sweeps, restrictions and injections give the same bits with any
		// number of warps)
		launch_k(pl.pdl, k_coarse5, pl.n, pl.coarse_nt, pl.coarse_smem, s, (const ProbDev *)pl.dp,
				pl.dst, pl.gl, pcg,
				use_p2, pl.p0, pl.nu); ++*pl.nl;
		KT_END(pl, s, "k_coarse5", pl.kt->cells() * BPC_COARSE5);
	}
	for (int l = pl.nfine_max - 1; l >= 0; l--) {
		if (!pl.nact[l]) continue;
		KT_BEGIN(pl, s);
		launch_k(pl.pdl, post, pl.nact[l], SP_THREADS, 0, s, (const ProbDev *)pl.dp, pl.dst,
				(const int4 *)pl.act[l], l, (const int *)pl.tbeg, (const int *)pl.tcnt, pl.partial, pl.gl, pcg);
		++*pl.nl;
		KT_END(pl, s, "k_post5", pl.kt->px(l) * BPX_POST5);
		if (l == 0 && pcg) {
			KT_BEGIN(pl, s);
			launch_k(pl.pdl, k_beta5, pl.n, SP_THREADS, 0, s, (const ProbDev *)pl.dp, pl.dst,
					(const int *)pl.tbeg, (const int *)pl.tcnt, (const double *)pl.partial, pl.gl, pl.p0);
			++*pl.nl;
			KT_END(pl, s, "k_beta5", 0.0);
		}
	}
}

// Biharmonic preconditioner: z = V(V(r)) with V the fused 5-point V-cycle on
// b0 = (float) r (written by k_resid64 or k_xr13), then rho = r . z and beta.
void launch_precond_bih(const Plan &pl, cudaStream_t s)
{
	const int nt = pl.nact[0];
	launch_vcycle_fused(pl, s, 0);
	{
		KT_BEGIN(pl, s);
		launch_k(pl.pdl, k_z2b, nt, SP_THREADS, 0, s, (const ProbDev *)pl.dp, (const ProbState *)pl.dst,
				(const int4 *)pl.act[0]); ++*pl.nl;
		KT_END(pl, s, "k_z2b", pl.kt->px(0) * BPX_Z2B);
	}
	launch_vcycle_fused(pl, s, 0);
	{
		KT_BEGIN(pl, s);
		launch_k(pl.pdl, k_rz13, nt, SP_THREADS, 0, s, (const ProbDev *)pl.dp, pl.dst, (const int4 *)pl.act[0],
				(const int *)pl.tbeg, (const int *)pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
		KT_END(pl, s, "k_rz13", pl.kt->px(0) * BPX_RZ13);
	}
}

// Two FP64 biharmonic PCG iterations (the search direction alternates between
// p64 and p64b).
void launch_iteration_bih(const Plan &pl, cudaStream_t s)
{
	const int nt = pl.nact[0];
	for (int par = 0; par < 2; par++) {
		kt_refresh(pl, s);
		{
			KT_BEGIN(pl, s);
			// the first launch of the loop body follows no kernel of the body
			launch_k(par ? pl.pdl : 0, k_pspmv13, nt, SP_THREADS, 0, s, (const ProbDev *)pl.dp, pl.dst,
					(const int4 *)pl.act[0], (const int *)pl.tbeg, (const int *)pl.tcnt, pl.partial, pl.gl,
					par); ++*pl.nl;
			KT_END(pl, s, "k_pspmv13", pl.kt->px(0) * BPX_PSPMV13);
		}
		{
			KT_BEGIN(pl, s);
			launch_k(pl.pdl, k_xr13, nt, SP_THREADS, 0, s, (const ProbDev *)pl.dp, pl.dst, (const int4 *)pl.act[0],
					(const int *)pl.tbeg, (const int *)pl.tcnt, pl.partial, pl.gl, par); ++*pl.nl;
			KT_END(pl, s, "k_xr13", pl.kt->px(0) * BPX_XR13);
		}
		launch_precond_bih(pl, s);
	}
}

// Two fused PCG iterations (the search direction alternates between p and p2).
void launch_iteration_fused(const Plan &pl, cudaStream_t s)
{
	const int nt = pl.nact[0];
	for (int parity = 0; parity < 2; parity++) {
		kt_refresh(pl, s);
		{
			KT_BEGIN(pl, s);
			// the first launch of the loop body follows no kernel of the body
			launch_k(parity ? pl.pdl : 0, k_spmv5, nt, SP_THREADS, 0, s, (const ProbDev *)pl.dp, pl.dst,
					(const int4 *)pl.act[0], (const int *)pl.tbeg, (const int *)pl.tcnt, pl.partial, pl.gl,
					parity); ++*pl.nl;
			KT_END(pl, s, "k_spmv5", pl.kt->px(0) * BPX_SPMV5);
		}
		{
			KT_BEGIN(pl, s);
			launch_k(pl.pdl, k_alpha5, pl.n, SP_THREADS, 0, s, pl.dst, (const int *)pl.tbeg, (const int *)pl.tcnt,
					(const double *)pl.partial, pl.gl, pl.p0); ++*pl.nl;
			KT_END(pl, s, "k_alpha5", 0.0);
		}
		launch_vcycle_fused(pl, s, 1, parity, 1);
	}
}

enum { MODE_PLAIN = 0, MODE_FUSED5 = 1, MODE_BIH64 = 2 };

// Signature of everything a solve graph bakes into its kernel parameters.
std::string plan_signature(const simpois_ctx *ctx, const Plan &pl, int K, int fused, const MgOptions &opt)
{
	std::string sig;
	char buf[96];
	snprintf(buf, sizeof buf, "%p/%d/%d/%d/%d/%d/%d/%d/%d/%d/%d|", (void *)ctx->arena, pl.n, K, (int)fused,
			pl.nfine_max, pl.nlev_max, pl.coarse_smem, opt.use_mg, pl.pdl, pl.nu, pl.coarse_nt);
	sig += buf;
	const int ng = fused == MODE_FUSED5 || fused == MODE_BIH64 ? pl.ngroups : 1;
	for (int g = 0; g < ng && ng > 1; g++) {
		snprintf(buf, sizeof buf, "g%d:%d+%d:%d:%d|", g, pl.gp0[g], pl.gpn[g], pl.gnfine[g], pl.gcoarse_nt[g]);
		sig += buf;
		for (int l = 0; l < pl.nlev_max; l++) {
			snprintf(buf, sizeof buf, "%d+%d,", pl.gbeg[g][l], pl.gcnt[g][l]);
			sig += buf;
		}
	}
	snprintf(buf, sizeof buf, "%p/%p/%p/%p/%p/%p|", (void *)pl.dp, (void *)pl.dst, (void *)pl.gl, (void *)pl.tbeg,
			(void *)pl.tcnt, (void *)pl.partial);
	sig += buf;
	for (int l = 0; l < pl.nlev_max; l++) {
		snprintf(buf, sizeof buf, "%p:%d,", (void *)pl.act[l], pl.nact[l]);
		sig += buf;
	}
	return sig;
}

// Build the whole converged solve as one graph with two nested device-side
// WHILE loops: refinement steps (k_resid64, first V-cycle, the PCG loop, U +=
// x) while a problem is still refining, and PCG iterations while a problem's
// inner solve runs.  Both loops are bounded (gmax) besides the per-problem
// caps the kernels enforce.  Returns cudaErrorNotSupported-like failures to
// the caller, which then drives the loops from the host.
// Add one problem group's loops to the solve graph G: the refinement WHILE
// node (no dependencies: groups run concurrently) with the PCG WHILE node in
// its body.  n_outer / n_inner: kernel nodes of the two bodies.
template <int K>
cudaError_t add_solve_loops(cudaGraph_t G, cudaStream_t cs, Plan &pl, const MgOptions &opt, int mode,
		long long *n_outer, long long *n_inner)
{
	const int nt = pl.nact[0];
	cudaError_t e;
	cudaGraphConditionalHandle ho, hi;
	cudaGraphNodeParams po = {};
	cudaGraphNode_t node_o, node_i;
	cudaGraph_t body_o = nullptr, body_i = nullptr;
	if ((e = cudaGraphConditionalHandleCreate(&ho, G, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
	po.type = cudaGraphNodeTypeConditional;
	po.conditional.handle = ho;
	po.conditional.type = cudaGraphCondTypeWhile;
	po.conditional.size = 1;
	if ((e = cudaGraphAddNode(&node_o, G, nullptr, nullptr, 0, &po)) != cudaSuccess) return e;
	body_o = po.conditional.phGraph_out[0];
	// refinement body
	if ((e = cudaStreamBeginCaptureToGraph(cs, body_o, nullptr, nullptr, 0,
			cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
	cudaError_t ce = cudaGraphConditionalHandleCreate(&hi, body_o, 0, cudaGraphCondAssignDefault);
	long long c0 = *pl.nl;
	launch_resid<K>(pl, nt, cs);
	if (mode == MODE_FUSED5) {
		launch_vcycle_fused(pl, cs);
	} else if (mode == MODE_BIH64) {
		launch_precond_bih(pl, cs);
	} else {
		launch_precond<K>(pl, opt, cs);
		k_rz<<<nt, SP_THREADS, 0, cs>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
	}
	const int gmax_inner = mode == MODE_BIH64 ? INNER_MAX13 + 4 : 4 * INNER_MAX;
	k_setcond<<<1, 32, 0, cs>>>(hi, pl.gl, 0, 1, gmax_inner); ++*pl.nl;
	cudaStreamCaptureStatus cst;
	cudaGraph_t cg;
	const cudaGraphNode_t *deps = nullptr;
	size_t ndeps = 0;
	if (ce == cudaSuccess) ce = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &ndeps);
	cudaGraphNodeParams pi = {};
	pi.type = cudaGraphNodeTypeConditional;
	pi.conditional.handle = hi;
	pi.conditional.type = cudaGraphCondTypeWhile;
	pi.conditional.size = 1;
	if (ce == cudaSuccess) ce = cudaGraphAddNode(&node_i, cg, deps, nullptr, ndeps, &pi);
	if (ce == cudaSuccess) ce = cudaStreamUpdateCaptureDependencies(cs, &node_i, nullptr, 1,
			cudaStreamSetCaptureDependencies);
	if (mode != MODE_BIH64) {   // the FP64 biharmonic PCG updates U itself
		k_uadd<<<nt, SP_THREADS, 0, cs>>>(pl.dp, pl.dst, pl.act[0]); ++*pl.nl;
	}
	k_setcond<<<1, 32, 0, cs>>>(ho, pl.gl, 1, 0, MAX_OUTER + 2); ++*pl.nl;
	*n_outer = *pl.nl - c0;
	e = cudaStreamEndCapture(cs, &body_o);
	if (ce != cudaSuccess) e = ce;
	if (e != cudaSuccess) return e;
	body_i = pi.conditional.phGraph_out[0];
	// PCG body
	if ((e = cudaStreamBeginCaptureToGraph(cs, body_i, nullptr, nullptr, 0,
			cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
	c0 = *pl.nl;
	if (mode == MODE_FUSED5)
		launch_iteration_fused(pl, cs);
	else if (mode == MODE_BIH64)
		launch_iteration_bih(pl, cs);
	else
		launch_iteration<K>(pl, opt, cs);
	k_setcond<<<1, 32, 0, cs>>>(hi, pl.gl, 0, 0, gmax_inner); ++*pl.nl;
	*n_inner = *pl.nl - c0;
	return cudaStreamEndCapture(cs, &body_i);
}

// Build the whole converged solve as one graph: per problem group (one group
// unless the fused batch was split), two nested device-side WHILE
// loops -- refinement steps (k_resid64, first V-cycle, the PCG loop, U += x)
// while a problem of the group is still refining, and PCG iterations while a
// problem's inner solve runs.  The groups' loops are independent branches, so
// one group's latency-bound coarse levels overlap another's fine-level work.
// Both loops are bounded (gmax) besides the per-problem caps the kernels
// enforce.  Returns the CUDA error of a failed build; the caller then drives
// the loops from the host.
template <int K>
cudaError_t build_solve_graph(simpois_ctx *ctx, Plan &pl, const MgOptions &opt, int mode)
{
	cudaGraph_t G = nullptr;
	cudaError_t e = cudaGraphCreate(&G, 0);
	if (e != cudaSuccess) return e;
	const long long n0 = *pl.nl;
	const int ng = mode == MODE_FUSED5 || mode == MODE_BIH64 ? pl.ngroups : 1;
	long long no[GMAX] = {}, ni[GMAX] = {};
	for (int g = 0; g < ng && e == cudaSuccess; g++) {
		if (ng > 1) {
			Plan v = group_view(pl, g);
			e = add_solve_loops<K>(G, ctx->capture_stream, v, opt, mode, no + g, ni + g);
		} else {
			e = add_solve_loops<K>(G, ctx->capture_stream, pl, opt, mode, no + g, ni + g);
		}
	}
	if (e == cudaSuccess) {
		// a graph of the same topology as the cached one (a new mask of the
		// same sizes usually changes only grid sizes and slices) updates it in
		// place, which costs a fraction of an instantiation; else a new one
		bool updated = false;
		if (ctx->solve_exec && ctx->solve_groups == ng) {
			cudaGraphExecUpdateResultInfo info;
			if (cudaGraphExecUpdate(ctx->solve_exec, G, &info) == cudaSuccess)
				updated = true;
			else
				cudaGetLastError();
		}
		cudaGraphExec_t ex = nullptr;
		if (!updated && (e = cudaGraphInstantiate(&ex, G, 0)) == cudaSuccess) {
			if (ctx->solve_exec) cudaGraphExecDestroy(ctx->solve_exec);
			ctx->solve_exec = ex;
		}
		if (e == cudaSuccess) {
			ctx->solve_groups = ng;
			for (int g = 0; g < ng; g++) {
				ctx->solve_nodes_outer[g] = no[g];
				ctx->solve_nodes_inner[g] = ni[g];
			}
		}
	}
	*pl.nl = n0;
	cudaGraphDestroy(G);
	if (e != cudaSuccess) cudaGetLastError();
	return e;
}

// The converged solve as one graph launch and one synchronisation.
template <int K>
int run_device_loop(simpois_ctx *ctx, Plan &pl, const MgOptions &opt, int mode, bool *done)
{
	*done = false;
	const std::string sig = plan_signature(ctx, pl, K, mode, opt);
	if (!ctx->solve_exec || ctx->solve_sig != sig) {
		ctx->solve_sig.clear();
		if (build_solve_graph<K>(ctx, pl, opt, mode) != cudaSuccess) return SIMPOIS_OK;  // host loop instead
		ctx->solve_sig = sig;
	}
	cudaStream_t s = ctx->stream;
	SP_CUDA(ctx, cudaGraphLaunch(ctx->solve_exec, s));
	Globals *hg = (Globals *)ctx->pinned;   // read with the final states
	SP_CUDA(ctx, cudaMemcpyAsync(hg, pl.gls, sizeof(Globals) * ctx->solve_groups, cudaMemcpyDeviceToHost, s));
	pl.hg = hg;
	*done = true;
	return SIMPOIS_OK;
}

template <int K>
int run_kind(simpois_ctx *ctx, Plan &pl, const MgOptions &opt)
{
	cudaStream_t s = ctx->stream;
	int *hcount = (int *)ctx->pinned;
	const int nt = pl.nact[0];
	if (nt == 0) return SIMPOIS_OK;
	// MODE_FUSED5: 5-point, fused V-cycle; MODE_BIH64: 13-point FP64 PCG with
	// the squared 5-point V-cycle; MODE_PLAIN: per-sweep kernels (or no MG)
	const int mode = !opt.use_mg || !pl.fused ? MODE_PLAIN : (K == 0 ? MODE_FUSED5 : MODE_BIH64);
	const bool fused = mode == MODE_FUSED5;
	pl.pdl = !pl.kt && pdl_enabled();
	if (opt.use_graph && !pl.kt && !verbose()) {
		bool done = false;
		int r = run_device_loop<K>(ctx, pl, opt, mode, &done);
		if (r != SIMPOIS_OK || done) return r;
	}
	auto iteration = [&](cudaStream_t st) {
		if (fused)
			launch_iteration_fused(pl, st);
		else if (mode == MODE_BIH64)
			launch_iteration_bih(pl, st);
		else
			launch_iteration<K>(pl, opt, st);
	};
	cudaGraphExec_t gexec = nullptr;
	long long per_iter = 0;   // kernel nodes of one captured graph
	if (opt.use_graph && !pl.kt) {
		cudaGraph_t graph;
		long long before = *pl.nl;
		SP_CUDA(ctx, cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal));
		iteration(ctx->capture_stream);
		SP_CUDA(ctx, cudaStreamEndCapture(ctx->capture_stream, &graph));
		per_iter = *pl.nl - before;
		*pl.nl = before;
		cudaError_t e = cudaGraphInstantiate(&gexec, graph, 0);
		cudaGraphDestroy(graph);
		if (e != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
	}
	int rc = SIMPOIS_OK;
	for (int outer = 0; outer <= MAX_OUTER; outer++) {
		if (pl.kt) {   // the refinement step runs for every problem not yet converged
			std::vector<ProbState> h(pl.n);
			cudaMemcpyAsync(h.data(), pl.dst, sizeof(ProbState) * pl.n, cudaMemcpyDeviceToHost, s);
			cudaStreamSynchronize(s);
			for (int p = 0; p < pl.n; p++) pl.kt->active[p] = h[p].outer_active != 0;
		}
		{
			KT_BEGIN(pl, s);
			launch_resid<K>(pl, nt, s);
			KT_END(pl, s, K == 0 ? "k_resid5" : "k_resid64", pl.kt->px(0) * BPX_RESID64);
		}
		if (fused) {
			launch_vcycle_fused(pl, s);
		} else if (mode == MODE_BIH64) {
			launch_precond_bih(pl, s);
		} else {
			launch_precond<K>(pl, opt, s);
			k_rz<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0], pl.tbeg, pl.tcnt, pl.partial, pl.gl); ++*pl.nl;
		}
		cudaError_t e = cudaMemcpyAsync(hcount, &pl.gl->inner_count, sizeof(int), cudaMemcpyDeviceToHost, s);
		if (e == cudaSuccess) e = cudaStreamSynchronize(s);
		if (e != cudaSuccess) { rc = ctx_fail(ctx, SIMPOIS_ECUDA, "refinement: %s", cudaGetErrorString(e)); break; }
		if (verbose()) {
			std::vector<ProbState> h(pl.n);
			cudaMemcpy(h.data(), pl.dst, sizeof(ProbState) * pl.n, cudaMemcpyDeviceToHost);
			for (int p = 0; p < pl.n && p < 8; p++)
				fprintf(stderr, "simpois: problem %d refinement %d: rel %.3e, PCG iterations %d, "
						"last inner |r|^2 ratio %.3e, status %d\n", p, h[p].outer, h[p].rel,
						h[p].total_iter, h[p].tau2 > 0 ? h[p].rr / (h[p].tau2) : 0.0, h[p].status);
		}
		if (*hcount == 0) break;
		int chunk = 4;
		for (int guard = 0; guard < 4 * INNER_MAX13; guard++) {
			for (int c = 0; c < chunk; c++) {
				if (gexec) {
					e = cudaGraphLaunch(gexec, s);
					*pl.nl += per_iter;
				} else
					iteration(s), e = cudaGetLastError();
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
		if (pl.kt) {   // U += x runs for every problem still in the refinement
			std::vector<ProbState> h(pl.n);
			cudaMemcpyAsync(h.data(), pl.dst, sizeof(ProbState) * pl.n, cudaMemcpyDeviceToHost, s);
			cudaStreamSynchronize(s);
			for (int p = 0; p < pl.n; p++) pl.kt->active[p] = h[p].outer_active != 0;
		}
		if (mode != MODE_BIH64) {
			KT_BEGIN(pl, s);
			k_uadd<<<nt, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.act[0]); ++*pl.nl;
			KT_END(pl, s, "k_uadd", pl.kt->px(0) * BPX_UADD);
		}
	}
	if (gexec) cudaGraphExecDestroy(gexec);
	return rc;
}

// Fold the timer's records into the context's per-kernel totals.
void kt_collect(simpois_ctx *ctx, KTimer &kt)
{
	cudaStreamSynchronize(ctx->stream);
	for (const auto &r : kt.recs) {
		float ms = 0;
		cudaEventElapsedTime(&ms, r.a, r.b);
		bool found = false;
		for (auto &k : ctx->kstats)
			if (k.name == r.name) {
				k.launches++;
				k.ms += ms;
				k.bytes += r.bytes;
				found = true;
			}
		if (!found) ctx->kstats.push_back({r.name, 1, (double)ms, r.bytes});
	}
}

}  // namespace

// cuTensorMapEncodeTiled from the driver (the runtime is linked statically;
// the driver entry point needs no link against libcuda); null if absent.
PFN_cuTensorMapEncodeTiled_v12000 tma_encoder()
{
	static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
		void *f = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
				cudaSuccess || q != cudaDriverEntryPointSuccess)
			f = nullptr;
		return (PFN_cuTensorMapEncodeTiled_v12000)f;
	}();
	return fn;
}

// A 2-D tile map of a w x h level array (elem 4: float, 1: byte) with box bw x
// bh, zero fill outside; false where the layout allows none (the row stride
// must be a multiple of 16 bytes) or the driver refuses it.
bool tma_map(CUtensorMap *m, void *base, int w, int h, int elem, int bw, int bh)
{
	PFN_cuTensorMapEncodeTiled_v12000 fn = tma_encoder();
	if (!fn || ((size_t)w * elem) % 16 != 0 || ((uintptr_t)base & 15) != 0) return false;
	cuuint64_t dims[2] = {(cuuint64_t)w, (cuuint64_t)h}, strides[1] = {(cuuint64_t)w * elem};
	cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh}, es[2] = {1, 1};
	return fn(m, elem == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims,
			strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
			CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int mg_handover_level(int w, int h, int coarse_max)
{
	int lw[MAXLEV], lh[MAXLEV];
	const int nl = level_dims(w, h, lw, lh);
	return handover_level(lw, lh, nl, coarse_max > 0 ? clamp_coarse_max(coarse_max) : default_coarse_max());
}

int mg_default_coarse_max() { return default_coarse_max(); }

int mg_solve(simpois_ctx *ctx, const MgProblem *probs, int n, const MgOptions &opt, simpois_report *rep,
		double *bnorm2)
{
	if (n <= 0) return SIMPOIS_OK;
	cudaStream_t s = ctx->stream;
	Plan pl;
	pl.nl = &ctx->launches;
	pl.n = n;
	if (opt.nu < 0 || opt.nu > NU_MAX) return ctx_fail(ctx, SIMPOIS_EINVAL, "sweeps per side %d outside 1..%d", opt.nu, NU_MAX);
	pl.nu = opt.nu > 0 ? opt.nu : NU5;
	std::vector<ProbDev> hp(n);   // host image of the problem table
	int kinds = 0;
	Layout Lo;
	std::vector<size_t> off_mask[MAXLEV], off_code[MAXLEV], off_b[MAXLEV], off_z[MAXLEV], off_z2[MAXLEV];
	std::vector<size_t> off_U(n), off_x(n), off_xlo(n), off_p(n), off_q(n), off_p2(n), off_balt(n);
	std::vector<size_t> off_r64(n, 0), off_p64(n, 0), off_p64b(n, 0), off_q64(n, 0);
	size_t ntl[MAXLEV] = {};   // tiles per level over all problems
	const int cmax = opt.coarse_max > 0 ? clamp_coarse_max(opt.coarse_max) : default_coarse_max();
	for (int k = 0; k < n; k++) {
		const MgProblem &q = probs[k];
		int lw[MAXLEV], lh[MAXLEV];
		int nl = level_dims(q.w, q.h, lw, lh);
		ProbDev &d = hp[k];
		memset(&d, 0, sizeof(d));
		d.nlev = nl;
		d.kind = q.kind;
		d.w = q.w;
		d.h = q.h;
		d.rtol = q.rtol;
		d.tau_min = tau_min();
		kinds |= 1 << q.kind;
		pl.nlev_max = std::max(pl.nlev_max, nl);
		for (int l = 0; l < nl; l++) {
			size_t px = (size_t)lw[l] * lh[l];
			d.lv[l].w = lw[l];
			d.lv[l].h = lh[l];
			off_mask[l].push_back(Lo.take(px));
			off_code[l].push_back(Lo.take(px));
			off_b[l].push_back(Lo.take(px * 4));
			off_z[l].push_back(Lo.take(px * 4));
			off_z2[l].push_back(Lo.take(px * 4));
			ntl[l] += (size_t)ntiles(lh[l]) * ntiles(lw[l]);
		}
		for (int l = nl; l < MAXLEV; l++) {
			off_mask[l].push_back(0);
			off_code[l].push_back(0);
			off_b[l].push_back(0);
			off_z[l].push_back(0);
			off_z2[l].push_back(0);
		}
		// fused path: the tile kernels cover the levels above the hand-over
		d.nfine = handover_level(lw, lh, nl, cmax);
		pl.nfine_max = std::max(pl.nfine_max, d.nfine);
		{
			const CoarseLayout cl = coarse_layout(lw, lh, d.nfine, nl);
			pl.coarse_smem = std::max(pl.coarse_smem, cl.bytes);
			for (int l = d.nfine; l < nl; l++) {
				d.coff_b[l] = cl.off_b[l];
				d.coff_z[l] = cl.off_z[l];
				d.coff_m[l] = cl.off_m[l];
			}
		}
		size_t px = (size_t)q.w * q.h;
		off_U[k] = Lo.take(px * 8);
		off_x[k] = Lo.take(px * 4);
		off_xlo[k] = Lo.take(px * 4);
		off_p[k] = Lo.take(px * 4);
		off_q[k] = Lo.take(px * 4);
		off_p2[k] = Lo.take(px * 4);
		off_balt[k] = Lo.take(px * 4);
		if (q.kind == 1 && opt.fused && opt.use_mg) {   // FP64 Krylov vectors of the biharmonic PCG
			off_r64[k] = Lo.take(px * 8);
			off_p64[k] = Lo.take(px * 8);
			off_p64b[k] = Lo.take(px * 8);
			off_q64[k] = Lo.take(px * 8);
		}
	}
	if (kinds == 3) return ctx_fail(ctx, SIMPOIS_EINVAL, "a batch mixes 5-point and 13-point problems");
	const int K = kinds == 2 ? 1 : 0;
	pl.fused = opt.fused;   // 13-point problems use the 5-point cycle as preconditioner
	if (pl.fused) {
		cudaError_t e = cudaFuncSetAttribute(k_coarse5, cudaFuncAttributeMaxDynamicSharedMemorySize,
				pl.coarse_smem);
		if (e != cudaSuccess)
			return ctx_fail(ctx, SIMPOIS_ECUDA, "coarse kernel shared memory (%d B): %s", pl.coarse_smem,
					cudaGetErrorString(e));
	}
	// the small tables -- problem table, states, loop counters, tile counts
	// and offsets, the lists' pointer tables -- in one block of the arena,
	// mirrored in the staging buffer and uploaded with one copy
	Layout Tl;
	const size_t t_dp = Tl.take(sizeof(ProbDev) * n, 16), t_st = Tl.take(sizeof(ProbState) * n, 16);
	const size_t t_gl = Tl.take(sizeof(Globals) * GMAX, 16), t_pcnt = Tl.take(sizeof(int) * MAXLEV * n, 16);
	const size_t t_trel = Tl.take(sizeof(int) * n, 16), t_dnall = Tl.take(sizeof(int) * MAXLEV, 16);
	const size_t t_dnact = Tl.take(sizeof(int) * MAXLEV, 16), t_dall = Tl.take(sizeof(int4 *) * MAXLEV, 16);
	const size_t t_dact = Tl.take(sizeof(int4 *) * MAXLEV, 16), t_dflag = Tl.take(sizeof(int *) * MAXLEV, 16);
	const size_t t_tbeg = Tl.take(sizeof(int) * n, 16), t_tcnt = Tl.take(sizeof(int) * n, 16);
	const size_t t_loff = Tl.take(sizeof(int) * (MAXLEV * ((size_t)n + 1) + MAXLEV + 1), 16);
	const size_t tab_bytes = (Tl.off + 15) / 16 * 16;
	const size_t o_tab = Lo.take(tab_bytes);
	const size_t o_dp = o_tab + t_dp, o_st = o_tab + t_st, o_gl = o_tab + t_gl, o_pcnt = o_tab + t_pcnt;
	const size_t o_trel = o_tab + t_trel, o_dnall = o_tab + t_dnall, o_dnact = o_tab + t_dnact;
	const size_t o_dall = o_tab + t_dall, o_dact = o_tab + t_dact, o_dflag = o_tab + t_dflag;
	const size_t o_tbeg = o_tab + t_tbeg, o_tcnt = o_tab + t_tcnt;
	size_t o_all[MAXLEV], o_act[MAXLEV], o_flag[MAXLEV];
	// every level's tile list in one block (level after level), so that one
	// copy uploads them all
	size_t lbeg[MAXLEV + 1] = {};
	for (int l = 0; l < pl.nlev_max; l++) lbeg[l + 1] = lbeg[l] + ntl[l];
	const size_t o_lists = Lo.take(sizeof(int4) * std::max<size_t>(1, lbeg[pl.nlev_max]));
	for (int l = 0; l < pl.nlev_max; l++) {
		pl.nall[l] = (int)ntl[l];
		o_all[l] = o_lists + sizeof(int4) * lbeg[l];
		o_act[l] = Lo.take(sizeof(int4) * ntl[l]);
		o_flag[l] = Lo.take(sizeof(int) * ntl[l]);
	}
	size_t o_part = Lo.take(sizeof(double) * 2 * std::max<size_t>(1, ntl[0]));
	size_t o_gptr = Lo.take(sizeof(void *) * 3 * n);
	// TMA maps (b and code) of the tile levels whose rows are 16-byte multiples
	int nmaps = 0;
	for (int k = 0; k < n && opt.tma; k++)
		for (int l = 0; l < hp[k].nfine; l++)
			if (hp[k].lv[l].w % 16 == 0) nmaps += l == 0 ? 3 : 2;   // level 0: also b_alt
	size_t o_tmap = Lo.take(sizeof(CUtensorMap) * std::max(1, nmaps), 128);
	size_t total = Lo.off;
	int rc = ctx_arena_reserve(ctx, total);
	if (rc) return rc;
	char *A = ctx->arena;

	// host images of the device tables, staged in pinned memory
	size_t stage_bytes = sizeof(ProbDev) * n + sizeof(ProbState) * n + sizeof(Globals) * GMAX;
	stage_bytes += 64 * MAXLEV + sizeof(void *) * 3 * n + sizeof(int) * n + 16 * (MAXLEV + 16) + 4096;
	stage_bytes += sizeof(CUtensorMap) * nmaps + 128;
	stage_bytes += sizeof(int) * (MAXLEV + 1) * n + 64;   // per-problem tile counts, group offsets
	stage_bytes += tab_bytes;                              // the table block
	rc = ctx_pinned_reserve(ctx, stage_bytes + 256 * GMAX);
	if (rc) return rc;
	char *stage = ctx->pinned + 256 * GMAX;  // the first bytes hold read-back scalars

	for (int k = 0; k < n; k++) {
		ProbDev &d = hp[k];
		const MgProblem &q = probs[k];
		d.g = q.g;
		d.out = q.out;
		d.vec4 = q.w % 4 == 0 && ((uintptr_t)q.g & 15) == 0 && ((uintptr_t)q.out & 15) == 0;
		if (opt.mode == MG_ADJOINT) {
			d.rhs = opt.grad_out[k];
			d.rhs_sign = 1.f;
			d.known_zero = 1;
		} else {
			d.rhs = q.f;
			d.rhs_sign = -1.f;
			d.known_zero = 0;
		}
		d.U = (double *)(A + off_U[k]);
		d.x = (float *)(A + off_x[k]);
		d.xlo = (float *)(A + off_xlo[k]);
		d.p = (float *)(A + off_p[k]);
		d.q = (float *)(A + off_q[k]);
		d.p2 = (float *)(A + off_p2[k]);
		d.b_alt = (float *)(A + off_balt[k]);
		d.r64 = off_r64[k] ? (double *)(A + off_r64[k]) : nullptr;
		d.p64 = off_p64[k] ? (double *)(A + off_p64[k]) : nullptr;
		d.p64b = off_p64b[k] ? (double *)(A + off_p64b[k]) : nullptr;
		d.q64 = off_q64[k] ? (double *)(A + off_q64[k]) : nullptr;
		for (int l = 0; l < d.nlev; l++) {
			d.lv[l].mask = (uint8_t *)(A + off_mask[l][k]);
			d.lv[l].code = (uint8_t *)(A + off_code[l][k]);
			d.lv[l].b = (float *)(A + off_b[l][k]);
			d.lv[l].z = (float *)(A + off_z[l][k]);
			d.lv[l].z2 = (float *)(A + off_z2[l][k]);
			d.lv[l].tmb = d.lv[l].tmc = nullptr;
		}
		d.tmb_alt = nullptr;
	}
	// the TMA maps: encoded on the host, uploaded with the tables
	std::vector<CUtensorMap> maps(std::max(1, nmaps));
	{
		CUtensorMap *dmaps = (CUtensorMap *)(A + o_tmap);
		int im = 0;
		for (int k = 0; k < n && opt.tma; k++) {
			ProbDev &d = hp[k];
			for (int l = 0; l < d.nfine; l++) {
				LevelDev &L = d.lv[l];
				if (L.w % 16 != 0) continue;
				const int nm = l == 0 ? 3 : 2;
				// level 0 swaps b with b_alt every PCG step, so both get a map
				constexpr int FR = Geo<2>::FR;   // the TMA boxes of the halo-4 region
				if (tma_map(&maps[im], L.b, L.w, L.h, 4, FR, FR) &&
						tma_map(&maps[im + 1], L.code, L.w, L.h, 1, 64, FR) &&
						(l != 0 || tma_map(&maps[im + 2], d.b_alt, L.w, L.h, 4, FR, FR))) {
					L.tmb = dmaps + im;
					L.tmc = dmaps + im + 1;
					if (l == 0) d.tmb_alt = dmaps + im + 2;
				}
				im += nm;
			}
		}
	}
	pl.dp = (ProbDev *)(A + o_dp);
	pl.dst = (ProbState *)(A + o_st);
	pl.gls = (Globals *)(A + o_gl);
	pl.gl = pl.gls;
	pl.pcnt = (int *)(A + o_pcnt);
	pl.tbeg_rel = (int *)(A + o_trel);
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

	// stage and upload: the table block, then (maps, adjoint pointers) after it
	size_t so = tab_bytes;
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
	{
		// loop counters, per-problem tile counts, group offsets, active
		// counts and tile counts start at 0; tile begins at INT_MAX
		char *tab = stage;
		memset(tab, 0, tab_bytes);
		memcpy(tab + t_dp, hp.data(), sizeof(ProbDev) * n);
		memcpy(tab + t_st, hst.data(), sizeof(ProbState) * n);
		memcpy(tab + t_dnall, pl.nall, sizeof(int) * MAXLEV);
		memcpy(tab + t_dall, pl.all, sizeof(int4 *) * MAXLEV);
		memcpy(tab + t_dact, pl.act, sizeof(int4 *) * MAXLEV);
		memcpy(tab + t_dflag, pl.flag, sizeof(int *) * MAXLEV);
		int *tb = (int *)(tab + t_tbeg);
		for (int k = 0; k < n; k++) tb[k] = INT_MAX;
		// the tile lists' layout: every level's first entry, then per level
		// each problem's first entry within it (a problem without the level
		// has none)
		int *lb = (int *)(tab + t_loff), *lo = lb + MAXLEV + 1;
		for (int l = 0; l <= MAXLEV; l++) lb[l] = (int)lbeg[std::min(l, pl.nlev_max)];
		for (int l = 0; l < pl.nlev_max; l++) {
			int *o = lo + (size_t)l * (n + 1);
			o[0] = 0;
			for (int k = 0; k < n; k++)
				o[k + 1] = o[k] + (l < hp[k].nlev ? ntiles(hp[k].lv[l].w) * ntiles(hp[k].lv[l].h) : 0);
		}
		SP_CUDA(ctx, cudaMemcpyAsync(A + o_tab, tab, tab_bytes, cudaMemcpyHostToDevice, s));
	}
	if (nmaps) SP_CUDA(ctx, put(A + o_tmap, maps.data(), sizeof(CUtensorMap) * nmaps));
	// the tile lists, problem after problem in every level, written on the device
	const size_t nlist = lbeg[pl.nlev_max];
	if (nlist) {
		const int *dlb = (const int *)(A + o_tab + t_loff);
		k_fill_lists<<<(unsigned)std::min<size_t>((nlist + 255) / 256, 8 * (size_t)std::max(1, ctx->sm_count)), 256,
				0, s>>>(pl.dp, n, pl.nlev_max, dlb, dlb + MAXLEV + 1, (int4 *)(A + o_lists));
		++*pl.nl;
	}

	if (opt.mode == MG_ADJOINT) {
		pl.gout = (const float **)(A + o_gptr);
		pl.gin = (float **)(A + o_gptr) + n;
		pl.gdat = (float **)(A + o_gptr) + 2 * n;
		SP_CUDA(ctx, put(pl.gout, opt.grad_out, sizeof(void *) * n));
		SP_CUDA(ctx, put(pl.gin, opt.grad_in, sizeof(void *) * n));
		SP_CUDA(ctx, put(pl.gdat, opt.grad_dat, sizeof(void *) * n));
	}

	// masks, tile flags, compacted lists
	k_setup0<<<(pl.nall[0] + TPB - 1) / TPB, SP_THREADS, 0, s>>>(pl.dp, pl.dst, pl.all[0], pl.nall[0], pl.flag[0]);
	++*pl.nl;
	k_codes0<<<(pl.nall[0] + TPB - 1) / TPB, SP_THREADS, 0, s>>>(pl.dp, pl.all[0], pl.nall[0]); ++*pl.nl;
	for (int l = 1; l < pl.nlev_max; l++) {
		k_mask_down<<<pl.nall[l], SP_THREADS, 0, s>>>(pl.dp, pl.all[l], l, pl.flag[l]); ++*pl.nl;
	}
	k_compact<<<pl.nlev_max, 1024, 0, s>>>(pl.dall, pl.dflag, pl.dnall, pl.dact, pl.dnact, pl.tbeg, pl.tcnt,
			pl.pcnt, n); ++*pl.nl;
	k_init_counts<<<1, 256, 0, s>>>(pl.dst, pl.tcnt, n, pl.gl); ++*pl.nl;
	SP_LAUNCH_CHECK(ctx);
	int *hn = (int *)ctx->pinned;
	SP_CUDA(ctx, cudaMemcpyAsync(hn, pl.dnact, sizeof(int) * MAXLEV, cudaMemcpyDeviceToHost, s));
	int *hpc = (int *)stage;   // the uploads above are done with the staging by now (stream order)
	const bool grouped = n > 1 && groups_max() > 1 && opt.use_graph && !opt.ktimer && !verbose() && opt.use_mg &&
			pl.fused;
	if (grouped)
		SP_CUDA(ctx, cudaMemcpyAsync(hpc, pl.pcnt, sizeof(int) * MAXLEV * n, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	for (int l = 0; l < pl.nlev_max; l++) pl.nact[l] = hn[l];
	pl.ngroups = 1;
	pl.gp0[0] = 0;
	pl.gpn[0] = n;
	pl.gnfine[0] = pl.nfine_max;
	const bool many = n > std::max(1, ctx->sm_count);
	bool l0 = false;
	for (int k = 0; k < n; k++) l0 = l0 || hp[k].nfine == 0;
	pl.coarse_nt = many && !l0 ? 256 : 1024;
	pl.gcoarse_nt[0] = pl.coarse_nt;
	for (int l = 0; l < MAXLEV; l++) pl.gcnt[0][l] = pl.nact[l];
	if (grouped) {
		// contiguous problem ranges with about equal level-0 active tiles
		const int G = std::min(n, groups_max());
		long long tot = 0, acc = 0;
		for (int k = 0; k < n; k++) tot += hpc[k];
		int g = 0;
		pl.gpn[0] = 0;
		for (int k = 0; k < n; k++) {
			acc += hpc[k];
			pl.gpn[g]++;
			if (g + 1 < G && k + 1 < n && acc * G >= tot * (g + 1)) {
				g++;
				pl.gp0[g] = k + 1;
				pl.gpn[g] = 0;
			}
		}
		pl.ngroups = g + 1;
		int *hrel = hpc + MAXLEV * n;
		for (int gg = 0; gg < pl.ngroups; gg++) {
			pl.gnfine[gg] = 0;
			for (int l = 0; l < MAXLEV; l++) {
				int b = 0, c = 0;
				for (int k = 0; k < pl.gp0[gg]; k++) b += l < pl.nlev_max ? hpc[(size_t)l * n + k] : 0;
				for (int k = pl.gp0[gg]; k < pl.gp0[gg] + pl.gpn[gg]; k++)
					c += l < pl.nlev_max ? hpc[(size_t)l * n + k] : 0;
				pl.gbeg[gg][l] = b;
				pl.gcnt[gg][l] = c;
			}
			int r = 0;
			for (int k = pl.gp0[gg]; k < pl.gp0[gg] + pl.gpn[gg]; k++) {
				hrel[k] = r;   // a problem's level-0 tiles from its group's first
				r += hpc[k];
				pl.gnfine[gg] = std::max(pl.gnfine[gg], hp[k].nfine);
			}
			bool gl0 = false;
			for (int k = pl.gp0[gg]; k < pl.gp0[gg] + pl.gpn[gg]; k++) gl0 = gl0 || hp[k].nfine == 0;
			pl.gcoarse_nt[gg] = many && !gl0 ? 256 : 1024;
		}
		SP_CUDA(ctx, cudaMemcpyAsync(pl.tbeg_rel, hrel, sizeof(int) * n, cudaMemcpyHostToDevice, s));
		for (int gg = 0; gg < pl.ngroups; gg++) {
			k_init_counts<<<1, 256, 0, s>>>(pl.dst + pl.gp0[gg], pl.tcnt + pl.gp0[gg], pl.gpn[gg], pl.gls + gg);
			++*pl.nl;
		}
		SP_LAUNCH_CHECK(ctx);
	}

	KTimer kt;
	if (opt.ktimer) {
		kt.ctx = ctx;
		kt.n = n;
		kt.active.assign(n, 1);
		kt.tiles.assign((size_t)MAXLEV * n, 0);
		kt.coarse_cells.assign(n, 0);
		for (int l = 0; l < pl.nlev_max; l++) {
			if (!pl.nact[l]) continue;
			std::vector<int4> h(pl.nact[l]);
			SP_CUDA(ctx, cudaMemcpyAsync(h.data(), pl.act[l], sizeof(int4) * h.size(), cudaMemcpyDeviceToHost, s));
			SP_CUDA(ctx, cudaStreamSynchronize(s));
			for (const int4 &t : h) kt.tiles[(size_t)l * n + t.x]++;
		}
		for (int k = 0; k < n; k++) {
			const LevelDev &c = hp[k].lv[hp[k].nfine];
			kt.coarse_cells[k] = c.w * c.h;
		}
		pl.kt = &kt;
	}
	if (ctx->rhs_pending) {   // the data term is still arriving: the loops read it
		SP_CUDA(ctx, cudaStreamWaitEvent(s, ctx->rhs_pending, 0));
		ctx->rhs_pending = nullptr;
	}
	rc = K == 0 ? run_kind<0>(ctx, pl, opt) : run_kind<1>(ctx, pl, opt);
	if (rc) return rc;
	if (pl.kt) kt_collect(ctx, kt);

	if (opt.mode == MG_ADJOINT) {
		k_adjoint_scatter<<<(pl.nall[0] + TPB - 1) / TPB, SP_THREADS, 0, s>>>(pl.dp, pl.all[0], pl.nall[0], pl.gout,
				pl.gin, pl.gdat); ++*pl.nl;
	}
	else {
		k_finalize<<<(pl.nall[0] + TPB - 1) / TPB, SP_THREADS, 0, s>>>(pl.dp, pl.all[0], pl.nall[0]); ++*pl.nl;
	}
	SP_LAUNCH_CHECK(ctx);
	ProbState *hs = (ProbState *)stage;
	Globals *hgl = (Globals *)(stage + ((sizeof(ProbState) * n + 15) / 16 * 16));
	SP_CUDA(ctx, cudaMemcpyAsync(hs, pl.dst, sizeof(ProbState) * n, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaMemcpyAsync(hgl, pl.gls, sizeof(Globals) * GMAX, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	if (pl.hg)
		for (int g = 0; g < ctx->solve_groups; g++)
			*pl.nl += ctx->solve_nodes_outer[g] * pl.hg[g].n_outer + ctx->solve_nodes_inner[g] * pl.hg[g].n_inner;
	for (int g = 0; g < GMAX; g++)
		if (hgl[g].tma_timeout) return ctx_fail(ctx, SIMPOIS_ECUDA, "a TMA region load did not complete in time");
	for (int k = 0; k < n; k++) {
		rep[k].status = hs[k].status;
		rep[k].unknowns = hs[k].nunknown;
		rep[k].iterations = hs[k].total_iter;
		rep[k].refinements = hs[k].outer;
		rep[k].rel_residual = hs[k].rel;
		rep[k].rel_residual_out = -1;
		if (bnorm2) bnorm2[k] = hs[k].bnorm2;
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
