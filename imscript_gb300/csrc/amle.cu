// AMLE (absolutely minimizing Lipschitz extension) fill on the GPU: the work
// of imscript's amle (src/amle.c:196-246) for every channel of a planar image.
//
// The reference keeps a lower and an upper iterate (tinf, tsup), starting at
// the image's minimum and maximum on the unknowns (amle_init,
// src/amle.c:89-112), and sweeps both in place, raster order, NITER times:
// each unknown becomes the distance-weighted midpoint of the smallest and the
// largest of its first NN in-image neighbours (amle_iteration,
// src/amle.c:66-87).  Here a sweep visits the colour classes (i + k j) mod m
// in turn, (m, k) chosen so that no neighbour offset of the first NN falls in
// a pixel's own class: a class updates in parallel, in place, and the result
// does not depend on the order inside the class.  The sweeps are blocked in
// time: one launch loads a 32 x 32 tile of both iterates with a halo of r S
// pixels (r the reach of the neighbourhood) into shared memory, sorts its
// unknowns into per-colour lists, and takes S class updates there, each on
// the cells still far enough from the region's edge; after them the tile is
// exact and alone is written back (double-buffered: a tile's halo is other
// tiles' pixels).  The launches of a call are one CUDA graph.  The kernel is
// instantiated for NN = 4, 6, 8, 16, 26 and 32 with the neighbour table as
// compile-time constants (any other NN reads it at run time), and a tile
// whose region lies wholly in the image skips the bounds tests.  Every float
// operation is the reference's, in its order (round-to-nearest intrinsics, no
// contraction; a division by 2 or 4 as the exact multiplication by its
// reciprocal), so the output is bit for bit the colour-ordered restatement of
// the reference.
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <string>

#include "common.cuh"
#include "solvers.h"

namespace {

// The neighbour table of get_nvals (src/amle.c:17-30): offsets and squared
// lengths, the weights of the midpoint.
constexpr int AMLE_MAXNN = 32;
// Target halo of the fused sweeps (pixels): how many iterations one launch
// takes.  The grouping changes no result bit; SIMPOIS_AMLE_HALO (1..32)
// overrides the default 8.
int amle_halo()
{
	static int v = [] {
		const char *e = getenv("SIMPOIS_AMLE_HALO");
		int x = e ? atoi(e) : 8;
		return x < 1 ? 1 : (x > 32 ? 32 : x);
	}();
	return v;
}
__constant__ int8_t c_adi[AMLE_MAXNN] = {1, 0, -1, 0, 1, -1, -1, 1, 2, 1, 2, 1, -2, -1, -2, -1,
	3, 1, 3, 1, -3, -1, -3, -1, 3, 2, 3, 2, -3, -2, -3, -2};
__constant__ int8_t c_adj[AMLE_MAXNN] = {0, 1, 0, -1, 1, -1, 1, -1, 1, 2, -1, -2, -1, -2, 1, 2,
	1, 3, -1, -3, -1, -3, 1, 3, 2, 3, -2, -3, -2, -3, 2, 3};
__constant__ float c_aw[AMLE_MAXNN] = {1, 1, 1, 1, 2, 2, 2, 2, 5, 5, 5, 5, 5, 5, 5, 5,
	10, 10, 10, 10, 10, 10, 10, 10, 13, 13, 13, 13, 13, 13, 13, 13};
const int h_adi[AMLE_MAXNN] = {1, 0, -1, 0, 1, -1, -1, 1, 2, 1, 2, 1, -2, -1, -2, -1,
	3, 1, 3, 1, -3, -1, -3, -1, 3, 2, 3, 2, -3, -2, -3, -2};
const int h_adj[AMLE_MAXNN] = {0, 1, 0, -1, 1, -1, 1, -1, 1, 2, -1, -2, -1, -2, 1, 2,
	1, 3, -1, -3, -1, -3, 1, 3, 2, 3, -2, -3, -2, -3, 2, 3};

// The smallest m >= 2 (and k < m) with (di + k dj) mod m != 0 for every
// offset of the first nn neighbours.
void colouring(int nn, int *m, int *k)
{
	for (int mm = 2; mm < 64; mm++)
		for (int kk = 0; kk < mm; kk++) {
			bool ok = true;
			for (int p = 0; p < nn && ok; p++) ok = (h_adi[p] + kk * h_adj[p]) % mm != 0;
			if (ok) {
				*m = mm;
				*k = kk;
				return;
			}
		}
	*m = 2;
	*k = 1;
}

struct AmleArgs {
	int w, h, pd, nn, m, k;
	const float *in, *init;
	float *out, *tinf, *tsup;
	float *tinf2, *tsup2;   // the second buffers of the fused sweeps
	uint8_t *unk;
	unsigned int *mm;    // per channel: sortable keys of the minimum and the maximum
	int *tflag;          // per channel and tile: the tile holds an unknown
	double *part;        // per channel and tile: partial sums of |tinf - tsup|
	int *pcnt;           // per channel and tile: unknown pixels
	unsigned int *gmax;  // per channel: max |tinf - tsup| (float bits)
};

// float <-> unsigned key with the same order (NaN excluded by the caller)
__device__ __forceinline__ unsigned int fkey(float f)
{
	const unsigned int b = __float_as_uint(f);
	return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fdekey(unsigned int k)
{
	return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ __forceinline__ int ntx(int w) { return (w + SP_TILE - 1) / SP_TILE; }

// Per channel: minimum and maximum over the non-NaN pixels (get_minmax,
// src/amle.c:48-57; the min and max of a set do not depend on the order).
__global__ void k_amle_minmax(AmleArgs a)
{
	const int c = blockIdx.y;
	const size_t n = (size_t)a.w * a.h;
	const float *x = a.in + n * c;
	unsigned int lo = 0xffffffffu, hi = 0u;
	for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
		const float v = x[i];
		if (v == v) {
			const unsigned int key = fkey(v);
			lo = min(lo, key);
			hi = max(hi, key);
		}
	}
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		lo = min(lo, __shfl_down_sync(0xffffffffu, lo, o));
		hi = max(hi, __shfl_down_sync(0xffffffffu, hi, o));
	}
	if ((threadIdx.x & 31) == 0) {
		atomicMin(&a.mm[2 * c], lo);
		atomicMax(&a.mm[2 * c + 1], hi);
	}
}

// tinf = tsup = x at the known pixels, the minimum and the maximum (or the
// init image) at the unknowns; unknown mask; per-tile flags.
__global__ void k_amle_init(AmleArgs a)
{
	__shared__ int any;
	const int c = blockIdx.y, t = blockIdx.x, tx = t % ntx(a.w), ty = t / ntx(a.w);
	const size_t n = (size_t)a.w * a.h;
	if (threadIdx.x == 0) any = 0;
	__syncthreads();
	// no non-NaN pixel: +inf and -inf, as the reference's get_minmax leaves them
	const unsigned int klo = a.mm[2 * c], khi = a.mm[2 * c + 1];
	const float lo = klo == 0xffffffffu ? INFINITY : fdekey(klo);
	const float hi = khi == 0u ? -INFINITY : fdekey(khi);
	const int i = tx * SP_TILE + (threadIdx.x & 31);
	int mine = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		const int j = ty * SP_TILE + (threadIdx.x >> 5) + SP_BLOCK_Y * r;
		if (i >= a.w || j >= a.h) continue;
		const size_t k = n * c + (size_t)j * a.w + i;
		const float v = a.in[k];
		const bool u = v != v;
		a.unk[k] = u;
		const float vi = u ? lo : v, vs = u ? (a.init ? a.init[k] : hi) : v;
		a.tinf[k] = vi;
		a.tsup[k] = vs;
		a.tinf2[k] = vi;
		a.tsup2[k] = vs;
		mine |= u;
	}
	if (__any_sync(0xffffffffu, mine) && (threadIdx.x & 31) == 0) atomicOr(&any, 1);
	__syncthreads();
	if (threadIdx.x == 0) a.tflag[(size_t)c * gridDim.x + t] = any;
}

// Several half-sweeps of both iterates of one tile in shared memory
// (temporal blocking): the tile and a halo of H = r x S pixels, r the reach
// of the neighbourhood, are loaded once; half-sweep s (global number s0 + s)
// updates the class ((s0 + s) mod m) cells at distance >= r (s + 1) from the
// region's edge, whose
// neighbours all still hold the values the sequential order gives them, so
// after S half-sweeps the tile itself (distance >= H) is exact; it alone is
// written back.  The same updates, in the same class order, as S / m calls of
// one-class-per-launch sweep, with the iterates read and written once.  Tiles of a launch run concurrently and a tile's halo is other tiles'
// pixels, so the iterates are double-buffered (src -> dst); both buffers hold
// the same values outside the tiles with unknowns, which no launch touches.
// NN > 0: the neighbourhood size known at compile time (the loop over the
// neighbours unrolls); NN == 0: a.nn at run time.
// The neighbour table again, as compile-time constants for the kernels'
// unrolled interior path (offsets in table order, and their weights).
__device__ __forceinline__ int k_di(int p)
{
	const int t[AMLE_MAXNN] = {1, 0, -1, 0, 1, -1, -1, 1, 2, 1, 2, 1, -2, -1, -2, -1,
		3, 1, 3, 1, -3, -1, -3, -1, 3, 2, 3, 2, -3, -2, -3, -2};
	return t[p];
}
__device__ __forceinline__ int k_dj(int p)
{
	const int t[AMLE_MAXNN] = {0, 1, 0, -1, 1, -1, 1, -1, 1, 2, -1, -2, -1, -2, 1, 2,
		1, 3, -1, -3, -1, -3, 1, 3, 2, 3, -2, -3, -2, -3, 2, 3};
	return t[p];
}
__device__ __forceinline__ float k_w(int p)
{
	const float t[AMLE_MAXNN] = {1, 1, 1, 1, 2, 2, 2, 2, 5, 5, 5, 5, 5, 5, 5, 5,
		10, 10, 10, 10, 10, 10, 10, 10, 13, 13, 13, 13, 13, 13, 13, 13};
	return t[p];
}

// (wmx v_min + wmn v_max) / (wmx + wmn), the reference's midpoint.  The
// weights are 1, 2, 5, 10 or 13, so a denominator of 2 or 4 is a power of
// two: multiplying by its reciprocal gives the same float as dividing.
__device__ __forceinline__ float amle_mid(float mn, float mx, float wmn, float wmx)
{
	const float num = __fadd_rn(__fmul_rn(wmx, mn), __fmul_rn(wmn, mx));
	const float den = __fadd_rn(wmx, wmn);
	if (den == 2.f) return __fmul_rn(num, 0.5f);
	if (den == 4.f) return __fmul_rn(num, 0.25f);
	return __fdiv_rn(num, den);
}

template <int NN>
__global__ void __launch_bounds__(SP_THREADS) k_amle_fused(AmleArgs a, const float *__restrict__ sinf,
		const float *__restrict__ ssup, float *__restrict__ dinf, float *__restrict__ dsup, int r, int s0, int S)
{
	const int nn = NN > 0 ? NN : a.nn;
	extern __shared__ __align__(16) unsigned char smem[];
	__shared__ int cnt[64];
	const int c = blockIdx.y, t = blockIdx.x;
	if (!a.tflag[(size_t)c * gridDim.x + t]) return;
	const int tx = t % ntx(a.w), ty = t / ntx(a.w);
	const size_t off = (size_t)a.w * a.h * c;
	const int H = r * S, R = SP_TILE + 2 * H, N = R * R, m = a.m;
	const int cap = R * ((R + m - 1) / m);   // cells of one colour in the region, at most
	float *zi = (float *)smem, *zs = zi + N;
	int *lists = (int *)(zs + N);            // per colour: unknown cells, packed (q | ring << 16)
	const int x0 = tx * SP_TILE - H, y0 = ty * SP_TILE - H;
	const bool interior = x0 >= 0 && y0 >= 0 && x0 + R <= a.w && y0 + R <= a.h;
	for (int q = threadIdx.x; q < m; q += blockDim.x) cnt[q] = 0;
	__syncthreads();
	for (int q = threadIdx.x; q < N; q += blockDim.x) {
		const int ry = q / R, rx = q - ry * R, gi = x0 + rx, gj = y0 + ry;
		const bool in = gi >= 0 && gi < a.w && gj >= 0 && gj < a.h;
		const size_t k = in ? off + (size_t)gj * a.w + gi : 0;
		zi[q] = in ? sinf[k] : 0.f;
		zs[q] = in ? ssup[k] : 0.f;
		if (in && a.unk[k]) {
			const int ring = min(min(rx, ry), min(R - 1 - rx, R - 1 - ry));
			if (ring >= r) {   // cells nearer the edge are never updated
				const int col = (gi + a.k * gj) % m;
				const int e = atomicAdd(&cnt[col], 1);
				lists[col * cap + e] = q | (ring << 16);
			}
		}
	}
	__syncthreads();
	for (int s = 0; s < S; s++) {
		const int colour = (s0 + s) % m, lo = r * (s + 1), n = cnt[colour];
		const int *list = lists + colour * cap;
		for (int e = threadIdx.x; e < n; e += blockDim.x) {
			const int v = list[e];
			if ((v >> 16) < lo) continue;
			const int q = v & 0xffff;
			// the reference's update (amle_iteration's body) of both iterates:
			// the first nn in-image neighbours in table order, the first
			// minimum and the first maximum, (a v_min + b v_max) / (a + b)
			// with a the weight of the maximum and b that of the minimum
			if (NN > 0 && interior) {
				// every neighbour exists: the same first-minimum and
				// first-maximum scan, in table order, without the tests
				float mn0 = zi[q + 1], mx0 = mn0, mn1 = zs[q + 1], mx1 = mn1;
				float wmn0 = 1.f, wmx0 = 1.f, wmn1 = 1.f, wmx1 = 1.f;
#pragma unroll
				for (int p = 1; p < (NN > 0 ? NN : 1); p++) {
					const int qq = q + k_dj(p) * R + k_di(p);
					const float v0 = zi[qq], v1 = zs[qq], wt = k_w(p);
					if (v0 < mn0) { mn0 = v0; wmn0 = wt; }
					if (v0 > mx0) { mx0 = v0; wmx0 = wt; }
					if (v1 < mn1) { mn1 = v1; wmn1 = wt; }
					if (v1 > mx1) { mx1 = v1; wmx1 = wt; }
				}
				if (NN == 4) {
					zi[q] = __fmul_rn(__fadd_rn(mn0, mx0), 0.5f);
					zs[q] = __fmul_rn(__fadd_rn(mn1, mx1), 0.5f);
				} else {
					zi[q] = amle_mid(mn0, mx0, wmn0, wmx0);
					zs[q] = amle_mid(mn1, mx1, wmn1, wmx1);
				}
				continue;
			}
			int gi = 0, gj = 0;
			if (!interior) {
				const int ry = q / R;
				gi = x0 + q - ry * R;
				gj = y0 + ry;
			}
			float mn0 = 0.f, mx0 = 0.f, mn1 = 0.f, mx1 = 0.f;
			float wmn0 = 0.f, wmx0 = 0.f, wmn1 = 0.f, wmx1 = 0.f;
			bool first = true;
#pragma unroll
			for (int p = 0; p < (NN > 0 ? NN : AMLE_MAXNN); p++) {
				if (NN == 0 && p >= nn) break;
				if (!interior) {
					const int ii = gi + c_adi[p], jj = gj + c_adj[p];
					if (ii < 0 || jj < 0 || ii >= a.w || jj >= a.h) continue;
				}
				const int qq = q + c_adj[p] * R + c_adi[p];
				const float v0 = zi[qq], v1 = zs[qq], wt = c_aw[p];
				if (first) {
					mn0 = mx0 = v0;
					mn1 = mx1 = v1;
					wmn0 = wmx0 = wmn1 = wmx1 = wt;
					first = false;
				} else {
					if (v0 < mn0) { mn0 = v0; wmn0 = wt; }
					if (v0 > mx0) { mx0 = v0; wmx0 = wt; }
					if (v1 < mn1) { mn1 = v1; wmn1 = wt; }
					if (v1 > mx1) { mx1 = v1; wmx1 = wt; }
				}
			}
			if (NN == 4 && !first) {
				// the 4-neighbourhood weighs every neighbour 1: (v_min + v_max) / 2
				zi[q] = __fmul_rn(__fadd_rn(mn0, mx0), 0.5f);
				zs[q] = __fmul_rn(__fadd_rn(mn1, mx1), 0.5f);
			} else {
				zi[q] = amle_mid(mn0, mx0, wmn0, wmx0);
				zs[q] = amle_mid(mn1, mx1, wmn1, wmx1);
			}
		}
		__syncthreads();
	}
	for (int q = threadIdx.x; q < SP_TILE * SP_TILE; q += blockDim.x) {
		const int i = tx * SP_TILE + (q & 31), j = ty * SP_TILE + (q >> 5);
		if (i < a.w && j < a.h) {
			const size_t k = off + (size_t)j * a.w + i;
			const int rq = ((q >> 5) + H) * R + (q & 31) + H;
			dinf[k] = zi[rq];
			dsup[k] = zs[rq];
		}
	}
}

// out = tsup; per tile the sum of |tinf - tsup| over its unknowns (double)
// and the channel's maximum.
__global__ void k_amle_finish(AmleArgs a)
{
	__shared__ double sh[32];
	const int c = blockIdx.y, t = blockIdx.x, tx = t % ntx(a.w), ty = t / ntx(a.w);
	const size_t off = (size_t)a.w * a.h * c;
	const int i = tx * SP_TILE + (threadIdx.x & 31);
	double s = 0;
	float mx = 0.f;
	int cu = 0;
	for (int r = 0; r < SP_ROWS; r++) {
		const int j = ty * SP_TILE + (threadIdx.x >> 5) + SP_BLOCK_Y * r;
		if (i >= a.w || j >= a.h) continue;
		const size_t k = off + (size_t)j * a.w + i;
		const float up = a.tsup[k];
		a.out[k] = up;
		if (a.unk[k]) {
			const float d = fabsf(__fsub_rn(a.tinf[k], up));
			s += d;
			mx = fmaxf(mx, d);
			cu++;
		}
	}
	s = block_sum<SP_THREADS>(s, sh);
	const double cd = block_sum<SP_THREADS>((double)cu, sh);
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
	if ((threadIdx.x & 31) == 0 && mx > 0.f) atomicMax(&a.gmax[c], __float_as_uint(mx));
	if (threadIdx.x == 0) {
		a.part[(size_t)c * gridDim.x + t] = s;
		a.pcnt[(size_t)c * gridDim.x + t] = (int)cd;
	}
}

}  // namespace

// dynamic shared memory of k_amle_fused for a region of side R, m colours:
// the two iterates and the per-colour cell lists
static int amle_smem(int R, int m) { return R * R * 8 + m * R * ((R + m - 1) / m) * 4; }

int amle_run(simpois_ctx *ctx, float *out, const float *in, int w, int h, int pd, int nn, int niter,
		const float *init, double *gap)
{
	if (nn < 0) nn = 0;
	if (nn > AMLE_MAXNN) nn = AMLE_MAXNN;
	if (niter < 0) niter = 0;
	cudaStream_t s = ctx->stream;
	const size_t n = (size_t)w * h * pd;
	const int ntiles = ((w + SP_TILE - 1) / SP_TILE) * ((h + SP_TILE - 1) / SP_TILE);
	Layout Lo;
	const size_t o_tinf = Lo.take(n * 4), o_tsup = Lo.take(n * 4), o_unk = Lo.take(n);
	const size_t o_tinf2 = Lo.take(n * 4), o_tsup2 = Lo.take(n * 4);
	const size_t o_mm = Lo.take(sizeof(unsigned int) * 2 * pd), o_gmax = Lo.take(sizeof(unsigned int) * pd);
	const size_t o_flag = Lo.take(sizeof(int) * (size_t)ntiles * pd);
	const size_t o_part = Lo.take(sizeof(double) * (size_t)ntiles * pd);
	const size_t o_pcnt = Lo.take(sizeof(int) * (size_t)ntiles * pd);
	int rc = ctx_arena_reserve(ctx, Lo.off);
	if (rc) return rc;
	char *A = ctx->arena;
	AmleArgs a;
	a.w = w;
	a.h = h;
	a.pd = pd;
	a.nn = nn;
	colouring(nn, &a.m, &a.k);
	a.in = in;
	a.init = init;
	a.out = out;
	a.tinf = (float *)(A + o_tinf);
	a.tsup = (float *)(A + o_tsup);
	a.tinf2 = (float *)(A + o_tinf2);
	a.tsup2 = (float *)(A + o_tsup2);
	a.unk = (uint8_t *)(A + o_unk);
	a.mm = (unsigned int *)(A + o_mm);
	a.gmax = (unsigned int *)(A + o_gmax);
	a.tflag = (int *)(A + o_flag);
	a.part = (double *)(A + o_part);
	a.pcnt = (int *)(A + o_pcnt);
	// min keys start at the top, max keys and the gap maxima at 0
	std::vector<unsigned int> mm0(2 * pd);
	for (int c = 0; c < pd; c++) {
		mm0[2 * c] = 0xffffffffu;
		mm0[2 * c + 1] = 0u;
	}
	SP_CUDA(ctx, cudaMemcpyAsync(a.mm, mm0.data(), sizeof(unsigned int) * 2 * pd, cudaMemcpyHostToDevice, s));
	SP_CUDA(ctx, cudaMemsetAsync(a.gmax, 0, sizeof(unsigned int) * pd, s));
	const dim3 gt(ntiles, pd);
	k_amle_minmax<<<dim3(std::max(1, std::min(ctx->sm_count * 4, (int)((size_t)w * h / 1024 + 1))), pd), 256, 0, s>>>(a);
	k_amle_init<<<gt, SP_THREADS, 0, s>>>(a);
	ctx->launches += 2;
	SP_LAUNCH_CHECK(ctx);
	// the sweeps: spl half-sweeps (colour classes, in order) per launch, a
	// halo of about amle_halo() pixels; the launches of a call in one graph,
	// cached while the call's pointers and sizes are unchanged
	int reach = 0;
	for (int p = 0; p < nn; p++) reach = std::max(reach, std::max(abs(h_adi[p]), abs(h_adj[p])));
	const long long total = (long long)niter * a.m;   // half-sweeps of the call
	const int spl = reach ? std::max(1, amle_halo() / reach) : (int)std::min<long long>(total, 1 << 20);
	const int launches = total > 0 ? (int)((total + spl - 1) / spl) : 0;
	if (total > 0) {
		const int Rmax = SP_TILE + 2 * reach * spl;
		const int smem_max = amle_smem(Rmax, a.m);
		auto kern = nn == 4 ? k_amle_fused<4> : nn == 6 ? k_amle_fused<6> : nn == 8 ? k_amle_fused<8>
				: nn == 16 ? k_amle_fused<16> : nn == 26 ? k_amle_fused<26> : nn == 32 ? k_amle_fused<32>
				: k_amle_fused<0>;
		SP_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
		char buf[256];
		snprintf(buf, sizeof buf, "%p/%p/%p/%p/%d/%d/%d/%d/%d/%d", (void *)A, (const void *)in,
				(const void *)init, (void *)out, w, h, pd, nn, niter, spl);
		if (!ctx->amle_exec || ctx->amle_sig != buf) {
			if (ctx->amle_exec) {
				cudaGraphExecDestroy(ctx->amle_exec);
				ctx->amle_exec = nullptr;
			}
			cudaStream_t cs = ctx->capture_stream;
			SP_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
			long long done = 0;
			for (int L = 0; L < launches; L++) {
				const int S = (int)std::min<long long>(spl, total - done), R = SP_TILE + 2 * reach * S;
				const bool even = (L & 1) == 0;
				kern<<<gt, SP_THREADS, amle_smem(R, a.m), cs>>>(a, even ? a.tinf : a.tinf2,
						even ? a.tsup : a.tsup2, even ? a.tinf2 : a.tinf, even ? a.tsup2 : a.tsup, reach,
						(int)(done % a.m), S);
				done += S;
			}
			cudaGraph_t g;
			SP_CUDA(ctx, cudaStreamEndCapture(cs, &g));
			cudaError_t e = cudaGraphInstantiate(&ctx->amle_exec, g, 0);
			cudaGraphDestroy(g);
			if (e != cudaSuccess) {
				ctx->amle_exec = nullptr;
				return ctx_fail(ctx, SIMPOIS_ECUDA, "AMLE graph: %s", cudaGetErrorString(e));
			}
			ctx->amle_sig = buf;
		}
		SP_CUDA(ctx, cudaGraphLaunch(ctx->amle_exec, s));
		ctx->launches += launches;
	}
	if (launches & 1) {   // the result is in the second buffers
		std::swap(a.tinf, a.tinf2);
		std::swap(a.tsup, a.tsup2);
	}
	k_amle_finish<<<gt, SP_THREADS, 0, s>>>(a);
	ctx->launches++;
	SP_LAUNCH_CHECK(ctx);
	if (gap) {
		std::vector<double> part((size_t)ntiles * pd);
		std::vector<int> pcnt((size_t)ntiles * pd);
		std::vector<unsigned int> gm(pd);
		SP_CUDA(ctx, cudaMemcpyAsync(part.data(), a.part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, s));
		SP_CUDA(ctx, cudaMemcpyAsync(pcnt.data(), a.pcnt, sizeof(int) * pcnt.size(), cudaMemcpyDeviceToHost, s));
		SP_CUDA(ctx, cudaMemcpyAsync(gm.data(), a.gmax, sizeof(unsigned int) * pd, cudaMemcpyDeviceToHost, s));
		SP_CUDA(ctx, cudaStreamSynchronize(s));
		for (int c = 0; c < pd; c++) {
			double sum = 0;
			long long cu = 0;
			for (int t = 0; t < ntiles; t++) {
				sum += part[(size_t)c * ntiles + t];
				cu += pcnt[(size_t)c * ntiles + t];
			}
			float mx;
			memcpy(&mx, &gm[c], sizeof mx);
			gap[2 * c] = mx;
			gap[2 * c + 1] = cu ? sum / (double)cu : 0.0;
		}
	}
	return SIMPOIS_OK;
}
