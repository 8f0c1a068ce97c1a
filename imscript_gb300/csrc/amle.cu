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
// does not depend on the order inside the class.  One launch updates one
// class of both iterates of every channel; the NITER x m launches of a call
// are one CUDA graph.  Every float operation is the reference's, in its order
// (round-to-nearest intrinsics, no contraction), so the output is bit for bit
// the colour-ordered restatement of the reference.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <string>

#include "common.cuh"
#include "solvers.h"

namespace {

// The neighbour table of get_nvals (src/amle.c:17-30): offsets and squared
// lengths, the weights of the midpoint.
constexpr int AMLE_MAXNN = 32;
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
		a.tinf[k] = u ? lo : v;
		a.tsup[k] = u ? (a.init ? a.init[k] : hi) : v;
		mine |= u;
	}
	if (__any_sync(0xffffffffu, mine) && (threadIdx.x & 31) == 0) atomicOr(&any, 1);
	__syncthreads();
	if (threadIdx.x == 0) a.tflag[(size_t)c * gridDim.x + t] = any;
}

// The reference's update of unknown (i, j) of x (amle_iteration's body):
// the first nn in-image neighbours in table order, the first minimum and the
// first maximum, (a v_min + b v_max) / (a + b) with a the weight of the
// maximum and b that of the minimum.
__device__ __forceinline__ float amle_new(const float *x, int w, int h, int i, int j, int nn)
{
	float vmin = 0.f, vmax = 0.f, wmin = 0.f, wmax = 0.f;
	int nv = 0;
	for (int p = 0; p < nn; p++) {
		const int ii = i + c_adi[p], jj = j + c_adj[p];
		if (ii < 0 || jj < 0 || ii >= w || jj >= h) continue;
		const float v = x[(size_t)jj * w + ii], wt = c_aw[p];
		if (nv == 0) {
			vmin = vmax = v;
			wmin = wmax = wt;
		} else {
			if (v < vmin) { vmin = v; wmin = wt; }
			if (v > vmax) { vmax = v; wmax = wt; }
		}
		nv++;
	}
	const float a = wmax, b = wmin;
	return __fdiv_rn(__fadd_rn(__fmul_rn(a, vmin), __fmul_rn(b, vmax)), __fadd_rn(a, b));
}

// One colour class of both iterates of every channel, in place.
__global__ void k_amle_sweep(AmleArgs a, int colour)
{
	const int c = blockIdx.y, t = blockIdx.x;
	if (!a.tflag[(size_t)c * gridDim.x + t]) return;
	const int tx = t % ntx(a.w), ty = t / ntx(a.w);
	const size_t off = (size_t)a.w * a.h * c;
	const int i = tx * SP_TILE + (threadIdx.x & 31);
	for (int r = 0; r < SP_ROWS; r++) {
		const int j = ty * SP_TILE + (threadIdx.x >> 5) + SP_BLOCK_Y * r;
		if (i >= a.w || j >= a.h) continue;
		const int col = (i + a.k * j) % a.m;
		const size_t k = off + (size_t)j * a.w + i;
		if (col != colour || !a.unk[k]) continue;
		const float ni = amle_new(a.tinf + off, a.w, a.h, i, j, a.nn);
		const float ns = amle_new(a.tsup + off, a.w, a.h, i, j, a.nn);
		a.tinf[k] = ni;
		a.tsup[k] = ns;
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
	// the sweeps: one graph of niter x m launches, cached while the call's
	// pointers and sizes are unchanged
	if (niter > 0) {
		char buf[256];
		snprintf(buf, sizeof buf, "%p/%p/%p/%p/%d/%d/%d/%d/%d", (void *)A, (const void *)in, (const void *)init,
				(void *)out, w, h, pd, nn, niter);
		if (!ctx->amle_exec || ctx->amle_sig != buf) {
			if (ctx->amle_exec) {
				cudaGraphExecDestroy(ctx->amle_exec);
				ctx->amle_exec = nullptr;
			}
			cudaStream_t cs = ctx->capture_stream;
			SP_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
			for (int it = 0; it < niter; it++)
				for (int c = 0; c < a.m; c++) k_amle_sweep<<<gt, SP_THREADS, 0, cs>>>(a, c);
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
		ctx->launches += (long long)niter * a.m;
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
