// noalloc.cu -- simpois_residual_device_noalloc: the FP64 relative residual
// of a float output, computed without allocating any memory.
//
// Why: simpois_residual_device takes its scratch (one pair of FP64 partial
// sums per block of 256 pixels, a completion counter and per-channel totals)
// from cudaMallocAsync.  Some callers cannot allocate device memory at the
// point where they check a result: processes whose device memory is fully
// reserved up front by another allocator or a fixed budget, code on a
// latency-critical path that must not enter the allocator, or any caller that
// forbids allocation calls between its own set-up and tear-down.  This entry
// point gives them the same numbers from a fixed scratch array that lives in
// the library itself.
//
// The scratch is the file-scope device array `g_resid_scratch` below:
// SCRATCH_BYTES = 1 MiB + 4 KiB, held on every GPU that loads the library until
// the process exits.  Limits that follow from it: at most 16,777,216 pixels
// per channel (one partial pair per 256 pixels, 65,536 pairs) and at most 64
// channels per call.  Larger requests are rejected with SIMPOIS_EINVAL before
// any work is issued.
//
// Every call shares that one array and leaves its contents behind; each call
// clears the counter it relies on before use.  Calls that overlap on the GPU
// (from two host threads, two contexts or two streams at the same time) race
// on the array: serialise them.
//
// Host code must not pass `g_resid_scratch` itself to a kernel: in host code
// that name is a host-side stand-in, not a device address.  The device address
// is looked up with cudaGetSymbolAddress once per device, on the first call
// made on that device, with that device current; make that first call before
// any stream capture begins on the device.
#include <mutex>

#include "common.cuh"

namespace {

constexpr int NA_THREADS = 256;
constexpr size_t NA_MAX_BLOCKS = 65536;                        // partial pairs
constexpr size_t NA_MAX_PIXELS = NA_MAX_BLOCKS * NA_THREADS;   // per channel
constexpr int NA_MAX_CHANNELS = 64;
constexpr int NA_MAX_DEVICES = 64;

// layout of the scratch array (in doubles)
constexpr size_t NA_PARTIAL_OFF = 0;                           // 2 per block
constexpr size_t NA_TOTAL_OFF = 2 * NA_MAX_BLOCKS;             // 2 per channel
constexpr size_t NA_COUNTER_OFF = NA_TOTAL_OFF + 2 * NA_MAX_CHANNELS;
constexpr size_t SCRATCH_DOUBLES = NA_COUNTER_OFF + 384;       // 1 MiB + 4 KiB
constexpr size_t SCRATCH_BYTES = SCRATCH_DOUBLES * sizeof(double);

static __device__ __align__(256) double g_resid_scratch[SCRATCH_DOUBLES];

__constant__ int8_t na_di13[12] = {1, 0, -1, 0, 1, 1, -1, -1, 2, 0, -2, 0};
__constant__ int8_t na_dj13[12] = {0, 1, 0, -1, 1, -1, 1, -1, 0, 2, 0, -2};
__constant__ float na_cf13[12] = {-8, -8, -8, -8, 2, 2, 2, 2, 1, 1, 1, 1};

// Per block: the FP64 sums over its unknown pixels of r^2 and b^2, where
// r = -f - A(u at the unknowns, g at the knowns) and b = -f - A(0 at the
// unknowns, g at the knowns), A the clamped 5-point -Laplacian (kind 0) or
// 13-point bilaplacian (kind 1); the last block of the grid to finish adds the
// partials in block order and writes the channel's totals.
template <int K>
__global__ void k_resid_noalloc(const float *__restrict__ u, const float *__restrict__ g,
		const float *__restrict__ f, int w, int h, double *scratch, int channel)
{
	__shared__ double sh[32];
	__shared__ bool am_last;
	double *partial = scratch + NA_PARTIAL_OFF;
	unsigned int *counter = (unsigned int *)(scratch + NA_COUNTER_OFF);
	size_t k = (size_t)blockIdx.x * NA_THREADS + threadIdx.x;
	double rr = 0, bb = 0;
	if (k < (size_t)w * h && isnan(g[k])) {
		const int i = (int)(k % w), j = (int)(k / w);
		auto at = [&](int a, int b, bool zero_unknown) -> double {
			int q = clampi(b, h) * w + clampi(a, w);
			float gv = g[q];
			if (isnan(gv)) return zero_unknown ? 0.0 : (double)u[q];
			return (double)gv;
		};
		auto apply = [&](bool zu) -> double {
			if (K == 0)
				return 4.0 * at(i, j, zu) - at(i + 1, j, zu) - at(i, j + 1, zu) - at(i - 1, j, zu) -
				       at(i, j - 1, zu);
			double r = 20.0 * at(i, j, zu);
			for (int s = 0; s < 12; s++) r += (double)na_cf13[s] * at(i + na_di13[s], j + na_dj13[s], zu);
			return r;
		};
		const double fk = f ? -(double)f[k] : 0.0;
		const double rk = fk - apply(false), bk = fk - apply(true);
		rr = rk * rk;
		bb = bk * bk;
	}
	const double s0 = block_sum<NA_THREADS>(rr, sh);
	const double s1 = block_sum<NA_THREADS>(bb, sh);
	if (threadIdx.x == 0) {
		partial[2 * blockIdx.x] = s0;
		partial[2 * blockIdx.x + 1] = s1;
		__threadfence();
		am_last = atomicAdd(counter, 1u) == gridDim.x - 1;
	}
	__syncthreads();
	if (!am_last) return;
	__threadfence();
	double a0 = 0, a1 = 0;
	for (int q = threadIdx.x; q < (int)gridDim.x; q += NA_THREADS) {
		a0 += __ldcg(partial + 2 * q);
		a1 += __ldcg(partial + 2 * q + 1);
	}
	a0 = block_sum<NA_THREADS>(a0, sh);
	a1 = block_sum<NA_THREADS>(a1, sh);
	if (threadIdx.x == 0) {
		scratch[NA_TOTAL_OFF + 2 * channel] = a0;
		scratch[NA_TOTAL_OFF + 2 * channel + 1] = a1;
		*counter = 0;
	}
}

std::mutex g_na_mu;
double *g_na_addr[NA_MAX_DEVICES];   // device address of the scratch, per device

// Device address of the scratch on the current device, looked up once per
// device and kept for the process's life.  A cudaDeviceReset unloads the
// library's module and with it this address: the entry point is not for use
// on a device after a reset (documented in the header).
int scratch_address(simpois_ctx *ctx, double **out)
{
	std::lock_guard<std::mutex> lock(g_na_mu);
	if (ctx->device < 0 || ctx->device >= NA_MAX_DEVICES)
		return ctx_fail(ctx, SIMPOIS_EINVAL, "device %d beyond the no-alloc table", ctx->device);
	if (!g_na_addr[ctx->device]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_resid_scratch);
		if (e != cudaSuccess || !p)
			return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
		g_na_addr[ctx->device] = (double *)p;
	}
	*out = g_na_addr[ctx->device];
	return SIMPOIS_OK;
}

}  // namespace

extern "C" int simpois_residual_device_noalloc(simpois_ctx *ctx, const float *u, const float *in,
		const float *dat, int w, int h, int pd, int kind, double *rel, double *bnorm)
{
	if (!ctx || !u || !in || !rel) return ctx_fail(ctx, SIMPOIS_EINVAL, "null context or buffer");
	if (w <= 0 || h <= 0 || pd <= 0)
		return ctx_fail(ctx, SIMPOIS_EINVAL, "bad image size %dx%dx%d", w, h, pd);
	if ((size_t)w * h > NA_MAX_PIXELS)
		return ctx_fail(ctx, SIMPOIS_EINVAL,
				"no-alloc residual: %dx%d = %zu pixels per channel exceeds the limit of %zu",
				w, h, (size_t)w * h, NA_MAX_PIXELS);
	if (pd > NA_MAX_CHANNELS)
		return ctx_fail(ctx, SIMPOIS_EINVAL, "no-alloc residual: %d channels exceed the limit of %d", pd,
				NA_MAX_CHANNELS);
	if (kind != 0 && kind != 1) return ctx_fail(ctx, SIMPOIS_EINVAL, "kind must be 0 or 1");
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	double *scratch = nullptr;
	int rc = scratch_address(ctx, &scratch);
	if (rc) return rc;
	cudaStream_t s = ctx->stream;
	// the completion counter must start at zero; a previous call leaves it at
	// zero, but the array's contents are not trusted across calls
	SP_CUDA(ctx, cudaMemsetAsync(scratch + NA_COUNTER_OFF, 0, sizeof(unsigned int), s));
	const size_t cs = (size_t)w * h;
	const unsigned nb = (unsigned)((cs + NA_THREADS - 1) / NA_THREADS);
	for (int l = 0; l < pd; l++) {
		const float *fl = dat ? dat + cs * l : nullptr;
		if (kind == 0)
			k_resid_noalloc<0><<<nb, NA_THREADS, 0, s>>>(u + cs * l, in + cs * l, fl, w, h, scratch, l);
		else
			k_resid_noalloc<1><<<nb, NA_THREADS, 0, s>>>(u + cs * l, in + cs * l, fl, w, h, scratch, l);
		ctx->launches++;
	}
	SP_LAUNCH_CHECK(ctx);
	double tot[2 * NA_MAX_CHANNELS];
	SP_CUDA(ctx, cudaMemcpyAsync(tot, scratch + NA_TOTAL_OFF, sizeof(double) * 2 * pd, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	for (int l = 0; l < pd; l++) {
		const double r2 = tot[2 * l], b2 = tot[2 * l + 1];
		if (bnorm) bnorm[l] = sqrt(b2);
		rel[l] = b2 > 0 ? sqrt(r2 / b2) : (r2 > 0 ? INFINITY : 0.0);
	}
	return SIMPOIS_OK;
}
