// common.cuh -- shared internals of libsimpois_gpu: the context, the device
// arena, error plumbing and the block-reduction helpers every solver kernel
// uses.  Target: sm_103a (GB300), one process per GPU.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/simpois_gpu.h"

// ---------------------------------------------------------------- context

struct simpois_ctx {
	int device = 0;
	cudaStream_t stream = nullptr;
	// private stream used only to capture CUDA graphs (capture is not
	// allowed on the legacy default stream); graphs replay on `stream`
	cudaStream_t capture_stream = nullptr;
	int sm_count = 0;
	std::string last_error;

	// device arena: one allocation reused by every solve on this context
	char *arena = nullptr;
	size_t arena_cap = 0;
	// largest arena the context may hold (simpois_set_memory_limit; 0: none)
	size_t arena_limit = 0;

	// pinned host staging for small read-backs (counts, flags, reports)
	char *pinned = nullptr;
	size_t pinned_cap = 0;

	// staging for the host-pointer entry point
	char *io = nullptr;
	size_t io_cap = 0;
	// the hole components of split biharmonic channels: labels, crops, table
	char *split = nullptr;
	size_t split_cap = 0;
	// its second stream (the output's known pixels go back while the solve
	// runs) and the events that order it with `stream`
	cudaStream_t aux_stream = nullptr;
	cudaEvent_t ev_in = nullptr, ev_out = nullptr, ev_rhs = nullptr;
	// set while the data term is still arriving on aux_stream: the next
	// converged solve waits for it before its first read of f (its setup
	// does not read f)
	cudaEvent_t rhs_pending = nullptr;


	// kernel launches issued (graph replays count their kernel nodes)
	long long launches = 0;

	// kernel timer (SIMPOIS_FLAG_KTIMER): per-kernel launches, CUDA-event
	// milliseconds and algorithmic bytes, accumulated across solves
	struct KStat {
		std::string name;
		long long launches;
		double ms, bytes;
	};
	std::vector<KStat> kstats;
	std::vector<cudaEvent_t> evpool;
	std::string kstats_json;

	// the last device-driven solve graph and the plan it was built for
	cudaGraphExec_t solve_exec = nullptr;
	std::string solve_sig;
	// kernel nodes of each problem group's refinement and PCG loop bodies
	long long solve_nodes_outer[16] = {}, solve_nodes_inner[16] = {};
	int solve_groups = 0;

	// fused V-cycle hand-over size: fixed by the caller (0: none), and the
	// autotuner's choice per batch shape
	int coarse_max_fixed = 0;
	// smoothing sweeps per side of the fused V-cycle: fixed by the caller (0:
	// none); with the hand-over, the autotuner's choice per batch shape
	int sweeps_fixed = 0;
	struct Tuned {
		int coarse_max, nu;
	};
	std::map<std::string, Tuned> tuned;
	// file the autotuner's choices are kept in ("": none)
	std::string tune_path;

	// the AMLE sweeps of the last call and the call they were captured for
	cudaGraphExec_t amle_exec = nullptr;
	std::string amle_sig;
};

// Record a message on the context and return the status.
int ctx_fail(simpois_ctx *ctx, int status, const char *fmt, ...);

// Ensure the arena holds at least `bytes`; the previous contents are lost.
int ctx_arena_reserve(simpois_ctx *ctx, size_t bytes);
int ctx_pinned_reserve(simpois_ctx *ctx, size_t bytes);
int ctx_io_reserve(simpois_ctx *ctx, size_t bytes);

#define SP_CUDA(ctx, call)                                                    \
	do {                                                                  \
		cudaError_t e_ = (call);                                      \
		if (e_ != cudaSuccess)                                        \
			return ctx_fail((ctx), SIMPOIS_ECUDA, "%s: %s (%s:%d)", \
				#call, cudaGetErrorString(e_), __FILE__,      \
				__LINE__);                                    \
	} while (0)

#define SP_LAUNCH_CHECK(ctx) SP_CUDA(ctx, cudaGetLastError())

// Bump allocator laid over the arena: offsets are planned on the host first
// (Layout::take), then bound to the arena base.
struct Layout {
	size_t off = 0;
	size_t take(size_t bytes, size_t align = 256)
	{
		off = (off + align - 1) / align * align;
		size_t o = off;
		off += bytes;
		return o;
	}
};

// ---------------------------------------------------------------- device helpers

#define SP_TILE 32          // tiles are 32 x 32 pixels
#define SP_BLOCK_X 32
#define SP_BLOCK_Y 8
#define SP_THREADS (SP_BLOCK_X * SP_BLOCK_Y)
#define SP_ROWS (SP_TILE / SP_BLOCK_Y)

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
	return v;
}

// Block sum of `v` over all threads of the block, returned to thread 0.
// Deterministic: fixed shuffle tree then a fixed order over the warps.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *sh)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	v = warp_sum(v);
	if (lane == 0) sh[warp] = v;
	__syncthreads();
	double r = 0;
	if (threadIdx.x == 0) {
#pragma unroll
		for (int k = 0; k < NT / 32; k++) r += sh[k];
	}
	__syncthreads();
	return r;
}

// ---------------------------------------------------------------- float-float sums
// A sum carried as hi + lo in two floats (about 48 significant bits) on the
// FP32 units.  FP64 arithmetic issues at about 1/70 of the FP32 rate on this
// GPU (and a float-to-double conversion costs as much), so the per-pixel
// terms of the FP32 PCG's dot products are accumulated this way and only the
// per-warp sums are converted to double for the rest of the reduction.
struct FF {
	float hi, lo;
};

// a + b exactly as hi + lo (TwoSum)
__device__ __forceinline__ FF ff_two_sum(float a, float b)
{
	const float s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	FF r;
	r.hi = s;
	r.lo = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
	return r;
}

// hi + lo with |lo| folded below half an ulp of hi (Fast2Sum)
__device__ __forceinline__ FF ff_norm(float hi, float lo)
{
	FF r;
	r.hi = __fadd_rn(hi, lo);
	r.lo = __fsub_rn(lo, __fsub_rn(r.hi, hi));
	return r;
}

// acc += a * b: the product split exactly by an FMA, added by TwoSum
__device__ __forceinline__ void ff_add_prod(FF &acc, float a, float b)
{
	const float p = __fmul_rn(a, b);
	const float e = __fmaf_rn(a, b, -p);
	const FF s = ff_two_sum(acc.hi, p);
	acc = ff_norm(s.hi, __fadd_rn(__fadd_rn(acc.lo, e), s.lo));
}

__device__ __forceinline__ FF ff_add(FF a, FF b)
{
	const FF s = ff_two_sum(a.hi, b.hi);
	return ff_norm(s.hi, __fadd_rn(__fadd_rn(a.lo, b.lo), s.lo));
}

// Block sum of float-float values (thread 0 gets the result): float-float
// across each warp and across the warps, on the FP32 pipe, and one conversion
// to double at the end.  (An FP64 instruction holds this GPU's FP64 pipe for
// tens of cycles: a double per warp made the reductions of the tile kernels
// occupy up to 30 % of it.)
template <int NT>
__device__ __forceinline__ double block_sum_ff(FF v, double *sh)
{
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		FF w;
		w.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
		w.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
		v = ff_add(v, w);
	}
	float2 *shf = reinterpret_cast<float2 *>(sh);   // NT / 32 <= 32 pairs
	if (lane == 0) shf[warp] = make_float2(v.hi, v.lo);
	__syncthreads();
	double r = 0;
	if (threadIdx.x == 0) {
		FF a = {shf[0].x, shf[0].y};
#pragma unroll
		for (int k = 1; k < NT / 32; k++) a = ff_add(a, FF{shf[k].x, shf[k].y});
		r = (double)a.hi + (double)a.lo;
	}
	__syncthreads();
	return r;
}

// Clamp-to-edge index (the Neumann extension of simpois.c:25-32).
__device__ __forceinline__ int clampi(int v, int n) { return v < 0 ? 0 : (v >= n ? n - 1 : v); }
