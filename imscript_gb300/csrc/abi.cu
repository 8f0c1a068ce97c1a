// abi.cu -- the C ABI of libsimpois_gpu (include/simpois_gpu.h): contexts,
// parameter handling, the host/device/batched entry points, the adjoint, and
// the drop-in poisson_solver_separable / poisson_rec symbols.
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <stdio.h>
#include <unistd.h>

#include "common.cuh"
#include "solvers.h"

// ------------------------------------------------------------------ context plumbing

int ctx_fail(simpois_ctx *ctx, int status, const char *fmt, ...)
{
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof buf, fmt, ap);
	va_end(ap);
	if (ctx) ctx->last_error = buf;
	return status;
}

int ctx_arena_reserve(simpois_ctx *ctx, size_t bytes)
{
	if (bytes <= ctx->arena_cap) return SIMPOIS_OK;
	// the caller's budget is checked before anything is freed or allocated
	if (ctx->arena_limit && bytes > ctx->arena_limit)
		return ctx_fail(ctx, SIMPOIS_ENOMEM, "%zu bytes of device memory needed, above the context's limit of %zu",
				bytes, ctx->arena_limit);
	if (ctx->arena) {
		cudaStreamSynchronize(ctx->stream);
		cudaFree(ctx->arena);
		ctx->arena = nullptr;
		ctx->arena_cap = 0;
	}
	size_t cap = bytes + bytes / 8 + (1 << 20);
	if (ctx->arena_limit && cap > ctx->arena_limit) cap = ctx->arena_limit;
	if (cudaMalloc((void **)&ctx->arena, cap) != cudaSuccess) {
		cudaGetLastError();
		return ctx_fail(ctx, SIMPOIS_ENOMEM, "cannot allocate %zu bytes of device memory", cap);
	}
	ctx->arena_cap = cap;
	return SIMPOIS_OK;
}

int ctx_pinned_reserve(simpois_ctx *ctx, size_t bytes)
{
	if (bytes <= ctx->pinned_cap) return SIMPOIS_OK;
	if (ctx->pinned) {
		cudaStreamSynchronize(ctx->stream);
		cudaFreeHost(ctx->pinned);
		ctx->pinned = nullptr;
		ctx->pinned_cap = 0;
	}
	size_t cap = bytes < 65536 ? 65536 : bytes + bytes / 4;
	if (cudaMallocHost((void **)&ctx->pinned, cap) != cudaSuccess) {
		cudaGetLastError();
		return ctx_fail(ctx, SIMPOIS_ENOMEM, "cannot allocate %zu bytes of pinned memory", cap);
	}
	ctx->pinned_cap = cap;
	return SIMPOIS_OK;
}

int ctx_io_reserve(simpois_ctx *ctx, size_t bytes)
{
	if (bytes <= ctx->io_cap) return SIMPOIS_OK;
	if (ctx->io) {
		cudaStreamSynchronize(ctx->stream);
		cudaFree(ctx->io);
		ctx->io = nullptr;
		ctx->io_cap = 0;
	}
	if (cudaMalloc((void **)&ctx->io, bytes) != cudaSuccess) {
		cudaGetLastError();
		return ctx_fail(ctx, SIMPOIS_ENOMEM, "cannot allocate %zu bytes of device memory", bytes);
	}
	ctx->io_cap = bytes;
	return SIMPOIS_OK;
}

namespace {

// per-channel NaN counts of a planar image
__global__ void k_count_nan(const float *__restrict__ g, size_t cs, int *__restrict__ counts)
{
	size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	int l = blockIdx.y;
	int c = (k < cs && isnan(g[cs * l + k])) ? 1 : 0;
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0 && c) atomicAdd(counts + l, c);
}

int check_dims(simpois_ctx *ctx, int w, int h, int pd)
{
	if (w <= 0 || h <= 0 || pd <= 0)
		return ctx_fail(ctx, SIMPOIS_EINVAL, "bad image size %dx%dx%d", w, h, pd);
	if ((long long)w * h >= (1LL << 31))
		return ctx_fail(ctx, SIMPOIS_EINVAL, "image of %dx%d exceeds 2^31 pixels per channel", w, h);
	return SIMPOIS_OK;
}

int worst(int a, int b) { return a > b ? a : b; }

// Reference schedule with per-channel unknown counts in the reports.
int run_reference(simpois_ctx *ctx, float *out, const float *in, const float *dat, int w, int h, int pd,
		const simpois_params *p, simpois_report *rep)
{
	size_t ws_bytes = ref_workspace_bytes(w, h, pd, dat != nullptr) + 256 * pd + 4096;
	int rc = ctx_arena_reserve(ctx, ws_bytes);
	if (rc) return rc;
	int *counts = (int *)(ctx->arena + ws_bytes - 256 * pd - 2048);
	SP_CUDA(ctx, cudaMemsetAsync(counts, 0, sizeof(int) * pd, ctx->stream));
	size_t cs = (size_t)w * h;
	dim3 G((unsigned)((cs + 255) / 256), pd);
	k_count_nan<<<G, 256, 0, ctx->stream>>>(in, cs, counts);
	ctx->launches++;
	SP_LAUNCH_CHECK(ctx);
	rc = ref_solve(ctx, out, in, dat, w, h, pd, p, rep, ctx->arena);
	if (rc) return rc;
	rc = ctx_pinned_reserve(ctx, 65536);
	if (rc) return rc;
	int *hc = (int *)ctx->pinned;
	SP_CUDA(ctx, cudaMemcpyAsync(hc, counts, sizeof(int) * pd, cudaMemcpyDeviceToHost, ctx->stream));
	SP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	for (int l = 0; l < pd; l++) {
		rep[l].unknowns = hc[l];
		rep[l].refinements = 0;
		rep[l].rel_residual = -1;
		rep[l].rel_residual_out = -1;
	}
	return SIMPOIS_OK;
}

// Converged schedule over the channels of several images; the singular
// channels (no known pixel) are redone with the reference schedule.
// Key of the tuning table: operator, V-cycle variant and every channel's shape.
std::string tune_key(const std::vector<MgProblem> &sub, int kind, const MgOptions &opt)
{
	std::string key = std::to_string(kind) + (opt.fused ? "f" : "u") + (opt.use_mg ? "m" : "c");
	char buf[32];
	for (const MgProblem &q : sub) {
		snprintf(buf, sizeof buf, "|%dx%d", q.w, q.h);
		key += buf;
	}
	return key;
}

// The autotuner: coordinate descent over the fused V-cycle's two launch
// choices.  First the hand-over size among the default, 32, 64 and 128 at the
// given sweeps per side (sizes that put the same levels in the same kernels
// are tried once; every size gives the same bits), then the sweeps per side,
// 1, 2 and 3, at the best hand-over (each count its own preconditioner: the
// iterates differ, every result meets the tolerance).  A candidate gets one
// untimed solve, which captures its solve graph, and the best of two timed
// ones (CUDA events on the context's stream around the whole call).  A choice
// the caller fixed is not tuned.  The batch is left solved with the chosen
// pair.
int tune_and_solve(simpois_ctx *ctx, const std::vector<MgProblem> &sub, MgOptions opt, simpois_report *r,
		double *bnorm2, bool tune_cm, bool tune_nu, int *chosen_cm, int *chosen_nu)
{
	cudaEvent_t a, b;
	SP_CUDA(ctx, cudaEventCreate(&a));
	if (cudaEventCreate(&b) != cudaSuccess) {
		cudaEventDestroy(a);
		return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaEventCreate");
	}
	int rc = SIMPOIS_OK;
	int last_cm = -1, last_nu = -1;   // the pair of the last solve
	auto timed = [&](int cm, int nu, float *best_ms) -> int {
		opt.coarse_max = cm;
		opt.nu = nu;
		int e = mg_solve(ctx, sub.data(), (int)sub.size(), opt, r, bnorm2);
		for (int k = 0; k < 2 && !e; k++) {
			float ms = 0;
			cudaEventRecord(a, ctx->stream);
			e = mg_solve(ctx, sub.data(), (int)sub.size(), opt, r, bnorm2);
			cudaEventRecord(b, ctx->stream);
			if (!e && (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess))
				e = ctx_fail(ctx, SIMPOIS_ECUDA, "autotuner timing: %s", cudaGetErrorString(cudaGetLastError()));
			*best_ms = k == 0 ? ms : std::min(*best_ms, ms);
		}
		last_cm = cm;
		last_nu = nu;
		return e;
	};
	const int nu0 = opt.nu > 0 ? opt.nu : 2;
	int best_cm = opt.coarse_max, best_nu = nu0;
	float best_ms = 0;
	bool have = false;
	if (tune_cm) {
		const int cands[] = {mg_default_coarse_max(), 32, 64, 128};
		std::vector<std::vector<int>> seen;
		for (int c : cands) {
			std::vector<int> nf;
			for (const MgProblem &q : sub) nf.push_back(mg_handover_level(q.w, q.h, c));
			if (std::find(seen.begin(), seen.end(), nf) != seen.end()) continue;
			seen.push_back(nf);
			float t = 0;
			if ((rc = timed(c, nu0, &t))) break;
			if (!have || t < best_ms) {
				best_ms = t;
				best_cm = c;
				have = true;
			}
		}
	}
	if (!rc && tune_nu) {
		for (int nu = 1; nu <= 3 && !rc; nu++) {
			if (have && nu == nu0) continue;   // measured above
			float t = 0;
			if ((rc = timed(best_cm, nu, &t))) break;
			if (!have || t < best_ms) {
				best_ms = t;
				best_nu = nu;
				have = true;
			}
		}
	}
	if (!rc && (last_cm != best_cm || last_nu != best_nu)) {
		opt.coarse_max = best_cm;
		opt.nu = best_nu;
		rc = mg_solve(ctx, sub.data(), (int)sub.size(), opt, r, bnorm2);
	}
	cudaEventDestroy(a);
	cudaEventDestroy(b);
	if (rc) return rc;
	*chosen_cm = best_cm;
	*chosen_nu = best_nu;
	return SIMPOIS_OK;
}

// ---------------------------------------------------------------- tuning file
// The autotuner's choices kept on disk, per device model: a text file
//
//   simpois-tune 1
//   device <compute capability> <SMs> <device name>
//   <hand-over> <sweeps> <batch-shape key>
//   ...
//
// A file written on another device model is read as empty (its timings do not
// carry over); a file whose first line is not the header, or with a malformed
// choice line, is an error.  Saving merges the file's current choices with the
// context's (the context's win) and replaces the file through a temporary one
// in the same directory, so concurrent writers lose at most each other's new
// entries, never the file.
static std::string device_line(const simpois_ctx *ctx)
{
	cudaDeviceProp pr;
	if (cudaGetDeviceProperties(&pr, ctx->device) != cudaSuccess) {
		cudaGetLastError();
		return "device unknown";
	}
	char buf[400];
	snprintf(buf, sizeof buf, "device %d.%d %d %s", pr.major, pr.minor, pr.multiProcessorCount, pr.name);
	return buf;
}

// Read the choices of `path` written for this device into `out`.  Returns
// SIMPOIS_OK (also for a missing file or another device's file).
static int tune_read(simpois_ctx *ctx, const std::string &path, std::map<std::string, simpois_ctx::Tuned> &out)
{
	FILE *f = fopen(path.c_str(), "r");
	if (!f) return SIMPOIS_OK;
	std::string line;
	auto getline = [&](std::string &l) -> bool {
		l.clear();
		int c;
		while ((c = fgetc(f)) != EOF && c != '\n') l.push_back((char)c);
		return c != EOF || !l.empty();
	};
	int rc = SIMPOIS_OK;
	if (!getline(line) || line != "simpois-tune 1") {
		rc = ctx_fail(ctx, SIMPOIS_EINVAL, "%s: not a tuning file", path.c_str());
	} else if (getline(line) && line == device_line(ctx)) {
		int ln = 2;
		while (getline(line)) {
			ln++;
			if (line.empty()) continue;
			int cm = 0, nu = 0, used = 0;
			if (sscanf(line.c_str(), "%d %d %n", &cm, &nu, &used) != 2 || used <= 0 ||
					(size_t)used >= line.size() || cm < 8 || cm > 128 || nu < 1 || nu > 3) {
				rc = ctx_fail(ctx, SIMPOIS_EINVAL, "%s:%d: malformed choice", path.c_str(), ln);
				break;
			}
			out[line.substr(used)] = {cm, nu};
		}
	}
	fclose(f);
	return rc;
}

static int tune_write(simpois_ctx *ctx)
{
	std::map<std::string, simpois_ctx::Tuned> all;
	tune_read(ctx, ctx->tune_path, all);   // a broken file is replaced
	for (const auto &kv : ctx->tuned) all[kv.first] = kv.second;
	char suffix[64];
	snprintf(suffix, sizeof suffix, ".tmp%ld.%p", (long)getpid(), (void *)ctx);
	const std::string tmp = ctx->tune_path + suffix;
	FILE *f = fopen(tmp.c_str(), "w");
	if (!f) return ctx_fail(ctx, SIMPOIS_EINVAL, "%s: cannot write", tmp.c_str());
	bool ok = fprintf(f, "simpois-tune 1\n%s\n", device_line(ctx).c_str()) > 0;
	for (const auto &kv : all)
		ok = ok && fprintf(f, "%d %d %s\n", kv.second.coarse_max, kv.second.nu, kv.first.c_str()) > 0;
	ok = (fclose(f) == 0) && ok;
	if (!ok || rename(tmp.c_str(), ctx->tune_path.c_str()) != 0) {
		remove(tmp.c_str());
		return ctx_fail(ctx, SIMPOIS_EINVAL, "%s: cannot write", ctx->tune_path.c_str());
	}
	return SIMPOIS_OK;
}

// ---------------------------------------------------------------- hole components
// A biharmonic channel whose unknowns form several groups that no stencil
// couples is several independent systems: the 13-point operator reaches 2
// pixels, the 5-point V-cycles of its preconditioner 1 (and their coarse
// levels only join cells whose children are all unknown).  Solved as one
// problem, every group iterates until the slowest converges (a thin scratch
// needs ~10 PCG iterations, a 1024-pixel hole hundreds); solved as separate
// problems in separate problem groups, each retires on its own.  The groups
// are found on a map of 8 x 8 pixel blocks: blocks holding an unknown, joined
// to their 8 neighbours (unknowns in blocks that do not touch are at least 9
// pixels apart).  Each group becomes a crop: its blocks' bounding box grown by
// the 13-point reach (2) and clipped to the image, so the known pixels its
// equations read are in the crop, and the image sides stay where they are (the
// operator's clamp).  In the crop, another group's unknowns read as known
// zeros: no equation of this group reaches them.  Each crop converges to the
// channel's relative residual, so the channel does: |r|^2 is the sum over the
// crops of |r_k|^2 <= rtol^2 |b_k|^2.
constexpr int HB = 8;   // block side of the component map
constexpr int SPLIT_MAX = 256;   // most components a channel is split into

// The block map: a thread per 8-pixel row of a block (two 16-byte loads when
// the image and its width keep rows aligned), the 8 rows of a block in 8
// consecutive lanes.
__global__ void k_block_any(const float *__restrict__ g, int w, int h, int bw, int nb, uint8_t *__restrict__ out)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	const int b = t >> 3, r = t & 7;
	bool u = false;
	if (b < nb) {
		const int bx = b % bw, by = b / bw, x = bx * HB, y = by * HB + r;
		if (y < h) {
			const float *row = g + (size_t)y * w + x;
			if ((w & 3) == 0 && ((uintptr_t)g & 15) == 0 && x + HB <= w) {
				const float4 a = *(const float4 *)row, c = *(const float4 *)(row + 4);
				u = isnan(a.x) || isnan(a.y) || isnan(a.z) || isnan(a.w) || isnan(c.x) || isnan(c.y) ||
						isnan(c.z) || isnan(c.w);
			} else {
				for (int k = 0; k < HB && x + k < w; k++) u = u || isnan(row[k]);
			}
		}
	}
	const unsigned any = __ballot_sync(0xffffffffu, u);
	if (r == 0 && b < nb) out[b] = (uint8_t)(((any >> (threadIdx.x & 24)) & 0xffu) != 0);
}

struct CropDev {
	const float *g, *f;         // the channel (device)
	float *out;                 // the channel's output
	float *cg, *cf, *cout;      // the crop's input, data term, output
	const int *label;           // the channel's block labels
	int w, x0, y0, cw, ch, bw, comp;
};

// crop input: the channel's pixels, another group's unknowns as known zeros
__global__ void k_crop_gather(const CropDev *__restrict__ cr)
{
	const CropDev c = cr[blockIdx.y];
	const size_t n = (size_t)c.cw * c.ch;
	for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
		const int y = (int)(k / c.cw), x = (int)(k - (size_t)y * c.cw);
		const int gx = c.x0 + x, gy = c.y0 + y;
		const size_t q = (size_t)gy * c.w + gx;
		float v = c.g[q];
		if (isnan(v) && c.label[(gy / HB) * c.bw + gx / HB] != c.comp) v = 0.f;
		c.cg[k] = v;
		if (c.cf) c.cf[k] = c.f[q];
	}
}

// the crop's unknowns into the channel's output
__global__ void k_crop_scatter(const CropDev *__restrict__ cr)
{
	const CropDev c = cr[blockIdx.y];
	const size_t n = (size_t)c.cw * c.ch;
	for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
		const int y = (int)(k / c.cw), x = (int)(k - (size_t)y * c.cw);
		const int gx = c.x0 + x, gy = c.y0 + y;
		const size_t q = (size_t)gy * c.w + gx;
		if (isnan(c.g[q]) && c.label[(gy / HB) * c.bw + gx / HB] == c.comp) c.out[q] = c.cout[k];
	}
}

struct HoleSplit {
	std::vector<MgProblem> probs;   // the problems to solve: whole channels and crops
	std::vector<int> owner;         // the channel (index into the input list) of each
	CropDev *table = nullptr;       // the crops (device), ncrop of them
	int ncrop = 0;
	unsigned gx = 1;                // blocks per crop of the gather and scatter
};

// Which operators' channels are split: SIMPOIS_SPLIT=0 none, 1 the
// biharmonic (the default), 2 both.
static bool split_enabled(int kind)
{
	static int v = [] {
		const char *e = getenv("SIMPOIS_SPLIT");
		return e ? atoi(e) : 1;
	}();
	return v >= 2 || (v == 1 && kind == 1);
}

// Split the channels of `sub` (one operator kind) into hole components;
// channels with one component stay whole.  The crops' inputs are gathered and
// the split channels' outputs hold their inputs (the known pixels) on return.
static int split_holes(simpois_ctx *ctx, const std::vector<MgProblem> &sub, HoleSplit &hs)
{
	cudaStream_t s = ctx->stream;
	const int n = (int)sub.size();
	std::vector<size_t> moff(n + 1, 0);
	std::vector<int> bws(n), bhs(n);
	for (int k = 0; k < n; k++) {
		bws[k] = (sub[k].w + HB - 1) / HB;
		bhs[k] = (sub[k].h + HB - 1) / HB;
		moff[k + 1] = moff[k] + (size_t)bws[k] * bhs[k];
	}
	int rc = ctx_pinned_reserve(ctx, moff[n] + 16);
	if (rc) return rc;
	uint8_t *maps = (uint8_t *)ctx->pinned;   // written by the kernel straight into page-locked memory
	for (int k = 0; k < n; k++) {
		const int nb = (int)(moff[k + 1] - moff[k]);
		k_block_any<<<(unsigned)((8 * (size_t)nb + 255) / 256), 256, 0, s>>>(sub[k].g, sub[k].w, sub[k].h, bws[k],
				nb, maps + moff[k]);
		ctx->launches++;
	}
	SP_LAUNCH_CHECK(ctx);
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	// components (8-neighbour flood fill) and their bounding boxes in blocks
	struct Comp { int ch, id, bx0, by0, bx1, by1; };
	std::vector<Comp> comps;
	std::vector<std::vector<int>> labels(n);
	std::vector<int> ncomp(n, 0), stack;
	for (int k = 0; k < n; k++) {
		const int bw = bws[k], bh = bhs[k];
		const uint8_t *m = maps + moff[k];
		std::vector<int> &lab = labels[k];
		lab.assign((size_t)bw * bh, -1);
		const size_t first = comps.size();
		for (int b0 = 0; b0 < bw * bh; b0++) {
			if (!m[b0] || lab[b0] >= 0) continue;
			Comp c = {k, ncomp[k]++, b0 % bw, b0 / bw, b0 % bw, b0 / bw};
			lab[b0] = c.id;
			stack.assign(1, b0);
			while (!stack.empty()) {
				const int b = stack.back();
				stack.pop_back();
				const int bx = b % bw, by = b / bw;
				c.bx0 = std::min(c.bx0, bx); c.bx1 = std::max(c.bx1, bx);
				c.by0 = std::min(c.by0, by); c.by1 = std::max(c.by1, by);
				for (int dy = -1; dy <= 1; dy++)
					for (int dx = -1; dx <= 1; dx++) {
						const int x = bx + dx, y = by + dy;
						if (x < 0 || y < 0 || x >= bw || y >= bh) continue;
						const int q = y * bw + x;
						if (m[q] && lab[q] < 0) {
							lab[q] = c.id;
							stack.push_back(q);
						}
					}
			}
			comps.push_back(c);
		}
		// one component (or none), or so many that the problems' overheads
		// would outweigh the retirements: solved whole (decided per channel,
		// so a channel's bits do not depend on the rest of the batch)
		if (ncomp[k] < 2 || ncomp[k] > SPLIT_MAX) {
			comps.resize(first);
			ncomp[k] = 1;
		}
	}
	hs.probs.clear();
	hs.owner.clear();
	hs.ncrop = (int)comps.size();
	for (int k = 0; k < n; k++)
		if (ncomp[k] < 2) {
			hs.probs.push_back(sub[k]);
			hs.owner.push_back(k);
		}
	if (!hs.ncrop) return SIMPOIS_OK;
	// device layout: labels of the split channels, the crops' buffers, the table
	Layout lo;
	std::vector<size_t> loff(n, 0), coff(comps.size());
	std::vector<CropDev> tab(comps.size());
	for (int k = 0; k < n; k++)
		if (ncomp[k] >= 2) loff[k] = lo.take(sizeof(int) * labels[k].size());
	for (size_t c = 0; c < comps.size(); c++) {
		const Comp &q = comps[c];
		const MgProblem &ch = sub[q.ch];
		CropDev &d = tab[c];
		d.x0 = std::max(0, q.bx0 * HB - 2);
		d.y0 = std::max(0, q.by0 * HB - 2);
		d.cw = std::min(ch.w, (q.bx1 + 1) * HB + 2) - d.x0;
		d.ch = std::min(ch.h, (q.by1 + 1) * HB + 2) - d.y0;
		d.w = ch.w;
		d.bw = bws[q.ch];
		d.comp = q.id;
		const size_t px = (size_t)d.cw * d.ch;
		coff[c] = lo.take(px * sizeof(float) * (ch.f ? 3 : 2));
	}
	const size_t otab = lo.take(sizeof(CropDev) * comps.size());
	if (lo.off > ctx->split_cap) {
		if (ctx->split) {
			cudaStreamSynchronize(s);
			cudaFree(ctx->split);
			ctx->split = nullptr;
			ctx->split_cap = 0;
		}
		const size_t cap = lo.off + lo.off / 8;
		if (cudaMalloc((void **)&ctx->split, cap) != cudaSuccess) {
			cudaGetLastError();
			return ctx_fail(ctx, SIMPOIS_ENOMEM, "cannot allocate %zu bytes of device memory", cap);
		}
		ctx->split_cap = cap;
	}
	char *B = ctx->split;
	for (int k = 0; k < n; k++) {
		if (ncomp[k] < 2) continue;
		SP_CUDA(ctx, cudaMemcpyAsync(B + loff[k], labels[k].data(), sizeof(int) * labels[k].size(),
				cudaMemcpyHostToDevice, s));
		// the known pixels of the output; the crops fill in the unknowns
		SP_CUDA(ctx, cudaMemcpyAsync(sub[k].out, sub[k].g, sizeof(float) * sub[k].w * sub[k].h,
				cudaMemcpyDeviceToDevice, s));
	}
	size_t most = 1;
	for (size_t c = 0; c < comps.size(); c++) {
		const MgProblem &ch = sub[comps[c].ch];
		CropDev &d = tab[c];
		const size_t px = (size_t)d.cw * d.ch;
		d.g = ch.g;
		d.f = ch.f;
		d.out = ch.out;
		d.label = (const int *)(B + loff[comps[c].ch]);
		d.cg = (float *)(B + coff[c]);
		d.cout = d.cg + px;
		d.cf = ch.f ? d.cout + px : nullptr;
		most = std::max(most, px);
		MgProblem q = ch;
		q.g = d.cg;
		q.f = d.cf;
		q.out = d.cout;
		q.w = d.cw;
		q.h = d.ch;
		hs.probs.push_back(q);
		hs.owner.push_back(comps[c].ch);
	}
	hs.table = (CropDev *)(B + otab);
	SP_CUDA(ctx, cudaMemcpyAsync(hs.table, tab.data(), sizeof(CropDev) * tab.size(), cudaMemcpyHostToDevice, s));
	hs.gx = (unsigned)std::min<size_t>(256, (most + 255) / 256);
	for (int c0 = 0; c0 < hs.ncrop; c0 += 65535) {   // the grid's y extent
		k_crop_gather<<<dim3(hs.gx, std::min(65535, hs.ncrop - c0)), 256, 0, s>>>(hs.table + c0);
		ctx->launches++;
	}
	SP_LAUNCH_CHECK(ctx);
	return SIMPOIS_OK;
}

// After the solve: the crops' unknowns into their channels' outputs, and one
// report per channel: the worst status, the largest iteration and refinement
// counts, the summed unknowns, and the channel's relative residual from its
// crops' (|r|^2 = sum |r_k|^2, |b|^2 = sum |b_k|^2); the residual of the float
// output, when asked for, is computed again on the whole channel.
static int split_finish(simpois_ctx *ctx, const HoleSplit &hs, const std::vector<simpois_report> &r,
		const std::vector<double> &bn2, const std::vector<MgProblem> &sub, simpois_report *out)
{
	const int n = (int)sub.size();
	for (int c0 = 0; c0 < hs.ncrop; c0 += 65535) {
		k_crop_scatter<<<dim3(hs.gx, std::min(65535, hs.ncrop - c0)), 256, 0, ctx->stream>>>(hs.table + c0);
		ctx->launches++;
	}
	SP_LAUNCH_CHECK(ctx);
	std::vector<int> parts(n, 0);
	std::vector<double> rr(n, 0.0), bb(n, 0.0);
	for (size_t q = 0; q < hs.probs.size(); q++) {
		const int c = hs.owner[q];
		simpois_report &o = out[c];
		const simpois_report &a = r[q];
		rr[c] += a.rel_residual * a.rel_residual * bn2[q];
		bb[c] += bn2[q];
		if (!parts[c]++) {
			o = a;
			continue;
		}
		if (a.status != SIMPOIS_OK && (o.status == SIMPOIS_OK || a.status == SIMPOIS_SINGULAR)) o.status = a.status;
		o.unknowns += a.unknowns;
		o.iterations = std::max(o.iterations, a.iterations);
		o.refinements = std::max(o.refinements, a.refinements);
	}
	std::vector<MgProblem> again;
	std::vector<int> which;
	for (int c = 0; c < n; c++) {
		if (parts[c] < 2) continue;
		out[c].rel_residual = bb[c] > 0 ? sqrt(rr[c] / bb[c]) : 0.0;
		if (out[c].rel_residual_out >= 0) {
			again.push_back(sub[c]);
			which.push_back(c);
		}
	}
	if (!again.empty()) {
		std::vector<const float *> u(again.size());
		std::vector<double> rel(again.size()), bn(again.size());
		for (size_t k = 0; k < again.size(); k++) u[k] = again[k].out;
		const int rc = mg_residual(ctx, again.data(), u.data(), (int)again.size(), rel.data(), bn.data());
		if (rc) return rc;
		for (size_t k = 0; k < again.size(); k++) out[which[k]].rel_residual_out = rel[k];
	}
	return SIMPOIS_OK;
}

int run_converged(simpois_ctx *ctx, const simpois_image *im, int n, const simpois_params *p,
		simpois_report *rep, int tune = 0, int *tuned_cm = nullptr, int *tuned_nu = nullptr)
{
	std::vector<MgProblem> probs;
	std::vector<int> img_of;
	for (int k = 0; k < n; k++) {
		float t = im[k].tstep;
		if (t < -1000)
			return ctx_fail(ctx, SIMPOIS_EINVAL,
				"the triharmonic operator (tstep < -1000) has no converged schedule; use rtol = 0");
		size_t cs = (size_t)im[k].w * im[k].h;
		for (int l = 0; l < im[k].pd; l++) {
			MgProblem q;
			q.g = im[k].in + cs * l;
			q.f = im[k].dat ? im[k].dat + cs * l : nullptr;
			q.out = im[k].out + cs * l;
			q.w = im[k].w;
			q.h = im[k].h;
			q.kind = t < 0 ? 1 : 0;
			q.rtol = im[k].rtol > 0 ? im[k].rtol : p->rtol;
			probs.push_back(q);
			img_of.push_back(k);
		}
	}
	MgOptions opt;
	opt.max_iter = p->max_iter > 0 ? p->max_iter : 500;
	opt.use_mg = !(p->flags & SIMPOIS_FLAG_NO_MG);
	// SIMPOIS_NO_GRAPH=1 issues every kernel eagerly (profilers cannot see
	// into graphs with conditional nodes); the kernels and results are the same
	const char *ng = getenv("SIMPOIS_NO_GRAPH");
	opt.use_graph = !(p->flags & SIMPOIS_FLAG_NO_GRAPH) && !(ng && atoi(ng) > 0);
	opt.out_resid = (p->flags & SIMPOIS_FLAG_OUT_RESID) != 0;
	opt.fused = !(p->flags & SIMPOIS_FLAG_UNFUSED);
	opt.ktimer = (p->flags & SIMPOIS_FLAG_KTIMER) != 0;
	opt.tma = (p->flags & SIMPOIS_FLAG_TMA) != 0;
	int rc = SIMPOIS_OK;
	// one batched solve per operator kind
	for (int kind = 0; kind < 2; kind++) {
		std::vector<MgProblem> sub;
		std::vector<int> where;
		for (size_t q = 0; q < probs.size(); q++)
			if (probs[q].kind == kind) {
				sub.push_back(probs[q]);
				where.push_back((int)q);
			}
		if (sub.empty()) continue;
		MgOptions o = opt;
		const std::string key = tune_key(sub, kind, opt);
		// biharmonic channels: each hole component its own problem
		HoleSplit hs;
		const bool split = o.fused && o.use_mg && split_enabled(kind);
		if (split) {
			if ((rc = split_holes(ctx, sub, hs))) return rc;
		} else {
			hs.probs = sub;
			for (size_t q = 0; q < sub.size(); q++) hs.owner.push_back((int)q);
		}
		std::vector<simpois_report> r(hs.probs.size());
		std::vector<double> bn2(hs.probs.size(), 0.0);
		const bool tunable = o.fused && o.use_mg && !o.ktimer;
		if (ctx->coarse_max_fixed > 0) o.coarse_max = ctx->coarse_max_fixed;
		if (ctx->sweeps_fixed > 0) o.nu = ctx->sweeps_fixed;
		const bool tune_cm = ctx->coarse_max_fixed <= 0, tune_nu = ctx->sweeps_fixed <= 0;
		// with a tuning file, a shape whose choice is known is not timed again
		const bool known = !ctx->tune_path.empty() && ctx->tuned.count(key);
		const bool tuning = tune && tunable && (tune_cm || tune_nu) && !known;
		if (tuning) {
			int bc = 0, bn = 0;
			rc = tune_and_solve(ctx, hs.probs, o, r.data(), bn2.data(), tune_cm, tune_nu, &bc, &bn);
			if (rc) return rc;
			ctx->tuned[key] = {bc, bn};
			o.coarse_max = bc;
			o.nu = bn;
			if (!ctx->tune_path.empty() && (rc = tune_write(ctx))) return rc;
		} else {
			auto it = ctx->tuned.find(key);
			if (it != ctx->tuned.end()) {
				if (tune_cm) o.coarse_max = it->second.coarse_max;
				if (tune_nu) o.nu = it->second.nu;
			}
			rc = mg_solve(ctx, hs.probs.data(), (int)hs.probs.size(), o, r.data(), bn2.data());
			if (rc) return rc;
		}
		std::vector<simpois_report> rs(sub.size());
		if ((rc = split_finish(ctx, hs, r, bn2, sub, rs.data()))) return rc;
		if (tuned_cm && (kind == 0 || tuned_cm[0] == 0))
			tuned_cm[0] = o.coarse_max > 0 ? o.coarse_max : mg_default_coarse_max();
		if (tuned_nu && (kind == 0 || tuned_nu[0] == 0)) tuned_nu[0] = o.nu > 0 ? o.nu : 2;
		for (size_t q = 0; q < sub.size(); q++) rep[where[q]] = rs[q];
	}
	// singular channels: the reference schedule, as the reference would run them
	for (size_t q = 0; q < probs.size(); q++) {
		if (rep[q].status != SIMPOIS_SINGULAR) continue;
		simpois_params pr = *p;
		pr.tstep = im[img_of[q]].tstep;
		pr.rtol = 0;
		simpois_report r1;
		rc = run_reference(ctx, probs[q].out, probs[q].g, probs[q].f, probs[q].w, probs[q].h, 1, &pr, &r1);
		if (rc) return rc;
		rep[q].iterations = r1.iterations;
	}
	return SIMPOIS_OK;
}

}  // namespace

// ------------------------------------------------------------------ public API

extern "C" {

void simpois_default_params(simpois_params *p)
{
	if (!p) return;
	memset(p, 0, sizeof *p);
	p->tstep = 0.25f;
	p->niter = 10;
	p->scale = 99;
	p->cgit = 0;
	p->pmsfac = 3;
	p->ponlit = 0;
	p->cg_eps = -1;
	p->rtol = 0;
	p->max_iter = 0;
	p->flags = 0;
}

static void env_double(const char *name, double *v)
{
	const char *s = getenv(name);
	double y;
	if (s && sscanf(s, "%lf", &y) == 1) *v = y;
}

void simpois_params_from_env(simpois_params *p)
{
	if (!p) return;
	env_double("PMSFAC", &p->pmsfac);
	env_double("PONLIT", &p->ponlit);
	env_double("CG_EPS", &p->cg_eps);
	env_double("SIMPOIS_RTOL", &p->rtol);
}

const char *simpois_strerror(int status)
{
	switch (status) {
	case SIMPOIS_OK: return "ok";
	case SIMPOIS_EINVAL: return "invalid argument";
	case SIMPOIS_ENOMEM: return "out of memory";
	case SIMPOIS_NOT_CONVERGED: return "tolerance not reached within the iteration cap";
	case SIMPOIS_BREAKDOWN: return "Krylov breakdown";
	case SIMPOIS_ECUDA: return "CUDA error";
	case SIMPOIS_ENODEV: return "no usable CUDA device";
	case SIMPOIS_SINGULAR: return "no known pixel: singular system";
	}
	return "unknown status";
}

const char *simpois_last_error(const simpois_ctx *ctx)
{
	return ctx ? ctx->last_error.c_str() : "";
}

int simpois_create(simpois_ctx **out, int device, void *stream)
{
	if (!out) return SIMPOIS_EINVAL;
	*out = nullptr;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		cudaGetLastError();
		return SIMPOIS_ENODEV;
	}
	if (device < 0 || device >= ndev) return SIMPOIS_EINVAL;
	if (cudaSetDevice(device) != cudaSuccess) {
		cudaGetLastError();
		return SIMPOIS_ENODEV;
	}
	simpois_ctx *c = new (std::nothrow) simpois_ctx();
	if (!c) return SIMPOIS_ENOMEM;
	c->device = device;
	c->stream = (cudaStream_t)stream;
	cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
	if (cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
		cudaGetLastError();
		delete c;
		return SIMPOIS_ECUDA;
	}
	// SIMPOIS_TUNE_CACHE=path: every context keeps its tuning in that file
	const char *tc = getenv("SIMPOIS_TUNE_CACHE");
	if (tc && *tc && simpois_set_tune_cache(c, tc) != SIMPOIS_OK)
		fprintf(stderr, "simpois: SIMPOIS_TUNE_CACHE ignored: %s\n", c->last_error.c_str());
	*out = c;
	return SIMPOIS_OK;
}

int simpois_destroy(simpois_ctx *ctx)
{
	if (!ctx) return SIMPOIS_OK;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	if (ctx->arena) cudaFree(ctx->arena);
	if (ctx->io) cudaFree(ctx->io);
	if (ctx->split) cudaFree(ctx->split);
	if (ctx->pinned) cudaFreeHost(ctx->pinned);
	if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
	if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
	if (ctx->ev_in) cudaEventDestroy(ctx->ev_in);
	if (ctx->ev_out) cudaEventDestroy(ctx->ev_out);
	if (ctx->ev_rhs) cudaEventDestroy(ctx->ev_rhs);
	for (cudaEvent_t e : ctx->evpool) cudaEventDestroy(e);
	if (ctx->solve_exec) cudaGraphExecDestroy(ctx->solve_exec);
	if (ctx->amle_exec) cudaGraphExecDestroy(ctx->amle_exec);
	delete ctx;
	return SIMPOIS_OK;
}

int simpois_solve_device(simpois_ctx *ctx, float *out, const float *in, const float *dat, int w, int h,
		int pd, const simpois_params *params, simpois_report *reports)
{
	if (!ctx || !out || !in) return ctx_fail(ctx, SIMPOIS_EINVAL, "null context or buffer");
	int rc = check_dims(ctx, w, h, pd);
	if (rc) return rc;
	simpois_params p;
	if (params) p = *params; else simpois_default_params(&p);
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	std::vector<simpois_report> rep(pd);
	memset(rep.data(), 0, sizeof(simpois_report) * pd);
	if (p.rtol > 0) {
		simpois_image im = {in, dat, out, w, h, pd, p.tstep, p.rtol};
		rc = run_converged(ctx, &im, 1, &p, rep.data());
	} else {
		rc = run_reference(ctx, out, in, dat, w, h, pd, &p, rep.data());
	}
	if (rc) return rc;
	SP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	int st = SIMPOIS_OK;
	for (int l = 0; l < pd; l++) st = worst(st, rep[l].status == SIMPOIS_SINGULAR ? SIMPOIS_OK : rep[l].status);
	if (reports) memcpy(reports, rep.data(), sizeof(simpois_report) * pd);
	return st;
}

// ---------------------------------------------- host entry point: direct I/O
//
// The converged schedule reads the data term f only at the unknowns, and the
// output equals the input g at every known pixel.  With page-locked host
// buffers the host entry point therefore moves, besides g itself, only the
// 4-pixel groups of f and of the output that hold an unknown (read and
// written in place by a kernel), and sends the output's known pixels back
// while the solve runs (the host link is idle then).

__global__ void k_fetch_rhs(const float4 *__restrict__ g, const float4 *__restrict__ hf, float4 *__restrict__ f,
		size_t n4)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
		const float4 v = g[i];
		const bool u = isnan(v.x) || isnan(v.y) || isnan(v.z) || isnan(v.w);
		f[i] = u ? hf[i] : make_float4(0.f, 0.f, 0.f, 0.f);
	}
}

__global__ void k_put_unknowns(const float4 *__restrict__ g, const float4 *__restrict__ out,
		float4 *__restrict__ hout, size_t n4)
{
	for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
		const float4 v = g[i];
		if (isnan(v.x) || isnan(v.y) || isnan(v.z) || isnan(v.w)) hout[i] = out[i];
	}
}

// The same two passes over every image of a batch, one launch each, the
// blocks shared out by size: image k takes blocks blk0 .. blk0 + ceil(n4 / ch)
// - 1 (blk0 ascending; an image with no groups takes none), block b of it the
// groups (b - blk0) ch .. + ch - 1.  fetch: dst = src at the groups of g
// holding an unknown (0 elsewhere), src a page-locked host buffer; put: dst
// (host) = src at those groups.
struct IoImg {
	const float4 *g;     // the image on the device
	const float4 *src;
	float4 *dst;
	size_t n4;           // 4-pixel groups
	unsigned blk0;       // first block
};

// The image of chunk b: the last one whose first chunk is at or below it
// (images without chunks share the next one's blk0).
__device__ __forceinline__ const IoImg &io_image(const IoImg *__restrict__ im, int n, unsigned b = blockIdx.x)
{
	int lo = 0, hi = n - 1;
	while (lo < hi) {
		const int mid = (lo + hi + 1) >> 1;
		if (im[mid].blk0 <= b) lo = mid;
		else hi = mid - 1;
	}
	return im[lo];
}

__global__ void k_fetch_rhs_batch(const IoImg *__restrict__ im, int n, unsigned ch)
{
	const IoImg &m = io_image(im, n);
	if (!m.src) return;   // no data term, or whole-buffer copies
	const size_t beg = (size_t)(blockIdx.x - m.blk0) * ch, end = min(beg + ch, m.n4);
	for (size_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
		const float4 v = m.g[i];
		const bool u = isnan(v.x) || isnan(v.y) || isnan(v.z) || isnan(v.w);
		m.dst[i] = u ? m.src[i] : make_float4(0.f, 0.f, 0.f, 0.f);
	}
}

__global__ void k_put_unknowns_batch(const IoImg *__restrict__ im, int n, unsigned ch)
{
	const IoImg &m = io_image(im, n);
	if (!m.dst) return;   // an image that took whole-buffer copies
	const size_t beg = (size_t)(blockIdx.x - m.blk0) * ch, end = min(beg + ch, m.n4);
	for (size_t i = beg + threadIdx.x; i < end; i += blockDim.x) {
		const float4 v = m.g[i];
		if (isnan(v.x) || isnan(v.y) || isnan(v.z) || isnan(v.w)) m.dst[i] = m.src[i];
	}
}

// The device address of a page-locked host buffer, 16-byte aligned; null for
// any other buffer.
static void *direct_ptr(const void *p)
{
	if (!p || ((uintptr_t)p & 15)) return nullptr;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	if (a.type != cudaMemoryTypeHost || !a.devicePointer || ((uintptr_t)a.devicePointer & 15)) return nullptr;
	return a.devicePointer;
}

// SIMPOIS_NO_DIRECT_IO=1: the host entry point copies whole buffers
static bool direct_io_enabled()
{
	static bool v = [] {
		const char *e = getenv("SIMPOIS_NO_DIRECT_IO");
		return !(e && atoi(e) > 0);
	}();
	return v;
}

// The second stream of the host entry points and its events (created once).
static int ensure_aux(simpois_ctx *ctx)
{
	if (ctx->aux_stream) return SIMPOIS_OK;
	SP_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
	SP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming));
	SP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_out, cudaEventDisableTiming));
	SP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ev_rhs, cudaEventDisableTiming));
	return SIMPOIS_OK;
}

int simpois_solve(simpois_ctx *ctx, float *out, const float *in, const float *dat, int w, int h, int pd,
		const simpois_params *params, simpois_report *reports)
{
	if (!ctx || !out || !in) return ctx_fail(ctx, SIMPOIS_EINVAL, "null context or buffer");
	int rc = check_dims(ctx, w, h, pd);
	if (rc) return rc;
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	size_t n = (size_t)w * h * pd;
	size_t bytes = n * sizeof(float);
	size_t slot = (bytes + 255) / 256 * 256;
	rc = ctx_io_reserve(ctx, slot * (dat ? 3 : 2));
	if (rc) return rc;
	float *din = (float *)ctx->io, *dout = (float *)(ctx->io + slot);
	float *ddat = dat ? (float *)(ctx->io + 2 * slot) : nullptr;
	cudaStream_t s = ctx->stream;
	const bool converged = params && params->rtol > 0;   // the default is the reference schedule
	float4 *hout = nullptr;
	const float4 *hdat = nullptr;
	if (converged && n % 4 == 0 && direct_io_enabled()) {
		hout = (float4 *)direct_ptr(out);
		hdat = dat ? (const float4 *)direct_ptr(dat) : nullptr;
		if (dat && !hdat) hout = nullptr;
	}
	const bool direct = hout != nullptr;
	if (direct && (rc = ensure_aux(ctx))) return rc;
	const int grid = 8 * (ctx->sm_count > 0 ? ctx->sm_count : 1);
	SP_CUDA(ctx, cudaMemcpyAsync(din, in, bytes, cudaMemcpyHostToDevice, s));
	if (direct) {
		// on the second stream, once g is in: the data term's groups that hold
		// an unknown (overlapping the solve's setup, which does not read f),
		// then the output's known pixels -- those of g -- while the solve runs
		SP_CUDA(ctx, cudaEventRecord(ctx->ev_in, s));
		SP_CUDA(ctx, cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_in, 0));
		if (dat) {
			k_fetch_rhs<<<grid, 256, 0, ctx->aux_stream>>>((const float4 *)din, hdat, (float4 *)ddat, n / 4);
			ctx->launches++;
			const cudaError_t e = cudaGetLastError();
			if (e != cudaSuccess) {
				cudaStreamSynchronize(ctx->aux_stream);
				return ctx_fail(ctx, SIMPOIS_ECUDA, "k_fetch_rhs: %s", cudaGetErrorString(e));
			}
			SP_CUDA(ctx, cudaEventRecord(ctx->ev_rhs, ctx->aux_stream));
			ctx->rhs_pending = ctx->ev_rhs;
		}
		SP_CUDA(ctx, cudaMemcpyAsync(out, din, bytes, cudaMemcpyDeviceToHost, ctx->aux_stream));
		SP_CUDA(ctx, cudaEventRecord(ctx->ev_out, ctx->aux_stream));
	} else if (dat) {
		SP_CUDA(ctx, cudaMemcpyAsync(ddat, dat, bytes, cudaMemcpyHostToDevice, s));
	}
	int st = simpois_solve_device(ctx, dout, din, ddat, w, h, pd, params, reports);
	if (ctx->rhs_pending) {   // a solve that stopped before its loops
		cudaStreamWaitEvent(s, ctx->rhs_pending, 0);
		ctx->rhs_pending = nullptr;
	}
	if (st != SIMPOIS_OK && st != SIMPOIS_NOT_CONVERGED && st != SIMPOIS_BREAKDOWN) {
		if (direct) cudaStreamSynchronize(ctx->aux_stream);   // the caller may free out
		return st;
	}
	if (direct) {
		SP_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_out, 0));
		k_put_unknowns<<<grid, 256, 0, s>>>((const float4 *)din, (const float4 *)dout, hout, n / 4);
		ctx->launches++;
		SP_CUDA(ctx, cudaGetLastError());
	} else {
		SP_CUDA(ctx, cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, s));
	}
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	return st;
}

static int solve_batch(simpois_ctx *ctx, const simpois_image *images, int n, const simpois_params *params,
		simpois_report *reports, int tune, int *coarse_max, int *sweeps = nullptr)
{
	if (!ctx || (!images && n > 0) || n < 0) return ctx_fail(ctx, SIMPOIS_EINVAL, "bad batch");
	simpois_params p;
	if (params) p = *params; else simpois_default_params(&p);
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	int total = 0;
	for (int k = 0; k < n; k++) {
		if (!images[k].in || !images[k].out) return ctx_fail(ctx, SIMPOIS_EINVAL, "image %d: null buffer", k);
		int rc = check_dims(ctx, images[k].w, images[k].h, images[k].pd);
		if (rc) return rc;
		total += images[k].pd;
	}
	std::vector<simpois_report> rep(total);
	memset(rep.data(), 0, sizeof(simpois_report) * total);
	// converged images share one batched solve; reference-schedule images run one by one
	std::vector<simpois_image> conv;
	std::vector<int> conv_first;
	int base = 0, rc = SIMPOIS_OK;
	for (int k = 0; k < n; k++) {
		double rtol = images[k].rtol > 0 ? images[k].rtol : p.rtol;
		if (rtol > 0) {
			conv.push_back(images[k]);
			conv_first.push_back(base);
		} else {
			simpois_params pk = p;
			pk.tstep = images[k].tstep;
			rc = run_reference(ctx, images[k].out, images[k].in, images[k].dat, images[k].w, images[k].h,
					images[k].pd, &pk, rep.data() + base);
			if (rc) return rc;
		}
		base += images[k].pd;
	}
	if (!conv.empty()) {
		int nch = 0;
		for (auto &im : conv) nch += im.pd;
		std::vector<simpois_report> r(nch);
		rc = run_converged(ctx, conv.data(), (int)conv.size(), &p, r.data(), tune, coarse_max, sweeps);
		if (rc) return rc;
		int q = 0;
		for (size_t k = 0; k < conv.size(); k++)
			for (int l = 0; l < conv[k].pd; l++) rep[conv_first[k] + l] = r[q++];
	}
	SP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	int st = SIMPOIS_OK;
	for (int l = 0; l < total; l++) st = worst(st, rep[l].status == SIMPOIS_SINGULAR ? SIMPOIS_OK : rep[l].status);
	if (reports) memcpy(reports, rep.data(), sizeof(simpois_report) * total);
	return st;
}

int simpois_solve_batch(simpois_ctx *ctx, const simpois_image *images, int n, const simpois_params *params,
		simpois_report *reports)
{
	return solve_batch(ctx, images, n, params, reports, 0, nullptr);
}

int simpois_solve_batch_host(simpois_ctx *ctx, const simpois_image *images, int n, const simpois_params *params,
		simpois_report *reports)
{
	if (!ctx || (!images && n > 0) || n < 0) return ctx_fail(ctx, SIMPOIS_EINVAL, "bad batch");
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	simpois_params p;
	if (params) p = *params; else simpois_default_params(&p);
	// device slots of every image's in, dat and out, one after the other, then
	// the tables of the direct passes
	std::vector<size_t> off(3 * (size_t)n);
	size_t total = 0;
	// direct I/O per image (as simpois_solve): converged, its size a multiple
	// of 4, out and dat page-locked and 16-byte aligned; the other images take
	// whole-buffer copies
	const bool may_direct = direct_io_enabled() && n <= 65535;
	std::vector<char> dir(n, 0);
	std::vector<IoImg> fetch(n), put(n);
	int ndir = 0;
	bool any_fetch = false;
	for (int k = 0; k < n; k++) {
		const simpois_image &im = images[k];
		if (!im.in || !im.out) return ctx_fail(ctx, SIMPOIS_EINVAL, "image %d: null buffer", k);
		int rc = check_dims(ctx, im.w, im.h, im.pd);
		if (rc) return rc;
		const size_t np = (size_t)im.w * im.h * im.pd, slot = (np * sizeof(float) + 255) / 256 * 256;
		off[3 * k] = total;
		total += slot;
		off[3 * k + 1] = total;
		total += im.dat ? slot : 0;
		off[3 * k + 2] = total;
		total += slot;
	}
	const size_t o_tab = total;
	total += may_direct ? 2 * sizeof(IoImg) * (size_t)n : 0;
	int rc = ctx_io_reserve(ctx, total > 0 ? total : 256);
	if (rc) return rc;
	cudaStream_t s = ctx->stream;
	std::vector<simpois_image> dev(images, images + n);
	// the inputs first: the pointer checks below run while they move
	for (int k = 0; k < n; k++) {
		const size_t bytes = (size_t)images[k].w * images[k].h * images[k].pd * sizeof(float);
		dev[k].in = (const float *)(ctx->io + off[3 * k]);
		dev[k].dat = images[k].dat ? (const float *)(ctx->io + off[3 * k + 1]) : nullptr;
		dev[k].out = (float *)(ctx->io + off[3 * k + 2]);
		SP_CUDA(ctx, cudaMemcpyAsync((void *)dev[k].in, images[k].in, bytes, cudaMemcpyHostToDevice, s));
	}
	for (int k = 0; k < n; k++) {
		const simpois_image &im = images[k];
		const size_t np = (size_t)im.w * im.h * im.pd;
		if (may_direct && (im.rtol > 0 || p.rtol > 0) && np % 4 == 0) {
			const float4 *hd = im.dat ? (const float4 *)direct_ptr(im.dat) : nullptr;
			float4 *ho = (float4 *)direct_ptr(im.out);
			if (ho && (!im.dat || hd)) {
				dir[k] = 1;
				ndir++;
				fetch[k].src = hd;
				any_fetch = any_fetch || hd;
				put[k].dst = ho;
			}
		}
	}
	size_t n4tot = 0;
	for (int k = 0; k < n; k++) {
		const size_t bytes = (size_t)images[k].w * images[k].h * images[k].pd * sizeof(float);
		if (images[k].dat && !dir[k])
			SP_CUDA(ctx, cudaMemcpyAsync((void *)dev[k].dat, images[k].dat, bytes, cudaMemcpyHostToDevice, s));
		if (dir[k]) {
			fetch[k].g = put[k].g = (const float4 *)dev[k].in;
			fetch[k].dst = (float4 *)dev[k].dat;
			put[k].src = (const float4 *)dev[k].out;
			fetch[k].n4 = put[k].n4 = bytes / 16;
			n4tot += bytes / 16;
		}
	}
	// blocks shared out by size: chunks of ch groups (a multiple of 1024, so
	// that each of the 256 threads takes 4 or more), about 32 blocks per SM
	// over the whole batch (at most 65535 images: nblk stays far below 2^31)
	const size_t target = 32 * (size_t)std::max(1, ctx->sm_count);
	const size_t ch = std::max<size_t>(1024, (n4tot / target + 1023) / 1024 * 1024);
	size_t nblk = 0;
	for (int k = 0; k < n; k++) {
		fetch[k].blk0 = put[k].blk0 = (unsigned)nblk;
		nblk += (fetch[k].n4 + ch - 1) / ch;
	}
	IoImg *dput = nullptr;
	if (ndir) {
		if ((rc = ensure_aux(ctx))) return rc;
		IoImg *dfetch = (IoImg *)(ctx->io + o_tab);
		dput = dfetch + n;
		// pageable sources: the copies are staged before the calls return
		SP_CUDA(ctx, cudaMemcpyAsync(dfetch, fetch.data(), sizeof(IoImg) * n, cudaMemcpyHostToDevice, s));
		SP_CUDA(ctx, cudaMemcpyAsync(dput, put.data(), sizeof(IoImg) * n, cudaMemcpyHostToDevice, s));
		// on the second stream, once the inputs are in: the direct images' data
		// terms at the groups that hold an unknown (overlapping the solve's
		// setup, which does not read them), then their outputs' known pixels --
		// those of the inputs -- while the solve runs
		SP_CUDA(ctx, cudaEventRecord(ctx->ev_in, s));
		SP_CUDA(ctx, cudaStreamWaitEvent(ctx->aux_stream, ctx->ev_in, 0));
		if (any_fetch) {
			k_fetch_rhs_batch<<<(unsigned)nblk, 256, 0, ctx->aux_stream>>>(dfetch, n, (unsigned)ch);
			ctx->launches++;
			const cudaError_t e = cudaGetLastError();
			if (e != cudaSuccess) {
				cudaStreamSynchronize(ctx->aux_stream);
				return ctx_fail(ctx, SIMPOIS_ECUDA, "k_fetch_rhs_batch: %s", cudaGetErrorString(e));
			}
			SP_CUDA(ctx, cudaEventRecord(ctx->ev_rhs, ctx->aux_stream));
			ctx->rhs_pending = ctx->ev_rhs;
		}
		// (copies on the copy engines: a kernel writing them competes with the
		// solve's kernels for the SMs and loses the overlap)
		for (int k = 0; k < n; k++) {
			if (!dir[k]) continue;
			const size_t bytes = (size_t)images[k].w * images[k].h * images[k].pd * sizeof(float);
			SP_CUDA(ctx, cudaMemcpyAsync(images[k].out, dev[k].in, bytes, cudaMemcpyDeviceToHost, ctx->aux_stream));
		}
		SP_CUDA(ctx, cudaEventRecord(ctx->ev_out, ctx->aux_stream));
	}
	const int st = solve_batch(ctx, dev.data(), n, params, reports, 0, nullptr);
	if (ctx->rhs_pending) {   // a solve that stopped before its loops
		cudaStreamWaitEvent(s, ctx->rhs_pending, 0);
		ctx->rhs_pending = nullptr;
	}
	if (st != SIMPOIS_OK && st != SIMPOIS_NOT_CONVERGED && st != SIMPOIS_BREAKDOWN) {
		if (ndir) cudaStreamSynchronize(ctx->aux_stream);   // the caller may free out
		cudaStreamSynchronize(s);
		return st;
	}
	for (int k = 0; k < n; k++) {
		if (dir[k]) continue;
		const size_t bytes = (size_t)images[k].w * images[k].h * images[k].pd * sizeof(float);
		SP_CUDA(ctx, cudaMemcpyAsync(images[k].out, dev[k].out, bytes, cudaMemcpyDeviceToHost, s));
	}
	if (ndir) {
		SP_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_out, 0));
		k_put_unknowns_batch<<<(unsigned)nblk, 256, 0, s>>>(dput, n, (unsigned)ch);
		ctx->launches++;
		SP_CUDA(ctx, cudaGetLastError());
	}
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	return st;
}

int simpois_autotune_ex(simpois_ctx *ctx, const simpois_image *images, int n, const simpois_params *params,
		simpois_report *reports, int *coarse_max, int *sweeps)
{
	int cm = 0, nu = 0;
	const int st = solve_batch(ctx, images, n, params, reports, 1, &cm, &nu);
	if (coarse_max) *coarse_max = cm;
	if (sweeps) *sweeps = nu;
	return st;
}

int simpois_autotune(simpois_ctx *ctx, const simpois_image *images, int n, const simpois_params *params,
		simpois_report *reports, int *coarse_max)
{
	return simpois_autotune_ex(ctx, images, n, params, reports, coarse_max, nullptr);
}

int simpois_set_sweeps(simpois_ctx *ctx, int sweeps)
{
	if (!ctx) return SIMPOIS_EINVAL;
	if (sweeps < 0 || sweeps > 3) return ctx_fail(ctx, SIMPOIS_EINVAL, "sweeps per side %d outside 1..3", sweeps);
	ctx->sweeps_fixed = sweeps;
	return SIMPOIS_OK;
}

int simpois_set_coarse_max(simpois_ctx *ctx, int coarse_max)
{
	if (!ctx) return SIMPOIS_EINVAL;
	if (coarse_max != 0 && (coarse_max < 8 || coarse_max > 128))
		return ctx_fail(ctx, SIMPOIS_EINVAL, "hand-over size %d outside 8..128", coarse_max);
	ctx->coarse_max_fixed = coarse_max;
	return SIMPOIS_OK;
}

int simpois_set_memory_limit(simpois_ctx *ctx, size_t bytes)
{
	if (!ctx) return SIMPOIS_EINVAL;
	ctx->arena_limit = bytes;
	return SIMPOIS_OK;
}

int simpois_set_tune_cache(simpois_ctx *ctx, const char *path)
{
	if (!ctx) return SIMPOIS_EINVAL;
	ctx->tune_path = path ? path : "";
	if (ctx->tune_path.empty()) return SIMPOIS_OK;
	std::map<std::string, simpois_ctx::Tuned> got;
	const int rc = tune_read(ctx, ctx->tune_path, got);
	if (rc) {
		ctx->tune_path.clear();
		return rc;
	}
	for (const auto &kv : got) ctx->tuned.insert(kv);   // the context's own choices stay
	return SIMPOIS_OK;
}

int simpois_residual_device(simpois_ctx *ctx, const float *u, const float *in, const float *dat, int w, int h,
		int pd, int kind, double *rel, double *bnorm)
{
	if (!ctx || !u || !in || !rel) return ctx_fail(ctx, SIMPOIS_EINVAL, "null context or buffer");
	int rc = check_dims(ctx, w, h, pd);
	if (rc) return rc;
	if (kind != 0 && kind != 1) return ctx_fail(ctx, SIMPOIS_EINVAL, "kind must be 0 or 1");
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	size_t cs = (size_t)w * h;
	std::vector<MgProblem> probs(pd);
	std::vector<const float *> us(pd);
	for (int l = 0; l < pd; l++) {
		probs[l].g = in + cs * l;
		probs[l].f = dat ? dat + cs * l : nullptr;
		probs[l].out = nullptr;
		probs[l].w = w;
		probs[l].h = h;
		probs[l].kind = kind;
		probs[l].rtol = 0;
		us[l] = u + cs * l;
	}
	std::vector<double> bn(pd);
	rc = mg_residual(ctx, probs.data(), us.data(), pd, rel, bn.data());
	if (rc) return rc;
	if (bnorm) memcpy(bnorm, bn.data(), sizeof(double) * pd);
	return SIMPOIS_OK;
}

int simpois_adjoint_device(simpois_ctx *ctx, const float *grad_out, const float *in, int w, int h, int pd,
		float *grad_in, float *grad_dat, const simpois_params *params, simpois_report *reports)
{
	if (!ctx || !grad_out || !in || !grad_in) return ctx_fail(ctx, SIMPOIS_EINVAL, "null context or buffer");
	int rc = check_dims(ctx, w, h, pd);
	if (rc) return rc;
	simpois_params p;
	if (params) p = *params; else simpois_default_params(&p);
	if (p.tstep < 0)
		return ctx_fail(ctx, SIMPOIS_EINVAL, "the adjoint covers the symmetric 5-point operator (tstep > 0)");
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	size_t cs = (size_t)w * h;
	std::vector<MgProblem> probs(pd);
	std::vector<const float *> go(pd);
	std::vector<float *> gi(pd), gd(pd);
	for (int l = 0; l < pd; l++) {
		probs[l].g = in + cs * l;
		probs[l].f = nullptr;
		probs[l].out = nullptr;
		probs[l].w = w;
		probs[l].h = h;
		probs[l].kind = 0;
		probs[l].rtol = p.rtol > 0 ? p.rtol : 1e-6;
		go[l] = grad_out + cs * l;
		gi[l] = grad_in + cs * l;
		gd[l] = grad_dat ? grad_dat + cs * l : nullptr;
	}
	MgOptions opt;
	opt.max_iter = p.max_iter > 0 ? p.max_iter : 500;
	opt.use_mg = !(p.flags & SIMPOIS_FLAG_NO_MG);
	opt.use_graph = !(p.flags & SIMPOIS_FLAG_NO_GRAPH);
	opt.fused = !(p.flags & SIMPOIS_FLAG_UNFUSED);
	opt.mode = MG_ADJOINT;
	opt.coarse_max = ctx->coarse_max_fixed;
	opt.nu = ctx->sweeps_fixed;
	{   // the forward fill's tuned choices, if any
		auto it = ctx->tuned.find(tune_key(probs, 0, opt));
		if (it != ctx->tuned.end()) {
			if (opt.coarse_max <= 0) opt.coarse_max = it->second.coarse_max;
			if (opt.nu <= 0) opt.nu = it->second.nu;
		}
	}
	opt.grad_out = go.data();
	opt.grad_in = gi.data();
	opt.grad_dat = gd.data();
	std::vector<simpois_report> rep(pd);
	memset(rep.data(), 0, sizeof(simpois_report) * pd);
	rc = mg_solve(ctx, probs.data(), pd, opt, rep.data());
	if (rc) return rc;
	SP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	int st = SIMPOIS_OK;
	for (int l = 0; l < pd; l++) st = worst(st, rep[l].status == SIMPOIS_SINGULAR ? SIMPOIS_OK : rep[l].status);
	if (reports) memcpy(reports, rep.data(), sizeof(simpois_report) * pd);
	return st;
}

long long simpois_launch_count(const simpois_ctx *ctx) { return ctx ? ctx->launches : 0; }

const char *simpois_kernel_stats(simpois_ctx *ctx)
{
	if (!ctx) return "{}";
	std::string j = "{";
	char buf[256];
	for (size_t k = 0; k < ctx->kstats.size(); k++) {
		const auto &st = ctx->kstats[k];
		snprintf(buf, sizeof buf, "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f, \"bytes\": %.0f}",
				k ? ", " : "", st.name.c_str(), st.launches, st.ms, st.bytes);
		j += buf;
	}
	j += "}";
	ctx->kstats_json = j;
	return ctx->kstats_json.c_str();
}

void simpois_reset_kernel_stats(simpois_ctx *ctx)
{
	if (ctx) ctx->kstats.clear();
}

void simpois_reset_launch_count(simpois_ctx *ctx)
{
	if (ctx) ctx->launches = 0;
}

// ------------------------------------------------------------------ drop-in symbols

static std::mutex g_dropin_mu;
static simpois_ctx *g_dropin_ctx = nullptr;
static simpois_params g_dropin_env;
static bool g_dropin_env_read = false;

static int dropin_solve(float *out, float *in, float *dat, int w, int h, int pd, float tstep, int niter,
		int scale, int cgit)
{
	std::lock_guard<std::mutex> lock(g_dropin_mu);
	if (!g_dropin_env_read) {
		simpois_default_params(&g_dropin_env);
		simpois_params_from_env(&g_dropin_env);
		g_dropin_env_read = true;
	}
	int rc = SIMPOIS_OK;
	if (!g_dropin_ctx) rc = simpois_create(&g_dropin_ctx, 0, nullptr);
	if (rc) {
		fprintf(stderr, "simpois: %s\n", simpois_strerror(rc));
		return rc;
	}
	simpois_params p = g_dropin_env;
	p.tstep = tstep;
	p.niter = niter;
	p.scale = scale;
	p.cgit = cgit;
	rc = simpois_solve(g_dropin_ctx, out, in, dat, w, h, pd, &p, nullptr);
	if (rc != SIMPOIS_OK)
		fprintf(stderr, "simpois: %s (%s)\n", simpois_strerror(rc), simpois_last_error(g_dropin_ctx));
	return rc;
}

void poisson_solver_separable(float *out, float *in, float *dat, int w, int h, int pd, float tstep, int niter,
		int scale, float cgrad)
{
	int rc = dropin_solve(out, in, dat, w, h, pd, tstep, niter, scale, (int)cgrad);
	if (rc != SIMPOIS_OK && rc != SIMPOIS_NOT_CONVERGED && rc != SIMPOIS_BREAKDOWN && out && in && out != in &&
			w > 0 && h > 0 && pd > 0)
		memcpy(out, in, sizeof(float) * (size_t)w * h * pd);
}

void poisson_recursive(float *u, float *g, float *f, int w, int h, float tstep, int niter, int scale)
{
	std::lock_guard<std::mutex> lock(g_dropin_mu);
	int rc = SIMPOIS_OK;
	if (!g_dropin_ctx) rc = simpois_create(&g_dropin_ctx, 0, nullptr);
	if (rc == SIMPOIS_OK) {
		simpois_params p;
		simpois_default_params(&p);   // this variant reads no smart parameter
		p.tstep = tstep;
		p.niter = niter;
		p.scale = scale;
		p.flags = SIMPOIS_FLAG_MINI;
		rc = simpois_solve(g_dropin_ctx, u, g, f, w, h, 1, &p, nullptr);
	}
	if (rc != SIMPOIS_OK) {
		fprintf(stderr, "simpois: %s\n", simpois_strerror(rc));
		if (u && g && u != g && w > 0 && h > 0) memcpy(u, g, sizeof(float) * (size_t)w * h);
	}
}

int simpois_amle_device(simpois_ctx *ctx, float *out, const float *in, int w, int h, int pd, int nn, int niter,
		const float *init, double *gap)
{
	if (!ctx || !out || !in) return ctx_fail(ctx, SIMPOIS_EINVAL, "null context or buffer");
	int rc = check_dims(ctx, w, h, pd);
	if (rc) return rc;
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	rc = amle_run(ctx, out, in, w, h, pd, nn, niter, init, gap);
	if (rc) return rc;
	SP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
	return SIMPOIS_OK;
}

int simpois_amle(simpois_ctx *ctx, float *out, const float *in, int w, int h, int pd, int nn, int niter,
		const float *init, double *gap)
{
	if (!ctx || !out || !in) return ctx_fail(ctx, SIMPOIS_EINVAL, "null context or buffer");
	int rc = check_dims(ctx, w, h, pd);
	if (rc) return rc;
	if (cudaSetDevice(ctx->device) != cudaSuccess) return ctx_fail(ctx, SIMPOIS_ECUDA, "cudaSetDevice");
	const size_t bytes = (size_t)w * h * pd * sizeof(float), slot = (bytes + 255) / 256 * 256;
	rc = ctx_io_reserve(ctx, slot * (init ? 3 : 2));
	if (rc) return rc;
	float *din = (float *)ctx->io, *dout = (float *)(ctx->io + slot);
	float *dini = init ? (float *)(ctx->io + 2 * slot) : nullptr;
	cudaStream_t s = ctx->stream;
	SP_CUDA(ctx, cudaMemcpyAsync(din, in, bytes, cudaMemcpyHostToDevice, s));
	if (init) SP_CUDA(ctx, cudaMemcpyAsync(dini, init, bytes, cudaMemcpyHostToDevice, s));
	rc = amle_run(ctx, dout, din, w, h, pd, nn, niter, dini, gap);
	if (rc) return rc;
	SP_CUDA(ctx, cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, s));
	SP_CUDA(ctx, cudaStreamSynchronize(s));
	return SIMPOIS_OK;
}

// A smart parameter as the reference reads it (smapa.h:19-41): a double
// scanned from the variable once per process, else the default, with the
// reference's message on stderr.
static double smart_parameter(const char *name, double def, bool *known, double *value)
{
	if (!*known) {
		fprintf(stderr, "scanning the environment for \"%s\"... ", name);
		const char *v = getenv(name);
		double y;
		if (v && sscanf(v, "%lf", &y) == 1) {
			fprintf(stderr, "got value %g\n", y);
			*value = y;
		} else {
			fprintf(stderr, "kept default value %g\n", def);
			*value = def;
		}
		*known = true;
	}
	return *value;
}

void amle(float *y, float *x, int w, int h)
{
	std::lock_guard<std::mutex> lock(g_dropin_mu);
	int rc = SIMPOIS_OK;
	if (!g_dropin_ctx) rc = simpois_create(&g_dropin_ctx, 0, nullptr);
	if (rc == SIMPOIS_OK) {
		if (getenv("AMLE_INIT"))
			fprintf(stderr, "amle: AMLE_INIT is read by the amle command, not by this function\n");
		static bool kn = false, ki = false;
		static double vn = 4, vi = 100;
		const int niter = (int)smart_parameter("AMLE_NITER", 100, &ki, &vi);
		const int nn = niter > 0 ? (int)smart_parameter("AMLE_NN", 4, &kn, &vn) : 4;
		rc = simpois_amle(g_dropin_ctx, y, x, w, h, 1, nn, niter, nullptr, nullptr);
	}
	if (rc != SIMPOIS_OK) {
		fprintf(stderr, "amle: %s\n", simpois_strerror(rc));
		if (y && x && y != x && w > 0 && h > 0) memcpy(y, x, sizeof(float) * (size_t)w * h);
	}
}

void poisson_rec(float *u, float *g, float *f, int w, int h, float tstep, int niter, int scale, int cgit)
{
	int rc = dropin_solve(u, g, f, w, h, 1, tstep, niter, scale, cgit);
	if (rc != SIMPOIS_OK && rc != SIMPOIS_NOT_CONVERGED && rc != SIMPOIS_BREAKDOWN && u && g && u != g && w > 0 &&
			h > 0)
		memcpy(u, g, sizeof(float) * (size_t)w * h);
}

}  // extern "C"
