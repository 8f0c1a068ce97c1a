// solvers.h -- internal interface between the C ABI (abi.cu) and the two
// solvers (ref_schedule.cu, mg_solver.cu).
#pragma once

#include "common.cuh"

// Reference schedule on one planar image (device pointers); `ws` is a device
// workspace of ref_workspace_bytes() bytes.
size_t ref_workspace_bytes(int w, int h, int pd, bool has_f);
int ref_solve(simpois_ctx *ctx, float *out, const float *in, const float *dat, int w, int h,
		int pd, const simpois_params *prm, simpois_report *rep, char *ws);

// One channel problem of the converged schedule.
struct MgProblem {
	const float *g;    // input channel (NaN = unknown), device
	const float *f;    // data term or nullptr, device
	float *out;        // output channel, device
	int w, h;
	int kind;          // 0: 5-point -Laplacian, 1: 13-point bilaplacian
	double rtol;
};

// What a batched solve does to the right-hand side.
enum MgMode {
	MG_FILL = 0,       // fill the unknowns of g (the simpois problem)
	MG_ADJOINT = 1,    // solve A lambda = grad_out on the unknowns of g
};

struct MgOptions {
	int max_iter = 500;    // PCG iterations per problem, all refinements
	int use_mg = 1;        // multigrid preconditioner (0: plain CG)
	int use_graph = 1;     // capture the PCG iteration in a CUDA graph
	int fused = 1;         // 5-point: fused V-cycle kernels (0: one launch per sweep)
	int ktimer = 0;        // time every main-loop launch with CUDA events (no graph)
	int out_resid = 0;     // FP64 residual of the float output
	int coarse_max = 0;    // fused V-cycle hand-over size (0: the default)
	int nu = 0;            // 5-point smoothing sweeps per side, 1..3 (0: the default, 2)
	int tma = 0;           // tile kernels load their regions through TMA
	int mode = MG_FILL;
	// MG_ADJOINT only: grad_out per problem (device), results
	const float *const *grad_out = nullptr;
	float *const *grad_in = nullptr;
	float *const *grad_dat = nullptr;
};

// Batched converged solve of n problems; rep receives n records and bnorm2,
// when given, each problem's |b|^2 (the denominator of its relative residual).
int mg_solve(simpois_ctx *ctx, const MgProblem *probs, int n, const MgOptions &opt,
		simpois_report *rep, double *bnorm2 = nullptr);

// Number of levels of a w x h problem that the fused V-cycle runs in the tile
// kernels for hand-over size coarse_max (0: the default).
int mg_handover_level(int w, int h, int coarse_max);

// The hand-over size used when a solve names none (64, or SIMPOIS_COARSE_MAX).
int mg_default_coarse_max();

// AMLE fill of a planar w x h x pd image (device pointers), nn neighbours,
// niter iterations, optional init planes; gap (may be null) receives per
// channel the max and the mean of |tinf - tsup| over the unknowns.
int amle_run(simpois_ctx *ctx, float *out, const float *in, int w, int h, int pd, int nn, int niter,
		const float *init, double *gap);

// FP64 relative residual of a float output for n problems (kind per problem).
int mg_residual(simpois_ctx *ctx, const MgProblem *probs, const float *const *u, int n,
		double *rel, double *bnorm);
