/*
 * simpois_main.c -- the `simpois` command on the GB300 library.
 *
 * A drop-in for imscript's `simpois` (simpois.c:305-443): the same options
 * with the same defaults (-i - -o - -m "" -f "" -t 0.25 -n 10 -s 99 -c 0),
 * the same argv consumption (pickopt.c:7-22), help texts, mask rule, size
 * checks and exit codes; the smart parameters PMSFAC, PONLIT and CG_EPS are
 * read from the environment as the reference does (smapa.h:44-60), plus
 * SIMPOIS_RTOL: when set > 0 the converged schedule solves every channel to
 * that FP64 relative residual.  The solve runs on GPU 0 through the C ABI
 * (include/simpois_gpu.h); there is no CPU path.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "imageio.h"
#include "simpois_gpu.h"

/* user-visible texts of the simpois command (simpois.c:307-347) */
static const char *help_name = "simpois";
static const char *help_version = "simpois 1.0\n\nWritten by mnhrdt";
static const char *help_oneliner = "a simple Poisson solver for images";
static const char *help_usage = "usage:\n\t"
	"simpois [options] [-m mask.png] [-f data.npy] [-i in.npy] [-o out.npy]";
static const char *help_long =
	"Simpois is a simple Poisson solver for image processing.\n"
	"\n"
	"This program can solve Poisson, Laplace and Biharmonic equations\n"
	"over an arbitrary part of the image domain, with arbitrary data terms\n"
	"and boundary conditions.  Fast approximations to the solution can be\n"
	"obtained by setting the parameters.  Solving over the whole image domain\n"
	"is discouraged, as it is always better to use fft-based methods.\n"
	"\n"
	"Usage: simpois [options] -i in.npy -o out.npy\n"
	"   or: simpois [options] -i in.npy > out.npy\n"
	"   or: cat in.npy | simpois [options] -o out.npy\n"
	"   or: cat in.npy | simpois [options] > out.npy\n"
	"\n"
	"Options:\n"
	" -i IMG\tInput image with boundary data (default=stdin)\n"
	" -f IMG\tPoisson data term (default=zeros)\n"
	" -m IMG\tMask for the region of interest (default=zeros)\n"
	" -o IMG\tOutput image (default=stdout)\n"
	" -t 0.25\tTime step for Gauss-Seidel iterations (negative=biharmonic)\n"
	" -n 10\tNumber of Gauss-Seidel iterations\n"
	" -s 99\tMaximum number of multi-scale octaves\n"
	" -c 0\tNumber of Conjugate Gradient iterations\n"
	" -h\tdisplay short help message\n"
	" --help\tdisplay longer help message\n"
	"\n"
	"Examples:\n"
	" cat in.npy | simpois > out.npy           Fill NANs by Laplace equation\n"
	" cat in.npy | simpois -n 1 > out.npy      Fill NANs, fast (one iteration)\n"
	" cat in.npy | simpois -t -0.08 > out.npy  Fill NANs, smooth (Biharmonic)\n"
	" simpois -i in.npy -o out.npy             Laplace, with explicit data\n"
	" simpois -m mask.png ...                  Use mask instead of NANs\n"
	" simpois -f lap.npy ...                   Poisson editor\n"
	"\n"
	"Report bugs to <enric.meinhardt@ens-paris-saclay.fr>.";

/* man page through help2man, as the imscript tools do (help_stuff.c:5-21) */
static int run_help2man(int raw)
{
	char cmd[512];
	snprintf(cmd, sizeof cmd, "help2man -N -S imscript -n \"%s\" %s%s %s", help_oneliner,
			raw > 0 ? "" : "./", help_name, abs(raw) > 1 ? "" : "|man -l -");
	return system(cmd);
}

/* -h, -?, --help, --version, --man... as the only argument (help_stuff.c:23-34) */
static void help_if_requested(const char *s)
{
	if (!s || !strcmp(s, "-h")) exit(0 * puts(help_usage));
	if (!strcmp(s, "-?")) exit(0 * puts(help_oneliner));
	if (!strcmp(s, "--help")) exit(0 * puts(help_long));
	if (!strcmp(s, "--version")) exit(0 * puts(help_version));
	if (!strcmp(s, "--man")) exit(run_help2man(1));
	if (!strcmp(s, "--manraw")) exit(run_help2man(2));
	if (!strcmp(s, "--man-x")) exit(run_help2man(-1));
	if (!strcmp(s, "--manraw-x")) exit(run_help2man(-2));
	if (!strcmp(s, "--help-oneliner")) puts(help_oneliner);
}

/* Take "-<name> <value>" out of argv; the value, or `def` when absent.  The
 * scan and the shift of the remaining arguments follow pickopt.c:7-22. */
static char *take_option(int *argc, char ***argv, const char *name, char *def)
{
	int c = *argc, has_value = def ? 1 : 0;
	char **v = *argv;
	for (int i = 0; i < c - has_value; i++) {
		if (v[i][0] != '-' || strcmp(v[i] + 1, name)) continue;
		char *r = v[i + has_value] + 1 - has_value;
		*argc -= has_value + 1;
		for (int j = i; j < c - has_value; j++) v[j] = v[j + has_value + 1];
		return r;
	}
	return def;
}

int main_simpois(int argc, char *argv[])
{
	if (argc == 2) help_if_requested(argv[1]);

	float tstep = atof(take_option(&argc, &argv, "t", "0.25"));
	float niter = atof(take_option(&argc, &argv, "n", "10"));
	float nscal = atof(take_option(&argc, &argv, "s", "99"));
	float cgrad = atof(take_option(&argc, &argv, "c", "0"));
	char *fname_i = take_option(&argc, &argv, "i", "-");
	char *fname_o = take_option(&argc, &argv, "o", "-");
	char *fname_m = take_option(&argc, &argv, "m", "");
	char *fname_f = take_option(&argc, &argv, "f", "");
	if (!strcmp(fname_f, "-") && !strcmp(fname_i, "-")) fname_i = "NAN";

	if (argc > 1) {
		fprintf(stderr, "Usage:\n\t%s [options]\n", *argv);
		fprintf(stderr, "\nComputes approximate solutions of Poisson"
				" or Laplace equations for images\n");
		fprintf(stderr, "\nOptions with their default values:\n"
				"\t-i stdin   Input image with boundary data\n"
				"\t-f (zeros) Optional image with Poisson data term\n"
				"\t-m (zeros) Optional image with region of interest\n"
				"\t-o stdout  Output image\n"
				"\t-t 0.25    Time step for Gauss-Seidel iterations\n"
				"\t-n 10      Number of Gauss-Seidel iterations\n"
				"\t-s 99      Number of Multi-Scale octaves\n"
				"\t-c 0       Number of Conjugate Gradient iterations\n");
		fprintf(stderr, "\nNote: NAN values in the input image"
				" are added to the region of interest\n");
		return 1;
	}

	int w = 0, h = 0, pd = 0;
	float *img_i = NULL;
	if (*fname_i && strcmp(fname_i, "NAN")) {
		img_i = imgio_read_split(fname_i, &w, &h, &pd);
		if (!img_i) return 1;
	}

	float *img_f = NULL;
	if (*fname_f) {
		int w2, h2, pd2;
		img_f = imgio_read_split(fname_f, &w2, &h2, &pd2);
		if (!img_f) return 1;
		if (!img_i) {
			w = w2; h = h2; pd = pd2;
			img_i = malloc(sizeof(float) * (size_t)w * h * pd);
			if (!img_i) return fprintf(stderr, "simpois: out of memory\n"), 1;
			for (size_t k = 0; k < (size_t)w * h * pd; k++) img_i[k] = NAN;
		} else if (w != w2 || h != h2 || pd != pd2) {
			return fprintf(stderr, "input sizes mismatch (i,f)");
		}
	}
	if (!img_i) return fprintf(stderr, "simpois: no input image\n"), 1;

	float *img_m = NULL;
	if (*fname_m) {
		int w2, h2;
		img_m = imgio_read_gray(fname_m, &w2, &h2);
		if (!img_m) return 1;
		if (w != w2 || h != h2) return fprintf(stderr, "input sizes mismatch (i,m)");
	}

	float *out = malloc(sizeof(float) * (size_t)w * h * pd);
	if (!out) return fprintf(stderr, "simpois: out of memory\n"), 1;

	if (img_m)
		for (size_t k = 0; k < (size_t)w * h * pd; k++)
			if (img_m[k % ((size_t)w * h)] > 0) img_i[k] = NAN;

	simpois_params prm;
	simpois_default_params(&prm);
	simpois_params_from_env(&prm);
	prm.tstep = tstep;
	prm.niter = (int)niter;
	prm.scale = (int)nscal;
	prm.cgit = (int)cgrad;

	simpois_ctx *ctx = NULL;
	int rc = simpois_create(&ctx, 0, NULL);
	if (rc) {
		fprintf(stderr, "simpois: %s\n", simpois_strerror(rc));
		return 1;
	}
	rc = simpois_solve(ctx, out, img_i, img_f, w, h, pd, &prm, NULL);
	if (rc != SIMPOIS_OK && rc != SIMPOIS_NOT_CONVERGED && rc != SIMPOIS_BREAKDOWN) {
		fprintf(stderr, "simpois: %s: %s\n", simpois_strerror(rc), simpois_last_error(ctx));
		simpois_destroy(ctx);
		return 1;
	}
	if (rc != SIMPOIS_OK)
		fprintf(stderr, "simpois: warning: %s\n", simpois_strerror(rc));
	simpois_destroy(ctx);

	int wr = imgio_write_split(fname_o, out, w, h, pd);

	free(out);
	free(img_i);
	free(img_m);
	free(img_f);
	return wr ? 1 : 0;
}

/* the im multi-tool compiles every tool with HIDE_ALL_MAINS and dispatches
 * to main_simpois itself (src/im.c, src/all_mains.inc) */
#ifndef HIDE_ALL_MAINS
int main(int c, char **v) { return main_simpois(c, v); }
#endif
