/*
 * amle_main.c -- the `amle` command on the GB300 library.
 *
 * A drop-in for imscript's `amle` (src/amle.c:330-367): `amle [in [mask
 * [out]]]` with "-" for stdin/stdout, the input read as one channel (colour
 * images converted to gray, as iio_read_image_float does), mask > 0 adding
 * pixels to the unknowns, the same help texts, usage message and exit codes;
 * AMLE_NN, AMLE_NITER and AMLE_INIT read from the environment as the
 * reference reads them (smapa.h:44-60, src/amle.c:100-110).  The fill runs on
 * GPU 0 through the C ABI (include/simpois_gpu.h); there is no CPU path.
 * Every tenth iteration the reference prints the gap between its lower and
 * upper iterates; this command prints that gap once, after the last one.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "imageio.h"
#include "simpois_gpu.h"

/* user-visible texts of the amle command (src/amle.c:291-327) */
static const char *help_name = "amle";
static const char *help_version = "amle 1.0\n\nWritten by mnhrdt";
static const char *help_oneliner = "Absolutely Minimizing Lipschitz Extension";
static const char *help_usage = "usage:\n\t"
	"simpois [in [mask [out]]]";
static const char *help_long =
	"Interpolate by AMLE (Absolutely Minimizing Lipschitz Extension).\n"
	"\n"
	"The pixels to fill-in are specified by NAN values in the input image\n"
	"or by a separate user-provided mask.  The interpolated is defined\n"
	"as that whose maximal slope is the lowest possible, recursively in all\n"
	"subsets on the region of interest.\n"
	"\n"
	"Usage: amle in.npy mask.png out.npy\n"
	"   or: amle in.npy mask.png > out.npy\n"
	"   or: amle in.npy > out.npy\n"
	"   or: cat in.npy | amle > out.npy\n"
	"\n"
	"Options:\n"
	" -h\tdisplay short help message\n"
	" --help\tdisplay longer help message\n"
	"\n"
	"Environement:\n"
	" AMLE_NN\tNeigborhood size (4, 6, 8, 16, 26 or 32, default=4)\n"
	" AMLE_TAU\tTimestep for the iterations (default=0.25)\n"
	" AMLE_NITER\tNumber of iterations at each scale (default=100)\n"
	" AMLE_INIT\tInitial image for the iterations (default=zeros)\n"
	"\n"
	"Examples:\n"
	" amle in.npy > out.npy               Fill-in the holes in a DSM\n"
	" AMLE_NN=32 amle in.npy > out.npy    More precise, slower solver\n"
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

/* the reference's fail(): message on stderr, exit status -1 (fail.c:64-80) */
static int fail_exit(char **v, const char *msg)
{
	fprintf(stderr, "\nFAIL(\"%s\"): %s\n\n", v[0], msg);
	exit(-1);
}

/* a smart parameter read as the reference reads it (smapa.h:19-41): a
 * double scanned from the variable, else the default, with its message */
static double smart_parameter(const char *name, double def)
{
	fprintf(stderr, "scanning the environment for \"%s\"... ", name);
	const char *s = getenv(name);
	double y;
	if (s && sscanf(s, "%lf", &y) == 1) {
		fprintf(stderr, "got value %g\n", y);
		return y;
	}
	fprintf(stderr, "kept default value %g\n", def);
	return def;
}

int main_amle(int c, char *v[])
{
	if (c == 2) help_if_requested(v[1]);

	if (c > 4 || (v[1] && v[1][0] == '-' && v[1][1] == 'h')) {
		fprintf(stderr, "usage:\n\t%s [in [mask [out]]]\n", *v);
		return 1;
	}
	const char *filename_in = c > 1 ? v[1] : "-";
	const char *filename_mask = c > 2 ? v[2] : "";
	const char *filename_out = c > 3 ? v[3] : "-";

	int w[2], h[2];
	float *in = imgio_read_gray(filename_in, w, h);
	if (!in) return fail_exit(v, "could not read image");
	float *mask = NULL;
	if (filename_mask[0]) {
		mask = imgio_read_gray(filename_mask, w + 1, h + 1);
		if (!mask) return fail_exit(v, "could not read image");
		if (w[0] != w[1] || h[0] != h[1]) return fail_exit(v, "image and mask file size mismatch");
	}
	size_t n = (size_t)*w * *h;
	float *out = malloc(sizeof(float) * n);
	if (!out) return fail_exit(v, "out of memory");
	if (mask)
		for (size_t i = 0; i < n; i++)
			if (mask[i] > 0) in[i] = NAN;

	/* AMLE_INIT: the start of the upper iterate at the unknowns */
	float *init = NULL;
	const char *fi = getenv("AMLE_INIT");
	if (fi) {
		int ww, hh;
		init = imgio_read_gray(fi, &ww, &hh);
		if (!init) return fail_exit(v, "could not read image");
		if ((size_t)ww * hh != n) return fail_exit(v, "init size mismatch");
	}

	simpois_ctx *ctx = NULL;
	int rc = simpois_create(&ctx, 0, NULL);
	if (rc) {
		fprintf(stderr, "amle: %s\n", simpois_strerror(rc));
		return 1;
	}
	/* the reference reads AMLE_NITER first (the loop bound), then AMLE_NN */
	const int niter = (int)smart_parameter("AMLE_NITER", 100);
	const int nn = niter > 0 ? (int)smart_parameter("AMLE_NN", 4) : 4;
	double gap[2] = {0, 0};
	rc = simpois_amle(ctx, out, in, *w, *h, 1, nn, niter, init, gap);
	if (rc) {
		fprintf(stderr, "amle: %s: %s\n", simpois_strerror(rc), simpois_last_error(ctx));
		simpois_destroy(ctx);
		return 1;
	}
	simpois_destroy(ctx);
	fprintf(stderr, "iter %d, e = {%g %g}\n", niter, gap[0], gap[1]);

	int wr = imgio_write_split(filename_out, out, *w, *h, 1);
	free(out);
	free(in);
	free(mask);
	free(init);
	return wr ? 1 : 0;
}

/* the im multi-tool compiles every tool with HIDE_ALL_MAINS and dispatches
 * to main_amle itself (src/im.c, src/all_mains.inc) */
#ifndef HIDE_ALL_MAINS
int main(int c, char **v) { return main_amle(c, v); }
#endif
