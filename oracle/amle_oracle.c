/*
 * amle_oracle.c -- CPU restatement of imscript's AMLE interpolator
 * (absolutely minimizing Lipschitz extension, src/amle.c) for the parity
 * tests.  Test infrastructure only: the product never links or calls it.
 *
 * amle_oracle() follows src/amle.c:196-246 (amle): the unknowns are the NaN
 * pixels; tinf starts at the image minimum and tsup at the maximum there
 * (amle_init, src/amle.c:89-112; an optional init image replaces tsup at the
 * unknowns, the AMLE_INIT file of the reference); every iteration sweeps tinf
 * then tsup (amle_iteration, src/amle.c:66-87), each unknown becoming the
 * distance-weighted midpoint of the smallest and largest of its first `nn`
 * in-image neighbours (get_nvals, src/amle.c:15-46, and get_minmax_idx,
 * src/amle.c:59-64, first index on ties); the output is tsup.
 *
 * order 0 sweeps the unknowns in raster order, in place, as the reference
 * does: bit for bit the reference's output.  order 1 sweeps the colour
 * classes (i + k j) mod m in turn (no pixel reads a pixel of its own class,
 * so a class can update in parallel): bit for bit the GPU's output.  The
 * float operations are the reference's, in its order; build with
 * -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>

/* The neighbour table of get_nvals (src/amle.c:17-30): {di, dj, di^2+dj^2}. */
static const int amle_nb[32][3] = {
	{+1, 0, 1}, {0, +1, 1}, {-1, 0, 1}, {0, -1, 1},
	{+1, +1, 2}, {-1, -1, 2}, {-1, +1, 2}, {+1, -1, 2},
	{+2, +1, 5}, {+1, +2, 5}, {+2, -1, 5}, {+1, -2, 5},
	{-2, -1, 5}, {-1, -2, 5}, {-2, +1, 5}, {-1, +2, 5},
	{+3, +1, 10}, {+1, +3, 10}, {+3, -1, 10}, {+1, -3, 10},
	{-3, -1, 10}, {-1, -3, 10}, {-3, +1, 10}, {-1, +3, 10},
	{+3, +2, 13}, {+2, +3, 13}, {+3, -2, 13}, {+2, -3, 13},
	{-3, -2, 13}, {-2, -3, 13}, {-3, +2, 13}, {-2, +3, 13},
};

/* The new value of unknown (i, j) of x (amle_iteration's body). */
static float amle_update(const float *x, int w, int h, int i, int j, int nn)
{
	float value[32] = {0}, weight[32] = {0};
	int nv = 0;
	for (int p = 0; p < nn; p++) {
		int ii = i + amle_nb[p][0], jj = j + amle_nb[p][1];
		if (ii >= 0 && jj >= 0 && ii < w && jj < h) {
			value[nv] = x[w * jj + ii];
			weight[nv] = amle_nb[p][2];
			nv += 1;
		}
	}
	int mn = 0, mx = 0;
	for (int q = 1; q < nv; q++) {
		if (value[q] < value[mn]) mn = q;
		if (value[q] > value[mx]) mx = q;
	}
	float a = weight[mx], b = weight[mn];
	return (a * value[mn] + b * value[mx]) / (a + b);
}

/* The smallest m >= 2 and k < m such that no offset of the first nn
 * neighbours has (di + k dj) mod m == 0: the colour classes (i + k j) mod m
 * of the parallel sweep. */
void amle_oracle_colouring(int nn, int *m, int *k)
{
	for (int mm = 2; mm < 64; mm++)
		for (int kk = 0; kk < mm; kk++) {
			int ok = 1;
			for (int p = 0; p < nn && ok; p++) {
				int r = (amle_nb[p][0] + kk * amle_nb[p][1]) % mm;
				if (r == 0) ok = 0;
			}
			if (ok) {
				*m = mm;
				*k = kk;
				return;
			}
		}
	*m = 2;
	*k = 1;
}

static int colour_of(int i, int j, int m, int k)
{
	int c = (i + k * j) % m;
	return c < 0 ? c + m : c;
}

static void sweep(float *x, const unsigned char *unk, int w, int h, int nn, int order, int m, int k)
{
	if (order == 0) {
		for (int j = 0; j < h; j++)
			for (int i = 0; i < w; i++)
				if (unk[j * w + i]) x[j * w + i] = amle_update(x, w, h, i, j, nn);
		return;
	}
	for (int c = 0; c < m; c++)
		for (int j = 0; j < h; j++)
			for (int i = 0; i < w; i++)
				if (unk[j * w + i] && colour_of(i, j, m, k) == c)
					x[j * w + i] = amle_update(x, w, h, i, j, nn);
}

/* One channel: y (w*h) from x (w*h, NaN = unknown); init may be NULL.
 * gap[0] = max |tinf - tsup| and gap[1] = their mean over the unknowns
 * after the last iteration (absolute_difference and mean_difference,
 * src/amle.c:114-142), when gap is not NULL. */
int amle_oracle(float *y, const float *x, int w, int h, int nn, int niter, const float *init, int order,
		double *gap)
{
	if (nn < 0) nn = 0;     /* no neighbour: 0/0, as the reference */
	if (nn > 32) nn = 32;   /* the reference reads past its table there */
	int m = 2, k = 1;
	amle_oracle_colouring(nn, &m, &k);
	size_t n = (size_t)w * h;
	float *tinf = malloc(n * sizeof(float)), *tsup = malloc(n * sizeof(float));
	unsigned char *unk = malloc(n);
	if (!tinf || !tsup || !unk) {
		free(tinf); free(tsup); free(unk);
		return 1;
	}
	float mn = INFINITY, mx = -INFINITY;
	for (size_t i = 0; i < n; i++) {
		if (x[i] < mn) mn = x[i];
		if (x[i] > mx) mx = x[i];
	}
	for (size_t i = 0; i < n; i++) {
		unk[i] = isnan(x[i]) ? 1 : 0;
		tinf[i] = unk[i] ? mn : x[i];
		tsup[i] = unk[i] ? (init ? init[i] : mx) : x[i];
	}
	for (int it = 0; it < niter; it++) {
		sweep(tinf, unk, w, h, nn, order, m, k);
		sweep(tsup, unk, w, h, nn, order, m, k);
	}
	if (gap) {
		float e = 0, ea = 0;
		int cnt = 0;
		for (size_t i = 0; i < n; i++)
			if (unk[i]) {
				float t = fabsf(tinf[i] - tsup[i]);
				if (t > e) e = t;
				ea += t;
				cnt++;
			}
		gap[0] = e;
		gap[1] = cnt ? ea / cnt : 0;
	}
	for (size_t i = 0; i < n; i++) y[i] = tsup[i];
	free(tinf);
	free(tsup);
	free(unk);
	return 0;
}
