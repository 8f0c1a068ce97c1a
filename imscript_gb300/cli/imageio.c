/*
 * imageio.c -- iio-compatible image input/output for the simpois command
 * (see imageio.h for the formats and conventions).
 */
#include "imageio.h"

#include <ctype.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

enum { T_F32, T_F64, T_U8, T_U16, T_U32, T_U64, T_I8, T_I16, T_I32, T_I64 };

/* an interleaved image as read: samples in their file type, plus float */
typedef struct {
	int w, h, pd;
	int type;       /* T_* of the samples on file                      */
	double *v;      /* w*h*pd interleaved samples, exact in double      */
} raw_image;

/* transformations of an image as read (defined with IIO_TRANS below) */
static void flip_leftright(raw_image *x);
static void flip_topdown(raw_image *x);
static int trim(raw_image *x, int left, int bottom, int right, int top);

static void *xcalloc(size_t n, size_t s)
{
	void *p = calloc(n ? n : 1, s ? s : 1);
	if (!p) fprintf(stderr, "imageio: out of memory\n");
	return p;
}

/* whole stream into memory */
static unsigned char *slurp(FILE *f, size_t *n)
{
	size_t cap = 1 << 16, len = 0;
	unsigned char *b = malloc(cap);
	if (!b) return NULL;
	for (;;) {
		if (len == cap) {
			unsigned char *nb = realloc(b, cap *= 2);
			if (!nb) { free(b); return NULL; }
			b = nb;
		}
		size_t r = fread(b + len, 1, cap - len, f);
		len += r;
		if (r == 0) break;
	}
	*n = len;
	return b;
}

static int type_size(int t)
{
	switch (t) {
	case T_U8: case T_I8: return 1;
	case T_U16: case T_I16: return 2;
	case T_F32: case T_U32: case T_I32: return 4;
	default: return 8;
	}
}

/* little-endian sample k of type t at p */
static double sample_le(const unsigned char *p, int t)
{
	uint64_t u = 0;
	int s = type_size(t);
	for (int k = s - 1; k >= 0; k--) u = (u << 8) | p[k];
	switch (t) {
	case T_U8: return (double)(uint8_t)u;
	case T_I8: return (double)(int8_t)u;
	case T_U16: return (double)(uint16_t)u;
	case T_I16: return (double)(int16_t)u;
	case T_U32: return (double)(uint32_t)u;
	case T_I32: return (double)(int32_t)u;
	case T_U64: return (double)u;
	case T_I64: return (double)(int64_t)u;
	case T_F32: { uint32_t b = (uint32_t)u; float f; memcpy(&f, &b, 4); return f; }
	default: { double d; memcpy(&d, &u, 8); return d; }
	}
}

/* ---- NumPy .npy 1.0 (iio.c:3216-3300: shape (h,w,pd); a (1,w,pd) array
 * with w>1 and pd>1 is read as (w,pd,1); fortran order transposes) */
static int read_npy(raw_image *x, const unsigned char *b, size_t n)
{
	if (n < 10 || b[6] != 1 || b[7] != 0) {
		fprintf(stderr, "imageio: only NPY 1.0 is supported\n");
		return 1;
	}
	size_t hl = b[8] + 256 * (size_t)b[9];
	if (10 + hl > n) return 1;
	char *hdr = xcalloc(hl + 1, 1);
	if (!hdr) return 1;
	memcpy(hdr, b + 10, hl);
	char descr[16] = {0}, order[16] = {0};
	int h = 1, w = 1, pd = 1;
	int r = sscanf(hdr, "{'descr': '%15[^']', 'fortran_order': %15[^,], 'shape': (%d, %d, %d",
			descr, order, &h, &w, &pd);
	free(hdr);
	if (r < 3) {
		fprintf(stderr, "imageio: badly formed npy header\n");
		return 2;
	}
	if (r < 5) pd = 1;
	if (r < 4) w = h, h = 1;   /* a 1-D array is one row */
	if (h <= 0 || w <= 0 || pd <= 0) {
		fprintf(stderr, "imageio: badly formed npy header (shape not positive)\n");
		return 2;
	}
	if (h == 1 && w > 1 && pd > 1) { h = w; w = pd; pd = 1; }
	const char *d = descr;
	if (*d == '<' || *d == '>' || *d == '=' || *d == '|') {
		if (*d == '>' && strcmp(d + 1, "u1") && strcmp(d + 1, "i1")) {
			fprintf(stderr, "imageio: big-endian npy is not supported\n");
			return 3;
		}
		d++;
	}
	int t;
	if (!strcmp(d, "f4")) t = T_F32;
	else if (!strcmp(d, "f8")) t = T_F64;
	else if (!strcmp(d, "u1") || !strcmp(d, "B1")) t = T_U8;
	else if (!strcmp(d, "u2")) t = T_U16;
	else if (!strcmp(d, "u4")) t = T_U32;
	else if (!strcmp(d, "u8")) t = T_U64;
	else if (!strcmp(d, "i1") || !strcmp(d, "b1")) t = T_I8;
	else if (!strcmp(d, "i2")) t = T_I16;
	else if (!strcmp(d, "i4")) t = T_I32;
	else if (!strcmp(d, "i8")) t = T_I64;
	else if (!strcmp(d, "c8")) { t = T_F32; pd *= 2; }
	else if (!strcmp(d, "c16")) { t = T_F64; pd *= 2; }
	else {
		fprintf(stderr, "imageio: unrecognized npy type \"%s\"\n", d);
		return 4;
	}
	if (order[0] == 'T') { int tmp = h; h = w; w = tmp; }
	size_t ns = (size_t)w * h * pd, ts = type_size(t);
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 5;
	size_t avail = (n - 10 - hl) / ts;
	if (avail < ns) fprintf(stderr, "imageio: npy file smaller than expected\n");
	for (size_t k = 0; k < ns && k < avail; k++) x->v[k] = sample_le(b + 10 + hl + k * ts, t);
	if (order[0] == 'T') {   /* stored column-major: transpose the pixels */
		double *tv = xcalloc(ns, sizeof(double));
		if (!tv) return 5;
		for (int j = 0; j < h; j++)
			for (int i = 0; i < w; i++)
				for (int l = 0; l < pd; l++)
					tv[((size_t)j * w + i) * pd + l] = x->v[((size_t)i * h + j) * pd + l];
		free(x->v);
		x->v = tv;
	}
	x->w = w; x->h = h; x->pd = pd; x->type = t;
	return 0;
}

/* ---- PFM: "Pf" gray or "PF" color, rows as stored, little-endian floats */
static int read_pfm(raw_image *x, const unsigned char *b, size_t n)
{
	int pd = b[1] == 'F' ? 3 : 1, w, h, used = 0;
	float scale;
	char tmp[128] = {0};
	memcpy(tmp, b, n < 127 ? n : 127);
	if (sscanf(tmp + 2, "%d %d %g%n", &w, &h, &scale, &used) != 3) return 1;
	size_t off = 2 + used + 1;
	size_t ns = (size_t)w * h * pd;
	if (off + 4 * ns > n) {
		fprintf(stderr, "imageio: truncated pfm\n");
		return 2;
	}
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 3;
	for (size_t k = 0; k < ns; k++) x->v[k] = sample_le(b + off + 4 * k, T_F32);
	x->w = w; x->h = h; x->pd = pd; x->type = T_F32;
	return 0;
}

/* ---- PNM: P2/P3 ascii, P5/P6 binary (8 or 16 bits, big-endian) */
static int pnm_int(const unsigned char *b, size_t n, size_t *p, int *v)
{
	while (*p < n) {
		if (b[*p] == '#') { while (*p < n && b[*p] != '\n') (*p)++; }
		else if (isspace(b[*p])) (*p)++;
		else break;
	}
	if (*p >= n || !isdigit(b[*p])) return 1;
	long r = 0;
	while (*p < n && isdigit(b[*p])) r = 10 * r + (b[(*p)++] - '0');
	*v = (int)r;
	return 0;
}

/* an ASCII sample: a float as "%f" reads it, after white space */
static int pnm_float(const unsigned char *b, size_t n, size_t *p, double *v)
{
	while (*p < n && isspace(b[*p])) (*p)++;
	char t[64];
	size_t k = 0;
	while (*p + k < n && k < sizeof t - 1 && !isspace(b[*p + k])) {
		t[k] = (char)b[*p + k];
		k++;
	}
	t[k] = 0;
	char *e;
	const float f = strtof(t, &e);
	if (e == t) return 1;
	*p += (size_t)(e - t);
	*v = f;
	return 0;
}

static int read_pnm(raw_image *x, const unsigned char *b, size_t n)
{
	char kind = b[1];
	int pd = (kind == '3' || kind == '6') ? 3 : 1, w, h, mx;
	size_t p = 2;
	if (pnm_int(b, n, &p, &w) || pnm_int(b, n, &p, &h)) return 1;
	/* iio's n-channel variants: "P7" (ASCII) and "P9" (binary) carry the
	 * channel count before the maximum value (iio.c:2291-2330) */
	if ((kind == '7' || kind == '9') && (pnm_int(b, n, &p, &pd) || pd <= 0)) return 1;
	if (pnm_int(b, n, &p, &mx)) return 1;
	if (kind == '7') kind = '2';
	if (kind == '9') kind = '5';
	size_t ns = (size_t)w * h * pd;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	if (kind == '2' || kind == '3') {
		for (size_t k = 0; k < ns; k++)
			if (pnm_float(b, n, &p, &x->v[k])) {
				fprintf(stderr, "imageio: fewer samples than the PNM header announces\n");
				return 1;
			}
	} else {
		p++;   /* the single whitespace after maxval */
		int bps = mx > 255 ? 2 : 1;
		for (size_t k = 0; k < ns && p + bps <= n; k++, p += bps)
			x->v[k] = bps == 1 ? b[p] : 256 * b[p] + b[p + 1];
	}
	x->w = w; x->h = h; x->pd = pd; x->type = mx > 255 ? T_U16 : T_U8;
	return 0;
}

/* ---- ASC: "w h 1 pd" header then planar samples (iio.c:2796-2830) */
static int read_asc(raw_image *x, const unsigned char *b, size_t n)
{
	char *s = xcalloc(n + 1, 1);
	if (!s) return 1;
	memcpy(s, b, n);
	int w, h, d, pd, used;
	if (sscanf(s, "%d %d %d %d%n", &w, &h, &d, &pd, &used) != 4 || d != 1) { free(s); return 1; }
	size_t ns = (size_t)w * h * pd;
	double *planar = xcalloc(ns, sizeof(double));
	x->v = xcalloc(ns, sizeof(double));
	if (!planar || !x->v) { free(s); free(planar); return 2; }
	char *save = NULL, *tok = strtok_r(s + used, " \n", &save);
	for (size_t k = 0; k < ns && tok; k++, tok = strtok_r(NULL, " \n", &save)) planar[k] = atof(tok);
	for (size_t i = 0; i < (size_t)w * h; i++)
		for (int l = 0; l < pd; l++) x->v[i * pd + l] = planar[(size_t)w * h * l + i];
	free(planar);
	free(s);
	x->w = w; x->h = h; x->pd = pd; x->type = T_F32;
	return 0;
}

/* ---- FLO (Middlebury flow: "PIEH", width, height, interleaved float
 * pairs) and JUV ("#UV {" text header padded to 255 bytes, then the u plane
 * and the v plane), 2 channels (iio.c:2619-2654) */
static int read_flo(raw_image *x, const unsigned char *b, size_t n)
{
	uint32_t w, h;
	if (n < 12) return 1;
	memcpy(&w, b + 4, 4);
	memcpy(&h, b + 8, 4);
	const size_t ns = (size_t)w * h * 2;
	if (n < 12 + 4 * ns) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t k = 0; k < ns; k++) {
		float v;
		memcpy(&v, b + 12 + 4 * k, 4);
		x->v[k] = v;
	}
	x->w = (int)w; x->h = (int)h; x->pd = 2; x->type = T_F32;
	return 0;
}

static int read_juv(raw_image *x, const unsigned char *b, size_t n)
{
	char head[256] = {0};
	int w, h;
	if (n < 255) return 1;
	memcpy(head, b, 255);
	if (sscanf(head, "#UV {\n dimx %d dimy %d\n}\n", &w, &h) != 2 || w <= 0 || h <= 0) return 1;
	const size_t np = (size_t)w * h;
	if (n < 255 + 8 * np) return 1;
	x->v = xcalloc(2 * np, sizeof(double));
	if (!x->v) return 2;
	for (size_t i = 0; i < np; i++) {
		float u, v;
		memcpy(&u, b + 255 + 4 * i, 4);
		memcpy(&v, b + 255 + 4 * (np + i), 4);
		x->v[2 * i] = u;
		x->v[2 * i + 1] = v;
	}
	x->w = w; x->h = h; x->pd = 2; x->type = T_F32;
	return 0;
}

/* ---- farbfeld ("farbfeld", big-endian 32-bit width and height, RGBA
 * 16-bit big-endian samples) and PCM ("PC", text width, height and scale,
 * then two float channels) (iio.c:2352-2375, 3164-3183) */
static int read_ffd(raw_image *x, const unsigned char *b, size_t n)
{
	if (n < 16) return 1;
	const uint32_t w = (uint32_t)b[8] << 24 | (uint32_t)b[9] << 16 | (uint32_t)b[10] << 8 | b[11];
	const uint32_t h = (uint32_t)b[12] << 24 | (uint32_t)b[13] << 16 | (uint32_t)b[14] << 8 | b[15];
	const size_t ns = (size_t)w * h * 4;
	if (n < 16 + 2 * ns) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t k = 0; k < ns; k++) x->v[k] = 256 * b[16 + 2 * k] + b[17 + 2 * k];
	x->w = (int)w; x->h = (int)h; x->pd = 4; x->type = T_U16;
	return 0;
}

static int read_pcm(raw_image *x, const unsigned char *b, size_t n)
{
	char head[128] = {0};
	memcpy(head, b, n < 127 ? n : 127);
	int w, h, used;
	float scale;
	if (sscanf(head + 2, " %d %d %g%n", &w, &h, &scale, &used) != 3 || w <= 0 || h <= 0) return 1;
	size_t p = 2 + (size_t)used;
	if (p >= n || !isspace(b[p])) return 1;
	p++;
	fprintf(stderr, "2 PCM w h scale = %d %d %g\n", w, h, scale);
	const size_t ns = (size_t)w * h * 2;
	if (n < p + 4 * ns) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t k = 0; k < ns; k++) {
		float v;
		memcpy(&v, b + p + 4 * k, 4);
		x->v[k] = v;
	}
	x->w = w; x->h = h; x->pd = 2; x->type = T_F32;
	return 0;
}

/* ---- MegaWave RIM images (iio.c:2400-2560): "IR"/"RI" float and "MI"/"IM"
 * byte images (comment length, width, height as 16-bit numbers, 56 bytes,
 * the comment, then the samples), "WE"/"VI" planar ccimage/cfimage (a tag,
 * then channels, rows, columns, band, form and comment size as 32-bit
 * numbers, then the planes).  The second spelling of each swaps bytes --
 * its 16-bit fields are little-endian and its 32-bit ones big-endian, the
 * first's the other way round -- and float samples are swapped with it,
 * except in a cfimage. */
static void swap_bytes(unsigned char *p, size_t words, int size);
static unsigned rim_short(const unsigned char *p, int swp) { return swp ? p[1] * 256u + p[0] : p[0] * 256u + p[1]; }
static uint32_t rim_int(const unsigned char *p, int swp)
{
	return swp ? (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]
	           : (uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | p[0];
}

static int read_rim(raw_image *x, const unsigned char *b, size_t n)
{
	const char a = (char)b[0], c = (char)b[1];
	const int fimage = (a == 'I' && c == 'R') || (a == 'R' && c == 'I');
	const int cimage = (a == 'M' && c == 'I') || (a == 'I' && c == 'M');
	const int swp = (a == 'R') || (a == 'I' && c == 'M') || a == 'V';
	if (fimage || cimage) {
		if (n < 64) return 1;
		const unsigned lencomm = rim_short(b + 2, swp), w = rim_short(b + 4, swp), h = rim_short(b + 6, swp);
		const size_t off = 8 + 56 + lencomm, ns = (size_t)w * h, ss = fimage ? 4 : 1;
		if (n < off + ns * ss) {
			fprintf(stderr, "imageio: could not read entire RIM file\n");
			return 1;
		}
		x->v = xcalloc(ns, sizeof(double));
		if (!x->v) return 2;
		for (size_t k = 0; k < ns; k++) {
			if (cimage) { x->v[k] = b[off + k]; continue; }
			unsigned char q[4];
			memcpy(q, b + off + 4 * k, 4);
			if (swp) swap_bytes(q, 1, 4);
			float v;
			memcpy(&v, q, 4);
			x->v[k] = v;
		}
		x->w = (int)w; x->h = (int)h; x->pd = 1; x->type = fimage ? T_F32 : T_U8;
		return 0;
	}
	/* ccimage / cfimage */
	if (n < 28) return 1;
	const unsigned iv = rim_short(b + 2, swp);
	if (iv != 0x4956 && iv != 0x5649 && iv != 0x4557 && iv != 0x5745) {
		fprintf(stderr, "imageio: bad ccimage header %x\n", iv);
		return 1;
	}
	const uint32_t np = rim_int(b + 4, swp), nrow = rim_int(b + 8, swp), ncol = rim_int(b + 12, swp);
	const uint32_t form = rim_int(b + 20, swp);
	const size_t ns = (size_t)np * nrow * ncol, ss = form == 0x8001 ? 1 : 4;
	if (form != 0x8001 && form != 0xc004) {
		fprintf(stderr, "imageio: unsupported PM_form %x\n", form);
		return 1;
	}
	if (n < 28 + ns * ss) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t j = 0; j < nrow; j++)
		for (size_t i = 0; i < ncol; i++)
			for (size_t l = 0; l < np; l++) {
				const size_t src = i + j * ncol + l * ncol * nrow, dst = l + (i + j * ncol) * np;
				if (ss == 1) {
					x->v[dst] = b[28 + src];
				} else {
					float v;
					memcpy(&v, b + 28 + 4 * src, 4);
					x->v[dst] = v;
				}
			}
	x->w = (int)ncol; x->h = (int)nrow; x->pd = (int)np; x->type = ss == 1 ? T_U8 : T_F32;
	return 0;
}

/* ---- FITS ("SIMPLE  "): after the first 80-byte line, lines "KEY = value"
 * up to "END " give BITPIX, NAXIS1 (width), NAXIS2 (height) and NAXIS3
 * (channels); after padding lines the big-endian samples follow, in file
 * order (iio.c:3453-3530) */
static int read_fit(raw_image *x, const unsigned char *b, size_t n)
{
	int bitpix = -1, w = -1, h = -1, pd = 1;
	size_t line = 0;   /* lines read after the first */
	for (;;) {
		line++;
		const size_t o = 80 * line;
		if (o + 80 > n) {
			fprintf(stderr, "imageio: FITS reader failed at line %zu\n", line);
			return 1;
		}
		char l[81] = {0}, k[81] = {0}, v[81] = {0};
		memcpy(l, b + o, 80);
		if (!memcmp(l, "END ", 4)) break;
		if (sscanf(l, "%80s = %80s", k, v) != 2) continue;
		if (!strcmp(k, "BITPIX")) bitpix = atoi(v);
		if (!strcmp(k, "NAXIS1")) w = atoi(v);
		if (!strcmp(k, "NAXIS2")) h = atoi(v);
		if (!strcmp(k, "NAXIS3")) pd = atoi(v);
	}
	/* the data starts at line ceil(n / 36) * 36 (n the lines after the first),
	 * right after "END" when n is a multiple of 36 */
	const size_t off = 80 * ((line % 36) ? (line / 36 + 1) * 36 : line + 1);
	int type, ss;
	switch (bitpix) {
	case 8: type = T_U8; ss = 1; break;
	case 16: type = T_I16; ss = 2; break;
	case 32: type = T_I32; ss = 4; break;
	case -32: type = T_F32; ss = 4; break;
	case -64: type = T_F64; ss = 8; break;
	default:
		fprintf(stderr, "imageio: unrecognized FITS BITPIX=%d\n", bitpix);
		return 1;
	}
	if (w <= 0 || h <= 0 || pd <= 0) return 1;
	const size_t ns = (size_t)w * h * pd;
	if (n < off + ns * ss) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t k = 0; k < ns; k++) {
		unsigned char q[8];
		memcpy(q, b + off + k * ss, ss);
		swap_bytes(q, 1, ss);   /* big-endian file, little-endian host */
		switch (type) {
		case T_U8: x->v[k] = q[0]; break;
		case T_I16: { int16_t t; memcpy(&t, q, 2); x->v[k] = t; break; }
		case T_I32: { int32_t t; memcpy(&t, q, 4); x->v[k] = t; break; }
		case T_F32: { float t; memcpy(&t, q, 4); x->v[k] = t; break; }
		default: { double t; memcpy(&t, q, 8); x->v[k] = t; break; }
		}
	}
	x->w = w; x->h = h; x->pd = pd; x->type = type;
	return 0;
}

/* ---- PDS ("PDS_"), and CCSD ("CCSD3Z" at byte 0, 1 or 2, the same label
 * language): "KEY = VALUE" label lines from byte 4 (8) (printable
 * characters only; a last line without newline is dropped; 1000 lines at
 * most): RECORD_BYTES (RECORD_TYPE UNDEFINED means 1), the record of the
 * object (^IMAGE, or IIO_PDS_OBJECT), and inside OBJECT = IMAGE: LINES,
 * LINE_SAMPLES, SAMPLE_BITS, BANDS, SAMPLE_TYPE (REAL is float, else
 * unsigned), the display directions (RIGHT flips left-right, DOWN top-down)
 * and LINE_PREFIX_BYTES / LINE_SUFFIX_BYTES (columns around each line, cut
 * off).  The samples, in this machine's byte order, start at record
 * ^IMAGE - 1 (iio.c:2863-2990). */
static int read_pds(raw_image *x, const unsigned char *b, size_t n, size_t start)
{
	const char *oid = getenv("IIO_PDS_OBJECT");
	if (!oid) oid = "^IMAGE";
	long rbytes = -1, w = -1, h = -1, spp = 1, bps = 1, obj = -1, cl = 0, cr = 0;
	int real = 0, in_object = 0, flip_h = 0, flip_v = 0;
	size_t p = start;
	for (int cx = 0; cx < 1000; cx++) {
		char line[1000], key[1000], value[1000];
		size_t i = 0;
		int end = 0;
		for (;;) {
			if (p >= n) { end = 1; break; }
			const unsigned char c = b[p++];
			if (c == '\n' || c == 0) break;
			if (isprint(c) && i < sizeof line - 1) line[i++] = (char)c;
		}
		if (end) break;
		line[i] = 0;
		if (sscanf(line, "%999s = %999s", key, value) != 2) continue;
		if (!strcmp(key, "RECORD_BYTES")) rbytes = atol(value);
		if (!strcmp(key, "RECORD_TYPE") && strstr(value, "UNDEFINED")) rbytes = 1;
		if (!strcmp(key, oid)) obj = atol(value);
		if (!strcmp(key, "OBJECT") && !strcmp(value, oid + 1)) in_object = 1;
		if (!in_object) continue;
		if (!strcmp(key, "LINES")) h = atol(value);
		if (!strcmp(key, "LINE_SAMPLES")) w = atol(value);
		if (!strcmp(key, "SAMPLE_BITS")) bps = atol(value);
		if (!strcmp(key, "BANDS")) spp = atol(value);
		if (!strcmp(key, "SAMPLE_TYPE")) {
			if (strstr(value, "REAL")) real = 1;
			if (strstr(value, "UNSIGNED")) real = 0;
			if (strstr(value, "INTEGER")) real = 0;
		}
		if (!strcmp(key, "SAMPLE_DISPLAY_DIRECTION")) flip_h = !strcmp(value, "RIGHT");
		if (!strcmp(key, "LINE_DISPLAY_DIRECTION")) flip_v = !strcmp(value, "DOWN");
		if (!strcmp(key, "LINE_PREFIX_BYTES")) cl = atol(value);
		if (!strcmp(key, "LINE_SUFFIX_BYTES")) cr = atol(value);
		if (!strcmp(key, "END_OBJECT") && !strcmp(value, oid + 1)) break;
	}
	w += cl + cr;
	int type = -1;
	if (real && bps == 32) type = T_F32;
	if (real && bps == 64) type = T_F64;
	if (!real && bps == 8) type = T_U8;
	if (!real && bps == 16) type = T_U16;
	if (!real && bps == 32) type = T_U32;
	if (type < 0 || w <= 0 || h <= 0 || spp <= 0 || rbytes < 0 || obj < 1) {
		fprintf(stderr, "imageio: unsupported or incomplete PDS label\n");
		return 1;
	}
	const size_t ss = (size_t)bps / 8, ns = (size_t)w * h * spp, off = (size_t)rbytes * (obj - 1);
	if (off + ns * ss > n) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t k = 0; k < ns; k++) {
		const unsigned char *q = b + off + k * ss;
		switch (type) {
		case T_U8: x->v[k] = q[0]; break;
		case T_U16: { uint16_t t; memcpy(&t, q, 2); x->v[k] = t; break; }
		case T_U32: { uint32_t t; memcpy(&t, q, 4); x->v[k] = t; break; }
		case T_F32: { float t; memcpy(&t, q, 4); x->v[k] = t; break; }
		default: { double t; memcpy(&t, q, 8); x->v[k] = t; break; }
		}
	}
	x->w = (int)w; x->h = (int)h; x->pd = (int)spp; x->type = type;
	if (flip_v) flip_topdown(x);
	if (flip_h) flip_leftright(x);
	return trim(x, (int)cl, 0, (int)cr, 0);
}

/* ---- VICAR ("LBLSIZE="): the 9 characters after the tag give the label
 * size n; the label up to byte n - 1 holds space-separated KEY=VALUE
 * tokens: TYPE 'IMAGE' and ORG 'BSQ' required, FORMAT (BYTE, HALF 16-bit
 * signed, FULL, REAL, DOUBL), NL lines, NS samples, NB bands, RECSIZE =
 * NBB + NS x sample size, NBB bytes before each line, NLB records skipped,
 * INTFMT 'HIGH' swapping 2- and 4-byte samples.  The NL x NB records
 * follow the label, band after band, read as they come (iio.c:3298-3418). */
static int read_vic(raw_image *x, const unsigned char *b, size_t n)
{
	if (n < 17) return 1;
	char sz[10] = {0};
	memcpy(sz, b + 8, 9);
	const long lbl = atol(sz);
	if (lbl < 18 || (size_t)lbl > n) return 1;
	char *l = malloc((size_t)lbl);
	if (!l) return 2;
	memcpy(l, b + 17, (size_t)lbl - 18);   /* the label's last byte is dropped */
	l[lbl - 18] = 0;
	long recsize = -1, nl = -1, ns = -1, nb = -1, nbb = 0, nlb = 0;
	char format[99] = "", type[99] = "", org[99] = "", ifmt[99] = "";
	char *save = NULL;
	for (char *tok = strtok_r(l, " ", &save); tok; tok = strtok_r(NULL, " ", &save)) {
		char *eq = strchr(tok, '=');
		if (!eq || eq == tok || !eq[1]) continue;
		*eq = 0;
		const char *k = tok, *v = eq + 1;
		char vv[99];
		sscanf(v, "%98s", vv);
		if (!strcmp(k, "RECSIZE")) recsize = atol(vv);
		if (!strcmp(k, "FORMAT")) snprintf(format, sizeof format, "%s", vv);
		if (!strcmp(k, "TYPE")) snprintf(type, sizeof type, "%s", vv);
		if (!strcmp(k, "ORG")) snprintf(org, sizeof org, "%s", vv);
		if (!strcmp(k, "INTFMT")) snprintf(ifmt, sizeof ifmt, "%s", vv);
		if (!strcmp(k, "NL")) nl = atol(vv);
		if (!strcmp(k, "NS")) ns = atol(vv);
		if (!strcmp(k, "NB")) nb = atol(vv);
		if (!strcmp(k, "NBB")) nbb = atol(vv);
		if (!strcmp(k, "NLB")) nlb = atol(vv);
	}
	free(l);
	int t = -1, ss = 0;
	if (!strcmp(format, "'BYTE'")) { t = T_U8; ss = 1; }
	if (!strcmp(format, "'HALF'")) { t = T_I16; ss = 2; }
	if (!strcmp(format, "'FULL'")) { t = T_I32; ss = 4; }
	if (!strcmp(format, "'REAL'")) { t = T_F32; ss = 4; }
	if (!strcmp(format, "'DOUBL'")) { t = T_F64; ss = 8; }
	if (strcmp(type, "'IMAGE'") || strcmp(org, "'BSQ'") || recsize <= 0 || t < 0 || nl <= 0 || ns <= 0 ||
			nb <= 0 || recsize != nbb + ns * ss) {
		fprintf(stderr, "imageio: unsupported VICAR label\n");
		return 1;
	}
	const size_t nrec = (size_t)nl * nb, off = (size_t)lbl + (size_t)nlb * recsize;
	if (off + nrec * recsize > n) return 1;
	const int swap = !strcmp(ifmt, "'HIGH'") && (ss == 2 || ss == 4);
	x->v = xcalloc(nrec * ns, sizeof(double));
	if (!x->v) return 2;
	size_t k = 0;
	for (size_t r = 0; r < nrec; r++)
		for (long i = 0; i < ns; i++, k++) {
			unsigned char q[8];
			memcpy(q, b + off + r * recsize + nbb + i * ss, ss);
			if (swap) swap_bytes(q, 1, ss);
			switch (t) {
			case T_U8: x->v[k] = q[0]; break;
			case T_I16: { int16_t v; memcpy(&v, q, 2); x->v[k] = v; break; }
			case T_I32: { int32_t v; memcpy(&v, q, 4); x->v[k] = v; break; }
			case T_F32: { float v; memcpy(&v, q, 4); x->v[k] = v; break; }
			default: { double v; memcpy(&v, q, 8); x->v[k] = v; break; }
			}
		}
	x->w = (int)ns; x->h = (int)nl; x->pd = (int)nb; x->type = t;
	return 0;
}

/* ---- RAT (radar): bytes 04 00 00 00, then 30 32-bit fields of which the
 * third to sixth are d, width, height and the variant (only 6), then
 * width x height pixels of 2 d^2 floats (iio.c:3185-3214) */
static int read_rat(raw_image *x, const unsigned char *b, size_t n)
{
	if (n < 124) return 1;
	int32_t d, w, h, var;
	memcpy(&d, b + 8, 4);
	memcpy(&w, b + 12, 4);
	memcpy(&h, b + 16, 4);
	memcpy(&var, b + 20, 4);
	if (var != 6) {
		fprintf(stderr, "imageio: RAT option var=%d not implemented\n", var);
		return 1;
	}
	if (d <= 0 || w <= 0 || h <= 0) return 1;
	const size_t pd = 2 * (size_t)d * d, ns = (size_t)w * h * pd;
	if (n < 124 + 4 * ns) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t k = 0; k < ns; k++) {
		float v;
		memcpy(&v, b + 124 + 4 * k, 4);
		x->v[k] = v;
	}
	x->w = w; x->h = h; x->pd = (int)pd; x->type = T_F32;
	return 0;
}

/* ---- LUM: "FLOA" at byte 8 -- big-endian 16-bit width and height at bytes
 * 2 and 6, big-endian floats from byte 3988 -- or "12LI" -- little-endian
 * 32-bit width and height at 0 and 4, 16-bit samples from byte 11968
 * (iio.c:2656-2697, 5290-5305) */
static int read_lum(raw_image *x, const unsigned char *b, size_t n)
{
	if (b[8] == '1') {
		uint32_t w, h;
		memcpy(&w, b, 4);
		memcpy(&h, b + 4, 4);
		const size_t ns = (size_t)w * h;
		if (n < 11968 + 2 * ns) return 1;
		x->v = xcalloc(ns, sizeof(double));
		if (!x->v) return 2;
		for (size_t k = 0; k < ns; k++) x->v[k] = b[11968 + 2 * k] + 256 * b[11969 + 2 * k];
		x->w = (int)w; x->h = (int)h; x->pd = 1; x->type = T_U16;
		return 0;
	}
	const int w = 256 * b[2] + b[3], h = 256 * b[6] + b[7];
	const size_t ns = (size_t)w * h;
	if (n < 0xf94 + 4 * ns) return 1;
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) return 2;
	for (size_t k = 0; k < ns; k++) {
		const unsigned char *q = b + 0xf94 + 4 * k;
		const uint32_t u = (uint32_t)q[0] << 24 | (uint32_t)q[1] << 16 | (uint32_t)q[2] << 8 | q[3];
		float v;
		memcpy(&v, &u, 4);
		x->v[k] = v;
	}
	x->w = w; x->h = h; x->pd = 1; x->type = T_F32;
	return 0;
}

/* ---- CSV and TXT: one image row per line, samples separated by commas
 * (CSV) or spaces (TXT); height = newlines, width = separators / height + 1,
 * samples parsed in order, any missing ones 0 (iio.c:2992-3071) */
static int read_text(raw_image *x, const unsigned char *b, size_t n, char sep)
{
	size_t h = 0, ns = 0;
	for (size_t i = 0; i < n; i++) {
		h += b[i] == '\n';
		ns += b[i] == (unsigned char)sep;
	}
	if (h == 0) return 1;
	const size_t w = ns / h + 1;
	char *s = xcalloc(n + 1, 1);
	x->v = xcalloc(w * h, sizeof(double));
	if (!s || !x->v) { free(s); return 2; }
	memcpy(s, b, n);
	const char delim[3] = {sep, '\n', 0};
	char *save = NULL, *tok = strtok_r(s, delim, &save);
	for (size_t k = 0; k < w * h && tok; k++, tok = strtok_r(NULL, delim, &save)) x->v[k] = (float)atof(tok);
	free(s);
	x->w = (int)w; x->h = (int)h; x->pd = 1; x->type = T_F32;
	return 0;
}

/* The text formats as iio tells them apart (iio.c:5260-5300, 5347-5400): on
 * the first 256 bytes (all of a shorter file), CSV when every byte is a
 * digit, ".e+-,", "naifNAIF" or a newline; else, when every byte is a digit,
 * ".eE+- ", "naifNAIF" or a newline, TXT when the first line does not hold
 * exactly three spaces or the second holds as many, else ASC when the first
 * line is "w h 1 pd".  0 = none of them. */
enum { TXT_NONE, TXT_CSV, TXT_TXT, TXT_ASC };
static int text_format(const unsigned char *b, size_t n)
{
	const size_t m = n < 256 ? n : 256;
	char head[257] = {0};
	memcpy(head, b, m);
	if (strspn(head, "0123456789.e+-,naifNAIF\n") == m) return TXT_CSV;
	if (strspn(head, "0123456789.eE+- naifNAIF\n") != m) return TXT_NONE;
	int a = 0, c = 0;
	size_t i = 0;
	for (; i < m && head[i] != '\n'; i++) a += head[i] == ' ';
	for (i++; i < m && head[i] != '\n'; i++) c += head[i] == ' ';
	if (a != 3 || a == c) return TXT_TXT;
	int t[4];
	if (sscanf(head, "%d %d %d %d", t, t + 1, t + 2, t + 3) == 4 && t[2] == 1) return TXT_ASC;
	return TXT_NONE;
}

/* iio's semantic names (iio.c:5604-5633): "zero:WxH[,pd]" and "one:WxH[,pd]"
 * (byte samples), "constant:V:WxH" (one float channel); 1 when `name` is
 * one (x filled, or a message on a malformed one), 0 otherwise. */
static int semantic_name(const char *name, raw_image *x, int *rc)
{
	int s[2], pd = 1;
	double value;
	if (name == strstr(name, "zero:") || name == strstr(name, "one:")) {
		const int one = name[0] == 'o';
		const char *q = name + (one ? 4 : 5);
		if (sscanf(q, "%dx%d,%d", s, s + 1, &pd) != 3 && sscanf(q, "%dx%d", s, s + 1) != 2) {
			fprintf(stderr, "imageio: bad semantical name \"%s\"\n", name);
			*rc = 1;
			return 1;
		}
		value = one;
		x->type = T_U8;
	} else if (name == strstr(name, "constant:")) {
		float v;
		if (sscanf(name + 9, "%g:%dx%d", &v, s, s + 1) != 3) {
			fprintf(stderr, "imageio: bad semantical name \"%s\"\n", name);
			*rc = 1;
			return 1;
		}
		value = v;
		x->type = T_F32;
	} else {
		return 0;
	}
	if (s[0] <= 0 || s[1] <= 0 || pd <= 0) {
		fprintf(stderr, "imageio: bad semantical name \"%s\"\n", name);
		*rc = 1;
		return 1;
	}
	x->w = s[0];
	x->h = s[1];
	x->pd = pd;
	size_t n = (size_t)s[0] * s[1] * pd;
	x->v = xcalloc(n, sizeof(double));
	if (!x->v) { *rc = 1; return 1; }
	for (size_t i = 0; i < n; i++) x->v[i] = value;
	*rc = 0;
	return 1;
}

/* ------------------------------------------- transformations on reading */

/* Exchange the samples of pixels (i, j) and (a, b). */
static void swap_pixels(raw_image *x, int i, int j, int a, int b)
{
	double *p = x->v + ((size_t)j * x->w + i) * x->pd, *q = x->v + ((size_t)b * x->w + a) * x->pd;
	for (int l = 0; l < x->pd; l++) {
		double t = p[l];
		p[l] = q[l];
		q[l] = t;
	}
}

static void flip_leftright(raw_image *x)
{
	for (int j = 0; j < x->h; j++)
		for (int i = 0; i < x->w / 2; i++) swap_pixels(x, i, j, x->w - 1 - i, j);
}

static void flip_topdown(raw_image *x)
{
	for (int j = 0; j < x->h / 2; j++)
		for (int i = 0; i < x->w; i++) swap_pixels(x, i, j, i, x->h - 1 - j);
}

/* out(i, j) = in(j, i); the image becomes h x w */
static int transpose(raw_image *x)
{
	const int nw = x->h, nh = x->w, pd = x->pd;
	double *y = xcalloc((size_t)nw * nh * pd, sizeof(double));
	if (!y) return 1;
	for (int j = 0; j < nh; j++)
		for (int i = 0; i < nw; i++)
			for (int l = 0; l < pd; l++)
				y[((size_t)j * nw + i) * pd + l] = x->v[((size_t)i * x->w + j) * pd + l];
	free(x->v);
	x->v = y;
	x->w = nw;
	x->h = nh;
	return 0;
}

/* iio's two-letter orientations (iio.c:814-823): an upper-case first letter
 * flips left-right, an upper-case second letter flips top-down, and the
 * letters in the order y, x transpose, in that order. */
static int reorient(raw_image *x, int orx, int ory)
{
	if (isupper(orx)) flip_leftright(x);
	if (isupper(ory)) flip_topdown(x);
	if (toupper(orx) > toupper(ory)) return transpose(x);
	return 0;
}

/* A permutation of the three axes of the interleaved samples, named "x"
 * (the channels), "y" (the columns) and "z" (the rows); the i-th letter of
 * t names the input axis that becomes output axis i, the first being the
 * new channel axis (iio.c:887-956). */
static int reorient3d(raw_image *x, const char *t)
{
	static const char *known[] = {"xyz", "yxz", "xzy", "zxy", "zyx", "yzx"};
	int ok = 0;
	for (int k = 0; k < 6; k++) ok |= !strcmp(t, known[k]);
	if (!ok) {
		fprintf(stderr, "imageio: unrecognized trasnposition string \"%s\"\n", t);
		return 1;
	}
	const int u[3] = {x->pd, x->w, x->h};
	int v[3], ax[3];
	for (int k = 0; k < 3; k++) {
		ax[k] = t[k] - 'x';
		v[k] = u[ax[k]];
	}
	double *y = xcalloc((size_t)u[0] * u[1] * u[2], sizeof(double));
	if (!y) return 1;
	int a[3];
	for (a[2] = 0; a[2] < v[2]; a[2]++)
		for (a[1] = 0; a[1] < v[1]; a[1]++)
			for (a[0] = 0; a[0] < v[0]; a[0]++) {
				int c[3];
				for (int k = 0; k < 3; k++) c[ax[k]] = a[k];
				y[((size_t)a[2] * v[1] + a[1]) * v[0] + a[0]] =
					x->v[((size_t)c[2] * u[1] + c[1]) * u[0] + c[0]];
			}
	free(x->v);
	x->v = y;
	x->pd = v[0];
	x->w = v[1];
	x->h = v[2];
	return 0;
}

/* The value of a sample outside the old image after a trim: NaN for float
 * samples, the bits of a float (double) NaN for 4-byte (8-byte) integer
 * samples, 0 for narrower ones (iio.c:832-870). */
static double pad_value(int type)
{
	switch (type) {
	case T_F32: case T_F64: return NAN;
	case T_I32: case T_U32: return 2143289344.0;            /* 0x7fc00000 */
	case T_I64: case T_U64: return 9221120237041090560.0;   /* 0x7ff8000000000000 */
	default: return 0;
	}
}

/* Remove `left` columns on the left, `right` on the right, `top` rows at the
 * top and `bottom` at the bottom; negative counts add padding. */
static int trim(raw_image *x, int left, int bottom, int right, int top)
{
	const int nw = x->w - left - right, nh = x->h - bottom - top, pd = x->pd;
	if (nw <= 0 || nh <= 0) {
		fprintf(stderr, "imageio: trim of a %dx%d image to %dx%d\n", x->w, x->h, nw, nh);
		return 1;
	}
	double *y = xcalloc((size_t)nw * nh * pd, sizeof(double));
	if (!y) return 1;
	const double pad = pad_value(x->type);
	for (int j = 0; j < nh; j++)
		for (int i = 0; i < nw; i++) {
			const int si = i + left, sj = j + top;
			const int in = si >= 0 && sj >= 0 && si < x->w && sj < x->h;
			for (int l = 0; l < pd; l++)
				y[((size_t)j * nw + i) * pd + l] = in ? x->v[((size_t)sj * x->w + si) * pd + l] : pad;
		}
	free(x->v);
	x->v = y;
	x->w = nw;
	x->h = nh;
	return 0;
}

static int flip(raw_image *x, const char *s)
{
	int r = 0;
	if (!strcmp(s, "leftright")) flip_leftright(x);
	if (!strcmp(s, "topdown")) flip_topdown(x);
	if (!strcmp(s, "transpose")) r |= transpose(x);
	if (!strcmp(s, "r270")) r |= reorient(x, 'y', 'X');
	if (!strcmp(s, "r90")) r |= reorient(x, 'Y', 'x');
	if (!strcmp(s, "r180")) r |= reorient(x, 'X', 'Y');
	if (!strcmp(s, "posetrans")) r |= reorient(x, 'Y', 'X');
	if (strlen(s) == 2) r |= reorient(x, s[0], s[1]);
	if (strlen(s) == 3 && tolower(s[0]) + tolower(s[1]) + tolower(s[2]) == 3 * 'y') r |= reorient3d(x, s);
	return r;
}

static int read_core(const char *name, raw_image *x);
static int read_raw(const char *name, raw_image *x);
static float gray_of(const double *p, int type);

/* ---- GDAL VRT ("<VRT"): the first line's rasterXSize and rasterYSize give
 * the size of one float channel; then every DstRect (xOff, yOff, xSize,
 * ySize) with a "<SourceFilename attributes>name<" tag pastes that image,
 * read as one gray channel from the VRT's directory, at the offset
 * (iio.c:3085-3160).  Pixels no tile covers read 0. */
static int xml_attr(int *out, const char *line, const char *tag, const char *attr)
{
	if (!strstr(line, tag)) return 0;
	const char *a = strstr(line, attr);
	if (!a) return 0;
	*out = atoi(a + 2 + strlen(attr));
	return 1;
}

static int read_vrt(raw_image *x, const unsigned char *b, size_t n, const char *name)
{
	char *text = malloc(n + 1);
	if (!text) return 2;
	memcpy(text, b, n);
	text[n] = 0;
	char *save = NULL, *line = strtok_r(text + 4, "\n", &save);   /* lines (empty ones skipped) */
	int w = 0, h = 0, cx = 0;
	if (line) {
		cx += xml_attr(&w, line, "Dataset", "rasterXSize");
		cx += xml_attr(&h, line, "Dataset", "rasterYSize");
	}
	if (!line || w <= 0 || h <= 0 || cx != 2) { free(text); return 1; }
	x->v = xcalloc((size_t)w * h, sizeof(double));
	if (!x->v) { free(text); return 2; }
	x->w = w; x->h = h; x->pd = 1; x->type = T_F32;
	char dir[4096];
	snprintf(dir, sizeof dir, "%s", strcmp(name, "-") ? name : ".");
	char *slash = strrchr(dir, '/');
	if (slash) *slash = 0; else snprintf(dir, sizeof dir, ".");
	int pos[4] = {0, 0, 0, 0}, pos_cx = 0, has_fname = 0, r = 0;
	char fname[4096] = "";
	while (!r && (line = strtok_r(NULL, "\n", &save))) {
		pos_cx += xml_attr(pos + 0, line, "DstRect", "xOff");
		pos_cx += xml_attr(pos + 1, line, "DstRect", "yOff");
		pos_cx += xml_attr(pos + 2, line, "DstRect", "xSize");
		pos_cx += xml_attr(pos + 3, line, "DstRect", "ySize");
		char tmp[4096];
		if (sscanf(line, " <SourceFilename %*[^>]>%4095[^<]s</SourceFilename>", tmp) == 1) {
			snprintf(fname, sizeof fname, "%s", tmp);
			has_fname++;
		}
		if (pos_cx == 4 && has_fname == 1) {
			pos_cx = has_fname = 0;
			char full[8200];
			snprintf(full, sizeof full, "%s/%s", dir, fname);
			raw_image t = {0};
			r = read_raw(full, &t);
			if (!r && t.pd != 1 && t.pd != 3 && t.pd != 4) {
				fprintf(stderr, "imageio: non-scalarizable image \"%s\"\n", full);
				r = 1;
			}
			for (int j = 0; !r && j < pos[3]; j++)
				for (int i = 0; i < pos[2]; i++) {
					const int ii = i + pos[0], jj = j + pos[1];
					if (ii < 0 || jj < 0 || ii >= w || jj >= h || i >= t.w || j >= t.h) continue;
					const double *q = t.v + ((size_t)j * t.w + i) * t.pd;
					x->v[(size_t)jj * w + ii] = t.pd == 1 ? (float)q[0] : gray_of(q, t.type);
				}
			free(t.v);
		}
	}
	free(text);
	return r;
}

/* ---- RAW: headerless binary samples described by a list of one-letter
 * fields, "RAW[w640,h480,p3,tuint16,e1]:file" or the IIO_RAW variable
 * (iio.c:3597-3777).  w, h, p (or d): sizes; o: header bytes; t: sample
 * type; e: swap bytes; i, y: image index and bytes between images; r: two-
 * letter orientation; b: ignored.  A value "@pos[/size]" is an integer read
 * from the file at byte pos (size 1, 2, 4 unsigned, negative signed; -4 by
 * default).  Missing sizes and offset are estimated from the file size. */
static int raw_type(const char *t, int *type, int *ss)
{
	char u[16] = {0};
	for (int i = 0; t[i] && i < 15; i++) u[i] = (char)toupper((unsigned char)t[i]);
	static const struct { const char *n; int t, s; } tab[] = {
		{"INT8", T_I8, 1}, {"UINT8", T_U8, 1}, {"CHAR", T_U8, 1}, {"INT16", T_I16, 2}, {"SHORT", T_I16, 2},
		{"UINT16", T_U16, 2}, {"INT32", T_I32, 4}, {"INT", T_I32, 4}, {"UINT32", T_U32, 4},
		{"INT64", T_I64, 8}, {"LONG", T_I64, 8}, {"LONGLONG", T_I64, 8}, {"UINT64", T_U64, 8},
		{"FLOAT", T_F32, 4}, {"DOUBLE", T_F64, 8}};
	for (size_t k = 0; k < sizeof tab / sizeof *tab; k++)
		if (!strcmp(u, tab[k].n)) {
			*type = tab[k].t;
			*ss = tab[k].s;
			return 0;
		}
	fprintf(stderr, "imageio: unrecognized typename \"%s\"\n", t);
	return 1;
}

static void swap_bytes(unsigned char *p, size_t words, int size)
{
	for (size_t k = 0; k < words; k++, p += size)
		for (int a = 0, b = size - 1; a < b; a++, b--) {
			unsigned char t = p[a];
			p[a] = p[b];
			p[b] = t;
		}
}

/* an integer field of the file (the reference swaps it in place) */
static int raw_field(unsigned char *d, size_t n, const char *tok, int swap, int *v)
{
	int pos, size = -4;
	if (sscanf(tok, "%d/%d", &pos, &size) != 2 && sscanf(tok, "%d", &pos) != 1) {
		*v = 0;
		return 0;
	}
	const int as = size < 0 ? -size : size;
	if (pos < 0 || (size_t)(as + pos) > n || (as != 1 && as != 2 && as != 4)) {
		fprintf(stderr, "imageio: can not read field beyond data size\n");
		return 1;
	}
	unsigned char *p = d + pos;
	if (swap && as > 1) swap_bytes(p, 1, as);
	uint32_t u = 0;
	memcpy(&u, p, as);   /* little-endian host */
	switch (size) {
	case 1: *v = (uint8_t)u; break;
	case 2: *v = (uint16_t)u; break;
	case 4: *v = (int)u; break;
	case -1: *v = (int8_t)u; break;
	case -2: *v = (int16_t)u; break;
	default: *v = (int32_t)u; break;
	}
	return 0;
}

static int read_raw_spec(const char *spec, const char *file, raw_image *x)
{
	FILE *f = strcmp(file, "-") ? fopen(file, "rb") : stdin;
	if (!f) {
		fprintf(stderr, "imageio: can not open file \"%s\" in mode \"r\"\n", file);
		return 1;
	}
	size_t n = 0;
	unsigned char *d = slurp(f, &n);
	if (f != stdin) fclose(f);
	if (!d) return 1;
	char *desc = malloc(strlen(spec) + 1);
	if (!desc) { free(d); return 1; }
	strcpy(desc, spec);
	long w = -1, h = -1, pd = 1, off = -1, index = 0, frame = 0;
	int swap = 0, type = T_U8, ss = 1, orient = 0, r = 0;
	for (char *tok = desc; tok && !r;) {
		char *next = strchr(tok, ',');
		if (next) *next++ = 0;
		if (*tok) {
			int v = 0;
			if (tok[1] == '@') r = raw_field(d, n, tok + 2, swap, &v);
			else v = atoi(tok + 1);
			switch (*tok) {
			case 'w': w = v; break;
			case 'h': h = v; break;
			case 'd': case 'p': pd = v; break;
			case 'o': off = v; break;
			case 'e': swap = v; break;
			case 'i': index = v; break;
			case 'y': frame = v; break;
			case 't': r = raw_type(tok + 1, &type, &ss); break;
			case 'r': orient = tok[1] ? tok[1] + 256 * tok[2] : 0; break;
			default: break;
			}
		}
		tok = next;
	}
	free(desc);
	if (r) { free(d); return r; }
	const long fs = (long)n, px = pd * ss;
	if (off < 0 && w > 0 && h > 0) off = fs - w * h * px;
	if (w < 0 && off > 0 && h > 0) w = (fs - off) / (h * px);
	if (h < 0 && off > 0 && w > 0) h = (fs - off) / (w * px);
	if (off < 0) off = 0;
	if (h < 0 && w > 0) h = fs / (w * px);
	if (w < 0 && h > 0) w = fs / (h * px);
	if (off < 0 || w <= 0 || h <= 0 || pd <= 0) {
		fprintf(stderr, "imageio: could not determine width, height and offset (got %ld,%ld,%ld)\n", w, h, off);
		free(d);
		return 1;
	}
	off += frame + index * (frame + w * h * px);
	const size_t ns = (size_t)w * h * pd;
	if ((size_t)off + ns * ss > n) {
		fprintf(stderr, "imageio: raw file is not large enough\n");
		free(d);
		return 1;
	}
	unsigned char *p = d + off;
	/* the reference swaps 2-byte samples, and 4-byte words -- one per
	 * sample, so only the first half of 8-byte samples -- for wider ones */
	if (swap && ss == 2) swap_bytes(p, ns, 2);
	if (swap && ss >= 4) swap_bytes(p, ns, 4);
	x->v = xcalloc(ns, sizeof(double));
	if (!x->v) { free(d); return 1; }
	for (size_t k = 0; k < ns; k++) {
		const unsigned char *q = p + k * ss;
		switch (type) {
		case T_U8: x->v[k] = q[0]; break;
		case T_I8: x->v[k] = (int8_t)q[0]; break;
		case T_U16: { uint16_t v; memcpy(&v, q, 2); x->v[k] = v; break; }
		case T_I16: { int16_t v; memcpy(&v, q, 2); x->v[k] = v; break; }
		case T_U32: { uint32_t v; memcpy(&v, q, 4); x->v[k] = v; break; }
		case T_I32: { int32_t v; memcpy(&v, q, 4); x->v[k] = v; break; }
		case T_U64: { uint64_t v; memcpy(&v, q, 8); x->v[k] = (double)v; break; }
		case T_I64: { int64_t v; memcpy(&v, q, 8); x->v[k] = (double)v; break; }
		case T_F32: { float v; memcpy(&v, q, 4); x->v[k] = v; break; }
		default: { double v; memcpy(&v, q, 8); x->v[k] = v; break; }
		}
	}
	free(d);
	x->w = (int)w; x->h = (int)h; x->pd = (int)pd; x->type = type;
	return orient ? reorient(x, orient & 0xff, orient >> 8) : 0;
}

/* "RAW[spec]:name" (iio.c:3597-3605): the colon after the closing bracket */
static const char *raw_prefix(const char *name)
{
	if (name != strstr(name, "RAW[")) return NULL;
	const char *colon = strchr(name, ':');
	return colon && colon[-1] == ']' ? colon : NULL;
}

/* Filter the image through a shell command: the image goes to the command's
 * standard input as a file, its standard output is read back as the image,
 * IIO_TRANS unset for it (iio.c:3826-3852); a command that fails leaves the
 * image as it was. */
static int pipe_through(raw_image *x, const char *cmd)
{
	char in[] = "/tmp/imageio_in_XXXXXX", out[] = "/tmp/imageio_out_XXXXXX";
	int fi = mkstemp(in);
	if (fi < 0) return 1;
	close(fi);
	int fo = mkstemp(out);
	if (fo < 0) { unlink(in); return 1; }
	close(fo);
	size_t np = (size_t)x->w * x->h;
	float *pl = xcalloc(np * x->pd, sizeof(float));
	int r = !pl;
	if (pl) {
		for (size_t i = 0; i < np; i++)
			for (int l = 0; l < x->pd; l++) pl[np * l + i] = (float)x->v[i * x->pd + l];
		r = imgio_write_split(in, pl, x->w, x->h, x->pd);
		free(pl);
	}
	if (!r) {
		size_t len = strlen(cmd) + strlen(in) + strlen(out) + 32;
		char *c = malloc(len);
		if (!c) r = 1;
		else {
			snprintf(c, len, "(unset IIO_TRANS; %s) <%s >%s", cmd, in, out);
			if (!system(c)) {
				raw_image y = {0};
				r = read_core(out, &y);
				if (!r) {
					free(x->v);
					*x = y;
				} else {
					free(y.v);
				}
			}
			free(c);
		}
	}
	unlink(in);
	unlink(out);
	return r;
}

/* Apply iio's list of transformations "op=value,op=value,..." (up to the
 * first ']') in order (iio.c:3854-3884): flip=leftright|topdown|transpose|
 * r90|r180|r270|posetrans|<two letters>|<three axes>, pipe=<command>, and
 * the trims x=V (drop V columns on the left), y=V (V rows at the top), w=V
 * (keep V columns), h=V (keep V rows).  Unknown operations are ignored. */
static int trans_apply(raw_image *x, const char *list)
{
	size_t n = strcspn(list, "]");
	char *t = malloc(n + 1);
	if (!t) return 1;
	memcpy(t, list, n);
	t[n] = 0;
	int r = 0;
	for (char *tok = t; tok && !r;) {
		char *next = strchr(tok, ',');
		if (next) *next++ = 0;
		char *eq = strchr(tok, '=');
		if (eq && eq != tok && eq[1]) {
			*eq = 0;
			const char *o = tok, *v = eq + 1;
			const int V = atoi(v), w = x->w, h = x->h;
			if (!strcmp(o, "flip")) r = flip(x, v);
			else if (!strcmp(o, "pipe")) r = pipe_through(x, v);
			else if (!strcmp(o, "x")) r = trim(x, V, 0, 0, 0);
			else if (!strcmp(o, "y")) r = trim(x, 0, 0, 0, V);
			else if (!strcmp(o, "w")) r = trim(x, 0, 0, w - V, 0);
			else if (!strcmp(o, "h")) r = trim(x, 0, h - V, 0, 0);
		}
		tok = next;
	}
	free(t);
	return r;
}

/* "TRANS[list]:name" (iio.c:3796-3808): the colon after the closing bracket */
static const char *trans_prefix(const char *name)
{
	if (name != strstr(name, "TRANS[")) return NULL;
	const char *colon = strchr(name, ':');
	return colon && colon[-1] == ']' ? colon : NULL;
}

/* A named image: semantic names as they are; "TRANS[list]:name" reads name
 * and applies the list; then every image read from a file gets the list in
 * IIO_TRANS, when set (iio.c:5587-5705). */
static int read_raw(const char *name, raw_image *x)
{
	int rc;
	if (semantic_name(name, x, &rc)) return rc;
	const char *colon = trans_prefix(name), *rcolon = raw_prefix(name);
	const char *iio_raw = getenv("IIO_RAW");
	if (colon) {
		rc = read_raw(colon + 1, x);
		if (!rc) rc = trans_apply(x, name + 6);
	} else if (rcolon) {
		const size_t len = (size_t)(rcolon - name) - 5;   /* between "RAW[" and "]:" */
		char *spec = malloc(len + 1);
		if (!spec) return 1;
		memcpy(spec, name + 4, len);
		spec[len] = 0;
		rc = read_raw_spec(spec, rcolon + 1, x);
		free(spec);
	} else if (iio_raw && strcmp(name, "-")) {
		rc = read_raw_spec(iio_raw, name, x);   /* IIO_RAW: every file is raw (iio.c:3777-3795) */
	} else {
		rc = read_core(name, x);
	}
	const char *env = getenv("IIO_TRANS");
	if (!rc && env && *env) rc = trans_apply(x, env);
	if (rc && colon) fprintf(stderr, "imageio: could not read image \"%s\"\n", name);
	return rc;
}

/* An image from a file or stdin, its format sniffed from the first bytes. */
static int read_core(const char *name, raw_image *x)
{
	FILE *f = strcmp(name, "-") ? fopen(name, "rb") : stdin;
	if (!f) {
		fprintf(stderr, "imageio: can not open file \"%s\" in mode \"r\"\n", name);
		return 1;
	}
	size_t n = 0;
	unsigned char *b = slurp(f, &n);
	if (f != stdin) fclose(f);
	if (!b) return 1;
	int r = 1;
	if (getenv("IIO_TXT")) r = read_text(x, b, n, ' ');   /* IIO_TXT: every file is TXT */
	else if (n >= 4 && b[0] == 0x93 && b[1] == 'N' && b[2] == 'U' && b[3] == 'M') r = read_npy(x, b, n);
	else if (n >= 2 && b[0] == 'P' && (b[1] == 'f' || b[1] == 'F')) r = read_pfm(x, b, n);
	else if (n >= 2 && b[0] == 'P' && b[1] && strchr("235679", b[1])) r = read_pnm(x, b, n);
	else if (n >= 2 && ((b[0] == 'I' && (b[1] == 'R' || b[1] == 'M')) || (b[0] == 'M' && b[1] == 'I') ||
			(b[0] == 'W' && b[1] == 'E') || (b[0] == 'V' && b[1] == 'I') ||
			(b[0] == 'R' && b[1] == 'I' && !(n >= 4 && b[2] == 'F' && b[3] == 'F'))))
		r = read_rim(x, b, n);
	else if (n >= 4 && !memcmp(b, "PIEH", 4)) r = read_flo(x, b, n);
	else if (n >= 4 && b[0] == 4 && b[1] == 0 && b[2] == 0 && b[3] == 0) r = read_rat(x, b, n);
	else if (n >= 8 && !memcmp(b, "SIMPLE  ", 8)) r = read_fit(x, b, n);
	else if (n >= 4 && !memcmp(b, "PDS_", 4)) r = read_pds(x, b, n, 4);
	else if (n >= 8 && (!memcmp(b, "CCSD3Z", 6) || !memcmp(b + 1, "CCSD3Z", 6) || !memcmp(b + 2, "CCSD3Z", 6)))
		r = read_pds(x, b, n, 8);
	else if (n >= 8 && !memcmp(b, "LBLSIZE=", 8)) r = read_vic(x, b, n);
	else if (n >= 4 && !memcmp(b, "<VRT", 4)) r = read_vrt(x, b, n, name);
	else if (n >= 4 && !memcmp(b, "farb", 4)) r = read_ffd(x, b, n);
	else if (n >= 2 && b[0] == 'P' && b[1] == 'C') r = read_pcm(x, b, n);
	else if (n >= 3 && !memcmp(b, "#UV", 3)) r = read_juv(x, b, n);
	else if (n >= 12 && !memchr(b, '\n', 8) && (!memcmp(b + 8, "FLOA", 4) || !memcmp(b + 8, "12LI", 4)))
		r = read_lum(x, b, n);
	else {
		const int tf = text_format(b, n);
		if (tf == TXT_CSV) r = read_text(x, b, n, ',');
		else if (tf == TXT_TXT) r = read_text(x, b, n, ' ');
		else if (tf == TXT_ASC) r = read_asc(x, b, n);
		else fprintf(stderr, "imageio: unrecognized format of \"%s\"\n", name);
	}
	free(b);
	if (r) fprintf(stderr, "imageio: could not read image \"%s\"\n", name);
	return r;
}

float *imgio_read_split(const char *name, int *w, int *h, int *pd)
{
	raw_image x = {0};
	if (read_raw(name, &x)) { free(x.v); return NULL; }
	size_t np = (size_t)x.w * x.h;
	float *o = xcalloc(np * x.pd, sizeof(float));
	if (o)
		for (size_t i = 0; i < np; i++)
			for (int l = 0; l < x.pd; l++) o[np * l + i] = (float)x.v[i * x.pd + l];
	free(x.v);
	*w = x.w; *h = x.h; *pd = x.pd;
	return o;
}

/* gray value in the sample type of the file, then float (iio.c:1230-1300) */
static float gray_of(const double *p, int type)
{
	double g = .299 * p[0] + .587 * p[1] + .114 * p[2];
	switch (type) {
	case T_U8: return (float)(uint8_t)g;
	case T_U16: return (float)(uint16_t)g;
	case T_F64: return (float)g;
	default: return (float)g;
	}
}

float *imgio_read_gray(const char *name, int *w, int *h)
{
	raw_image x = {0};
	if (read_raw(name, &x)) { free(x.v); return NULL; }
	size_t np = (size_t)x.w * x.h;
	float *o = NULL;
	if (x.pd == 1 || x.pd == 3 || x.pd == 4) {
		o = xcalloc(np, sizeof(float));
		if (o)
			for (size_t i = 0; i < np; i++)
				o[i] = x.pd == 1 ? (float)x.v[i] : gray_of(x.v + i * x.pd, x.type);
	} else {
		fprintf(stderr, "imageio: non-scalarizable image \"%s\"\n", name);
	}
	free(x.v);
	*w = x.w; *h = x.h;
	return o;
}

/* ---------------------------------------------------------------- writing */

static int suffix(const char *s, const char *suf)
{
	size_t a = strlen(s), b = strlen(suf);
	return a >= b && !strcmp(s + a - b, suf);
}

static FILE *open_out(const char *name)
{
	FILE *f = strcmp(name, "-") ? fopen(name, "wb") : stdout;
	if (!f) fprintf(stderr, "imageio: can not open file \"%s\" in mode \"w\"\n", name);
	return f;
}

static int close_out(FILE *f)
{
	if (f == stdout) return fflush(f) ? 1 : 0;
	return fclose(f) ? 1 : 0;
}

/* one row of w samples a line ("%.9g", spaces); a single row or column of
 * pd-vectors one pixel a line (iio.c:4277-4304) */
static void write_txt(FILE *f, const float *v, int w, size_t ns, int pd)
{
	const size_t rw = pd == 1 ? (size_t)w : (size_t)pd;
	for (size_t k = 0; k < ns; k++) fprintf(f, "%.9g%c", v[k], (k + 1) % rw ? ' ' : '\n');
}

int imgio_write_split(const char *name, const float *x, int w, int h, int pd)
{
	size_t np = (size_t)w * h, ns = np * pd;
	/* "TXT:name" and "RAW:name" (iio.c:6292-6307) */
	const int txt_prefix = name == strstr(name, "TXT:"), raw_prefix_w = name == strstr(name, "RAW:");
	if ((txt_prefix || raw_prefix_w) && strlen(name) > 4) {
		if (txt_prefix && !(pd == 1 || w == 1 || h == 1)) {
			fprintf(stderr, "imageio: TXT needs one channel, or one row or column\n");
			return 1;
		}
		float *v = malloc(sizeof(float) * (ns ? ns : 1));
		if (!v) return 1;
		for (size_t i = 0; i < np; i++)
			for (int l = 0; l < pd; l++) v[i * pd + l] = x[np * l + i];
		FILE *f = open_out(name + 4);
		int rc = !f;
		if (f) {
			if (txt_prefix) write_txt(f, v, w, ns, pd);
			else rc = fwrite(v, sizeof(float), ns, f) != ns;
			rc |= close_out(f);
		}
		free(v);
		if (rc) fprintf(stderr, "imageio: error writing \"%s\"\n", name + 4);
		return rc;
	}
	if (!strcmp(name, "-") && isatty(1)) {
		printf("IMAGE %dx%d,%d float\n", w, h, pd);
		return 0;
	}
	float *v = malloc(sizeof(float) * (ns ? ns : 1));   /* interleaved */
	if (!v) return 1;
	for (size_t i = 0; i < np; i++)
		for (int l = 0; l < pd; l++) v[i * pd + l] = x[np * l + i];
	int rc = 0;
	FILE *f = open_out(name);
	if (!f) { free(v); return 1; }
	if (suffix(name, ".uv") && pd == 2) {
		/* JUV: a 255-byte text header (the text, its NUL, spaces), u, v */
		char head[255];
		memset(head, ' ', sizeof head);
		snprintf(head, sizeof head, "#UV {\n dimx %d dimy %d\n}\n", w, h);
		rc = fwrite(head, 1, 255, f) != 255;
		rc |= fwrite(x, sizeof(float), ns, f) != ns;   /* the planes: u then v */
	} else if (suffix(name, ".flo") && pd == 2) {
		const uint32_t dims[2] = {(uint32_t)w, (uint32_t)h};
		rc = fwrite("PIEH", 1, 4, f) != 4;
		rc |= fwrite(dims, 4, 2, f) != 2;
		rc |= fwrite(v, sizeof(float), ns, f) != ns;
	} else if ((suffix(name, ".pfm")) && (pd == 1 || pd == 3)) {
		fprintf(f, "P%c\n%d %d\n%g\n", pd > 1 ? 'F' : 'f', w, h, -1.0);
		rc = fwrite(v, sizeof(float), ns, f) != ns;
	} else if ((suffix(name, ".ppm") || suffix(name, ".pgm")) && (pd == 1 || pd == 3)) {
		fprintf(f, "P%c\n%d %d\n%g\n", pd > 1 ? '3' : '2', w, h, 255.0);
		for (size_t k = 0; k < ns; k++) fprintf(f, "%d\n", (int)v[k]);
	} else if (suffix(name, ".csv") && pd == 1) {
		for (size_t k = 0; k < ns; k++) fprintf(f, "%.9g%c", v[k], (k + 1) % w ? ',' : '\n');
	} else if (suffix(name, ".txt") && (pd == 1 || w == 1 || h == 1)) {
		write_txt(f, v, w, ns, pd);
	} else if (suffix(name, ".raw")) {
		rc = fwrite(v, sizeof(float), ns, f) != ns;   /* the samples, interleaved */
	} else if (suffix(name, ".mw") && pd == 1) {
		/* MegaWave fimage: "IR", comment length 2, width, height, 29 zero
		 * 16-bit fields (big-endian), the floats (iio.c:4376-4406) */
		unsigned char hd[66] = {'I', 'R', 0, 2};
		hd[4] = (unsigned char)(w >> 8); hd[5] = (unsigned char)w;
		hd[6] = (unsigned char)(h >> 8); hd[7] = (unsigned char)h;
		rc = fwrite(hd, 1, sizeof hd, f) != sizeof hd;
		rc |= fwrite(v, sizeof(float), ns, f) != ns;
	} else if (suffix(name, ".asc")) {
		fprintf(f, "%d %d 1 %d\n", w, h, pd);
		for (size_t k = 0; k < ns; k++) fprintf(f, "%.9g\n", x[k]);   /* planar */
	} else {
		char hdr[256];
		int n = snprintf(hdr, sizeof hdr,
				"{'descr': '<f4', 'fortran_order': False, 'shape': (%d, %d, %d)}", h, w, pd);
		int total = ((10 + n + 1 + 15) / 16) * 16;
		unsigned char pre[10] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0, 0, 0};
		pre[8] = (total - 10) % 256;
		pre[9] = (total - 10) / 256;
		fwrite(pre, 1, 10, f);
		fwrite(hdr, 1, n, f);
		for (int k = 10 + n; k < total - 1; k++) fputc(' ', f);
		fputc('\n', f);
		rc = fwrite(v, sizeof(float), ns, f) != ns;
	}
	rc |= close_out(f);
	free(v);
	if (rc) fprintf(stderr, "imageio: error writing \"%s\"\n", name);
	return rc;
}
