/*
 * imageio.h -- the image reading and writing the simpois command needs,
 * following iio's conventions (iio.h:33-43, iio.c:5164-5346, 6166-6300):
 *
 *  - images are returned "split": planar float, x[w*h*l + w*j + i];
 *  - "-" names stdin (reading) or stdout (writing); iio's semantic names
 *    "zero:WxH[,pd]", "one:WxH[,pd]" and "constant:V:WxH" read as images;
 *  - every image read from a file (not a semantic name) gets the list of
 *    transformations in IIO_TRANS, and a name "TRANS[list]:file" gets that
 *    list as well (iio.c:3796-3884, 5677-5705): flips and reorientations,
 *    trims (negative ones pad with NaN), a pipe through a shell command;
 *  - "RAW[fields]:file" reads headerless binary samples (sizes, header,
 *    type, byte swap, orientation, image index, fields read from the file),
 *    and so does every file while IIO_RAW holds the fields; IIO_TXT reads
 *    every file as TXT (iio.c:3597-3795, 5164-5180);
 *  - the input format is sniffed from the first bytes: NumPy .npy (1.0,
 *    every numeric dtype), PFM ("Pf"/"PF"), PNM ("P2","P3","P5","P6", and
 *    iio's n-channel "P7"/"P9"; ASCII samples read as floats), and
 *    the text formats told apart as iio does -- CSV and TXT (one row per
 *    line, commas or spaces) and ASC ("w h 1 pd" header, planar samples);
 *  - the output format follows the file-name suffix: .uv and .flo (2
 *    channels), .pfm (1 or 3 channels), .ppm/.pgm (1 or 3 channels, ASCII
 *    integers), .csv, .txt, .raw (the samples, interleaved), .asc, .npy, or
 *    the prefixes "TXT:" and "RAW:"; any other name, and a stdout that is not
 *    a terminal, get NumPy .npy.  A terminal stdout gets the one-line
 *    "IMAGE wxh,pd float" summary.  FLO, JUV (.uv), farbfeld, PCM, LUM, RAT,
 *    FITS, PDS, CCSD, VICAR, GDAL VRT and MegaWave RIM files are read too,
 *    and ".mw" writes a RIM float image.  Not read: the formats for which
 *    iio needs libraries (PNG, TIFF, JPEG, EXR, WebP, HEIF, HDF5); BMP and
 *    DLM are not read by iio either.
 *
 * Errors print a message and return NULL / nonzero; nothing exits.
 */
#ifndef SIMPOIS_IMAGEIO_H
#define SIMPOIS_IMAGEIO_H

/* Planar float image of *w x *h x *pd, or NULL with a message on stderr. */
float *imgio_read_split(const char *name, int *w, int *h, int *pd);

/* Single-channel float image; 3 (RGB) and 4 (RGBA) channel images are
 * converted to gray with the weights .299 .587 .114 (iio.c:1230-1300). */
float *imgio_read_gray(const char *name, int *w, int *h);

/* Write a planar float image; returns 0 on success. */
int imgio_write_split(const char *name, const float *x, int w, int h, int pd);

#endif
