/* Test harness for the CLI's image I/O (imscript_gb300/cli/imageio.c):
 *   imageio_harness read  IN  OUT.npy   read any format, write npy
 *   imageio_harness gray  IN  OUT.npy   read as one gray channel, write npy
 *   imageio_harness write IN.npy OUT    read npy, write by OUT's suffix
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "imageio.h"

int main(int argc, char **argv)
{
	if (argc != 4) return 2;
	int w, h, pd = 1;
	float *x = !strcmp(argv[1], "gray") ? imgio_read_gray(argv[2], &w, &h)
	                                    : imgio_read_split(argv[2], &w, &h, &pd);
	if (!x) return 1;
	int r = imgio_write_split(argv[3], x, w, h, pd);
	free(x);
	return r;
}
