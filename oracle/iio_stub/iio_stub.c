/* Test infrastructure only (oracle): failing stand-ins for file I/O, see iio.h. */
#include <stdio.h>
#include <stdlib.h>
#include "iio.h"

float *iio_read_image_float(const char *fname, int *w, int *h)
{
	(void)w; (void)h;
	fprintf(stderr, "oracle: image file input is not available (%s)\n", fname);
	return NULL;
}

float *iio_read_image_float_vec(const char *fname, int *w, int *h, int *pd)
{
	(void)w; (void)h; (void)pd;
	fprintf(stderr, "oracle: image file input is not available (%s)\n", fname);
	return NULL;
}

void iio_save_image_float_vec(char *filename, float *x, int w, int h, int pd)
{
	(void)x; (void)w; (void)h; (void)pd;
	fprintf(stderr, "oracle: image file output is not available (%s)\n", filename);
}

void iio_save_image_float(char *filename, float *x, int w, int h)
{
	(void)x; (void)w; (void)h;
	fprintf(stderr, "oracle: image file output is not available (%s)\n", filename);
}
