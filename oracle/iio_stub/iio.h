/*
 * Test infrastructure only (oracle).  Stand-in for the reference's vendored
 * image I/O header (3rdparty/iio/iio.h), which forces libpng/libjpeg/libtiff
 * on (iio.h:290-292) and therefore cannot be compiled on this image.  The
 * oracle never reads or writes image files: io_utility.cpp is linked only for
 * IOUtility::separate / IOUtility::cat, which PatchNonLocalDepth::update calls
 * (patch_non_local_depth.cpp:46-53).  These four prototypes are the ones
 * io_utility.cpp:124,152,194,226 call; iio_stub.c makes every call fail.
 */
#ifndef NLI_ORACLE_IIO_STUB_H
#define NLI_ORACLE_IIO_STUB_H

float *iio_read_image_float(const char *fname, int *w, int *h);
float *iio_read_image_float_vec(const char *fname, int *w, int *h, int *pd);
void iio_save_image_float_vec(char *filename, float *x, int w, int h, int pd);
void iio_save_image_float(char *filename, float *x, int w, int h);

#endif
