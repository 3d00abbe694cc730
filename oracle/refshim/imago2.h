/* imago2.h -- TEST INFRASTRUCTURE: stand-in for libimago (image files).
 * Saving writes a portable float map; loading always fails (the scenes of
 * the test suite use no textures). */
#ifndef SHIM_IMAGO2_H_
#define SHIM_IMAGO2_H_

#ifdef __cplusplus
extern "C" {
#endif

enum { IMG_FMT_GREY8, IMG_FMT_RGB24, IMG_FMT_RGBA32, IMG_FMT_GREYF, IMG_FMT_RGBF, IMG_FMT_RGBAF };

void *img_load_pixels(const char *fname, int *xsz, int *ysz, int fmt);
int img_save_pixels(const char *fname, void *pix, int xsz, int ysz, int fmt);
void img_free_pixels(void *pix);

#ifdef __cplusplus
}
#endif

#endif
