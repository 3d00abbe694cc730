/* imago2.h -- TEST INFRASTRUCTURE: stand-in for libimago (image files).
 * Saving writes a portable float map; loading reads binary PPM (P6) as RGBA
 * floats (the texture test scenes use that format). */
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
