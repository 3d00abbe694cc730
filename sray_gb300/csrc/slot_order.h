/* slot_order.h -- the order in which a sample batch's slots take pixels
 * (shared by the camera and finish kernels and the host checks). */
#ifndef SRAY_SLOT_ORDER_H_
#define SRAY_SLOT_ORDER_H_

#ifdef __CUDACC__
#define SRAY_HD __host__ __device__
#else
#define SRAY_HD
#endif

namespace sray {

/* The pixel of active slot a: the batch's list when there is one, else --
 * the first batch -- for a single frame of tw x th pixels the pixels in
 * bands of four rows, column-major within a band, so that the 32 rays of a
 * warp leave from an 8 x 4 patch (and the rays they spawn keep that order;
 * the last band has the rows that are left); tw = 0: slot a is pixel a (a
 * batch of jobs) */
SRAY_HD inline int slot_pixel(const int *active, int a, int tw, int th)
{
	if(active) return active[a];
	if(tw <= 0) return a;
	const int band = a / (4 * tw), r = a - band * 4 * tw;
	const int hb = th - 4 * band < 4 ? th - 4 * band : 4;
	return (4 * band + r % hb) * tw + r / hb;
}

}  // namespace sray

#endif
