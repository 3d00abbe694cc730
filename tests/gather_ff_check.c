/* gather_ff_check.c -- compares the float-float range decisions of the
 * photon gather (sray_gb300/csrc/range_ff.h, the code the GPU kernel runs)
 * with the double computation of the reference's kd-tree rule, on random
 * and adversarial cases: points placed within rounding of the radius,
 * points almost on the query, coordinates of very different magnitudes.
 * Prints "cases fallback mismatches"; a mismatch is a decided case whose
 * in-range flag or float-rounded key differs from double. */
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <stdint.h>
#include "range_ff.h"

static uint64_t rs = 0x9E3779B97F4A7C15ull;
static double urand(void)
{
	rs ^= rs << 13;
	rs ^= rs >> 7;
	rs ^= rs << 17;
	return (double)(rs >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char **argv)
{
	long n = argc > 1 ? atol(argv[1]) : 2000000;
	long fall = 0, bad = 0;
	const float radii[3] = {0.5f, 0.013f, 3.7f};
	for(long i = 0; i < n; i++) {
		float rad = radii[i % 3];
		double r2 = (double)rad * (double)rad;
		float r2_hi = (float)r2, r2_lo = (float)(r2 - (double)r2_hi);
		float q[3], p[3];
		for(int k = 0; k < 3; k++) q[k] = (float)(urand() * 120.0 - 60.0);
		int mode = (int)(i % 5);
		for(int k = 0; k < 3; k++) {
			double d = urand() * 2.0 - 1.0;
			if(mode == 0) p[k] = (float)(q[k] + d * rad * 1.2);
			else if(mode == 1) p[k] = (float)(q[k] + d * 1e-3 * rad);
			else if(mode == 2) p[k] = (float)(q[k] + d * rad * 0.58);
			else if(mode == 3) p[k] = k == 0 ? q[k] : (float)(q[k] + d * rad);
			else p[k] = (float)(q[k] + d * rad);
		}
		if(mode == 3 && (i & 8)) {
			q[0] = (float)(1e-12 * (urand() - 0.5));
			p[0] = (float)((urand() - 0.5) * rad);
		}
		if(mode == 4) {
			/* onto the sphere of the radius, within float rounding */
			double dx = (double)p[0] - q[0], dy = (double)p[1] - q[1], dz = (double)p[2] - q[2];
			double d = sqrt(dx * dx + dy * dy + dz * dz);
			if(d > 0.0) {
				double sc = rad / d;
				p[0] = (float)(q[0] + dx * sc);
				p[1] = (float)(q[1] + dy * sc);
				p[2] = (float)(q[2] + dz * sc);
			}
		}
		double dx = (double)p[0] - (double)q[0], dy = (double)p[1] - (double)q[1], dz = (double)p[2] - (double)q[2];
		double d2 = dx * dx + dy * dy + dz * dz;
		int in_d = d2 <= r2;
		float kf = (float)d2;
		uint32_t key_d;
		memcpy(&key_d, &kf, 4);
		int in = 0;
		uint32_t key = 0;
		if(!sray_range_ff(p[0], p[1], p[2], q[0], q[1], q[2], r2_hi, r2_lo, &in, &key)) {
			fall++;
			continue;
		}
		if(in != in_d || (in && key != key_d)) {
			if(bad < 5) fprintf(stderr, "mismatch p=%a %a %a q=%a %a %a in %d/%d key %08x/%08x\n", p[0], p[1], p[2], q[0], q[1], q[2], in,
					in_d, key, key_d);
			bad++;
		}
	}
	printf("%ld %ld %ld\n", n, fall, bad);
	return 0;
}
