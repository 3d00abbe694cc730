/* range_ff.h -- exact photon-gather range decisions without double arithmetic.
 *
 * The reference decides "within range" and orders neighbours on the double
 * sum of squares d2 = (px-qx)^2 + (py-qy)^2 + (pz-qz)^2 of float positions,
 * rounded to float (kd_nearest_range3f; the k-nearest selection uses the
 * float-rounded key).  This GPU has little double throughput, so d2 is
 * evaluated in float-float arithmetic (Dekker's two-sum and the fma
 * two-product): the unevaluated sum H + L is within 2^-43 of the exact value
 * and the double evaluation within 2^-50, so with a margin of 2^-36 both the
 * range test and the float rounding of d2 come out as the double computation
 * gives them, unless H + L lies within the margin of the radius or of a float
 * rounding boundary; those rare cases (and tiny or non-finite sums) are left
 * to the caller to recompute in double.
 *
 * Host and device share this file: the CPU test suite compiles it with
 * -ffp-contract=off and compares it with double arithmetic.  fmaf is the
 * correctly rounded fused multiply-add on both sides.
 */
#ifndef SRAY_RANGE_FF_H_
#define SRAY_RANGE_FF_H_

#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define SRAY_FF __host__ __device__ __forceinline__
#else
#define SRAY_FF static inline
#endif

SRAY_FF uint32_t sray_ff_bits(float f)
{
	uint32_t u;
	memcpy(&u, &f, 4);
	return u;
}

SRAY_FF float sray_ff_float(uint32_t u)
{
	float f;
	memcpy(&f, &u, 4);
	return f;
}

SRAY_FF void sray_two_sum(float a, float b, float *s, float *e)
{
	float ss = a + b;
	float bb = ss - a;
	*s = ss;
	*e = (a - (ss - bb)) + (b - bb);
}

SRAY_FF void sray_fast_two_sum(float a, float b, float *s, float *e)
{
	float ss = a + b;
	*s = ss;
	*e = b - (ss - a);
}

/* (p - q)^2 as h + l */
SRAY_FF void sray_diff_sq_ff(float p, float q, float *h, float *l)
{
	float s, e;
	sray_two_sum(p, -q, &s, &e);      /* s + e = p - q exactly */
	float hh = s * s;
	float ll = fmaf(s, s, -hh);       /* hh + ll = s^2 exactly */
	*h = hh;
	*l = ll + ((2.0f * s) * e + e * e);
}

SRAY_FF void sray_add_ff(float h1, float l1, float h2, float l2, float *h, float *l)
{
	float s, e;
	sray_two_sum(h1, h2, &s, &e);
	e = e + (l1 + l2);
	sray_fast_two_sum(s, e, h, l);
}

/* returns 0 when the double computation must decide; otherwise 1 with *in
 * (d2 <= range^2 in double, range^2 = r2_hi + r2_lo exactly) and *key (bits
 * of (float)d2 when in range) */
SRAY_FF int sray_range_ff(float px, float py, float pz, float qx, float qy, float qz, float r2_hi, float r2_lo, int *in,
		uint32_t *key)
{
	float hx, lx, hy, ly, hz, lz, h, l;
	sray_diff_sq_ff(px, qx, &hx, &lx);
	sray_diff_sq_ff(py, qy, &hy, &ly);
	sray_diff_sq_ff(pz, qz, &hz, &lz);
	sray_add_ff(hx, lx, hy, ly, &h, &l);
	sray_add_ff(h, l, hz, lz, &h, &l);
	if(!(h >= 8.673617e-19f && h <= 1e30f)) return 0;        /* 2^-60 .. overflow-safe */
	float delta = h * 1.4551915e-11f;                          /* 2^-36 */
	float diff = (h - r2_hi) + (l - r2_lo);
	if(diff > delta) {
		*in = 0;
		*key = 0;
		return 1;
	}
	if(!(diff < -delta)) return 0;
	/* rounding of d2 to float: h unless d2 may cross half an ulp of h */
	uint32_t hb = sray_ff_bits(h);
	float ulp = sray_ff_float(hb & 0x7f800000u) * 1.1920929e-7f;   /* 2^-23 */
	float ulp_dn = (hb & 0x007fffffu) ? ulp : 0.5f * ulp;
	if(!(l + delta < 0.5f * ulp) || !(l - delta > -0.5f * ulp_dn)) return 0;
	*in = 1;
	*key = hb;
	return 1;
}

#endif
