/* sray_rng.h -- the counter-based random stream and the deterministic float
 * trigonometry shared by the GPU renderer, its CPU oracle and the harness that
 * drives the compiled reference.
 *
 * The reference draws every random number from the C library's global rand()
 * state (frand/sphrand in libvmath, rand() in src/scene.cc:594,639 and
 * src/camera.cc:233), so two runs never see the same photon or pixel-sample
 * set.  Here every draw comes from a Philox4x32-10 counter generator
 * (J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11), keyed by a 64-bit seed and addressed by a 128-bit
 * counter whose upper three words name the stream (photon index, pixel
 * sample, shading-tree path) and whose lowest word counts draws.  Any thread
 * on any device can therefore regenerate any stream without shared state.
 *
 * Uniforms are 24-bit: u = (x >> 8) * 2^-24, exactly representable in float
 * and double, so the FP32 and FP64 code paths consume identical values.
 *
 * The float trigonometry below (sincos of an angle given in turns, atan2) is
 * written from the Taylor series of sin, cos and atan with octant / tan(pi/8)
 * argument reduction, using only IEEE add, subtract, multiply and divide.
 * Built without FMA contraction (-ffp-contract=off on the host, -fmad=false
 * on the device) it returns bit-identical results on x86, Arm and the GPU,
 * which is what lets photon paths and projection-map cell choices agree
 * exactly between the CUDA kernels and the FP32 oracle.
 */
#ifndef SRAY_RNG_H_
#define SRAY_RNG_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define SRAY_HD __host__ __device__ __forceinline__
#else
#define SRAY_HD static inline
#endif

/* stream domains: the top word of the Philox counter */
enum {
	SRAY_DOM_PIXEL = 1,       /* camera jitter + shading draws of one pixel sample */
	SRAY_DOM_CAUST = 2,       /* one caustic photon */
	SRAY_DOM_GLOBAL = 3,      /* one global-illumination photon */
	SRAY_DOM_PROJMAP = 4,     /* light sample positions used to build projection maps */
	SRAY_DOM_USER = 5,
	SRAY_DOM_NRC = 6          /* final-gather directions of a radiance-cache record (keyed per frame) */
};

typedef struct sray_rng {
	uint32_t k0, k1;          /* key (seed) */
	uint32_t c1, c2, c3;      /* stream address */
	uint32_t n;               /* draws taken so far */
	uint32_t buf[4];          /* last Philox block */
} sray_rng;

SRAY_HD void sray_philox4x32_10(const uint32_t ctr_in[4], uint32_t k0, uint32_t k1, uint32_t out[4])
{
	uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
	for(int r = 0; r < 10; r++) {
		if(r) {
			k0 += 0x9E3779B9u;
			k1 += 0xBB67AE85u;
		}
		uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
		uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
		uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
		uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
		c0 = hi1 ^ c1 ^ k0;
		c1 = lo1;
		c2 = hi0 ^ c3 ^ k1;
		c3 = lo0;
	}
	out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

SRAY_HD void sray_rng_init(sray_rng *s, uint64_t seed, uint32_t dom, uint32_t a, uint32_t b)
{
	s->k0 = (uint32_t)seed;
	s->k1 = (uint32_t)(seed >> 32);
	s->c1 = a;
	s->c2 = b;
	s->c3 = dom;
	s->n = 0;
	s->buf[0] = s->buf[1] = s->buf[2] = s->buf[3] = 0;
}

SRAY_HD uint32_t sray_rng_u32(sray_rng *s)
{
	uint32_t lane = s->n & 3u;
	if(lane == 0) {
		uint32_t ctr[4];
		ctr[0] = s->n >> 2;
		ctr[1] = s->c1;
		ctr[2] = s->c2;
		ctr[3] = s->c3;
		sray_philox4x32_10(ctr, s->k0, s->k1, s->buf);
	}
	s->n++;
	return s->buf[lane];
}

/* continue a stream after `n` draws (the state of a stream is its address
 * and its draw count) */
SRAY_HD void sray_rng_seek(sray_rng *s, uint32_t n)
{
	s->n = n;
	if(n & 3u) {
		uint32_t ctr[4];
		ctr[0] = n >> 2;
		ctr[1] = s->c1;
		ctr[2] = s->c2;
		ctr[3] = s->c3;
		sray_philox4x32_10(ctr, s->k0, s->k1, s->buf);
	}
}

/* uniform in [0, 1 - 2^-24], exact in float and double */
SRAY_HD float sray_rng_uniform_f(sray_rng *s)
{
	return (float)(sray_rng_u32(s) >> 8) * (1.0f / 16777216.0f);
}

SRAY_HD double sray_rng_uniform_d(sray_rng *s)
{
	return (double)(sray_rng_u32(s) >> 8) * (1.0 / 16777216.0);
}

/* rand()-style 31-bit integer draw */
SRAY_HD int sray_rng_int(sray_rng *s)
{
	return (int)(sray_rng_u32(s) >> 1);
}

/* ---- deterministic float trigonometry ---- */

#define SRAY_PI_F      3.14159265358979323846f
#define SRAY_TWO_PI_F  6.28318530717958647692f
#define SRAY_HALF_PI_F 1.57079632679489661923f
#define SRAY_QUARTER_PI_F 0.78539816339744830962f

/* sin and cos of 2*pi*u, u in turns (any u with |u| < 2^20) */
SRAY_HD void sray_sincos_turns_f(float u, float *s_out, float *c_out)
{
	float q = u * 4.0f;                       /* quarter turns, exact */
	float kf = (float)(int)(q + (q >= 0.0f ? 0.5f : -0.5f));
	int k = (int)kf;
	float r = (q - kf) * 0.25f;               /* exact: |r| <= 1/8 turn */
	float a = r * SRAY_TWO_PI_F;              /* |a| <= pi/4 */
	float a2 = a * a;
	/* Taylor series of sin and cos, Horner form */
	float sp = 1.0f / 362880.0f;
	sp = sp * a2 + (-1.0f / 5040.0f);
	sp = sp * a2 + (1.0f / 120.0f);
	sp = sp * a2 + (-1.0f / 6.0f);
	float sa = a + a * (a2 * sp);
	float cp = 1.0f / 3628800.0f;
	cp = cp * a2 + (-1.0f / 40320.0f);
	cp = cp * a2 + (1.0f / 720.0f);
	cp = cp * a2 + (-1.0f / 24.0f);
	cp = cp * a2 + 0.5f;
	float ca = 1.0f - a2 * cp;
	switch(k & 3) {
	case 0: *s_out = sa; *c_out = ca; break;
	case 1: *s_out = ca; *c_out = -sa; break;
	case 2: *s_out = -sa; *c_out = -ca; break;
	default: *s_out = -ca; *c_out = sa; break;
	}
}

/* sin and cos of an angle in radians (reduced through turns) */
SRAY_HD void sray_sincos_f(float ang, float *s_out, float *c_out)
{
	sray_sincos_turns_f(ang * (1.0f / SRAY_TWO_PI_F), s_out, c_out);
}

/* atan2(y, x) in (-pi, pi]; atan2(0, 0) = 0 */
SRAY_HD float sray_atan2_f(float y, float x)
{
	float ax = x < 0.0f ? -x : x;
	float ay = y < 0.0f ? -y : y;
	if(ax == 0.0f && ay == 0.0f) {
		return (x < 0.0f) ? SRAY_PI_F : 0.0f;
	}
	int swap = ay > ax;
	float t = swap ? ax / ay : ay / ax;       /* t in [0, 1] */
	float base = 0.0f;
	if(t > 0.41421356237309504880f) {         /* tan(pi/8) */
		t = (t - 1.0f) / (t + 1.0f);
		base = SRAY_QUARTER_PI_F;
	}
	float t2 = t * t;
	/* atan(t) = t - t^3/3 + t^5/5 - ... ; |t| <= tan(pi/8) */
	float p = 1.0f / 19.0f;
	p = p * t2 + (-1.0f / 17.0f);
	p = p * t2 + (1.0f / 15.0f);
	p = p * t2 + (-1.0f / 13.0f);
	p = p * t2 + (1.0f / 11.0f);
	p = p * t2 + (-1.0f / 9.0f);
	p = p * t2 + (1.0f / 7.0f);
	p = p * t2 + (-1.0f / 5.0f);
	p = p * t2 + (1.0f / 3.0f);
	float a = base + (t - t * (t2 * p));
	if(swap) a = SRAY_HALF_PI_F - a;
	if(x < 0.0f) a = SRAY_PI_F - a;
	if(y < 0.0f) a = -a;
	return a;
}

#endif /* SRAY_RNG_H_ */
