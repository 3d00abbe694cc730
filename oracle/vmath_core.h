/* vmath_core.h -- TEST INFRASTRUCTURE.  Double-precision restatement of the
 * parts of libvmath (gfxtools, by the reference's author; not vendored in
 * the reference and not pinned to a version) that S-ray's rendering path
 * calls.  Used by the CPU oracle and by the shim that lets the reference's
 * own sources compile here, so that both compute set-up math identically.
 *
 * Conventions (restated from the call sites, which fix them):
 *  - 4x4 matrices are row-major and act on column vectors: p' = M p, the
 *    translation is in column 3 (src/camera.cc:216-234 builds the camera
 *    matrix that way).
 *  - XFormNode composes pivot * T * R * S * -pivot (src/anim.cc:391-419).
 *  - quaternions are (s, x, y, z); Quaternion(axis, angle) is
 *    (cos(a/2), axis sin(a/2)); rotation matrices are right-handed.
 *  - SphVector: theta = atan2(z, x), phi = acos(y / r); back to Cartesian
 *    x = r cos(theta) sin(phi), y = r cos(phi), z = r sin(theta) sin(phi).
 *    src/projmap.cc:146-209 only needs the two directions to be inverses.
 *  - reflection(v, n) = v - 2 (v.n) n: the mirror direction of a vector
 *    travelling towards the surface (src/shader.cc:192-200 sends reflection
 *    rays with it and src/shader.cc:270-276 builds the Phong lobe with it).
 *  - refraction(v, n, eta) = eta v + (eta c - sqrt(1 - eta^2 (1 - c^2))) n
 *    with c = -v.n, and the mirror direction on total internal reflection,
 *    which is what the TIR test of src/shader.cc:221-229 expects.
 *  - sphrand(r): a uniform point on the sphere of radius r from two
 *    uniforms, z = 2 u1 - 1, phi = 2 pi u0.
 *  - ERROR_MARGIN = 1e-6, XSMALL_NUMBER = 1e-8.
 */
#ifndef VMATH_CORE_H_
#define VMATH_CORE_H_

#include <math.h>
#include <string.h>
#include "sray_rng.h"

#define VMC_ERROR_MARGIN 1e-6
#define VMC_XSMALL_NUMBER 1e-8
#define VMC_SMALL_NUMBER 1e-4

static inline void vmc_mat_identity(double m[4][4])
{
	memset(m, 0, 16 * sizeof(double));
	m[0][0] = m[1][1] = m[2][2] = m[3][3] = 1.0;
}

static inline void vmc_mat_mul(double out[4][4], const double a[4][4], const double b[4][4])
{
	double r[4][4];
	for(int i = 0; i < 4; i++) {
		for(int j = 0; j < 4; j++) {
			r[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j] + a[i][3] * b[3][j];
		}
	}
	memcpy(out, r, sizeof r);
}

static inline void vmc_mat_translation(double m[4][4], double x, double y, double z)
{
	vmc_mat_identity(m);
	m[0][3] = x; m[1][3] = y; m[2][3] = z;
}

static inline void vmc_mat_scaling(double m[4][4], double x, double y, double z)
{
	vmc_mat_identity(m);
	m[0][0] = x; m[1][1] = y; m[2][2] = z;
}

/* rotation matrix of the quaternion (s, x, y, z) */
static inline void vmc_mat_quat(double m[4][4], double s, double x, double y, double z)
{
	vmc_mat_identity(m);
	m[0][0] = 1.0 - 2.0 * y * y - 2.0 * z * z;
	m[0][1] = 2.0 * x * y - 2.0 * s * z;
	m[0][2] = 2.0 * z * x + 2.0 * s * y;
	m[1][0] = 2.0 * x * y + 2.0 * s * z;
	m[1][1] = 1.0 - 2.0 * x * x - 2.0 * z * z;
	m[1][2] = 2.0 * y * z - 2.0 * s * x;
	m[2][0] = 2.0 * z * x - 2.0 * s * y;
	m[2][1] = 2.0 * y * z + 2.0 * s * x;
	m[2][2] = 1.0 - 2.0 * x * x - 2.0 * y * y;
}

static inline void vmc_mat_transpose(double out[4][4], const double m[4][4])
{
	double r[4][4];
	for(int i = 0; i < 4; i++)
		for(int j = 0; j < 4; j++)
			r[i][j] = m[j][i];
	memcpy(out, r, sizeof r);
}

static inline double vmc_det3(double a, double b, double c, double d, double e, double f,
		double g, double h, double i)
{
	return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

/* inverse by the adjugate: inv = adj(M) / det(M), cofactors from 3x3 minors */
static inline void vmc_mat_inverse(double out[4][4], const double m[4][4])
{
	double cof[4][4];
	for(int i = 0; i < 4; i++) {
		for(int j = 0; j < 4; j++) {
			double sub[9];
			int k = 0;
			for(int r = 0; r < 4; r++) {
				if(r == i) continue;
				for(int c = 0; c < 4; c++) {
					if(c == j) continue;
					sub[k++] = m[r][c];
				}
			}
			double minor = vmc_det3(sub[0], sub[1], sub[2], sub[3], sub[4], sub[5], sub[6], sub[7], sub[8]);
			cof[i][j] = ((i + j) & 1) ? -minor : minor;
		}
	}
	double det = m[0][0] * cof[0][0] + m[0][1] * cof[0][1] + m[0][2] * cof[0][2] + m[0][3] * cof[0][3];
	for(int i = 0; i < 4; i++)
		for(int j = 0; j < 4; j++)
			out[i][j] = cof[j][i] / det;
}

static inline void vmc_xform_point(double out[3], const double m[4][4], const double p[3])
{
	double x = m[0][0] * p[0] + m[0][1] * p[1] + m[0][2] * p[2] + m[0][3];
	double y = m[1][0] * p[0] + m[1][1] * p[1] + m[1][2] * p[2] + m[1][3];
	double z = m[2][0] * p[0] + m[2][1] * p[1] + m[2][2] * p[2] + m[2][3];
	out[0] = x; out[1] = y; out[2] = z;
}

static inline void vmc_xform_dir(double out[3], const double m[4][4], const double v[3])
{
	double x = m[0][0] * v[0] + m[0][1] * v[1] + m[0][2] * v[2];
	double y = m[1][0] * v[0] + m[1][1] * v[1] + m[1][2] * v[2];
	double z = m[2][0] * v[0] + m[2][1] * v[1] + m[2][2] * v[2];
	out[0] = x; out[1] = y; out[2] = z;
}

/* quaternion helpers: q = {s, x, y, z} */
static inline void vmc_quat_axis_angle(double q[4], const double axis[3], double angle)
{
	double half = angle * 0.5;
	double sn = sin(half);
	q[0] = cos(half);
	q[1] = axis[0] * sn;
	q[2] = axis[1] * sn;
	q[3] = axis[2] * sn;
}

static inline void vmc_quat_normalize(double q[4])
{
	double len = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
	if(len > 0.0) {
		q[0] /= len; q[1] /= len; q[2] /= len; q[3] /= len;
	}
}

static inline void vmc_quat_mul(double out[4], const double a[4], const double b[4])
{
	double s = a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
	double x = a[0] * b[1] + b[0] * a[1] + (a[2] * b[3] - a[3] * b[2]);
	double y = a[0] * b[2] + b[0] * a[2] + (a[3] * b[1] - a[1] * b[3]);
	double z = a[0] * b[3] + b[0] * a[3] + (a[1] * b[2] - a[2] * b[1]);
	out[0] = s; out[1] = x; out[2] = y; out[3] = z;
}

static inline void vmc_quat_slerp(double out[4], const double a[4], const double b[4], double t)
{
	double dot = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
	double bb[4] = {b[0], b[1], b[2], b[3]};
	if(dot < 0.0) {
		dot = -dot;
		bb[0] = -bb[0]; bb[1] = -bb[1]; bb[2] = -bb[2]; bb[3] = -bb[3];
	}
	double wa, wb;
	if(dot > 0.9999) {
		wa = 1.0 - t;
		wb = t;
	} else {
		double ang = acos(dot);
		double sn = sin(ang);
		wa = sin((1.0 - t) * ang) / sn;
		wb = sin(t * ang) / sn;
	}
	for(int i = 0; i < 4; i++) out[i] = a[i] * wa + bb[i] * wb;
}

/* SphVector <-> Cartesian */
static inline void vmc_sph_from_vec(double *theta, double *phi, double *r, const double v[3])
{
	*r = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
	*theta = atan2(v[2], v[0]);
	*phi = acos(v[1] / *r);
}

static inline void vmc_vec_from_sph(double out[3], double theta, double phi, double r)
{
	out[0] = r * cos(theta) * sin(phi);
	out[1] = r * cos(phi);
	out[2] = r * sin(theta) * sin(phi);
}

/* random draws on a Philox stream, double precision */
static inline double vmc_frand(sray_rng *s, double range)
{
	return range * sray_rng_uniform_d(s);
}

static inline void vmc_sphrand(double out[3], sray_rng *s, double rad)
{
	double u0 = sray_rng_uniform_d(s);
	double u1 = sray_rng_uniform_d(s);
	double z = 2.0 * u1 - 1.0;
	double sxy = sqrt(1.0 - z * z);
	double ang = 2.0 * M_PI * u0;
	out[0] = rad * cos(ang) * sxy;
	out[1] = rad * sin(ang) * sxy;
	out[2] = rad * z;
}

static inline double vmc_gaussian(double x, double mean, double sdev)
{
	double d = x - mean;
	return exp(-(d * d) / (2.0 * sdev * sdev)) / (sdev * sqrt(2.0 * M_PI));
}

#endif
