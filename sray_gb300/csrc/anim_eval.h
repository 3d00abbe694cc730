/* anim_eval.h -- keyframe tracks and node transforms, one implementation for
 * the host (scene loading, per-frame object bounds, projection maps, the
 * camera) and the device (the per-frame table of object transforms and
 * light positions, k_xforms in render.cu).
 *
 * Track evaluation follows Track<T>::operator() (src/anim.inl:189-263):
 * keys sorted by time; outside the keys' range the repeat extrapolator wraps
 * the time (ping-pong and clamp hold the end key); the key interval is
 * found by the nearest-key search of get_key_interval (src/anim.inl:70-110);
 * step holds the interval's start, linear interpolates component-wise
 * (quaternions included), cubic is Catmull-Rom for vectors and a slerp of
 * the interval's keys for quaternions (src/anim.inl:268-273).  The node
 * matrix is XFormNode::get_xform_matrix: pivot * T * R * S * -pivot
 * (src/anim.cc:391-419).  All in double, as the reference computes them.
 */
#ifndef SRAY_ANIM_EVAL_H_
#define SRAY_ANIM_EVAL_H_

#include <math.h>
#include <string.h>

#ifdef __CUDACC__
#define SRAY_HD __host__ __device__
#else
#define SRAY_HD
#endif

namespace sray {

enum { INTERP_STEP, INTERP_LINEAR, INTERP_CUBIC };
enum { EXTRAP_CLAMP, EXTRAP_REPEAT, EXTRAP_PINGPONG };

/* a track as flat arrays: n key times (ascending) and n values of dim
 * doubles (3: a vector x y z; 4: a quaternion s x y z); def when n == 0 */
struct KeyView {
	const int *time;
	const double *val;
	const double *def;
	int n, dim, interp, extrap;
};

SRAY_HD inline int key_iabs(int v) { return v < 0 ? -v : v; }

/* the key nearest to `time` in [s, e] (the search of get_key_interval) */
SRAY_HD inline int key_nearest(const int *time, int s, int e, int t)
{
	for(;;) {
		if(s == e) return s;
		if(e - s == 1) return key_iabs(t - time[s]) < key_iabs(time[e] - t) ? s : e;
		int mid = (s + e) / 2;
		if(t < time[mid]) e = mid;
		else if(t > time[mid]) s = mid + 1;
		else return mid;
	}
}

/* the track's value at `time` into out[dim] */
SRAY_HD inline void key_eval(const KeyView &k, int time, double *out)
{
	int n = k.n, dim = k.dim;
	if(!n) {
		for(int i = 0; i < dim; i++) out[i] = k.def[i];
		return;
	}
	if(n > 1) {
		int first = k.time[0], last = k.time[n - 1];
		if(first != last && (time < first || time > last) && k.extrap == EXTRAP_REPEAT) {
			while(time < first) time += last - first;
			time = (time - first) % (last - first) + first;
		}
	}
	int nk = key_nearest(k.time, 0, n - 1, time);
	int s = nk, e = -1;
	if(time < k.time[nk] && k.time[nk] != k.time[0]) { s = nk - 1; e = nk; }
	else if(time > k.time[nk] && k.time[nk] != k.time[n - 1]) { s = nk; e = nk + 1; }
	const double *vs = k.val + (size_t)s * dim;
	if(e < 0 || k.interp == INTERP_STEP || (k.interp != INTERP_LINEAR && k.interp != INTERP_CUBIC)) {
		for(int i = 0; i < dim; i++) out[i] = vs[i];
		return;
	}
	const double *ve = k.val + (size_t)e * dim;
	double t = (double)(time - k.time[s]) / (double)(k.time[e] - k.time[s]);
	if(k.interp == INTERP_LINEAR) {
		for(int i = 0; i < dim; i++) out[i] = vs[i] + (ve[i] - vs[i]) * t;
		return;
	}
	if(dim == 4) {
		/* slerp of the interval's keys, taking the shorter arc */
		double d = vs[0] * ve[0] + vs[1] * ve[1] + vs[2] * ve[2] + vs[3] * ve[3];
		double b[4] = {ve[0], ve[1], ve[2], ve[3]};
		if(d < 0.0) { d = -d; b[0] = -b[0]; b[1] = -b[1]; b[2] = -b[2]; b[3] = -b[3]; }
		double wa, wb;
		if(d > 0.9999) { wa = 1.0 - t; wb = t; }
		else {
			double ang = acos(d), sn = sin(ang);
			wa = sin((1.0 - t) * ang) / sn;
			wb = sin(t * ang) / sn;
		}
		for(int i = 0; i < 4; i++) out[i] = vs[i] * wa + b[i] * wb;
		return;
	}
	/* Catmull-Rom through the interval's neighbours (end keys repeated) */
	const double *v0 = k.val + (size_t)(s > 0 ? s - 1 : s) * dim;
	const double *v3 = k.val + (size_t)(e < n - 1 ? e + 1 : e) * dim;
	double t2 = t * t, t3 = t2 * t;
	for(int i = 0; i < dim; i++) {
		double a = v0[i], bb = vs[i], c = ve[i], dd = v3[i];
		out[i] = (bb * 2.0 + (c - a) * t + (a * 2.0 - bb * 5.0 + c * 4.0 - dd) * t2 + (bb * 3.0 - a - c * 3.0 + dd) * t3) * 0.5;
	}
}

/* ---- 4x4 matrices, row-major, acting on column vectors ---- */
SRAY_HD inline void m4_ident(double m[4][4])
{
	for(int i = 0; i < 4; i++) for(int j = 0; j < 4; j++) m[i][j] = i == j ? 1.0 : 0.0;
}
SRAY_HD inline void m4_mul(double o[4][4], const double a[4][4], const double b[4][4])
{
	double r[4][4];
	for(int i = 0; i < 4; i++)
		for(int j = 0; j < 4; j++)
			r[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j] + a[i][3] * b[3][j];
	for(int i = 0; i < 4; i++) for(int j = 0; j < 4; j++) o[i][j] = r[i][j];
}
/* the rotation of quaternion (s, x, y, z), not renormalised */
SRAY_HD inline void m4_quat(double m[4][4], const double *q)
{
	m4_ident(m);
	double s = q[0], x = q[1], y = q[2], z = q[3];
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
SRAY_HD inline double m4_det3(double a, double b, double c, double d, double e, double f, double g, double h, double i)
{
	return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}
/* general inverse by the adjugate */
SRAY_HD inline void m4_inverse(double out[4][4], const double m[4][4])
{
	double cof[4][4];
	for(int i = 0; i < 4; i++) {
		for(int j = 0; j < 4; j++) {
			double s[9];
			int k = 0;
			for(int r = 0; r < 4; r++) {
				if(r == i) continue;
				for(int c = 0; c < 4; c++) if(c != j) s[k++] = m[r][c];
			}
			double mn = m4_det3(s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], s[8]);
			cof[i][j] = ((i + j) & 1) ? -mn : mn;
		}
	}
	double det = m[0][0] * cof[0][0] + m[0][1] * cof[0][1] + m[0][2] * cof[0][2] + m[0][3] * cof[0][3];
	for(int i = 0; i < 4; i++)
		for(int j = 0; j < 4; j++)
			out[i][j] = cof[j][i] / det;
}

/* XFormNode::get_xform_matrix from the evaluated tracks */
SRAY_HD inline void node_matrix(const double *p, const double *q, const double *s, const double *pivot, double m[4][4])
{
	double pm[4][4], npm[4][4], tm[4][4], rm[4][4], sm[4][4], a[4][4];
	m4_ident(pm); pm[0][3] = pivot[0]; pm[1][3] = pivot[1]; pm[2][3] = pivot[2];
	m4_ident(npm); npm[0][3] = -pivot[0]; npm[1][3] = -pivot[1]; npm[2][3] = -pivot[2];
	m4_ident(tm); tm[0][3] = p[0]; tm[1][3] = p[1]; tm[2][3] = p[2];
	m4_quat(rm, q);
	m4_ident(sm); sm[0][0] = s[0]; sm[1][1] = s[1]; sm[2][2] = s[2];
	m4_mul(a, pm, tm);
	m4_mul(a, a, rm);
	m4_mul(a, a, sm);
	m4_mul(m, a, npm);
}

/* the per-time record of an object's transform (XF_STRIDE floats):
 * forward 3x4, inverse 3x4, inverse-transpose 3x3, zero padding */
SRAY_HD inline void pack_transform(const double m[4][4], float *dst, int stride)
{
	double inv[4][4];
	m4_inverse(inv, m);
	for(int i = 0; i < 3; i++) for(int j = 0; j < 4; j++) dst[i * 4 + j] = (float)m[i][j];
	for(int i = 0; i < 3; i++) for(int j = 0; j < 4; j++) dst[12 + i * 4 + j] = (float)inv[i][j];
	for(int r = 0; r < 3; r++) for(int c = 0; c < 3; c++) dst[24 + r * 3 + c] = (float)inv[c][r];
	for(int k = 33; k < stride; k++) dst[k] = 0.0f;
}

}  // namespace sray

#endif
