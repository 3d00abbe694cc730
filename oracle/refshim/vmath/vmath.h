/* vmath.h -- TEST INFRASTRUCTURE: a stand-in for libvmath (gfxtools), which
 * the reference includes as <vmath/vmath.h> but does not ship.  It provides
 * the types and functions the reference's sources call, with the semantics
 * documented in vmath_core.h, so the reference's own files compile here and
 * serve as the pin of the CPU oracle.  Random draws come from the Philox
 * stream that the harness selects per photon / pixel sample.
 */
#ifndef SHIM_VMATH_H_
#define SHIM_VMATH_H_

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <assert.h>
#include "vmath_core.h"

typedef double scalar_t;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#define TWO_PI (2.0 * M_PI)
#define HALF_PI (0.5 * M_PI)
#define QUARTER_PI (0.25 * M_PI)
#define DEG_TO_RAD(a) (((a) * M_PI) / 180.0)
#define RAD_TO_DEG(a) (((a) * 180.0) / M_PI)
#define SQ(x) ((x) * (x))
#ifndef MIN
#define MIN(a, b)	((a) < (b) ? (a) : (b))
#endif
#ifndef MAX
#define MAX(a, b)	((a) > (b) ? (a) : (b))
#endif
#define ERROR_MARGIN VMC_ERROR_MARGIN
#define SMALL_NUMBER VMC_SMALL_NUMBER
#define XSMALL_NUMBER VMC_XSMALL_NUMBER

/* the stream the harness selected for the current photon / pixel sample */
sray_rng *shim_rng_current(void);

class Vector3;
class Vector4;
class Matrix3x3;
class Matrix4x4;
class Quaternion;
class SphVector;

class Vector2 {
public:
	scalar_t x, y;
	Vector2(scalar_t x = 0, scalar_t y = 0) : x(x), y(y) {}
	Vector2(const Vector3 &v);
	scalar_t &operator[](int i) { return i ? y : x; }
	const scalar_t &operator[](int i) const { return i ? y : x; }
};

class SphVector {
public:
	scalar_t theta, phi, r;
	SphVector(scalar_t theta = 0, scalar_t phi = 0, scalar_t r = 1) : theta(theta), phi(phi), r(r) {}
	SphVector(const Vector3 &v);
};

class Vector3 {
public:
	scalar_t x, y, z;
	Vector3(scalar_t x = 0, scalar_t y = 0, scalar_t z = 0) : x(x), y(y), z(z) {}
	Vector3(const Vector2 &v) : x(v.x), y(v.y), z(1) {}
	Vector3(const Vector4 &v);
	Vector3(const SphVector &s)
	{
		double o[3];
		vmc_vec_from_sph(o, s.theta, s.phi, s.r);
		x = o[0]; y = o[1]; z = o[2];
	}
	scalar_t &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
	const scalar_t &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }

	scalar_t length() const { return sqrt(x * x + y * y + z * z); }
	scalar_t length_sq() const { return x * x + y * y + z * z; }
	void normalize() { scalar_t l = length(); x /= l; y /= l; z /= l; }
	Vector3 normalized() const { scalar_t l = length(); return Vector3(x / l, y / l, z / l); }
	void transform(const Matrix4x4 &m);
	Vector3 transformed(const Matrix4x4 &m) const;
	void transform(const Matrix3x3 &m);
	Vector3 transformed(const Matrix3x3 &m) const;
	void transform(const Quaternion &q);
	Vector3 transformed(const Quaternion &q) const;
	Vector3 reflection(const Vector3 &n) const;
	Vector3 refraction(const Vector3 &n, scalar_t ior) const;

	Vector3 &operator+=(const Vector3 &v) { x += v.x; y += v.y; z += v.z; return *this; }
	Vector3 &operator-=(const Vector3 &v) { x -= v.x; y -= v.y; z -= v.z; return *this; }
	Vector3 &operator*=(const Vector3 &v) { x *= v.x; y *= v.y; z *= v.z; return *this; }
	Vector3 &operator*=(scalar_t s) { x *= s; y *= s; z *= s; return *this; }
	Vector3 &operator/=(scalar_t s) { x /= s; y /= s; z /= s; return *this; }
};

inline Vector2::Vector2(const Vector3 &v) : x(v.x), y(v.y) {}
inline SphVector::SphVector(const Vector3 &v)
{
	double in[3] = {v.x, v.y, v.z};
	vmc_sph_from_vec(&theta, &phi, &r, in);
}

inline Vector3 operator+(const Vector3 &a, const Vector3 &b) { return Vector3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline Vector3 operator-(const Vector3 &a, const Vector3 &b) { return Vector3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline Vector3 operator-(const Vector3 &a) { return Vector3(-a.x, -a.y, -a.z); }
inline Vector3 operator*(const Vector3 &a, const Vector3 &b) { return Vector3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline Vector3 operator*(const Vector3 &a, scalar_t s) { return Vector3(a.x * s, a.y * s, a.z * s); }
inline Vector3 operator*(scalar_t s, const Vector3 &a) { return Vector3(s * a.x, s * a.y, s * a.z); }
inline Vector3 operator/(const Vector3 &a, scalar_t s) { return Vector3(a.x / s, a.y / s, a.z / s); }
inline Vector3 operator/(const Vector3 &a, const Vector3 &b) { return Vector3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline bool operator==(const Vector3 &a, const Vector3 &b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

inline scalar_t dot_product(const Vector3 &a, const Vector3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vector3 cross_product(const Vector3 &a, const Vector3 &b)
{
	return Vector3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

inline Vector3 Vector3::reflection(const Vector3 &n) const { return *this - n * (2.0 * dot_product(*this, n)); }
inline Vector3 Vector3::refraction(const Vector3 &n, scalar_t ior) const
{
	scalar_t cos_inc = dot_product(*this, -n);
	scalar_t radical = 1.0 + (ior * ior) * (cos_inc * cos_inc - 1.0);
	if(radical < 0.0) return reflection(n);
	scalar_t beta = ior * cos_inc - sqrt(radical);
	return *this * ior + n * beta;
}

class Vector4 {
public:
	scalar_t x, y, z, w;
	Vector4(scalar_t x = 0, scalar_t y = 0, scalar_t z = 0, scalar_t w = 0) : x(x), y(y), z(z), w(w) {}
	Vector4(const Vector3 &v) : x(v.x), y(v.y), z(v.z), w(1) {}
	scalar_t &operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
	const scalar_t &operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
	scalar_t length() const { return sqrt(x * x + y * y + z * z + w * w); }
	scalar_t length_sq() const { return x * x + y * y + z * z + w * w; }
	void transform(const Matrix4x4 &m);
	Vector4 &operator+=(const Vector4 &v) { x += v.x; y += v.y; z += v.z; w += v.w; return *this; }
	Vector4 &operator-=(const Vector4 &v) { x -= v.x; y -= v.y; z -= v.z; w -= v.w; return *this; }
	Vector4 &operator*=(const Vector4 &v) { x *= v.x; y *= v.y; z *= v.z; w *= v.w; return *this; }
	Vector4 &operator*=(scalar_t s) { x *= s; y *= s; z *= s; w *= s; return *this; }
	Vector4 &operator/=(scalar_t s) { x /= s; y /= s; z /= s; w /= s; return *this; }
};

inline Vector3::Vector3(const Vector4 &v) : x(v.x), y(v.y), z(v.z) {}

inline Vector4 operator+(const Vector4 &a, const Vector4 &b) { return Vector4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline Vector4 operator-(const Vector4 &a, const Vector4 &b) { return Vector4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline Vector4 operator-(const Vector4 &a) { return Vector4(-a.x, -a.y, -a.z, -a.w); }
inline Vector4 operator*(const Vector4 &a, const Vector4 &b) { return Vector4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline Vector4 operator*(const Vector4 &a, scalar_t s) { return Vector4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline Vector4 operator*(scalar_t s, const Vector4 &a) { return Vector4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline Vector4 operator/(const Vector4 &a, scalar_t s) { return Vector4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline Vector4 operator-(const Vector4 &a, scalar_t s) { return Vector4(a.x - s, a.y - s, a.z - s, a.w - s); }
inline Vector4 operator+(const Vector4 &a, scalar_t s) { return Vector4(a.x + s, a.y + s, a.z + s, a.w + s); }

class Matrix3x3 {
public:
	scalar_t m[3][3];
	Matrix3x3() { memset(m, 0, sizeof m); m[0][0] = m[1][1] = m[2][2] = 1.0; }
	Matrix3x3(scalar_t m00, scalar_t m01, scalar_t m02, scalar_t m10, scalar_t m11, scalar_t m12,
			scalar_t m20, scalar_t m21, scalar_t m22)
	{
		m[0][0] = m00; m[0][1] = m01; m[0][2] = m02;
		m[1][0] = m10; m[1][1] = m11; m[1][2] = m12;
		m[2][0] = m20; m[2][1] = m21; m[2][2] = m22;
	}
	Matrix3x3(const Matrix4x4 &m4);
	scalar_t *operator[](int i) { return m[i]; }
	const scalar_t *operator[](int i) const { return m[i]; }
	Matrix3x3 transposed() const
	{
		return Matrix3x3(m[0][0], m[1][0], m[2][0], m[0][1], m[1][1], m[2][1], m[0][2], m[1][2], m[2][2]);
	}
};

class Matrix4x4 {
public:
	scalar_t m[4][4];
	Matrix4x4() { vmc_mat_identity(m); }
	Matrix4x4(scalar_t m00, scalar_t m01, scalar_t m02, scalar_t m03, scalar_t m10, scalar_t m11, scalar_t m12, scalar_t m13,
			scalar_t m20, scalar_t m21, scalar_t m22, scalar_t m23, scalar_t m30, scalar_t m31, scalar_t m32, scalar_t m33)
	{
		m[0][0] = m00; m[0][1] = m01; m[0][2] = m02; m[0][3] = m03;
		m[1][0] = m10; m[1][1] = m11; m[1][2] = m12; m[1][3] = m13;
		m[2][0] = m20; m[2][1] = m21; m[2][2] = m22; m[2][3] = m23;
		m[3][0] = m30; m[3][1] = m31; m[3][2] = m32; m[3][3] = m33;
	}
	Matrix4x4(const Matrix3x3 &m3)
	{
		vmc_mat_identity(m);
		for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) m[i][j] = m3.m[i][j];
	}
	scalar_t *operator[](int i) { return m[i]; }
	const scalar_t *operator[](int i) const { return m[i]; }
	void set_translation(const Vector3 &t) { vmc_mat_translation(m, t.x, t.y, t.z); }
	void set_scaling(const Vector3 &s) { vmc_mat_scaling(m, s.x, s.y, s.z); }
	Matrix4x4 inverse() const { Matrix4x4 r; vmc_mat_inverse(r.m, m); return r; }
	Matrix4x4 transposed() const { Matrix4x4 r; vmc_mat_transpose(r.m, m); return r; }
};

inline Matrix3x3::Matrix3x3(const Matrix4x4 &m4)
{
	for(int i = 0; i < 3; i++) for(int j = 0; j < 3; j++) m[i][j] = m4.m[i][j];
}

inline Matrix4x4 operator*(const Matrix4x4 &a, const Matrix4x4 &b) { Matrix4x4 r; vmc_mat_mul(r.m, a.m, b.m); return r; }

inline void Vector3::transform(const Matrix4x4 &mat)
{
	double in[3] = {x, y, z}, o[3];
	vmc_xform_point(o, mat.m, in);
	x = o[0]; y = o[1]; z = o[2];
}
inline Vector3 Vector3::transformed(const Matrix4x4 &mat) const { Vector3 v = *this; v.transform(mat); return v; }
inline void Vector3::transform(const Matrix3x3 &mat)
{
	double nx = mat.m[0][0] * x + mat.m[0][1] * y + mat.m[0][2] * z;
	double ny = mat.m[1][0] * x + mat.m[1][1] * y + mat.m[1][2] * z;
	double nz = mat.m[2][0] * x + mat.m[2][1] * y + mat.m[2][2] * z;
	x = nx; y = ny; z = nz;
}
inline Vector3 Vector3::transformed(const Matrix3x3 &mat) const { Vector3 v = *this; v.transform(mat); return v; }
inline void Vector4::transform(const Matrix4x4 &mat)
{
	double nx = mat.m[0][0] * x + mat.m[0][1] * y + mat.m[0][2] * z + mat.m[0][3] * w;
	double ny = mat.m[1][0] * x + mat.m[1][1] * y + mat.m[1][2] * z + mat.m[1][3] * w;
	double nz = mat.m[2][0] * x + mat.m[2][1] * y + mat.m[2][2] * z + mat.m[2][3] * w;
	double nw = mat.m[3][0] * x + mat.m[3][1] * y + mat.m[3][2] * z + mat.m[3][3] * w;
	x = nx; y = ny; z = nz; w = nw;
}

class Quaternion {
public:
	scalar_t s;
	Vector3 v;
	Quaternion() : s(1), v(0, 0, 0) {}
	Quaternion(scalar_t s, scalar_t x, scalar_t y, scalar_t z) : s(s), v(x, y, z) {}
	Quaternion(const Vector3 &axis, scalar_t angle) { set_rotation(axis, angle); }
	void set_rotation(const Vector3 &axis, scalar_t angle)
	{
		double a[3] = {axis.x, axis.y, axis.z}, q[4];
		vmc_quat_axis_angle(q, a, angle);
		s = q[0]; v = Vector3(q[1], q[2], q[3]);
	}
	void normalize()
	{
		double q[4] = {s, v.x, v.y, v.z};
		vmc_quat_normalize(q);
		s = q[0]; v = Vector3(q[1], q[2], q[3]);
	}
	Quaternion conjugate() const { return Quaternion(s, -v.x, -v.y, -v.z); }
	Matrix3x3 get_rotation_matrix() const
	{
		double m[4][4];
		vmc_mat_quat(m, s, v.x, v.y, v.z);
		return Matrix3x3(m[0][0], m[0][1], m[0][2], m[1][0], m[1][1], m[1][2], m[2][0], m[2][1], m[2][2]);
	}
};

inline Quaternion operator*(const Quaternion &a, const Quaternion &b)
{
	double qa[4] = {a.s, a.v.x, a.v.y, a.v.z}, qb[4] = {b.s, b.v.x, b.v.y, b.v.z}, o[4];
	vmc_quat_mul(o, qa, qb);
	return Quaternion(o[0], o[1], o[2], o[3]);
}
inline Quaternion operator+(const Quaternion &a, const Quaternion &b) { return Quaternion(a.s + b.s, a.v.x + b.v.x, a.v.y + b.v.y, a.v.z + b.v.z); }
inline Quaternion operator-(const Quaternion &a, const Quaternion &b) { return Quaternion(a.s - b.s, a.v.x - b.v.x, a.v.y - b.v.y, a.v.z - b.v.z); }
inline Quaternion operator*(const Quaternion &a, scalar_t t) { return Quaternion(a.s * t, a.v.x * t, a.v.y * t, a.v.z * t); }

inline void Vector3::transform(const Quaternion &q)
{
	Matrix3x3 m = q.get_rotation_matrix();
	transform(m);
}
inline Vector3 Vector3::transformed(const Quaternion &q) const { Vector3 r = *this; r.transform(q); return r; }

inline Quaternion slerp(const Quaternion &a, const Quaternion &b, scalar_t t)
{
	double qa[4] = {a.s, a.v.x, a.v.y, a.v.z}, qb[4] = {b.s, b.v.x, b.v.y, b.v.z}, o[4];
	vmc_quat_slerp(o, qa, qb, t);
	return Quaternion(o[0], o[1], o[2], o[3]);
}

inline scalar_t lerp(scalar_t a, scalar_t b, scalar_t t) { return a + (b - a) * t; }
inline Vector3 lerp(const Vector3 &a, const Vector3 &b, scalar_t t) { return a + (b - a) * t; }
inline Vector4 lerp(const Vector4 &a, const Vector4 &b, scalar_t t) { return a + (b - a) * t; }
inline Quaternion lerp(const Quaternion &a, const Quaternion &b, scalar_t t)
{
	return Quaternion(a.s + (b.s - a.s) * t, a.v.x + (b.v.x - a.v.x) * t, a.v.y + (b.v.y - a.v.y) * t, a.v.z + (b.v.z - a.v.z) * t);
}

inline Vector3 catmull_rom_spline(const Vector3 &v0, const Vector3 &v1, const Vector3 &v2, const Vector3 &v3, scalar_t t)
{
	double t2 = t * t, t3 = t2 * t;
	return (v1 * 2.0 + (v2 - v0) * t + (v0 * 2.0 - v1 * 5.0 + v2 * 4.0 - v3) * t2 + (v1 * 3.0 - v0 - v2 * 3.0 + v3) * t3) * 0.5;
}

/* ray with an index-of-refraction stack of depth 4 */
class Ray {
public:
	static scalar_t env_ior;
	Vector3 origin, dir;
	scalar_t energy;
	int iter;
	scalar_t ior;
	long time;
	scalar_t stack[4];
	int sp;

	Ray() : origin(0, 0, 0), dir(0, 0, 1), energy(1.0), iter(0), ior(env_ior), time(0), sp(0) {}
	Ray(const Vector3 &o, const Vector3 &d) : origin(o), dir(d), energy(1.0), iter(0), ior(env_ior), time(0), sp(0) {}

	Ray transformed(const Matrix4x4 &m) const
	{
		Ray r = *this;
		double o[3], d[3], oi[3] = {origin.x, origin.y, origin.z}, di[3] = {dir.x, dir.y, dir.z};
		vmc_xform_point(o, m.m, oi);
		vmc_xform_dir(d, m.m, di);
		r.origin = Vector3(o[0], o[1], o[2]);
		r.dir = Vector3(d[0], d[1], d[2]);
		return r;
	}
	void enter(scalar_t n) { ior = n; if(sp < 4) stack[sp++] = n; }
	void leave()
	{
		if(sp == 0) return;
		sp--;
		ior = sp ? stack[sp - 1] : env_ior;
	}
	scalar_t calc_ior(bool entering, scalar_t mat_ior = 1.0) const
	{
		scalar_t from = ior;
		if(entering) return from / mat_ior;
		Ray t = *this;
		t.leave();
		return from / t.ior;
	}
};

inline Ray reflect_ray(const Ray &in, const Vector3 &n)
{
	Ray r = in;
	r.dir = in.dir.reflection(n);
	return r;
}

inline Ray refract_ray(const Ray &in, const Vector3 &n, scalar_t mat_ior, bool entering, scalar_t ray_mag)
{
	Ray r = in;
	scalar_t ior = r.calc_ior(entering, mat_ior);
	if(entering) r.enter(mat_ior);
	else r.leave();
	r.dir = (r.dir / ray_mag).refraction(n, ior) * ray_mag;
	if(dot_product(r.dir, n) > 0.0) {
		if(entering) r.leave();
		else r.enter(mat_ior);
	}
	return r;
}

inline scalar_t frand(scalar_t range) { return vmc_frand(shim_rng_current(), range); }
inline Vector3 sphrand(scalar_t rad)
{
	double o[3];
	vmc_sphrand(o, shim_rng_current(), rad);
	return Vector3(o[0], o[1], o[2]);
}
inline scalar_t gaussian(scalar_t x, scalar_t mean, scalar_t sdev) { return vmc_gaussian(x, mean, sdev); }

#endif
