/* sray_oracle.cc -- TEST INFRASTRUCTURE: CPU restatement of S-ray's rendering
 * path (the checker of the GPU library; never linked into the product).
 *
 * Each function follows the reference routine cited beside it (paths are
 * relative to the reference project root).  The structure stays the
 * reference's: recursive octree traversal over all eight children with no
 * ordering or early out, recursive Whitted/photon-map shading, recursive
 * photon tracing with Russian roulette, fixed-radius photon gathers.
 * Random numbers come from the Philox streams of include/sray_rng.h instead
 * of the C library's global rand() state, so every run draws the same
 * photon and pixel-sample sets.
 *
 * The photon map keeps the kdtree library's semantics (positions and query
 * point rounded to float, squared distances compared in double against the
 * float-rounded radius), behind a uniform grid instead of a kd-tree, since
 * only the set of photons in range matters for the sums.
 */
#include <chrono>
#include <math.h>
#include <float.h>
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>
#include <vector>
#include <algorithm>
#include <thread>
#include <atomic>
#include <memory>
#include <unistd.h>
#include "sray_oracle.h"
#include "sray_rng.h"
#include "vmath_core.h"

namespace {

const double RAY_MAG = 10000.0;   /* src/opt.h:21 */

/* ------------------------------------------------------------------ */
/* small vector types, precision R                                      */
/* ------------------------------------------------------------------ */
template <class R> struct V3 {
	R x, y, z;
	V3() : x(0), y(0), z(0) {}
	V3(R a, R b, R c) : x(a), y(b), z(c) {}
	R &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
	R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return V3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return V3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> inline V3<R> operator-(V3<R> a) { return V3<R>(-a.x, -a.y, -a.z); }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return V3<R>(a.x * s, a.y * s, a.z * s); }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return V3<R>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return V3<R>(a.x / s, a.y / s, a.z / s); }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b)
{
	return V3<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> inline R rsqrt_(R v);
template <> inline float rsqrt_(float v) { return sqrtf(v); }
template <> inline double rsqrt_(double v) { return sqrt(v); }
template <class R> inline R length(V3<R> a) { return rsqrt_<R>(dot(a, a)); }
template <class R> inline V3<R> normalized(V3<R> a) { R l = length(a); return V3<R>(a.x / l, a.y / l, a.z / l); }
template <class R> inline V3<R> reflection(V3<R> v, V3<R> n) { return v - n * ((R)2 * dot(v, n)); }
template <class R> inline V3<R> refraction(V3<R> v, V3<R> n, R ior)
{
	R cos_inc = dot(v, -n);
	R radical = (R)1 + (ior * ior) * (cos_inc * cos_inc - (R)1);
	if(radical < (R)0) {
		return reflection(v, n);
	}
	R beta = ior * cos_inc - rsqrt_<R>(radical);
	return v * ior + n * beta;
}

template <class R> struct V4 {
	R x, y, z, w;
	V4() : x(0), y(0), z(0), w(0) {}
	V4(R a, R b, R c, R d) : x(a), y(b), z(c), w(d) {}
};
template <class R> inline V4<R> operator+(V4<R> a, V4<R> b) { return V4<R>(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
template <class R> inline V4<R> operator-(V4<R> a, V4<R> b) { return V4<R>(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
template <class R> inline V4<R> operator*(V4<R> a, V4<R> b) { return V4<R>(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
template <class R> inline V4<R> operator*(V4<R> a, R s) { return V4<R>(a.x * s, a.y * s, a.z * s, a.w * s); }
template <class R> inline V4<R> operator*(R s, V4<R> a) { return V4<R>(s * a.x, s * a.y, s * a.z, s * a.w); }
template <class R> inline V4<R> operator/(V4<R> a, R s) { return V4<R>(a.x / s, a.y / s, a.z / s, a.w / s); }
template <class R> inline R length_sq(V4<R> a) { return a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w; }

typedef V3<double> V3d;

/* ------------------------------------------------------------------ */
/* XML: a minimal DOM with the reference's attribute typing            */
/* ------------------------------------------------------------------ */
enum { AT_STR, AT_INT, AT_FLT, AT_VEC };

struct XAttr {
	std::string name, str;
	int type;
	int ival;
	double fval;
	double vval[4];
};

struct XNode {
	std::string name;
	std::vector<XAttr> attr;
	std::vector<XNode> chld;
	const XAttr *get(const char *n) const
	{
		for(size_t i = 0; i < attr.size(); i++) {
			if(attr[i].name == n) return &attr[i];
		}
		return 0;
	}
};

/* src/xmltree.c:51-95: a value starting with a digit (or sign + digit) is
 * numeric: FLT if it contains '.', else INT; with more than one
 * whitespace-separated number it becomes a VEC, padded with 1.0.  The
 * numbers are kept as float (struct xml_attr, src/xmltree.h:31-33). */
static void type_attr(XAttr &a)
{
	const char *val = a.str.c_str();
	a.type = AT_STR;
	a.ival = 0;
	a.fval = 0.0;
	a.vval[0] = a.vval[1] = a.vval[2] = a.vval[3] = 0.0;
	if(isdigit((unsigned char)val[0]) || ((val[0] == '+' || val[0] == '-') && isdigit((unsigned char)val[1]))) {
		a.type = strchr(val, '.') ? AT_FLT : AT_INT;
		a.ival = atoi(val);
		a.fval = (float)atof(val);
		a.vval[0] = a.vval[1] = a.vval[2] = a.vval[3] = 1.0;
		int i;
		for(i = 0; i < 4; i++) {
			if(!*val) break;
			a.vval[i] = (float)atof(val);
			while(*val && !isspace((unsigned char)*val)) val++;
			while(*val && isspace((unsigned char)*val)) val++;
		}
		if(i > 1) a.type = AT_VEC;
	}
}

struct XmlParser {
	const char *p, *end;
	std::string err;

	void skip_ws() { while(p < end && isspace((unsigned char)*p)) p++; }

	static void decode(std::string &s)
	{
		if(s.find('&') == std::string::npos) return;
		std::string o;
		for(size_t i = 0; i < s.size(); i++) {
			if(s[i] == '&') {
				size_t semi = s.find(';', i);
				if(semi != std::string::npos) {
					std::string ent = s.substr(i + 1, semi - i - 1);
					if(ent == "lt") { o += '<'; i = semi; continue; }
					if(ent == "gt") { o += '>'; i = semi; continue; }
					if(ent == "amp") { o += '&'; i = semi; continue; }
					if(ent == "quot") { o += '"'; i = semi; continue; }
					if(ent == "apos") { o += '\''; i = semi; continue; }
				}
			}
			o += s[i];
		}
		s.swap(o);
	}

	/* skip text, comments, processing instructions; stop at '<' of an element or '</' */
	bool skip_misc()
	{
		for(;;) {
			while(p < end && *p != '<') p++;
			if(p >= end) return false;
			if(p + 3 < end && p[1] == '!' && p[2] == '-' && p[3] == '-') {
				const char *e = strstr(p, "-->");
				if(!e || e >= end) { err = "unterminated comment"; return false; }
				p = e + 3;
				continue;
			}
			if(p + 1 < end && (p[1] == '?' || p[1] == '!')) {
				while(p < end && *p != '>') p++;
				if(p < end) p++;
				continue;
			}
			return true;
		}
	}

	bool parse_element(XNode &node)
	{
		/* at '<' */
		p++;
		const char *ns = p;
		while(p < end && !isspace((unsigned char)*p) && *p != '/' && *p != '>') p++;
		node.name.assign(ns, p - ns);
		for(;;) {
			skip_ws();
			if(p >= end) { err = "unexpected end in tag"; return false; }
			if(*p == '/') {
				if(p + 1 < end && p[1] == '>') { p += 2; return true; }
				err = "bad '/' in tag";
				return false;
			}
			if(*p == '>') { p++; break; }
			const char *an = p;
			while(p < end && *p != '=' && !isspace((unsigned char)*p)) p++;
			XAttr a;
			a.name.assign(an, p - an);
			skip_ws();
			if(p >= end || *p != '=') { err = "attribute without value: " + a.name; return false; }
			p++;
			skip_ws();
			if(p >= end || (*p != '"' && *p != '\'')) { err = "unquoted attribute: " + a.name; return false; }
			char q = *p++;
			const char *vs = p;
			while(p < end && *p != q) p++;
			if(p >= end) { err = "unterminated attribute"; return false; }
			a.str.assign(vs, p - vs);
			p++;
			decode(a.str);
			type_attr(a);
			node.attr.push_back(a);
		}
		/* children */
		for(;;) {
			if(!skip_misc()) { err = err.empty() ? "unexpected end of document in <" + node.name + ">" : err; return false; }
			if(p[1] == '/') {
				p += 2;
				const char *cn = p;
				while(p < end && *p != '>') p++;
				std::string cname(cn, p - cn);
				while(!cname.empty() && isspace((unsigned char)cname.back())) cname.pop_back();
				if(cname != node.name) { err = "mismatched </" + cname + "> for <" + node.name + ">"; return false; }
				if(p < end) p++;
				return true;
			}
			node.chld.push_back(XNode());
			if(!parse_element(node.chld.back())) return false;
		}
	}

	bool parse(const char *text, size_t len, XNode &root)
	{
		p = text;
		end = text + len;
		if(!skip_misc()) { err = "no root element"; return false; }
		return parse_element(root);
	}
};

/* ------------------------------------------------------------------ */
/* animation tracks and transforms (src/anim.inl, src/anim.cc)          */
/* ------------------------------------------------------------------ */
enum { INTERP_STEP, INTERP_LINEAR, INTERP_CUBIC };
enum { EXTRAP_CLAMP, EXTRAP_REPEAT, EXTRAP_PINGPONG };

struct Quat { double q[4]; };

static inline V3d lerp_v(const V3d &a, const V3d &b, double t) { return a + (b - a) * t; }

template <class T> struct Track {
	T def;
	std::vector<std::pair<int, T> > keys;
	int interp = INTERP_LINEAR, extrap = EXTRAP_CLAMP;

	void reset(const T &v) { keys.clear(); interp = INTERP_LINEAR; extrap = EXTRAP_CLAMP; def = v; }

	/* src/anim.inl:70-84: binary search for the key nearest to time */
	int nearest(int s, int e, int time) const
	{
		if(s == e) return s;
		if(e - s == 1) {
			return abs(time - keys[s].first) < abs(keys[e].first - time) ? s : e;
		}
		int mid = (s + e) / 2;
		if(time < keys[mid].first) return nearest(s, mid, time);
		if(time > keys[mid].first) return nearest(mid + 1, e, time);
		return mid;
	}

	/* XFormNode::set_position & co (src/anim.cc:220-287) through Track::add_key (src/anim.inl:146-159) */
	void set_key(int time, const T &v)
	{
		if(!keys.empty()) {
			int n = nearest(0, (int)keys.size() - 1, time);
			if(keys[n].first == time) {
				keys[n].second = v;
				return;
			}
		}
		keys.push_back(std::make_pair(time, v));
		std::stable_sort(keys.begin(), keys.end(),
				[](const std::pair<int, T> &a, const std::pair<int, T> &b) { return a.first < b.first; });
	}
};

template <class T> static T interp_val(const Track<T> &tr, const T &a, const T &b, double t);
template <> V3d interp_val(const Track<V3d> &, const V3d &a, const V3d &b, double t) { return lerp_v(a, b, t); }
template <> Quat interp_val(const Track<Quat> &, const Quat &a, const Quat &b, double t)
{
	Quat r;
	for(int i = 0; i < 4; i++) r.q[i] = a.q[i] + (b.q[i] - a.q[i]) * t;
	return r;
}

static V3d catmull(const V3d &v0, const V3d &v1, const V3d &v2, const V3d &v3, double t)
{
	double t2 = t * t, t3 = t2 * t;
	return (v1 * 2.0 + (v2 - v0) * t + (v0 * 2.0 - v1 * 5.0 + v2 * 4.0 - v3) * t2 +
			(v1 * 3.0 - v0 - v2 * 3.0 + v3) * t3) * 0.5;
}
static Quat catmull(const Quat &, const Quat &v1, const Quat &v2, const Quat &, double t)
{
	Quat r;
	vmc_quat_slerp(r.q, v1.q, v2.q, t);
	return r;
}

/* Track::operator()(int) -- src/anim.inl:189-263 */
template <class T> static T track_eval(const Track<T> &tr, int time)
{
	if(tr.keys.empty()) return tr.def;
	const std::vector<std::pair<int, T> > &k = tr.keys;
	if(k.size() > 1) {
		int first = k.front().first, last = k.back().first;
		if(first != last && (time < first || time > last)) {
			if(tr.extrap == EXTRAP_REPEAT) {
				while(time < first) time += last - first;
				time = (time - first) % (last - first) + first;
			}
		}
	}
	int n = tr.nearest(0, (int)k.size() - 1, time);
	int s = n, e = -1;
	if(time < k[n].first && k[n].first != k[0].first) {
		s = n - 1;
		e = n;
	} else if(time > k[n].first && k[n].first != k[k.size() - 1].first) {
		s = n;
		e = n + 1;
	}
	switch(tr.interp) {
	case INTERP_STEP:
		return k[s].second;
	case INTERP_LINEAR:
		if(e >= 0) {
			double t = (double)(time - k[s].first) / (double)(k[e].first - k[s].first);
			return interp_val(tr, k[s].second, k[e].second, t);
		}
		return k[s].second;
	case INTERP_CUBIC:
		if(e >= 0) {
			double t = (double)(time - k[s].first) / (double)(k[e].first - k[s].first);
			const T &v0 = k[s > 0 ? s - 1 : s].second;
			const T &v3 = k[e < (int)k.size() - 1 ? e + 1 : e].second;
			return catmull(v0, k[s].second, k[e].second, v3, t);
		}
		return k[s].second;
	default:
		return k[s].second;
	}
}

struct XForm {
	Track<V3d> ptrack, strack;
	Track<Quat> rtrack;
	V3d pivot;

	XForm() { reset(); }
	void reset()
	{
		ptrack.reset(V3d(0, 0, 0));
		Quat id = {{1, 0, 0, 0}};
		rtrack.reset(id);
		strack.reset(V3d(1, 1, 1));
		pivot = V3d(0, 0, 0);
	}
	void set_interp(int i) { ptrack.interp = rtrack.interp = strack.interp = i; }
	void set_extrap(int e) { ptrack.extrap = rtrack.extrap = strack.extrap = e; }

	/* XFormNode::load_xml -- src/anim.cc:68-121 */
	void load_xml(const XNode &node)
	{
		const XAttr *a;
		int msec = 0;
		if((a = node.get("interpolate"))) {
			if(a->str == "linear") set_interp(INTERP_LINEAR);
			else if(a->str == "step") set_interp(INTERP_STEP);
			else if(a->str == "cubic") set_interp(INTERP_CUBIC);
		}
		if((a = node.get("extrapolate"))) {
			if(a->str == "clamp") set_extrap(EXTRAP_CLAMP);
			else if(a->str == "repeat") set_extrap(EXTRAP_REPEAT);
			else if(a->str == "pingpong") set_extrap(EXTRAP_PINGPONG);
		}
		if((a = node.get("time")) && a->type == AT_INT) msec = a->ival;
		if((a = node.get("pos")) && a->type == AT_VEC) ptrack.set_key(msec, V3d(a->vval[0], a->vval[1], a->vval[2]));
		if((a = node.get("rot")) && a->type == AT_VEC) {
			Quat q = {{a->vval[0], a->vval[1], a->vval[2], a->vval[3]}};
			vmc_quat_normalize(q.q);
			rtrack.set_key(msec, q);
		}
		if((a = node.get("axisrot")) && a->type == AT_VEC) {
			double ang = (a->vval[0] * M_PI) / 180.0;
			double axis[3] = {a->vval[1], a->vval[2], a->vval[3]};
			Quat q;
			vmc_quat_axis_angle(q.q, axis, ang);
			rtrack.set_key(msec, q);
		}
		if((a = node.get("scale")) && a->type == AT_VEC) strack.set_key(msec, V3d(a->vval[0], a->vval[1], a->vval[2]));
		if((a = node.get("pivot")) && a->type == AT_VEC) pivot = V3d(a->vval[0], a->vval[1], a->vval[2]);
	}

	V3d position(int t) const { return track_eval(ptrack, t); }
	V3d scaling(int t) const { return track_eval(strack, t); }

	/* XFormNode::get_xform_matrix -- src/anim.cc:391-419 */
	void matrix(int time, double m[4][4]) const
	{
		V3d pos = track_eval(ptrack, time);
		Quat rot = track_eval(rtrack, time);
		V3d sc = track_eval(strack, time);
		double pm[4][4], npm[4][4], tm[4][4], rm[4][4], sm[4][4];
		vmc_mat_translation(pm, pivot.x, pivot.y, pivot.z);
		vmc_mat_translation(npm, -pivot.x, -pivot.y, -pivot.z);
		vmc_mat_translation(tm, pos.x, pos.y, pos.z);
		vmc_mat_quat(rm, rot.q[0], rot.q[1], rot.q[2], rot.q[3]);
		vmc_mat_scaling(sm, sc.x, sc.y, sc.z);
		double a[4][4];
		vmc_mat_mul(a, pm, tm);
		vmc_mat_mul(a, a, rm);
		vmc_mat_mul(a, a, sm);
		vmc_mat_mul(m, a, npm);
	}
};

static V3d xform_pt(const double m[4][4], const V3d &p)
{
	double in[3] = {p.x, p.y, p.z}, o[3];
	vmc_xform_point(o, m, in);
	return V3d(o[0], o[1], o[2]);
}

/* ------------------------------------------------------------------ */
/* materials (src/material.cc)                                          */
/* ------------------------------------------------------------------ */
struct MatAttr {
	std::string name;
	double col[4];
	int tex = -1;                /* index into Scene::texs, -1 = none */
};

/* Texture (src/texture.cc): an RGBA float image, rows top first, looked up
 * with the 5-tap filter and repeat wrapping. */
struct Tex {
	int xsz = 0, ysz = 0;
	std::vector<float> pix;
};

struct Material {
	std::string name;
	int phong = 0;
	std::vector<MatAttr> attr;   /* sorted by name (src/material.cc:91-111) */

	Material()
	{
		/* src/material.cc:68-76 */
		set("diffuse", 1.0, 1.0, 1.0, 0.0);
		set("specular", 0.0, 0.0, 0.0, 0.0);
		set("reflect", 0.0, 0.0, 0.0, 0.0);
		set("refract", 0.0, 0.0, 0.0, 0.0);
		set("ior", 1.5, 0.0, 0.0, 0.0);
	}
	/* set_attribute replaces both the colour and the texture (src/material.cc:140-151) */
	void set(const char *n, double r, double g, double b, double a, int tex = -1)
	{
		for(size_t i = 0; i < attr.size(); i++) {
			if(attr[i].name == n) {
				attr[i].col[0] = r; attr[i].col[1] = g; attr[i].col[2] = b; attr[i].col[3] = a;
				attr[i].tex = tex;
				return;
			}
		}
		MatAttr m;
		m.name = n;
		m.col[0] = r; m.col[1] = g; m.col[2] = b; m.col[3] = a;
		m.tex = tex;
		attr.push_back(m);
		std::sort(attr.begin(), attr.end(), [](const MatAttr &x, const MatAttr &y) { return x.name < y.name; });
	}
	const MatAttr *find(const char *n) const
	{
		for(size_t i = 0; i < attr.size(); i++) if(attr[i].name == n) return &attr[i];
		return 0;
	}
	bool have(const char *n) const { return find(n) != 0; }
	/* get_attribute returns a default (1,1,1,1) attribute when missing (src/material.cc:161-165) */
	const double *get(const char *n) const
	{
		static const double def[4] = {1.0, 1.0, 1.0, 1.0};
		const MatAttr *a = find(n);
		return a ? a->col : def;
	}
	int tex_of(const char *n) const
	{
		const MatAttr *a = find(n);
		return a ? a->tex : -1;
	}
};

/* ------------------------------------------------------------------ */
/* octree build (src/octree.inl:119-191)                                */
/* ------------------------------------------------------------------ */
struct Box { double mn[3], mx[3]; };

static inline bool box_overlap(const Box &a, const Box &b)   /* AABox::in_box, src/aabb.cc:53-65 */
{
	for(int i = 0; i < 3; i++) {
		if(a.mn[i] > b.mx[i] || b.mn[i] > a.mx[i]) return false;
	}
	return true;
}

struct OctNode {
	Box box;
	std::vector<int> items;
	int child = -1;   /* index of the first of 8 consecutive children; -1 = leaf */
};

struct Octree {
	std::vector<OctNode> nodes;
	std::vector<Box> item_box;
	int max_depth = 5, max_items = 5;

	void clear() { nodes.clear(); item_box.clear(); }

	void subdivide(int ni, int lvl)
	{
		if((int)nodes[ni].items.size() <= max_items || lvl >= max_depth) return;
		Box b = nodes[ni].box;
		double c[3];
		for(int i = 0; i < 3; i++) c[i] = (b.mn[i] + b.mx[i]) * 0.5;
		Box cb[8];
		/* child layout of src/octree.inl:160-168 */
		const int lo[8][3] = {{0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1}};
		for(int k = 0; k < 8; k++) {
			for(int i = 0; i < 3; i++) {
				cb[k].mn[i] = lo[k][i] ? c[i] : b.mn[i];
				cb[k].mx[i] = lo[k][i] ? b.mx[i] : c[i];
			}
		}
		int first = (int)nodes.size();
		nodes.resize(first + 8);
		nodes[ni].child = first;
		for(int k = 0; k < 8; k++) {
			OctNode &ch = nodes[first + k];
			ch.box = cb[k];
			const std::vector<int> &pitems = nodes[ni].items;
			for(size_t j = 0; j < pitems.size(); j++) {
				if(box_overlap(item_box[pitems[j]], ch.box)) ch.items.push_back(pitems[j]);
			}
			subdivide(first + k, lvl + 1);
		}
		nodes[ni].items.clear();
		nodes[ni].items.shrink_to_fit();
	}

	void build(const std::vector<Box> &boxes, int depth, int items)
	{
		clear();
		max_depth = depth;
		max_items = items;
		item_box = boxes;
		Box bounds;
		for(int i = 0; i < 3; i++) { bounds.mn[i] = FLT_MAX; bounds.mx[i] = -FLT_MAX; }
		for(size_t k = 0; k < boxes.size(); k++) {
			for(int i = 0; i < 3; i++) {
				if(boxes[k].mn[i] < bounds.mn[i]) bounds.mn[i] = boxes[k].mn[i];
				if(boxes[k].mx[i] > bounds.mx[i]) bounds.mx[i] = boxes[k].mx[i];
			}
		}
		nodes.resize(1);
		nodes[0].box = bounds;
		nodes[0].items.resize(boxes.size());
		for(size_t k = 0; k < boxes.size(); k++) nodes[0].items[k] = (int)k;
		if((int)boxes.size() > max_items) subdivide(0, 0);
	}
};

/* ------------------------------------------------------------------ */
/* scene objects                                                         */
/* ------------------------------------------------------------------ */
enum { OBJ_SPHERE, OBJ_CYLINDER, OBJ_MESH };
enum { LT_POINT, LT_SPHERE, LT_BOX };

struct Face {
	V3d p[3], n[3], tg[3];
	double tex[3][2];
};

struct Object {
	int type = OBJ_SPHERE;
	std::string name;
	int mat = -1;
	XForm xf;
	double rad = 1.0, start = -1.0, end = 1.0;
	std::vector<Face> faces;
	Octree oct;

	/* calc_bounds: src/sphere.cc:70-77, src/cylinder.cc:125-146, src/mesh.cc:238-257 */
	Box bounds(int msec) const
	{
		Box b;
		double m[4][4];
		xf.matrix(msec, m);
		if(type == OBJ_SPHERE) {
			V3d c = xform_pt(m, V3d(0, 0, 0));
			for(int i = 0; i < 3; i++) { b.mn[i] = c[i] - rad; b.mx[i] = c[i] + rad; }
		} else if(type == OBJ_CYLINDER) {
			V3d s1 = xform_pt(m, V3d(0, start, 0)), s2 = xform_pt(m, V3d(0, end, 0));
			for(int i = 0; i < 3; i++) {
				double a0 = s1[i] - radius(), a1 = s2[i] - radius();
				double c0 = s1[i] + radius(), c1 = s2[i] + radius();
				b.mn[i] = a0 < a1 ? a0 : a1;
				b.mx[i] = c0 > c1 ? c0 : c1;
			}
		} else {
			for(int i = 0; i < 3; i++) { b.mn[i] = FLT_MAX; b.mx[i] = -FLT_MAX; }
			for(size_t f = 0; f < faces.size(); f++) {
				for(int v = 0; v < 3; v++) {
					V3d p = xform_pt(m, faces[f].p[v]);
					for(int i = 0; i < 3; i++) {
						if(p[i] < b.mn[i]) b.mn[i] = p[i];
						if(p[i] > b.mx[i]) b.mx[i] = p[i];
					}
				}
			}
		}
		return b;
	}
	double radius() const { return rad; }
};

/* projection map, src/projmap.cc */
struct ProjMap {
	int udiv = 64, vdiv = 32;
	std::vector<char> cells;
	double coverage = 0.0;
	std::vector<double> cell_area;
	double total_area = 0.0;

	ProjMap() { set_subdiv(64, 32); }

	void corner_dir(int uc, int vc, int corner, double out[3]) const
	{
		static const int offs[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
		double du = 1.0 / udiv, dv = 1.0 / vdiv;
		double u = (uc + offs[corner][0]) * du;
		double v = (vc + offs[corner][1]) * dv;
		vmc_vec_from_sph(out, u * M_PI * 2.0, v * M_PI, 1.0);
	}
	void set_subdiv(int u, int v)
	{
		udiv = u;
		vdiv = v;
		cells.assign(u * v, 0);
		cell_area.resize(u * v);
		total_area = 0.0;
		for(int i = 0; i < u * v; i++) {
			int uc = i % udiv, vc = i / udiv;
			double c[4][3];
			for(int j = 0; j < 4; j++) corner_dir(uc, vc, j, c[j]);
			V3d v0(c[0][0], c[0][1], c[0][2]), v1(c[1][0], c[1][1], c[1][2]);
			V3d v2(c[2][0], c[2][1], c[2][2]), v3(c[3][0], c[3][1], c[3][2]);
			double area = length(cross(v1 - v0, v2 - v0)) * 0.5;
			area += length(cross(v2 - v0, v3 - v0)) * 0.5;
			cell_area[i] = area;
			total_area += area;
		}
	}
	void clear() { std::fill(cells.begin(), cells.end(), 0); coverage = 0.0; }
	void set_all(bool val) { std::fill(cells.begin(), cells.end(), val ? 1 : 0); coverage = val ? 1.0 : 0.0; }
	void set_cell(int uc, int vc, bool val)
	{
		int idx = vc * udiv + uc;
		if((bool)cells[idx] != val) {
			double change = cell_area[idx] / total_area;
			coverage += val ? change : -change;
		}
		cells[idx] = val;
	}
	double get_coverage() const { return coverage < 0.0 ? 0.0 : (coverage > 1.0 ? 1.0 : coverage); }
	/* cell_from_dir (src/projmap.cc:146-160), double; indices clamped to the grid */
	void cell_from_dir(const double d[3], int *uc, int *vc) const
	{
		double theta, phi, r;
		vmc_sph_from_vec(&theta, &phi, &r, d);
		if(theta < 0.0) theta = M_PI * 2.0 + theta;
		double u = theta / (M_PI * 2.0), v = phi / M_PI;
		int a = (int)(u * udiv), b = (int)(v * vdiv);
		*uc = a < 0 ? 0 : (a >= udiv ? udiv - 1 : a);
		*vc = b < 0 ? 0 : (b >= vdiv ? vdiv - 1 : b);
	}
};

/* ::build_projmap -- src/light.cc:392-432 */
static void build_projmap(ProjMap *map, const V3d &lpos, const std::vector<Box> &boxes)
{
	for(size_t i = 0; i < boxes.size(); i++) {
		const Box &b = boxes[i];
		if(lpos.x >= b.mn[0] && lpos.y >= b.mn[1] && lpos.z >= b.mn[2] &&
				lpos.x < b.mx[0] && lpos.y < b.mx[1] && lpos.z < b.mx[2]) {
			map->set_all(true);
			return;
		}
		V3d mn(b.mn[0], b.mn[1], b.mn[2]), mx(b.mx[0], b.mx[1], b.mx[2]);
		V3d center = (mn + mx) / 2.0;
		V3d dm = mn - center;
		double rad_sq = dot(dm, dm);
		V3d v = center - lpos;
		double objdist = length(v);
		int uc, vc;
		double vv[3] = {v.x, v.y, v.z};
		map->cell_from_dir(vv, &uc, &vc);
		map->set_cell(uc, vc, true);
		int num = map->udiv * map->vdiv;
		for(int j = 0; j < num; j++) {
			uc = j % map->udiv;
			vc = j / map->udiv;
			for(int k = 0; k < 4; k++) {
				double cd[3];
				map->corner_dir(uc, vc, k, cd);
				V3d corner = V3d(cd[0], cd[1], cd[2]) * objdist;
				V3d d = (lpos + corner) - center;
				if(dot(d, d) <= rad_sq) {
					map->set_cell(uc, vc, true);
					break;
				}
			}
		}
	}
}

struct Light {
	int type = LT_POINT;
	double col[4] = {1, 1, 1, 1};
	XForm xf;
	float radius = 1.0f;
	V3d dim = V3d(1, 1, 1);
	ProjMap pm, spm;
};

struct Camera {
	int target = 0;
	XForm xf, txf;
	double vfov = M_PI / 4.0, aspect = 1.0, max_dist = RAY_MAG;
	int shutter = 0;

	/* Camera::get_matrix / TargetCamera::get_matrix (src/camera.cc:113-116, 216-234) */
	void matrix(int time, double m[4][4]) const
	{
		if(!target) {
			xf.matrix(time, m);
			return;
		}
		V3d pos = xf.position(time), targ = txf.position(time);
		V3d up(0, 1, 0);
		V3d dir = normalized(targ - pos);
		V3d right = normalized(cross(up, dir));
		up = cross(dir, right);
		double roll = txf.scaling(time).x;
		double q[4], axis[3] = {dir.x, dir.y, dir.z};
		vmc_quat_axis_angle(q, axis, roll);
		double rm[4][4];
		vmc_mat_quat(rm, q[0], q[1], q[2], q[3]);
		double u[3] = {up.x, up.y, up.z}, r[3] = {right.x, right.y, right.z};
		vmc_xform_dir(u, rm, u);
		vmc_xform_dir(r, rm, r);
		vmc_mat_identity(m);
		m[0][0] = r[0]; m[0][1] = u[0]; m[0][2] = dir.x; m[0][3] = pos.x;
		m[1][0] = r[1]; m[1][1] = u[1]; m[1][2] = dir.y; m[1][3] = pos.y;
		m[2][0] = r[2]; m[2][1] = u[2]; m[2][2] = dir.z; m[2][3] = pos.z;
	}
};

struct Scene {
	std::vector<Material> mats;
	std::vector<Object> objs;
	std::vector<Light> lights;
	Camera cam;
	bool have_cam = false;
	double env_ior = 1.0;
	double env_col[4] = {0, 0, 0, 0};
	double env_amb[4] = {0, 0, 0, 0};
	Material default_mat;
	std::vector<Tex> texs;
	Octree oct;
	double gather_dist = 0.001;
	int64_t n_tris = 0;
};

/* ------------------------------------------------------------------ */
/* scene loading (src/scene.cc:93-183 and the per-class load_xml)       */
/* ------------------------------------------------------------------ */
static bool load_object_common(Scene &sc, Object &o, const XNode &node, std::string &err)
{
	const XAttr *a;
	if((a = node.get("name"))) o.name = a->str;
	for(size_t i = 0; i < node.chld.size(); i++) {
		const XNode &c = node.chld[i];
		if(c.name == "matref") {
			if(!(a = c.get("name"))) { err = "invalid material reference in object " + o.name; return false; }
			int found = -1;
			for(size_t m = 0; m < sc.mats.size(); m++) if(sc.mats[m].name == a->str) { found = (int)m; break; }
			if(found < 0) { err = "material " + a->str + " referenced by object " + o.name + " does not exist"; return false; }
			o.mat = found;
		} else if(c.name == "xform") {
			o.xf.load_xml(c);
		}
	}
	return true;
}

/* Mesh::load_xml -- src/meshload.cc:55-157 */
static bool load_mesh(Object &o, const XNode &node, std::string &err)
{
	const XNode *mesh = 0;
	for(size_t i = 0; i < node.chld.size(); i++) if(node.chld[i].name == "mesh") { mesh = &node.chld[i]; break; }
	if(!mesh) { err = "<mesh> not found in mesh object " + o.name; return false; }
	static const char *ename[4] = {"vertex", "normal", "texcoord", "tangent"};
	struct Elem { V3d v; int id; };
	std::vector<Elem> el[4];
	bool ordered[4] = {true, true, true, true};
	int cur[4] = {0, 0, 0, 0};
	struct FRef { int vi[3], ni[3], ti[3], gi[3]; };
	std::vector<FRef> frefs;
	for(size_t i = 0; i < mesh->chld.size(); i++) {
		const XNode &c = mesh->chld[i];
		int e = -1;
		for(int k = 0; k < 4; k++) if(c.name == ename[k]) e = k;
		if(e >= 0) {
			Elem x;
			const XAttr *a;
			if((a = c.get("id")) && a->type == AT_INT) x.id = a->ival;
			else x.id = cur[e];
			if((a = c.get("val")) && a->type == AT_VEC) x.v = V3d(a->vval[0], a->vval[1], a->vval[2]);
			if(x.id != cur[e]++) ordered[e] = false;
			el[e].push_back(x);
		} else if(c.name == "face") {
			FRef f;
			memset(&f, 0, sizeof f);
			int k = 0;
			for(size_t j = 0; j < c.chld.size() && k < 3; j++) {
				const XNode &vr = c.chld[j];
				if(vr.name != "vref") continue;
				const XAttr *a;
				f.vi[k] = ((a = vr.get("vertex")) && a->type == AT_INT) ? a->ival : 0;
				f.ni[k] = ((a = vr.get("normal")) && a->type == AT_INT) ? a->ival : 0;
				f.gi[k] = ((a = vr.get("tangent")) && a->type == AT_INT) ? a->ival : 0;
				f.ti[k] = ((a = vr.get("texcoord")) && a->type == AT_INT) ? a->ival : 0;
				k++;
			}
			frefs.push_back(f);
		}
	}
	for(int e = 0; e < 4; e++) {
		if(!ordered[e]) std::stable_sort(el[e].begin(), el[e].end(), [](const Elem &a, const Elem &b) { return a.id < b.id; });
		if(!el[e].empty() && el[e].back().id != (int)el[e].size() - 1) {
			err = "error loading mesh " + o.name + ": missing vertex elements";
			return false;
		}
	}
	o.faces.resize(frefs.size());
	for(size_t i = 0; i < frefs.size(); i++) {
		Face &f = o.faces[i];
		for(int j = 0; j < 3; j++) {
			int vi = frefs[i].vi[j], ni = frefs[i].ni[j], gi = frefs[i].gi[j], ti = frefs[i].ti[j];
			if(vi < 0 || vi >= (int)el[0].size()) { err = "face vertex index out of range in " + o.name; return false; }
			f.p[j] = el[0][vi].v;
			if(el[1].empty()) f.n[j] = V3d(0, 0, 0);
			else { if(ni < 0 || ni >= (int)el[1].size()) { err = "normal index out of range"; return false; } f.n[j] = el[1][ni].v; }
			if(el[3].empty()) f.tg[j] = V3d(0, 0, 0);
			else { if(gi < 0 || gi >= (int)el[3].size()) { err = "tangent index out of range"; return false; } f.tg[j] = el[3][gi].v; }
			if(el[2].empty()) { f.tex[j][0] = f.tex[j][1] = 0.0; }
			else { if(ti < 0 || ti >= (int)el[2].size()) { err = "texcoord index out of range"; return false; } f.tex[j][0] = el[2][ti].v.x; f.tex[j][1] = el[2][ti].v.y; }
		}
	}
	return true;
}

/* Mesh::build_tree -- src/mesh.cc:210-226 (object space) */
static void build_mesh_tree(Object &o, int depth, int items)
{
	std::vector<Box> boxes(o.faces.size());
	for(size_t i = 0; i < o.faces.size(); i++) {
		Box &b = boxes[i];
		for(int k = 0; k < 3; k++) { b.mn[k] = FLT_MAX; b.mx[k] = -FLT_MAX; }
		for(int v = 0; v < 3; v++) {
			for(int k = 0; k < 3; k++) {
				double c = o.faces[i].p[v][k];
				if(c < b.mn[k]) b.mn[k] = c;
				if(c > b.mx[k]) b.mx[k] = c;
			}
		}
	}
	o.oct.build(boxes, depth, items);
}

/* find_file (src/datapath.c:57-77): "<dir>/<name>" for the directories of
 * SRAY_DATA_PATH that exist as a file.  The list parser (src/datapath.c:
 * 79-113) writes its terminator over the first ':' and then tests that same
 * byte, so only the first entry of the list is ever searched. */
static bool find_data_file(const char *name, std::string &path)
{
	const char *env = getenv("SRAY_DATA_PATH");
	if(!env || !*env) return false;
	path.assign(env, strcspn(env, ":"));
	path += "/";
	path += name;
	return access(path.c_str(), F_OK) == 0;
}

static int ppm_number(FILE *fp)
{
	int c, v = 0, any = 0;
	while((c = fgetc(fp)) != EOF) {
		if(c == '#') { while((c = fgetc(fp)) != EOF && c != '\n') {} continue; }
		if(c >= '0' && c <= '9') { v = v * 10 + (c - '0'); any = 1; }
		else if(any) break;
	}
	return any ? v : -1;
}

/* Texture::load (src/texture.cc:28-36) -> Image::load (src/img.cc:60-74):
 * the image as RGBA floats.  Binary PPM (P6, maxval <= 255), channel / 255
 * and alpha 1, is the one file format read here. */
static bool load_texture(const char *name, Tex &t)
{
	std::string path;
	if(!find_data_file(name, path)) return false;
	FILE *fp = fopen(path.c_str(), "rb");
	if(!fp) return false;
	char magic[2];
	bool ok = fread(magic, 1, 2, fp) == 2 && magic[0] == 'P' && magic[1] == '6';
	int w = ok ? ppm_number(fp) : -1, h = ok ? ppm_number(fp) : -1, maxv = ok ? ppm_number(fp) : -1;
	ok = ok && w > 0 && h > 0 && maxv > 0 && maxv <= 255 && (int64_t)w * h < ((int64_t)1 << 28);
	std::vector<unsigned char> rgb;
	if(ok) {
		rgb.resize((size_t)w * h * 3);
		ok = fread(rgb.data(), 1, rgb.size(), fp) == rgb.size();
	}
	fclose(fp);
	if(!ok) return false;
	t.xsz = w;
	t.ysz = h;
	t.pix.resize((size_t)w * h * 4);
	for(size_t i = 0; i < (size_t)w * h; i++) {
		for(int k = 0; k < 3; k++) t.pix[i * 4 + k] = rgb[i * 3 + k] / 255.0f;
		t.pix[i * 4 + 3] = 1.0f;
	}
	return true;
}

static bool load_scene(Scene &sc, const sray_opts &opt, const char *text, size_t len, std::string &err)
{
	XmlParser xp;
	XNode root;
	if(!xp.parse(text, len, root)) { err = "xml: " + xp.err; return false; }
	sc = Scene();
	for(size_t i = 0; i < root.chld.size(); i++) {
		const XNode &n = root.chld[i];
		if(n.name != "material") continue;
		Material m;
		const XAttr *a;
		if(!(a = n.get("name"))) { err = "invalid material: name attribute not found"; return false; }
		m.name = a->str;
		if((a = n.get("shader"))) m.phong = a->str == "phong";
		for(size_t j = 0; j < n.chld.size(); j++) {
			const XNode &c = n.chld[j];
			if(c.name != "mattr") continue;
			const XAttr *an = c.get("name"), *av = c.get("value");
			if(!an || !av) continue;
			double col[4];
			if(av->type == AT_VEC) { col[0] = av->vval[0]; col[1] = av->vval[1]; col[2] = av->vval[2]; }
			else if(av->type == AT_FLT || av->type == AT_INT) col[0] = col[1] = col[2] = av->fval;
			else continue;
			col[3] = 1.0;
			/* a "map" loads a texture of its own; one that fails to load
			 * leaves the attribute untextured (src/material.cc:64-72) */
			int tex = -1;
			if((a = c.get("map"))) {
				Tex t;
				if(load_texture(a->str.c_str(), t)) {
					tex = (int)sc.texs.size();
					sc.texs.push_back(std::move(t));
				} else {
					fprintf(stderr, "failed to load texture: %s\n", a->str.c_str());
				}
			}
			m.set(an->str.c_str(), col[0], col[1], col[2], col[3], tex);
		}
		sc.mats.push_back(m);
	}
	for(size_t i = 0; i < root.chld.size(); i++) {
		const XNode &n = root.chld[i];
		const XAttr *a;
		if(n.name == "env") {
			if((a = n.get("ambient"))) {
				if(a->type == AT_VEC) { sc.env_amb[0] = a->vval[0]; sc.env_amb[1] = a->vval[1]; sc.env_amb[2] = a->vval[2]; sc.env_amb[3] = 1.0; }
				else if(a->type == AT_INT || a->type == AT_FLT) { sc.env_amb[0] = sc.env_amb[1] = sc.env_amb[2] = a->fval; sc.env_amb[3] = 1.0; }
			}
			if((a = n.get("bgcolor")) && a->type == AT_VEC) {
				sc.env_col[0] = a->vval[0]; sc.env_col[1] = a->vval[1]; sc.env_col[2] = a->vval[2]; sc.env_col[3] = 1.0;
			}
			if((a = n.get("ior")) && a->type == AT_FLT) sc.env_ior = a->fval;
		} else if(n.name == "object") {
			if(!(a = n.get("type"))) { err = "invalid object: no type attribute."; return false; }
			Object o;
			if(a->str == "sphere") o.type = OBJ_SPHERE;
			else if(a->str == "cylinder") o.type = OBJ_CYLINDER;
			else if(a->str == "mesh") o.type = OBJ_MESH;
			else { err = "invalid object: unknown type: " + a->str; return false; }
			if(!load_object_common(sc, o, n, err)) return false;
			if(o.type == OBJ_SPHERE) {
				bool res = false;
				for(size_t j = 0; j < n.chld.size(); j++) {
					if(n.chld[j].name == "sphere") {
						if((a = n.chld[j].get("rad"))) o.rad = a->fval;
						res = true;
					}
				}
				if(!res) { err = "sphere object without <sphere>"; return false; }
			} else if(o.type == OBJ_CYLINDER) {
				bool res = false;
				for(size_t j = 0; j < n.chld.size(); j++) {
					if(n.chld[j].name == "cylinder") {
						if((a = n.chld[j].get("rad"))) o.rad = a->fval;
						if((a = n.chld[j].get("start"))) o.start = a->fval;
						if((a = n.chld[j].get("end"))) o.end = a->fval;
						res = true;
					}
				}
				if(!res) { err = "cylinder object without <cylinder>"; return false; }
			} else {
				if(!load_mesh(o, n, err)) return false;
				build_mesh_tree(o, opt.meshoct_max_depth, opt.meshoct_max_items);
				sc.n_tris += (int64_t)o.faces.size();
			}
			sc.objs.push_back(o);
		} else if(n.name == "light") {
			if(!(a = n.get("type"))) { err = "invalid light: no type attribute."; return false; }
			Light l;
			if(a->str == "point") l.type = LT_POINT;
			else if(a->str == "sphere") l.type = LT_SPHERE;
			else if(a->str == "box") l.type = LT_BOX;
			else { err = "invalid light: unknown type: " + a->str; return false; }
			if((a = n.get("color"))) {
				if(a->type == AT_VEC) { l.col[0] = a->vval[0]; l.col[1] = a->vval[1]; l.col[2] = a->vval[2]; l.col[3] = 1.0; }
				else if(a->type == AT_INT || a->type == AT_FLT) { l.col[0] = l.col[1] = l.col[2] = a->fval; l.col[3] = 1.0; }
			}
			for(size_t j = 0; j < n.chld.size(); j++) {
				const XNode &c = n.chld[j];
				if(c.name == "xform") l.xf.load_xml(c);
				else if(c.name == "sphere" && l.type == LT_SPHERE) {
					if(!(a = c.get("rad"))) { err = "sphere light without rad"; return false; }
					l.radius = (float)a->fval;
				} else if(c.name == "aabox" && l.type == LT_BOX) {
					const XAttr *mn = c.get("min"), *mx = c.get("max");
					if(!mn || mn->type != AT_VEC || !mx || mx->type != AT_VEC) { err = "bad aabox"; return false; }
					l.dim = V3d(mx->vval[0] - mn->vval[0], mx->vval[1] - mn->vval[1], mx->vval[2] - mn->vval[2]);
				}
			}
			sc.lights.push_back(l);
		} else if(n.name == "camera") {
			if(!(a = n.get("type"))) { err = "invalid camera: no type attribute."; return false; }
			Camera c;
			c.aspect = (double)opt.width / (double)opt.height;
			c.shutter = opt.shutter;
			if(a->str == "free") c.target = 0;
			else if(a->str == "target") {
				c.target = 1;
				c.xf.ptrack.set_key(0, V3d(0, 5, 10));
				c.txf.ptrack.set_key(0, V3d(0, 0, 0));
				c.txf.strack.set_key(0, V3d(0, 0, 0));
			} else { err = "invalid camera: unknown type: " + a->str; return false; }
			if((a = n.get("shutter"))) c.shutter = (int)a->fval;
			if((a = n.get("fov")) && (a->type == AT_FLT || a->type == AT_INT)) c.vfov = (a->fval * M_PI) / 180.0;
			bool have_target = false;
			for(size_t j = 0; j < n.chld.size(); j++) {
				const XNode &ch = n.chld[j];
				if(ch.name == "xform") c.xf.load_xml(ch);
			}
			if(c.target) {
				for(size_t j = 0; j < n.chld.size(); j++) {
					const XNode &ch = n.chld[j];
					if(ch.name == "target") {
						have_target = true;
						for(size_t k = 0; k < ch.chld.size(); k++) if(ch.chld[k].name == "xform") c.txf.load_xml(ch.chld[k]);
						break;
					}
				}
				if(!have_target) { err = "failed to load target camera, no <target> child"; return false; }
			}
			if(!sc.have_cam) {
				sc.cam = c;
				sc.have_cam = true;
			}
		}
	}
	if(!sc.have_cam) {
		sc.cam = Camera();
		sc.cam.aspect = (double)opt.width / (double)opt.height;
		sc.cam.shutter = opt.shutter;
		sc.have_cam = true;
	}
	return true;
}

/* Scene::build_tree -- src/scene.cc:353-390 */
static void build_scene_tree(Scene &sc, const sray_opts &opt, int t0, int t1)
{
	std::vector<Box> boxes(sc.objs.size());
	for(size_t i = 0; i < sc.objs.size(); i++) {
		Box s = sc.objs[i].bounds(t0), e = sc.objs[i].bounds(t1);
		for(int k = 0; k < 3; k++) {
			boxes[i].mn[k] = s.mn[k] < e.mn[k] ? s.mn[k] : e.mn[k];
			boxes[i].mx[k] = s.mx[k] > e.mx[k] ? s.mx[k] : e.mx[k];
		}
	}
	sc.oct.build(boxes, opt.scnoct_max_depth, opt.scnoct_max_items);
	const Box &rb = sc.oct.nodes[0].box;
	V3d d(rb.mx[0] - rb.mn[0], rb.mx[1] - rb.mn[1], rb.mx[2] - rb.mn[2]);
	sc.gather_dist = length(d) * opt.gather_dist;
}

/* ------------------------------------------------------------------ */
/* precision-specific frame data and tracing                            */
/* ------------------------------------------------------------------ */
template <class R> struct Ray {
	V3<R> o, d;
	int time = 0;
	int iter = 0;
	R energy = (R)1;
	R ior = (R)1;
	R stack[4];
	int sp = 0;

	/* Ray::enter / leave / calc_ior (libvmath ray.cc), as used by
	 * src/shader.cc:212,244-267 and src/scene.cc:601-634 */
	void enter(R n) { ior = n; if(sp < 4) stack[sp++] = n; }
	void leave()
	{
		if(sp == 0) return;
		sp--;
		ior = sp ? stack[sp - 1] : (R)1;
	}
	R calc_ior(bool entering, R mat_ior) const
	{
		R from = ior;
		if(entering) return from / mat_ior;
		Ray t = *this;
		t.leave();
		return from / t.ior;
	}
};

template <class R> struct SurfPoint {
	R dist;
	V3<R> pos, normal, tangent;
	V3<R> gn;         /* geometric normal (world space, unit): where float light samples start */
	R tex[2];
};

template <class R> struct Photon {
	V3<R> p;          /* stored position, full precision */
	float pos[3];     /* position as the kd-tree holds it (kd_insert3f rounds to float) */
	V3<R> dir, norm;
	V4<R> col;
	int type;
};
enum { DIRECT_PHOTON, CAUST_PHOTON, GI_PHOTON };

struct Counters {
	int64_t rays = 0, nodes = 0, prims = 0, shadow = 0, gathers = 0;
};

template <class R> static inline R maxr(R a, R b) { return a > b ? a : b; }
#define SHADOW_OFFSET 3.814697265625e-06   /* 2^-18 */
template <class R> static inline R powr(R a, R b);
template <> inline float powr(float a, float b) { return powf(a, b); }
template <> inline double powr(double a, double b) { return pow(a, b); }
template <class R> static inline R fabsr(R a) { return a < (R)0 ? -a : a; }

struct FrameBase {
	virtual ~FrameBase() {}
	virtual int render_rows(int y0, int y1, float *fb, int nthreads, int quirk, int *spp) = 0;
	virtual int render_row_list(int n, const int *rows, float *fb, int nthreads, int quirk, int *spp) = 0;
	virtual int primary_hits(int *obj, int *prim, double *t, unsigned char *tie) = 0;
	virtual int cast_rays(int n, const double *o, const double *d, const int *tm, int *obj, int *prim, double *t, unsigned char *tie) = 0;
	virtual int photons(int which, float *out, int cap) = 0;
	virtual void photon_counts(int *c, int *g) = 0;
	virtual int gather(int which, int n, const double *pos, const double *norm, double *out) = 0;
	Counters ctr;
	std::string err;
	/* pixel index added to every pixel's stream key (a job of a batch keys
	 * its pixels by their place in the batch's pixel space) */
	uint32_t pix_base = 0;
	/* wall time of the phases of the last prepare, ms: scene tree and
	 * frame tables, projection maps, photon tracing and map build */
	double ms_build = 0.0, ms_proj = 0.0, ms_photons = 0.0;
};

template <class R> struct Frame : FrameBase {
	typedef V3<R> V;
	typedef V4<R> C;

	const Scene &sc;
	const sray_opts opt;
	int rng_mode;
	long msec;
	int t0, t1;
	int tlo, thi;                       /* time table range */

	struct ObjR { int type, mat; R rad, start, end; };
	std::vector<ObjR> objs;
	std::vector<R> xf;                  /* per object per time: fwd 12, inv 12, invT 9 */
	int nt;
	struct TriR { V p[3]; V vn[3], vt[3]; R tex[3][2]; };
	std::vector<std::vector<TriR> > tris;
	struct NodeR { R mn[3], mx[3]; };
	std::vector<std::vector<NodeR> > mesh_boxes;
	std::vector<NodeR> scene_boxes;
	/* attributes that can carry a texture, in MatR::tex order */
	enum { TA_DIFFUSE, TA_SPECULAR, TA_SHININESS, TA_REFLECT, TA_REFRACT, TA_IOR, TA_NORMAL, TA_COUNT };
	struct MatR {
		int phong;
		C kd, ks;
		R shin, refl, refr, ior;
		bool have_spec, have_shin, have_normal;
		int tex[TA_COUNT];               /* texture per attribute, -1 = none */
		R scol[TA_COUNT];                /* the attribute colour's x (textured scalars, bump scale) */
		bool textured;
	};
	std::vector<MatR> mats;
	MatR defmat;
	struct LightR { int type; C col; R radius; V dim; R box_m[12]; };
	std::vector<LightR> lights;
	std::vector<R> light_pos;           /* per light per time: xyz */
	std::vector<R> cam_m;               /* per time: 12 */
	R cam_f, cam_xsz, cam_ysz, cam_maxd;
	C env_col, env_amb;
	R eps, xsmall;
	R gather_r;
	double gather_d;
	std::vector<Photon<R> > caust, gi;
	struct Grid {
		double cell = 1.0;
		double org[3] = {0, 0, 0};
		std::vector<std::pair<uint64_t, int> > keys;
		void build(const std::vector<Photon<R> > &ph, double cellsz)
		{
			cell = cellsz > 0.0 ? cellsz : 1.0;
			keys.resize(ph.size());
			org[0] = org[1] = org[2] = 0.0;
			for(size_t i = 0; i < ph.size(); i++) keys[i] = std::make_pair(key(ph[i].pos[0], ph[i].pos[1], ph[i].pos[2]), (int)i);
			std::sort(keys.begin(), keys.end());
		}
		int64_t cidx(double v) const { return (int64_t)floor(v / cell); }
		static uint64_t pack(int64_t x, int64_t y, int64_t z)
		{
			return ((uint64_t)(x & 0x1fffff) << 42) | ((uint64_t)(y & 0x1fffff) << 21) | (uint64_t)(z & 0x1fffff);
		}
		uint64_t key(double x, double y, double z) const { return pack(cidx(x), cidx(y), cidx(z)); }
	};
	Grid caust_grid, gi_grid;

	Frame(const Scene &s, const sray_opts &o, int mode, long ms) : sc(s), opt(o), rng_mode(mode), msec(ms) {}

	void mat_r(const double m[4][4], R *out) const
	{
		for(int i = 0; i < 3; i++) for(int j = 0; j < 4; j++) out[i * 4 + j] = (R)m[i][j];
	}

	int tindex(int time) const
	{
		if(time < tlo || time > thi) return -1;
		return time - tlo;
	}

	void setup(int time_lo, int time_hi)
	{
		tlo = time_lo;
		thi = time_hi;
		nt = thi - tlo + 1;
		eps = (R)VMC_ERROR_MARGIN;
		xsmall = (R)VMC_XSMALL_NUMBER;
		objs.resize(sc.objs.size());
		xf.assign(sc.objs.size() * nt * 33, (R)0);
		tris.resize(sc.objs.size());
		mesh_boxes.resize(sc.objs.size());
		for(size_t i = 0; i < sc.objs.size(); i++) {
			const Object &o = sc.objs[i];
			objs[i].type = o.type;
			objs[i].mat = o.mat;
			objs[i].rad = (R)o.rad;
			objs[i].start = (R)o.start;
			objs[i].end = (R)o.end;
			for(int t = 0; t < nt; t++) {
				double m[4][4], inv[4][4], it[4][4];
				o.xf.matrix(tlo + t, m);
				vmc_mat_inverse(inv, m);
				vmc_mat_transpose(it, inv);
				R *dst = &xf[(i * nt + t) * 33];
				mat_r(m, dst);
				mat_r(inv, dst + 12);
				for(int r = 0; r < 3; r++) for(int c = 0; c < 3; c++) dst[24 + r * 3 + c] = (R)it[r][c];
			}
			if(o.type == OBJ_MESH) {
				tris[i].resize(o.faces.size());
				for(size_t f = 0; f < o.faces.size(); f++) {
					TriR &t = tris[i][f];
					for(int v = 0; v < 3; v++) {
						t.p[v] = V((R)o.faces[f].p[v].x, (R)o.faces[f].p[v].y, (R)o.faces[f].p[v].z);
						t.vn[v] = V((R)o.faces[f].n[v].x, (R)o.faces[f].n[v].y, (R)o.faces[f].n[v].z);
						t.vt[v] = V((R)o.faces[f].tg[v].x, (R)o.faces[f].tg[v].y, (R)o.faces[f].tg[v].z);
						t.tex[v][0] = (R)o.faces[f].tex[v][0];
						t.tex[v][1] = (R)o.faces[f].tex[v][1];
					}
				}
				mesh_boxes[i].resize(o.oct.nodes.size());
				for(size_t n = 0; n < o.oct.nodes.size(); n++) {
					for(int k = 0; k < 3; k++) {
						mesh_boxes[i][n].mn[k] = (R)o.oct.nodes[n].box.mn[k];
						mesh_boxes[i][n].mx[k] = (R)o.oct.nodes[n].box.mx[k];
					}
				}
			}
		}
		scene_boxes.resize(sc.oct.nodes.size());
		for(size_t n = 0; n < sc.oct.nodes.size(); n++) {
			for(int k = 0; k < 3; k++) {
				scene_boxes[n].mn[k] = (R)sc.oct.nodes[n].box.mn[k];
				scene_boxes[n].mx[k] = (R)sc.oct.nodes[n].box.mx[k];
			}
		}
		mats.resize(sc.mats.size());
		for(size_t i = 0; i < sc.mats.size(); i++) mats[i] = mat_of(sc.mats[i]);
		defmat = mat_of(sc.default_mat);
		lights.resize(sc.lights.size());
		light_pos.resize(sc.lights.size() * nt * 3);
		for(size_t i = 0; i < sc.lights.size(); i++) {
			const Light &l = sc.lights[i];
			lights[i].type = l.type;
			lights[i].col = C((R)l.col[0], (R)l.col[1], (R)l.col[2], (R)l.col[3]);
			lights[i].radius = (R)l.radius;
			lights[i].dim = V((R)l.dim.x, (R)l.dim.y, (R)l.dim.z);
			double m0[4][4];
			l.xf.matrix(0, m0);
			mat_r(m0, lights[i].box_m);
			for(int t = 0; t < nt; t++) {
				V3d p = l.xf.position(tlo + t);
				light_pos[(i * nt + t) * 3 + 0] = (R)p.x;
				light_pos[(i * nt + t) * 3 + 1] = (R)p.y;
				light_pos[(i * nt + t) * 3 + 2] = (R)p.z;
			}
		}
		cam_m.resize(nt * 12);
		for(int t = 0; t < nt; t++) {
			double m[4][4];
			sc.cam.matrix(tlo + t, m);
			mat_r(m, &cam_m[t * 12]);
		}
		cam_f = (R)(1.0 / tan(0.5 * sc.cam.vfov));
		cam_xsz = (R)(sc.cam.aspect * 2.0);
		cam_ysz = (R)2.0;
		cam_maxd = (R)sc.cam.max_dist;
		env_col = C((R)sc.env_col[0], (R)sc.env_col[1], (R)sc.env_col[2], (R)sc.env_col[3]);
		env_amb = C((R)sc.env_amb[0], (R)sc.env_amb[1], (R)sc.env_amb[2], (R)sc.env_amb[3]);
		gather_d = sc.gather_dist;
		gather_r = (R)sc.gather_dist;
	}

	MatR mat_of(const Material &m) const
	{
		MatR r;
		r.phong = m.phong;
		const double *c = m.get("diffuse");
		r.kd = C((R)c[0], (R)c[1], (R)c[2], (R)c[3]);
		c = m.get("specular");
		r.ks = C((R)c[0], (R)c[1], (R)c[2], (R)c[3]);
		r.have_spec = m.have("specular");
		r.shin = (R)(float)m.get("shininess")[0];
		r.have_shin = m.have("shininess");
		r.refl = (R)(float)m.get("reflect")[0];
		r.refr = (R)(float)m.get("refract")[0];
		r.ior = (R)(float)m.get("ior")[0];
		r.have_normal = m.have("normal");
		static const char *names[TA_COUNT] = {"diffuse", "specular", "shininess", "reflect", "refract", "ior", "normal"};
		r.textured = false;
		for(int k = 0; k < TA_COUNT; k++) {
			r.tex[k] = m.tex_of(names[k]);
			r.scol[k] = (R)m.get(names[k])[0];
			if(r.tex[k] >= 0) r.textured = true;
		}
		return r;
	}

	/* ------------------ textures ------------------ */
	/* Texture::lookup (src/texture.cc:60-83) with the texture's identity
	 * transform: texel (int)(tc * size), the average of it and its four
	 * edge neighbours, each wrapped by Texture::get_texel's repeat mode
	 * (src/texture.cc:85-101). */
	C tex_lookup(int ti, const R tc[2]) const
	{
		const Tex &t = sc.texs[ti];
		int tx = (int)(tc[0] * (R)t.xsz);
		int ty = (int)(tc[1] * (R)t.ysz);
		static const int off[5][2] = {{0, 0}, {1, 0}, {-1, 0}, {0, 1}, {0, -1}};
		C sum;
		for(int i = 0; i < 5; i++) {
			int x = (tx + off[i][0]) % t.xsz, y = (ty + off[i][1]) % t.ysz;
			if(x < 0) x += t.xsz;
			if(y < 0) y += t.ysz;
			const float *p = &t.pix[((size_t)y * t.xsz + x) * 4];
			C c((R)p[0], (R)p[1], (R)p[2], (R)p[3]);
			sum = i ? sum + c : c;
		}
		return sum / (R)5;
	}
	/* MatAttrib::get_color / get_value (src/material.inl:18-29) */
	C attr_color(const MatR &m, int a, const C &col, const R tc[2]) const
	{
		return m.tex[a] >= 0 ? tex_lookup(m.tex[a], tc) * col : col;
	}
	R attr_value(const MatR &m, int a, R val, const R tc[2]) const
	{
		return m.tex[a] >= 0 ? (R)(float)(tex_lookup(m.tex[a], tc).x * m.scol[a]) : val;
	}
	/* get_bump_normal (src/shader.cc:296-318): the unflipped surface normal,
	 * tilted by the normal map's texel in the frame (tangent, normal x
	 * tangent, normal) when the attribute has a texture */
	V bump_normal(const MatR &m, const SurfPoint<R> &sp) const
	{
		V normal = sp.normal;
		if(m.tex[TA_NORMAL] < 0) return normal;
		C nc = tex_lookup(m.tex[TA_NORMAL], sp.tex);
		V n(nc.x * (R)2 - (R)1, nc.y * (R)2 - (R)1, nc.z * (R)2 - (R)1);
		n.x = n.x * m.scol[TA_NORMAL];
		n.y = n.y * m.scol[TA_NORMAL];
		n = normalized(n);
		V bitan = cross(normal, sp.tangent);
		return V(sp.tangent.x * n.x + bitan.x * n.y + normal.x * n.z,
				sp.tangent.y * n.x + bitan.y * n.y + normal.y * n.z,
				sp.tangent.z * n.x + bitan.z * n.y + normal.z * n.z);
	}

	const MatR &mat_for(int obj) const
	{
		int m = objs[obj].mat;
		return m >= 0 ? mats[m] : defmat;
	}

	/* ------------------ random draws ------------------ */
	R frand(sray_rng *s, R range) const;
	V sphrand(sray_rng *s, R rad) const;

	/* ------------------ intersection ------------------ */
	/* AABox::intersect (src/aabb.cc:81-125) */
	bool box_hit(const NodeR &b, const Ray<R> &ray) const
	{
		const R *bb[2] = {b.mn, b.mx};
		int xs = ray.d.x < (R)0;
		R idx = (R)1 / ray.d.x;
		R tmin = (bb[xs][0] - ray.o.x) * idx;
		R tmax = (bb[1 - xs][0] - ray.o.x) * idx;
		int ys = ray.d.y < (R)0;
		R idy = (R)1 / ray.d.y;
		R tymin = (bb[ys][1] - ray.o.y) * idy;
		R tymax = (bb[1 - ys][1] - ray.o.y) * idy;
		if((tmin > tymax) || (tymin > tmax)) return false;
		if(tymin > tmin) tmin = tymin;
		if(tymax < tmax) tmax = tymax;
		int zs = ray.d.z < (R)0;
		R idz = (R)1 / ray.d.z;
		R tzmin = (bb[zs][2] - ray.o.z) * idz;
		R tzmax = (bb[1 - zs][2] - ray.o.z) * idz;
		if((tmin > tzmax) || (tzmin > tmax)) return false;
		if(tzmin > tmin) tmin = tzmin;
		if(tzmax < tmax) tmax = tzmax;
		return (tmin < (R)1) && (tmax > (R)0);
	}

	/* Triangle::intersect (src/mesh.cc:117-165) */
	bool tri_hit(const TriR &tr, const Ray<R> &ray, SurfPoint<R> *sp) const
	{
		V v1 = tr.p[1] - tr.p[0];
		V v2 = tr.p[2] - tr.p[0];
		V normal = cross(v1, v2);
		R ndd = dot(normal, ray.d);
		if(fabsr(ndd) < eps) return false;
		V vo = ray.o - tr.p[0];
		R t = -dot(normal, vo) / ndd;
		if(t < eps || t > (R)1) return false;
		V pos = ray.o + ray.d * t;
		for(int i = 0; i < 3; i++) {
			V test = cross(tr.p[(i + 1) % 3] - tr.p[i], pos - tr.p[i]);
			if(!(dot(test, normal) >= (R)0)) return false;
		}
		if(sp) {
			sp->dist = t;
			sp->pos = pos;
			V n, tg;
			R tc[2];
			interp_face(tr, pos, normal, &n, &tg, tc);
			sp->tex[0] = tc[0];
			sp->tex[1] = tc[1];
			sp->normal = dot(n, n) < xsmall ? normal : n;
			sp->tangent = tg;
			sp->gn = normal;
		}
		return true;
	}

	/* The patch inversion's discriminant.  Where the hit lies on the patch's
	 * fold the exact value is ~0; float rounding can make it negative, and
	 * the reference's sqrt would give NaN (a NaN normal).  Float clamps it
	 * to 0 (the GPU does the same); double keeps the reference's sqrt. */
	static R root_disc(R d)
	{
		if(sizeof(R) == 4) d = d > (R)0 ? d : (R)0;
		return rsqrt_<R>(d);
	}

	/* interp_face (src/mesh.cc:321-445): bilinear-patch inversion after Haines */
	void interp_face(const TriR &tri, const V &ispos, const V &normal, V *onorm, V *otang, R *otex) const
	{
		V p00 = tri.p[0], p10 = tri.p[1], p01 = tri.p[2], p11 = tri.p[2];
		V pa = (p00 - p10) + (p11 - p01);
		V pb = p10 - p00;
		V pc = p01 - p00;
		V pd = p00;
		V na = cross(pa, normal), nb = cross(pb, normal), nc = cross(pc, normal);
		R du0 = dot(nc, pd);
		R du1 = dot(na, pd) + dot(nc, pb);
		R du2 = dot(na, pb);
		R dv0 = dot(nb, pd);
		R dv1 = dot(na, pd) + dot(nb, pc);
		R dv2 = dot(na, pc);
		R rx, ry;
		if(fabsr(du2) <= xsmall) {
			R divisor = du1 - dot(na, ispos);
			rx = fabsr(divisor) > xsmall ? ((dot(nc, ispos) - du0) / divisor) : (R)0;
		} else {
			V qux = na / ((R)2 * du2);
			V quy = -nc / du2;
			R dux = -du1 / ((R)2 * du2);
			R duy = du0 / du2;
			R ka = dux + dot(qux, ispos);
			R kb = duy + dot(quy, ispos);
			R sq = root_disc(ka * ka - kb);
			R u0 = ka - sq;
			R u1 = ka + sq;
			rx = (u0 < (R)0 || u0 > (R)1) ? u1 : u0;
		}
		if(fabsr(dv2) <= xsmall) {
			R divisor = dv1 - dot(na, ispos);
			ry = fabsr(divisor) > xsmall ? ((dot(nb, ispos) - dv0) / divisor) : (R)0;
		} else {
			V qvx = na / ((R)2 * dv2);
			V qvy = -nb / dv2;
			R dvx = -dv1 / ((R)2 * dv2);
			R dvy = dv0 / dv2;
			R ka = dvx + dot(qvx, ispos);
			R kb = dvy + dot(qvy, ispos);
			R sq = root_disc(ka * ka - kb);
			R v0 = ka - sq;
			R v1 = ka + sq;
			ry = (v0 < (R)0 || v0 > (R)1) ? v1 : v0;
		}
#define OLERP(a, b, t) ((a) + ((b) - (a)) * (t))
		for(int k = 0; k < 2; k++) {
			R s0 = OLERP(tri.tex[0][k], tri.tex[2][k], ry);
			R s1 = OLERP(tri.tex[1][k], tri.tex[2][k], ry);
			otex[k] = OLERP(s0, s1, rx);
		}
		for(int k = 0; k < 3; k++) {
			R n0 = OLERP(tri.vn[0][k], tri.vn[2][k], ry);
			R n1 = OLERP(tri.vn[1][k], tri.vn[2][k], ry);
			(*onorm)[k] = OLERP(n0, n1, rx);
			R g0 = OLERP(tri.vt[0][k], tri.vt[2][k], ry);
			R g1 = OLERP(tri.vt[1][k], tri.vt[2][k], ry);
			(*otang)[k] = OLERP(g0, g1, rx);
		}
#undef OLERP
	}

	const R *xfm(int obj, int time) const
	{
		int ti = tindex(time);
		if(ti < 0) ti = time < tlo ? 0 : nt - 1;
		return &xf[(obj * nt + ti) * 33];
	}
	static V mul_pt(const R *m, const V &p)
	{
		return V(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
				m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
				m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
	}
	static V mul_dir(const R *m, const V &p)
	{
		return V(m[0] * p.x + m[1] * p.y + m[2] * p.z,
				m[4] * p.x + m[5] * p.y + m[6] * p.z,
				m[8] * p.x + m[9] * p.y + m[10] * p.z);
	}
	static V mul_n(const R *m, const V &p)   /* 3x3 */
	{
		return V(m[0] * p.x + m[1] * p.y + m[2] * p.z,
				m[3] * p.x + m[4] * p.y + m[5] * p.z,
				m[6] * p.x + m[7] * p.y + m[8] * p.z);
	}

	/* mesh octree closest hit, src/octree.inl:201-241 (all children, in order) */
	void mesh_rec(int obj, int ni, const Ray<R> &ray, SurfPoint<R> &best, int &bprim, bool &tie, bool &found, Counters &c) const
	{
		const Object &o = sc.objs[obj];
		c.nodes++;
		if(!box_hit(mesh_boxes[obj][ni], ray)) return;
		const OctNode &n = o.oct.nodes[ni];
		if(!n.items.empty()) {
			for(size_t k = 0; k < n.items.size(); k++) {
				SurfPoint<R> pt;
				c.prims++;
				int f = n.items[k];
				if(tri_hit(tris[obj][f], ray, &pt)) {
					if(!found || pt.dist < best.dist) {
						tie = false;
						best = pt;
						bprim = f;
						found = true;
					} else if(pt.dist == best.dist && f != bprim) {
						tie = true;
					}
				}
			}
		} else if(n.child >= 0) {
			for(int k = 0; k < 8; k++) mesh_rec(obj, n.child + k, ray, best, bprim, tie, found, c);
		}
	}

	/* Object::intersect: Sphere (src/sphere.cc:85-131), Cylinder (src/cylinder.cc:125-185),
	 * Mesh (src/mesh.cc:252-308).  Returns the world-space surface point. */
	bool obj_hit(int oi, const Ray<R> &wray, SurfPoint<R> *sp, int *prim, bool *tie, Counters &c) const
	{
		const ObjR &o = objs[oi];
		const R *m = xfm(oi, wray.time);
		const R *inv = m + 12, *it = m + 24;
		Ray<R> ray = wray;
		ray.o = mul_pt(inv, wray.o);
		ray.d = mul_dir(inv, wray.d);
		*prim = 0;
		*tie = false;
		if(o.type == OBJ_SPHERE) {
			c.prims++;
			R t1, t2;
			if(sizeof(R) == 4) {
				/* float: the roots in a form without cancellation (the
				 * discriminant from the ray's closest approach to the centre,
				 * the near root as c / q), as the GPU computes them */
				R a = dot(ray.d, ray.d);
				R bh = dot(ray.o, ray.d);
				V pp = ray.o - ray.d * (bh / a);
				R dh = o.rad * o.rad - dot(pp, pp);
				if(dh < (R)0) return false;
				R sq = std::sqrt(dh * a);
				R cc = dot(ray.o, ray.o) - o.rad * o.rad;
				R q = -(bh + (bh < (R)0 ? -sq : sq));
				R ta = q / a, tb = q != (R)0 ? cc / q : ta;
				t1 = ta > tb ? ta : tb;
				t2 = ta > tb ? tb : ta;
			} else {
			R a = dot(ray.d, ray.d);
			R b = (R)2 * ray.d.x * ray.o.x + (R)2 * ray.d.y * ray.o.y + (R)2 * ray.d.z * ray.o.z;
			R cc = dot(ray.o, ray.o) - o.rad * o.rad;
			R d = b * b - (R)4 * a * cc;
			if(d < (R)0) return false;
			R sq = rsqrt_<R>(d);
			t1 = (-b + sq) / ((R)2 * a);
			t2 = (-b - sq) / ((R)2 * a);
			}
			if((t1 < eps && t2 < eps) || (t1 > (R)1 && t2 > (R)1)) return false;
			if(t1 < eps) t1 = t2;
			if(t2 < eps) t2 = t1;
			sp->dist = t1 < t2 ? t1 : t2;
			sp->pos = ray.o + ray.d * sp->dist;
			sp->normal = sp->pos / o.rad;
			sp->tangent = cross(V(0, 1, 0), sp->normal);
			sph_tex(sp->pos, sp->tex, false);
			sp->pos = mul_pt(m, sp->pos);
			sp->normal = mul_n(it, sp->normal);
			sp->gn = normalized(sp->normal);
			sp->tangent = mul_n(it, sp->tangent);
			return true;
		}
		if(o.type == OBJ_CYLINDER) {
			c.prims++;
			R t1, t2;
			R a = ray.d.x * ray.d.x + ray.d.z * ray.d.z;
			if(sizeof(R) == 4 && a > (R)0) {
				R bh = ray.d.x * ray.o.x + ray.d.z * ray.o.z;
				R px = ray.o.x - ray.d.x * (bh / a), pz = ray.o.z - ray.d.z * (bh / a);
				R dh = o.rad * o.rad - (px * px + pz * pz);
				if(dh < (R)0) return false;
				R sq = std::sqrt(dh * a);
				R cc = ray.o.x * ray.o.x + ray.o.z * ray.o.z - o.rad * o.rad;
				R q = -(bh + (bh < (R)0 ? -sq : sq));
				R ta = q / a, tb = q != (R)0 ? cc / q : ta;
				t1 = ta > tb ? ta : tb;
				t2 = ta > tb ? tb : ta;
			} else {
			R b = (R)2 * ray.d.x * ray.o.x + (R)2 * ray.d.z * ray.o.z;
			R cc = ray.o.x * ray.o.x + ray.o.z * ray.o.z - o.rad * o.rad;
			R d = b * b - (R)4 * a * cc;
			if(d < (R)0) return false;
			R sq = rsqrt_<R>(d);
			t1 = (-b + sq) / ((R)2 * a);
			t2 = (-b - sq) / ((R)2 * a);
			}
			if((t1 < eps && t2 < eps) || (t1 > (R)1 && t2 > (R)1)) return false;
			V p1 = ray.o + ray.d * t1;
			V p2 = ray.o + ray.d * t2;
			bool v0 = true, v1 = true;
			if(t1 < eps || p1.y < o.start || p1.y >= o.end) { v0 = false; t1 = t2; }
			if(t2 < eps || p2.y < o.start || p2.y >= o.end) { v1 = false; t2 = t1; }
			if(!v0 && !v1) return false;
			sp->dist = t1 < t2 ? t1 : t2;
			sp->pos = ray.o + ray.d * sp->dist;
			sp->normal = (V((R)1, (R)0, (R)1) * sp->pos) / o.rad;
			sp->tangent = cross(V(0, 1, 0), sp->normal);
			sph_tex(sp->pos, sp->tex, true);
			sp->pos = mul_pt(m, sp->pos);
			sp->normal = mul_n(it, sp->normal);
			sp->gn = normalized(sp->normal);
			sp->tangent = mul_n(it, sp->tangent);
			return true;
		}
		/* mesh */
		const Object &ob = sc.objs[oi];
		if(ob.oct.nodes.empty()) return false;
		SurfPoint<R> best;
		best.dist = (R)DBL_MAX;
		int bprim = -1;
		bool found = false, t = false;
		mesh_rec(oi, 0, ray, best, bprim, t, found, c);
		if(!found) return false;
		*sp = best;
		*prim = bprim;
		*tie = t;
		sp->pos = mul_pt(m, sp->pos);
		sp->normal = normalized(mul_n(it, sp->normal));
		sp->tangent = normalized(mul_n(it, sp->tangent));
		sp->gn = normalized(mul_n(it, sp->gn));
		return true;
	}

	void sph_tex(const V &p, R *tex, bool cyl) const
	{
		/* SphVector(pos): theta = atan2(z, x) + pi; u = theta / 2pi; v = phi / pi (or y for the cylinder) */
		double th = atan2((double)p.z, (double)p.x) + M_PI;
		double r = sqrt((double)p.x * p.x + (double)p.y * p.y + (double)p.z * p.z);
		double ph = acos((double)p.y / r);
		tex[0] = (R)(th / (2.0 * M_PI));
		tex[1] = cyl ? p.y : (R)(ph / M_PI);
	}

	/* scene octree closest hit (src/octree.inl:201-241 over objects) */
	void scene_rec(int ni, const Ray<R> &ray, SurfPoint<R> &best, int &bobj, int &bprim, bool &tie, bool &found, Counters &c) const
	{
		c.nodes++;
		if(!box_hit(scene_boxes[ni], ray)) return;
		const OctNode &n = sc.oct.nodes[ni];
		if(!n.items.empty()) {
			for(size_t k = 0; k < n.items.size(); k++) {
				SurfPoint<R> pt;
				int prim;
				bool otie;
				int oi = n.items[k];
				if(obj_hit(oi, ray, &pt, &prim, &otie, c)) {
					if(!found || pt.dist < best.dist) {
						best = pt;
						bobj = oi;
						bprim = prim;
						tie = otie;
						found = true;
					} else if(pt.dist == best.dist && (oi != bobj || prim != bprim)) {
						tie = true;
					}
				}
			}
		} else if(n.child >= 0) {
			for(int k = 0; k < 8; k++) scene_rec(n.child + k, ray, best, bobj, bprim, tie, found, c);
		}
	}

	/* Scene::cast_ray (src/scene.cc:764-794) */
	bool cast(const Ray<R> &ray, SurfPoint<R> *sp, int *obj, int *prim, bool *tie, Counters &c) const
	{
		c.rays++;
		SurfPoint<R> best;
		best.dist = (R)FLT_MAX;
		int bo = -1, bp = -1;
		bool t = false, found = false;
		if(!sc.oct.nodes.empty()) scene_rec(0, ray, best, bo, bp, t, found, c);
		if(!found) return false;
		if(best.dist >= (R)FLT_MAX) return false;
		if(sp) *sp = best;
		if(obj) *obj = bo;
		if(prim) *prim = bp;
		if(tie) *tie = t;
		return true;
	}

	/* ------------------ lights ------------------ */
	V light_point(int li, int time, sray_rng *s) const
	{
		const LightR &l = lights[li];
		int ti = tindex(time);
		if(ti < 0) ti = time < tlo ? 0 : nt - 1;
		const R *p = &light_pos[(li * nt + ti) * 3];
		V pos(p[0], p[1], p[2]);
		if(l.type == LT_SPHERE) return pos + sphrand(s, l.radius);
		if(l.type == LT_BOX) {
			V v;
			v.x = frand(s, l.dim.x) - (R)0.5 * l.dim.x;
			v.y = frand(s, l.dim.y) - (R)0.5 * l.dim.y;
			v.z = frand(s, l.dim.z) - (R)0.5 * l.dim.z;
			return mul_pt(l.box_m, v);
		}
		return pos;
	}

	/* ------------------ photon maps ------------------ */
	/* kd_nearest_range3f semantics: float positions and query, double distances */
	template <class F> void range_query(const std::vector<Photon<R> > &ph, const Grid &g, const V &pos, double max_dist, F f) const
	{
		float qf[3] = {(float)pos.x, (float)pos.y, (float)pos.z};
		double q[3] = {qf[0], qf[1], qf[2]};
		double range = (double)(float)max_dist;
		double r2 = range * range;
		int64_t lo[3], hi[3];
		for(int k = 0; k < 3; k++) { lo[k] = g.cidx(q[k] - range); hi[k] = g.cidx(q[k] + range); }
		for(int64_t x = lo[0]; x <= hi[0]; x++)
		for(int64_t y = lo[1]; y <= hi[1]; y++)
		for(int64_t z = lo[2]; z <= hi[2]; z++) {
			uint64_t key = Grid::pack(x, y, z);
			auto it = std::lower_bound(g.keys.begin(), g.keys.end(), std::make_pair(key, INT_MIN));
			for(; it != g.keys.end() && it->first == key; ++it) {
				const Photon<R> &p = ph[it->second];
				double d2 = 0.0;
				for(int k = 0; k < 3; k++) { double dx = (double)p.pos[k] - q[k]; d2 += dx * dx; }
				if(d2 <= r2) f(p, d2);
			}
		}
	}

	/* candidate set of a gather: the fixed-radius range of the reference, or
	 * (k > 0) the k nearest within the radius cap */
	void gather_set(const std::vector<Photon<R> > &ph, const Grid &g, const V &pos, double rad, int k,
			std::vector<std::pair<double, const Photon<R> *> > &out) const
	{
		out.clear();
		range_query(ph, g, pos, rad, [&](const Photon<R> &p, double d2) {
			/* k-nearest selection orders photons by the float-rounded squared distance */
			out.push_back(std::make_pair(k > 0 ? (double)(float)d2 : d2, &p));
		});
		if(k > 0 && (int)out.size() > k) {
			std::nth_element(out.begin(), out.begin() + (k - 1), out.end(),
					[](const std::pair<double, const Photon<R> *> &a, const std::pair<double, const Photon<R> *> &b) { return a.first < b.first; });
			double dk = out[k - 1].first;
			size_t w = 0;
			for(size_t i = 0; i < out.size(); i++) if(out[i].first <= dk) out[w++] = out[i];
			out.resize(w);
		}
	}

	/* PhotonMap::irradiance_est (src/pmap.cc:109-139) */
	C irradiance_est(const V &pos, const V &norm, Counters &c) const
	{
		c.gathers++;
		C irrad(0, 0, 0, 0);
		std::vector<std::pair<double, const Photon<R> *> > set;
		int k = opt.caust_k;
		double rad = k > 0 ? (double)opt.gather_rcap : gather_d;
		gather_set(caust, caust_grid, pos, rad, k, set);
		if(set.size() < 8) return irrad;
		double r2max = 0.0;
		for(size_t i = 0; i < set.size(); i++) {
			const Photon<R> *p = set[i].second;
			if(set[i].first > r2max) r2max = set[i].first;
			if(dot(p->dir, norm) < (R)0) irrad = irrad + p->col;
		}
		double r2 = k > 0 ? r2max : gather_d * gather_d;
		irrad = irrad * (R)(1.0 / (M_PI * r2));
		return irrad;
	}

	/* PhotonMap::radiance_est (src/pmap.cc:143-178) */
	C radiance_est(const V &pos, const V &norm, Counters &c) const
	{
		c.gathers++;
		C flux(0, 0, 0, 0);
		std::vector<std::pair<double, const Photon<R> *> > set;
		int k = opt.gi_k;
		double rad = k > 0 ? (double)opt.gather_rcap : gather_d;
		gather_set(gi, gi_grid, pos, rad, k, set);
		if(set.empty()) return flux;
		const R max_cos = (R)cos(M_PI / 2.5);
		double r2max = 0.0;
		for(size_t i = 0; i < set.size(); i++) {
			const Photon<R> *p = set[i].second;
			if(set[i].first > r2max) r2max = set[i].first;
			R ndotl = dot(-p->dir, norm);
			if(ndotl > (R)0 && dot(p->norm, norm) > max_cos) flux = flux + p->col * ndotl;
		}
		double r2 = k > 0 ? r2max : gather_d * gather_d;
		flux = flux * (R)(1.0 / (M_PI * r2));
		return flux;
	}

	/* ------------------ shading ------------------ */
	struct Ctx {
		sray_rng rng;
		uint32_t pixel, sample;
		Counters *c;
	};

	/* path-keyed streams: root node 1, reflection child 4p, refraction child
	 * 4p+1, diffuse child 4p+2 (its sample index in the high half of the
	 * sample word) */
	void node_rng(Ctx &ctx, uint32_t path, uint32_t dsub) const
	{
		if(rng_mode == 1) {
			sray_rng_init(&ctx.rng, opt.seed, SRAY_DOM_PIXEL | (path << 4), ctx.pixel, ctx.sample | (dsub << 16));
		}
	}

	static R fresnel(R r, R cosa)   /* src/shader.cc:285-291 */
	{
		R inv = (R)1 - cosa;
		R inv_sq = inv * inv;
		return r + ((R)1 - r) * inv_sq * inv_sq * inv;
	}

	/* The origin of a light sample's shadow ray.  The reference starts it at
	 * the surface point and ignores hits closer than ERROR_MARGIN (in units
	 * of the segment); in double the surface's own hit is ~1e-15 away, in
	 * float the point is off the surface by a few ulps and a segment leaving
	 * at a shallow angle can hit its own surface beyond the margin.  In
	 * float the ray therefore starts 2^-18 (|p|max + 1) off the surface
	 * along the geometric normal, on the side it leaves to (the GPU does
	 * the same); double keeps the reference's origin. */
	V shadow_origin(const V &pt, const V &gn, const V &dir) const
	{
		if(sizeof(R) != 4) return pt;
		R side = dot(dir, gn);
		if(side == (R)0) return pt;
		R off = (maxr(maxr(fabsr(pt.x), fabsr(pt.y)), fabsr(pt.z)) + (R)1) * (R)SHADOW_OFFSET;
		if(side < (R)0) off = -off;
		return pt + gn * off;
	}

	/* calc_lighting (src/shader.cc:250-283) */
	void calc_lighting(C *diff, C *spec, int li, R shininess, const V &pt, const V &norm, const V &gn, const V &vdir, int tm,
			Ctx &ctx) const
	{
		const LightR &lt = lights[li];
		int ns = lt.type != LT_POINT ? opt.shadow_samples : 1;
		*diff = *spec = C(0, 0, 0, 0);
		for(int i = 0; i < ns; i++) {
			V lpos = light_point(li, tm, &ctx.rng);
			V ldir = lpos - pt;
			R ldist = length(ldir);
			Ray<R> shadow;
			shadow.o = shadow_origin(pt, gn, ldir);
			shadow.d = ldir;
			shadow.time = tm;
			ldir = ldir / ldist;
			ctx.c->shadow++;
			if(!cast(shadow, 0, 0, 0, 0, *ctx.c)) {
				V vref = reflection(vdir, norm);
				R ndotl = maxr(dot(norm, ldir), (R)0);
				R rdotl = maxr(dot(vref, ldir), (R)0);
				C lcol = lt.col * (R)1;
				*diff = *diff + ndotl * lcol;
				*spec = *spec + powr(rdotl, shininess) * lcol;
			}
		}
		if(ns > 1) {
			R scale = (R)1 / (R)ns;
			*diff = *diff * scale;
			*spec = *spec * scale;
		}
	}

	/* shade_undef (src/shader.cc:36-73) */
	C shade_undef(const Ray<R> &ray, const SurfPoint<R> &sp, Ctx &ctx) const
	{
		int x = (int)(sp.tex[0] * (R)20);
		int y = (int)(sp.tex[1] * (R)10);
		C texcol = ((x % 2) == (y % 2)) ? C((R)1, (R)0.3, (R)0.2, (R)1) : C((R)0.2, (R)0.3, (R)1, (R)1);
		C diff((R)0.1, (R)0.1, (R)0.1, (R)1), spec(0, 0, 0, (R)1);
		for(size_t i = 0; i < lights.size(); i++) {
			V lpos = light_point((int)i, ray.time, &ctx.rng);
			V ldir = lpos - sp.pos;
			R ldist = length(ldir);
			Ray<R> shadow;
			shadow.o = shadow_origin(sp.pos, sp.gn, ldir);
			shadow.d = ldir;
			shadow.time = ray.time;
			ldir = ldir / ldist;
			V vdir = -normalized(ray.d);
			V hdir = normalized(ldir + vdir);
			ctx.c->shadow++;
			if(!cast(shadow, 0, 0, 0, 0, *ctx.c)) {
				R ndotl = maxr(dot(sp.normal, ldir), (R)0);
				R ndoth = maxr(dot(sp.normal, hdir), (R)0);
				diff = diff + ndotl * lights[i].col * (R)1;
				spec = spec + powr(ndoth, (R)50) * lights[i].col * (R)1;
			}
		}
		return diff * texcol + spec;
	}

	/* shade_phong (src/shader.cc:83-247) */
	C shade_phong(const Ray<R> &ray, const SurfPoint<R> &sp, const MatR &mat, Ctx &ctx, uint32_t path) const
	{
		bool entering;
		V normal;
		if(dot(ray.d, sp.normal) > (R)0) {
			normal = -sp.normal;
			entering = false;
		} else {
			normal = sp.normal;
			entering = true;
		}
		R ray_mag = length(ray.d);
		V incident = ray.d / ray_mag;
		C ks(0, 0, 0, (R)1);
		R refl_fact = 0, trans_fact = 0;
		C kd = attr_color(mat, TA_DIFFUSE, mat.kd, sp.tex);
		if(mat.have_spec) ks = attr_color(mat, TA_SPECULAR, mat.ks, sp.tex);
		R shininess = attr_value(mat, TA_SHININESS, mat.shin, sp.tex);

		if(ray.iter == INT_MAX) {
			C rad = radiance_est(sp.pos, normal, *ctx.c);
			return rad * kd;
		}
		node_rng(ctx, path, 0);
		refl_fact = attr_value(mat, TA_REFLECT, mat.refl, sp.tex);
		trans_fact = attr_value(mat, TA_REFRACT, mat.refr, sp.tex);
		R mat_ior = attr_value(mat, TA_IOR, mat.ior, sp.tex);
		R ior = ray.calc_ior(entering, mat_ior);
		if(mat.have_normal) normal = bump_normal(mat, sp);

		C diff = env_amb * kd;
		C spec(0, 0, 0, (R)1);
		for(size_t i = 0; i < lights.size(); i++) {
			C d, s;
			calc_lighting(&d, &s, (int)i, shininess, sp.pos, normal, sp.gn, incident, ray.time, ctx);
			diff = diff + d;
			spec = spec + s;
		}

		C gi(0, 0, 0, 0);
		if(opt.gi_photons) {
			for(int i = 0; i < opt.diffuse_samples; i++) {
				V dir = sphrand(&ctx.rng, (R)1);
				R ndotl;
				if((ndotl = dot(dir, normal)) < (R)0) dir = -dir;
				R diff_energy = ndotl * ray.energy;
				if(diff_energy > (R)opt.min_energy) {
					Ray<R> dr = ray;
					dr.iter = INT_MAX;
					dr.energy = diff_energy;
					dr.o = sp.pos;
					dr.d = dir * ray_mag;
					if(rng_mode == 1) {
						sray_rng saved = ctx.rng;
						gi = gi + trace_ray(dr, ctx, path * 4 + 2, (uint32_t)i) * ndotl;
						ctx.rng = saved;
					} else {
						gi = gi + trace_ray(dr, ctx, path * 4 + 2, (uint32_t)i) * ndotl;
					}
				}
			}
			if(opt.diffuse_samples > 1) gi = gi / (R)opt.diffuse_samples;
		}

		C refl(0, 0, 0, 0), refr(0, 0, 0, 0);
		R refl_energy = refl_fact * ray.energy;
		if(refl_energy > (R)opt.min_energy && ray.iter > 0) {
			Ray<R> rr = ray;
			rr.energy = refl_energy;
			rr.iter--;
			rr.o = sp.pos;
			rr.d = reflection(rr.d, normal);
			refl = trace_ray(rr, ctx, path * 4, 0) * refl_fact;
		}
		R trans_energy = trans_fact * ray.energy;
		if(trans_energy > (R)opt.min_energy && ray.iter > 0) {
			Ray<R> tr = ray;
			if(entering) tr.enter(mat_ior);
			else tr.leave();
			tr.energy = trans_energy;
			tr.iter--;
			tr.o = sp.pos;
			tr.d = refraction(ray.d / ray_mag, normal, ior) * ray_mag;
			if(dot(tr.d, normal) > (R)0) {
				if(entering) tr.leave();
				else tr.enter(mat_ior);
			}
			refr = trace_ray(tr, ctx, path * 4 + 1, 0) * trans_fact;
		}

		C irrad(0, 0, 0, 0);
		if(opt.caust_photons) irrad = irradiance_est(sp.pos, normal, *ctx.c);

		R ray_dot_n = dot(-ray.d / ray_mag, normal);
		R sqrt_fres_0 = trans_fact > (R)0 ? (ior - (R)1) / (ior + (R)1) : (R)1;
		R fres = fresnel(sqrt_fres_0 * sqrt_fres_0, ray_dot_n);
		C reflrefr = refr + (refl - refr) * fres;
		return (diff + gi) * kd + (spec + reflrefr) * ks + irrad;
	}

	/* Scene::trace_ray (src/scene.cc:551-569) */
	C trace_ray(const Ray<R> &ray, Ctx &ctx, uint32_t path, uint32_t dsub) const
	{
		SurfPoint<R> sp;
		int obj;
		if(cast(ray, &sp, &obj, 0, 0, *ctx.c)) {
			const MatR &m = mat_for(obj);
			C col;
			if(m.phong) col = shade_phong(ray, sp, m, ctx, path);
			else {
				node_rng(ctx, path, dsub);
				col = shade_undef(ray, sp, ctx);
			}
			col.w = (R)1;
			return col;
		}
		return env_col;
	}

	/* Camera::get_primary_ray (src/camera.cc:119-142) */
	Ray<R> primary(int x, int y, int sub, int time, sray_rng *s) const
	{
		R px = ((R)x / (R)opt.width) * cam_xsz - cam_xsz / (R)2;
		R py = (R)1 - ((R)y / (R)opt.height) * cam_ysz;
		if(sub > 0) {
			px = px + cam_xsz * (frand(s, (R)1) - (R)0.5) / (R)opt.width;
			py = py + cam_ysz * (frand(s, (R)1) - (R)0.5) / (R)opt.height;
		}
		Ray<R> r;
		r.o = V(0, 0, 0);
		r.d = V(px, py, cam_f) * cam_maxd;
		r.time = time;
		if(opt.mblur && sub > 0 && sc.cam.shutter > 0) r.time += sray_rng_int(s) % sc.cam.shutter - sc.cam.shutter / 2;
		int ti = tindex(r.time);
		if(ti < 0) ti = r.time < tlo ? 0 : nt - 1;
		const R *m = &cam_m[ti * 12];
		r.o = mul_pt(m, r.o);
		r.d = mul_dir(m, r.d);
		r.energy = (R)1;
		return r;
	}

	/* ------------------ photon tracing ------------------ */
	/* Scene::trace_caustics_photon (src/scene.cc:571-647), loop form */
	bool trace_caust(Ray<R> ray, Photon<R> *ph, sray_rng *s, Counters &c) const
	{
		for(int guard = 0; guard < 100000; guard++) {
			if(ray.iter <= 0) return false;
			SurfPoint<R> sp;
			int obj;
			if(!cast(ray, &sp, &obj, 0, 0, c)) return false;
			const MatR &m = mat_for(obj);
			C spec = attr_color(m, TA_SPECULAR, m.ks, sp.tex);
			R refl = attr_value(m, TA_REFLECT, m.refl, sp.tex);
			R refr = attr_value(m, TA_REFRACT, m.refr, sp.tex);
			R mat_ior = attr_value(m, TA_IOR, m.ior, sp.tex);
			bool entering;
			V normal;
			R ray_mag = length(ray.d);
			if(dot(ray.d, sp.normal) > (R)0) { normal = -sp.normal; entering = false; }
			else { normal = sp.normal; entering = true; }
			R ior = ray.calc_ior(entering, mat_ior);
			if(m.have_normal) normal = bump_normal(m, sp);
			R ray_dot_n = dot(-ray.d / ray_mag, normal);
			R sf0 = refr > (R)0 ? (ior - (R)1) / (ior + (R)1) : (R)1;
			R fres = fresnel(sf0 * sf0, ray_dot_n);
			refl = fres * refl;
			refr = ((R)1 - fres) * refr;
			R rnum = frand(s, (R)1);
			if(rnum < refl) {
				Ray<R> nr = ray;
				nr.d = reflection(ray.d, normal);
				nr.iter--;
				nr.o = sp.pos;
				ph->type = CAUST_PHOTON;
				ph->col = ph->col * spec;
				ray = nr;
			} else if(rnum < refr) {
				Ray<R> nr = refract_ray(ray, normal, mat_ior, entering, ray_mag);
				nr.o = sp.pos;
				ph->type = CAUST_PHOTON;
				ph->col = ph->col * spec;
				ray = nr;
			} else {
				ph->dir = normalized(ray.d);
				ph->pos[0] = (float)sp.pos.x;
				ph->pos[1] = (float)sp.pos.y;
				ph->pos[2] = (float)sp.pos.z;
				ph->norm = normal;
				ph->p = sp.pos;
				return true;
			}
		}
		return false;
	}

	/* refraction of a ray (libvmath refract_ray, same steps as src/shader.cc:244-267) */
	Ray<R> refract_ray(const Ray<R> &in, const V &n, R mat_ior, bool entering, R ray_mag) const
	{
		Ray<R> r = in;
		R ior = r.calc_ior(entering, mat_ior);
		if(entering) r.enter(mat_ior);
		else r.leave();
		r.d = refraction(r.d / ray_mag, n, ior) * ray_mag;
		if(dot(r.d, n) > (R)0) {
			if(entering) r.leave();
			else r.enter(mat_ior);
		}
		return r;
	}

	/* Scene::trace_global_photon (src/scene.cc:650-760), loop form */
	bool trace_global(Ray<R> ray, Photon<R> *ph, sray_rng *s, Counters &c) const
	{
		for(int guard = 0; guard < 100000; guard++) {
			if(ray.iter <= 0) return false;
			V incident = normalized(ray.d);
			SurfPoint<R> sp;
			int obj;
			if(!cast(ray, &sp, &obj, 0, 0, c)) return false;
			V normal;
			bool entering;
			R ray_mag = length(ray.d);
			if(dot(ray.d, sp.normal) > (R)0) { normal = -sp.normal; entering = false; }
			else { normal = sp.normal; entering = true; }
			const MatR &m = mat_for(obj);
			C diff = attr_color(m, TA_DIFFUSE, m.kd, sp.tex);
			R diff_avg = (diff.x + diff.y + diff.z) / (R)3;
			C spec = attr_color(m, TA_SPECULAR, m.ks, sp.tex);
			R spec_avg = (spec.x + spec.y + spec.z) / (R)3;
			R rnum = frand(s, (R)1);
			if(rnum < diff_avg) {
				V dir = sphrand(s, (R)1);
				if(dot(dir, normal) < (R)0) dir = -dir;
				R ndotl = dot(-incident, normal);
				Ray<R> nr = ray;
				nr.d = dir * (R)RAY_MAG;
				nr.iter--;
				nr.o = sp.pos;
				ph->type = GI_PHOTON;
				ph->col = ph->col * (ndotl * (diff / diff_avg));
				ray = nr;
			} else if(rnum < diff_avg + spec_avg) {
				R refl = attr_value(m, TA_REFLECT, m.refl, sp.tex);
				R refr = attr_value(m, TA_REFRACT, m.refr, sp.tex);
				R mat_ior = attr_value(m, TA_IOR, m.ior, sp.tex);
				R ior = ray.calc_ior(entering, mat_ior);
				R ray_dot_n = dot(-ray.d / ray_mag, normal);
				R sf0 = refr > (R)0 ? (ior - (R)1) / (ior + (R)1) : (R)1;
				R fres = fresnel(sf0 * sf0, ray_dot_n);
				refl = fres * refl;
				refr = ((R)1 - fres) * refr;
				R rn2 = frand(s, (R)1);
				if(rn2 < refl) {
					Ray<R> nr = ray;
					nr.d = reflection(ray.d, normal);
					nr.iter--;
					nr.o = sp.pos;
					ph->type = CAUST_PHOTON;
					ph->col = ph->col * spec;
					return trace_caust(nr, ph, s, c);
				} else if(rn2 < refr) {
					Ray<R> nr = refract_ray(ray, normal, mat_ior, entering, ray_mag);
					nr.o = sp.pos;
					ph->type = CAUST_PHOTON;
					ph->col = ph->col * spec;
					return trace_caust(nr, ph, s, c);
				}
				return false;
			} else {
				ph->dir = incident;
				ph->pos[0] = (float)sp.pos.x;
				ph->pos[1] = (float)sp.pos.y;
				ph->pos[2] = (float)sp.pos.z;
				ph->norm = normal;
				ph->p = sp.pos;
				return true;
			}
		}
		return false;
	}

	/* ProjMap::gen_dir(true) (src/projmap.cc:193-209), with an iteration bound */
	bool gen_dir(const ProjMap &pm, sray_rng *s, V *out) const;

	/* Light::gen_photon (src/light.cc:111-148) */
	bool gen_photon(int li, int time, int sampling, sray_rng *s, Photon<R> *p) const
	{
		const LightR &lt = lights[li];
		const Light &L = sc.lights[li];
		V pos = light_point(li, time, s);
		p->p = pos;
		p->pos[0] = (float)pos.x; p->pos[1] = (float)pos.y; p->pos[2] = (float)pos.z;
		p->col = lt.col * (R)opt.photon_energy;
		p->type = DIRECT_PHOTON;
		const ProjMap *proj = sampling == 1 ? &L.pm : &L.spm;
		p->col = p->col * (R)proj->get_coverage();
		if(proj->get_coverage() == 0.0) {
			proj = 0;
			p->col = lt.col * (R)opt.photon_energy;
		}
		V dir;
		if(proj) {
			if(!gen_dir(*proj, s, &dir)) return false;
		} else {
			dir = sphrand(s, (R)1);
		}
		p->dir = dir * (R)RAY_MAG;
		return true;
	}

	/* shoot_photons (src/render.cc:67-122) with build_caustics_map / build_global_map
	 * (src/scene.cc:445-534); every photon on its own stream */
	void shoot(Scene &msc)
	{
		auto t_shoot = std::chrono::steady_clock::now();
		ms_proj = ms_photons = 0.0;
		caust.clear();
		gi.clear();
		if(!opt.caust_photons && !opt.gi_photons) return;
		int nl = (int)msc.lights.size();
		if(!nl) return;
		std::vector<double> intensity(nl), power(nl);
		double acc = 0.0;
		for(int i = 0; i < nl; i++) {
			const double *c = msc.lights[i].col;
			intensity[i] = (c[0] + c[1] + c[2]) / 3.0;
			acc += intensity[i];
			if(!msc.objs.empty()) build_proj(msc, i);
		}
		auto tp = std::chrono::steady_clock::now();
		ms_proj = std::chrono::duration<double, std::milli>(tp - t_shoot).count();
		for(int i = 0; i < nl; i++) power[i] = intensity[i] / acc;
		shoot_map(0, power);
		shoot_map(1, power);
		ms_photons = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tp).count();
	}

	/* Light::build_proj_intern (src/light.cc:151-200) */
	void build_proj(Scene &msc, int li)
	{
		Light &L = msc.lights[li];
		int tm[3] = {t0, t1, -1};
		if(t0 == t1) tm[1] = -1;
		L.pm.clear();
		L.spm.clear();
		int samples = L.type == LT_SPHERE ? 8 : 1;
		/* one stream per light, drawn in order over both shutter ends */
		sray_rng s;
		sray_rng_init(&s, opt.seed, SRAY_DOM_PROJMAP, (uint32_t)li, 0);
		for(int tidx = 0; tm[tidx] != -1 && tidx < 2; tidx++) {
			std::vector<Box> boxes(msc.objs.size()), cboxes;
			for(size_t i = 0; i < msc.objs.size(); i++) {
				const Object &o = msc.objs[i];
				const Material &m = o.mat >= 0 ? msc.mats[o.mat] : msc.default_mat;
				bool spec = m.get("reflect")[0] > 0.0 || m.get("refract")[0] > 0.0;
				boxes[i] = o.bounds(tm[tidx]);
				if(spec) cboxes.push_back(boxes[i]);
			}
			for(int k = 0; k < samples; k++) {
				V3d lpos = L.xf.position(tm[tidx]);
				if(L.type == LT_SPHERE) {
					double r[3];
					vmc_sphrand(r, &s, (double)L.radius);
					lpos = lpos + V3d(r[0], r[1], r[2]);
				} else if(L.type == LT_BOX) {
					double m0[4][4];
					L.xf.matrix(0, m0);
					V3d v;
					v.x = vmc_frand(&s, L.dim.x) - 0.5 * L.dim.x;
					v.y = vmc_frand(&s, L.dim.y) - 0.5 * L.dim.y;
					v.z = vmc_frand(&s, L.dim.z) - 0.5 * L.dim.z;
					lpos = xform_pt(m0, v);
				}
				build_projmap(&L.pm, lpos, boxes);
				build_projmap(&L.spm, lpos, cboxes);
			}
		}
	}

	void shoot_map(int global, const std::vector<double> &power)
	{
		std::vector<Photon<R> > &map = global ? gi : caust;
		int num = global ? opt.gi_photons : opt.caust_photons;
		int nthreads = opt.threads > 0 ? opt.threads : (int)std::thread::hardware_concurrency();
		if(nthreads <= 0) nthreads = 1;
		for(size_t li = 0; li < lights.size(); li++) {
			int nphot = (int)ceil((double)num * power[li]);
			size_t first = map.size();
			/* photons are independent (each on its own stream): trace them on
			 * all threads, keep the stored ones in emission order */
			std::vector<Photon<R> > res(nphot > 0 ? nphot : 0);
			std::vector<char> ok(nphot > 0 ? nphot : 0, 0);
			std::atomic<int> next(0);
			auto work = [&]() {
				Counters c;
				for(;;) {
					int j0 = next.fetch_add(256);
					if(j0 >= nphot) break;
					for(int j = j0; j < j0 + 256 && j < nphot; j++) {
						sray_rng s;
						sray_rng_init(&s, opt.seed, global ? SRAY_DOM_GLOBAL : SRAY_DOM_CAUST, (uint32_t)j, (uint32_t)li);
						int ms = t0 == t1 ? t0 : (sray_rng_int(&s) % (t1 - t0) + t0);
						Photon<R> &p = res[j];
						if(!gen_photon((int)li, ms, global ? 1 : 2, &s, &p)) continue;
						Ray<R> ray;
						ray.o = p.p;
						ray.d = p.dir;
						ray.time = ms;
						ray.iter = opt.iter;
						if(global) ok[j] = trace_global(ray, &p, &s, c);
						else ok[j] = trace_caust(ray, &p, &s, c) && p.type == CAUST_PHOTON;
					}
				}
			};
			std::vector<std::thread> th;
			for(int t = 1; t < nthreads; t++) th.push_back(std::thread(work));
			work();
			for(auto &t : th) t.join();
			for(int j = 0; j < nphot; j++) if(ok[j]) map.push_back(res[j]);
			if(nphot) {
				double scale = 1.0 / (double)nphot;
				for(size_t i = first; i < map.size(); i++) {
					map[i].col.x *= (R)scale;
					map[i].col.y *= (R)scale;
					map[i].col.z *= (R)scale;
				}
			}
		}
		if(global) gi_grid.build(gi, opt.gi_k > 0 ? (double)opt.gather_rcap : gather_d);
		else caust_grid.build(caust, opt.caust_k > 0 ? (double)opt.gather_rcap : gather_d);
	}

	/* ------------------ pixels ------------------ */
	/* variance (src/render.cc:261-270), in float as the reference */
	static float variance(const C *samples, const C &sum, int num, float rcp_num)
	{
		C mean = sum * (R)rcp_num;
		float sqdist = 0.0f;
		for(int i = 0; i < num; i++) sqdist = (float)((R)sqdist + length_sq(mean - samples[i]));
		return sqdist * rcp_num;
	}

	/* render_block (src/render.cc:194-244) for one tile */
	void render_block(int bx, int by, int y0, int y1, float *fb, int quirk, int *spp, Counters &c) const
	{
		int bsz = opt.blk_sz;
		int xs = bx * bsz, ys = by * bsz;
		int xsz = std::min(bsz, opt.width - xs), ysz = std::min(bsz, opt.height - ys);
		std::vector<C> sub(opt.max_samples > 0 ? opt.max_samples : 1);
		for(int y = 0; y < ysz; y++) {
			int py = ys + y;
			if(py < y0 || py >= y1) continue;
			float *img = fb + ((size_t)py * opt.width + xs) * 4;
			for(int x = 0; x < xsz; x++) {
				int px = xs + x;
				uint32_t lpix = (uint32_t)(py * opt.width + px), pix = pix_base + lpix;
				img[x * 4] = img[x * 4 + 1] = img[x * 4 + 2] = img[x * 4 + 3] = 0.0f;
				int i = 0;
				C pixel;
				while(i < opt.max_samples) {
					Ctx ctx;
					ctx.pixel = pix;
					ctx.sample = (uint32_t)i;
					ctx.c = &c;
					sray_rng_init(&ctx.rng, opt.seed, SRAY_DOM_PIXEL, pix, (uint32_t)i);
					Ray<R> ray = primary(px, py, i, t0, &ctx.rng);
					ray.iter = opt.iter;
					sub[i] = trace_ray(ray, ctx, 1, 0);
					pixel.x = img[x * 4] = (float)(img[x * 4] + sub[i].x);
					pixel.y = img[x * 4 + 1] = (float)(img[x * 4 + 1] + sub[i].y);
					pixel.z = img[x * 4 + 2] = (float)(img[x * 4 + 2] + sub[i].z);
					pixel.w = img[x * 4 + 3] = (float)(img[x * 4 + 3] + sub[i].w);
					i++;
					if(i >= opt.min_samples && i > 1) {
						float v = variance(sub.data(), pixel, i, (float)(1.0 / (double)i));
						if(v < opt.max_var) break;
					}
				}
				if(spp) spp[lpix] = i;
				double rcp = 1.0 / (double)i;
				if(quirk) {
					img[x] = (float)(img[x] * rcp);
				} else {
					for(int k = 0; k < 4; k++) img[x * 4 + k] = (float)(img[x * 4 + k] * rcp);
				}
			}
		}
	}

	int render_rows(int y0, int y1, float *fb, int nthreads, int quirk, int *spp) override
	{
		int bsz = opt.blk_sz > 0 ? opt.blk_sz : 48;
		int xb = (opt.width + bsz - 1) / bsz, yb = (opt.height + bsz - 1) / bsz;
		int by0 = y0 / bsz, by1 = (y1 + bsz - 1) / bsz;
		if(by1 > yb) by1 = yb;
		std::vector<std::pair<int, int> > blocks;
		for(int by = by0; by < by1; by++) for(int bx = 0; bx < xb; bx++) blocks.push_back(std::make_pair(bx, by));
		if(nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
		if(nthreads <= 0) nthreads = 1;
		std::atomic<size_t> next(0);
		std::vector<Counters> cs(nthreads);
		auto work = [&](int tid) {
			for(;;) {
				size_t b = next.fetch_add(1);
				if(b >= blocks.size()) break;
				render_block(blocks[b].first, blocks[b].second, y0, y1, fb, quirk, spp, cs[tid]);
			}
		};
		std::vector<std::thread> th;
		for(int i = 1; i < nthreads; i++) th.push_back(std::thread(work, i));
		work(0);
		for(auto &t : th) t.join();
		ctr = Counters();
		for(auto &c : cs) {
			ctr.rays += c.rays; ctr.nodes += c.nodes; ctr.prims += c.prims; ctr.shadow += c.shadow; ctr.gathers += c.gathers;
		}
		return 0;
	}

	/* the listed rows, one task per row and tile column (a thin sample of
	 * rows spread over the image keeps every thread busy) */
	int render_row_list(int n, const int *rows, float *fb, int nthreads, int quirk, int *spp) override
	{
		int bsz = opt.blk_sz > 0 ? opt.blk_sz : 48;
		int xb = (opt.width + bsz - 1) / bsz;
		std::vector<std::pair<int, int> > tasks;
		for(int i = 0; i < n; i++) {
			if(rows[i] < 0 || rows[i] >= opt.height) return SRAY_EINVAL;
			for(int bx = 0; bx < xb; bx++) tasks.push_back(std::make_pair(bx, rows[i]));
		}
		if(nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
		if(nthreads <= 0) nthreads = 1;
		std::atomic<size_t> next(0);
		std::vector<Counters> cs(nthreads);
		auto work = [&](int tid) {
			for(;;) {
				size_t k = next.fetch_add(1);
				if(k >= tasks.size()) break;
				int y = tasks[k].second;
				render_block(tasks[k].first, y / bsz, y, y + 1, fb, quirk, spp, cs[tid]);
			}
		};
		std::vector<std::thread> th;
		for(int i = 1; i < nthreads; i++) th.push_back(std::thread(work, i));
		work(0);
		for(auto &t : th) t.join();
		ctr = Counters();
		for(auto &c : cs) {
			ctr.rays += c.rays; ctr.nodes += c.nodes; ctr.prims += c.prims; ctr.shadow += c.shadow; ctr.gathers += c.gathers;
		}
		return 0;
	}

	int primary_hits(int *obj, int *prim, double *t, unsigned char *tie) override
	{
		ctr = Counters();
		int n = opt.width * opt.height;
		int nth = (int)std::thread::hardware_concurrency();
		if(nth <= 0) nth = 1;
		std::vector<Counters> cs(nth);
		std::atomic<int> next(0);
		auto work = [&](int tid) {
			for(;;) {
				int row = next.fetch_add(1);
				if(row >= opt.height) break;
				for(int x = 0; x < opt.width; x++) {
					int i = row * opt.width + x;
					sray_rng s;
					sray_rng_init(&s, opt.seed, SRAY_DOM_PIXEL, pix_base + (uint32_t)i, 0);
					Ray<R> ray = primary(x, row, 0, t0, &s);
					SurfPoint<R> sp;
					int o = -1, p = -1;
					bool tt = false;
					if(cast(ray, &sp, &o, &p, &tt, cs[tid])) {
						obj[i] = o; prim[i] = p; t[i] = (double)sp.dist; tie[i] = tt;
					} else {
						obj[i] = -1; prim[i] = -1; t[i] = 0.0; tie[i] = 0;
					}
				}
			}
		};
		std::vector<std::thread> th;
		for(int i = 1; i < nth; i++) th.push_back(std::thread(work, i));
		work(0);
		for(auto &x : th) x.join();
		for(auto &c : cs) { ctr.rays += c.rays; ctr.nodes += c.nodes; ctr.prims += c.prims; }
		(void)n;
		return 0;
	}

	int cast_rays(int n, const double *o, const double *d, const int *tm, int *obj, int *prim, double *t, unsigned char *tie) override
	{
		Counters c;
		for(int i = 0; i < n; i++) {
			Ray<R> ray;
			ray.o = V((R)o[i * 3], (R)o[i * 3 + 1], (R)o[i * 3 + 2]);
			ray.d = V((R)d[i * 3], (R)d[i * 3 + 1], (R)d[i * 3 + 2]);
			ray.time = tm ? tm[i] : t0;
			SurfPoint<R> sp;
			int oo = -1, pp = -1;
			bool tt = false;
			if(cast(ray, &sp, &oo, &pp, &tt, c)) {
				obj[i] = oo; prim[i] = pp; t[i] = (double)sp.dist; tie[i] = tt;
			} else {
				obj[i] = -1; prim[i] = -1; t[i] = 0.0; tie[i] = 0;
			}
		}
		ctr = c;
		return 0;
	}

	int photons(int which, float *out, int cap) override
	{
		const std::vector<Photon<R> > &m = which ? gi : caust;
		int n = (int)m.size();
		for(int i = 0; i < n && i < cap; i++) {
			float *f = out + (size_t)i * 16;
			const Photon<R> &p = m[i];
			f[0] = p.pos[0]; f[1] = p.pos[1]; f[2] = p.pos[2];
			f[3] = (float)p.dir.x; f[4] = (float)p.dir.y; f[5] = (float)p.dir.z;
			f[6] = (float)p.norm.x; f[7] = (float)p.norm.y; f[8] = (float)p.norm.z;
			f[9] = (float)p.col.x; f[10] = (float)p.col.y; f[11] = (float)p.col.z; f[12] = (float)p.col.w;
			f[13] = (float)p.type; f[14] = f[15] = 0.0f;
		}
		return n;
	}

	void photon_counts(int *c, int *g) override { *c = (int)caust.size(); *g = (int)gi.size(); }

	int gather(int which, int n, const double *pos, const double *norm, double *out) override
	{
		Counters c;
		for(int i = 0; i < n; i++) {
			V p((R)pos[i * 3], (R)pos[i * 3 + 1], (R)pos[i * 3 + 2]);
			V nn((R)norm[i * 3], (R)norm[i * 3 + 1], (R)norm[i * 3 + 2]);
			C r = which ? radiance_est(p, nn, c) : irradiance_est(p, nn, c);
			out[i * 4] = r.x; out[i * 4 + 1] = r.y; out[i * 4 + 2] = r.z; out[i * 4 + 3] = r.w;
		}
		return 0;
	}
};

/* random draws: double precision uses libm (as the compiled reference does
 * through its shim), float precision the deterministic float series */
template <> double Frame<double>::frand(sray_rng *s, double range) const { return range * sray_rng_uniform_d(s); }
template <> float Frame<float>::frand(sray_rng *s, float range) const { return range * sray_rng_uniform_f(s); }
template <> V3<double> Frame<double>::sphrand(sray_rng *s, double rad) const
{
	double r[3];
	vmc_sphrand(r, s, rad);
	return V3<double>(r[0], r[1], r[2]);
}
template <> V3<float> Frame<float>::sphrand(sray_rng *s, float rad) const
{
	float u0 = sray_rng_uniform_f(s);
	float u1 = sray_rng_uniform_f(s);
	float z = 2.0f * u1 - 1.0f;
	float sxy = sqrtf(1.0f - z * z);
	float sn, cs;
	sray_sincos_turns_f(u0, &sn, &cs);
	return V3<float>(rad * cs * sxy, rad * sn * sxy, rad * z);
}

template <> bool Frame<double>::gen_dir(const ProjMap &pm, sray_rng *s, V3<double> *out) const
{
	for(int it = 0; it < (1 << 20); it++) {
		V3<double> v = sphrand(s, 1.0);
		int uc, vc;
		double vv[3] = {v.x, v.y, v.z};
		pm.cell_from_dir(vv, &uc, &vc);
		if(pm.cells[vc * pm.udiv + uc]) { *out = v; return true; }
	}
	return false;
}

template <> bool Frame<float>::gen_dir(const ProjMap &pm, sray_rng *s, V3<float> *out) const
{
	for(int it = 0; it < (1 << 20); it++) {
		V3<float> v = sphrand(s, 1.0f);
		/* cell_from_dir in float: theta = atan2(z, x), phi = atan2(sqrt(x^2 + z^2), y) */
		float theta = sray_atan2_f(v.z, v.x);
		float phi = sray_atan2_f(sqrtf(v.x * v.x + v.z * v.z), v.y);
		if(theta < 0.0f) theta = SRAY_TWO_PI_F + theta;
		float u = theta / SRAY_TWO_PI_F, w = phi / SRAY_PI_F;
		int uc = (int)(u * (float)pm.udiv), vc = (int)(w * (float)pm.vdiv);
		uc = uc < 0 ? 0 : (uc >= pm.udiv ? pm.udiv - 1 : uc);
		vc = vc < 0 ? 0 : (vc >= pm.vdiv ? pm.vdiv - 1 : vc);
		if(pm.cells[vc * pm.udiv + uc]) { *out = v; return true; }
	}
	return false;
}

struct Oracle {
	sray_opts opt;
	int fp64, rng_mode;
	Scene sc;
	bool loaded = false;
	std::unique_ptr<FrameBase> frame;
	long frame_msec = LONG_MIN;
	uint32_t pix_base = 0;
	std::string err;
};

static int prepare(Oracle *o, long msec)
{
	if(!o->loaded) { o->err = "no scene loaded"; return SRAY_ESTATE; }
	if(o->frame && o->frame_msec == msec) return 0;
	int shutter = o->sc.cam.shutter;
	int t0 = (int)(msec - shutter / 2), t1 = t0 + shutter;
	auto tb = std::chrono::steady_clock::now();
	build_scene_tree(o->sc, o->opt, t0, t1);
	int lo = t0 - shutter - 2, hi = t1 + shutter + 2;
	if(o->fp64) {
		Frame<double> *f = new Frame<double>(o->sc, o->opt, o->rng_mode, msec);
		f->t0 = t0; f->t1 = t1;
		f->setup(lo, hi);
		f->ms_build = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
		f->shoot(o->sc);
		o->frame.reset(f);
	} else {
		Frame<float> *f = new Frame<float>(o->sc, o->opt, o->rng_mode, msec);
		f->t0 = t0; f->t1 = t1;
		f->setup(lo, hi);
		f->ms_build = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
		f->shoot(o->sc);
		o->frame.reset(f);
	}
	o->frame_msec = msec;
	return 0;
}

} /* namespace */

extern "C" {

void *orc_create(const sray_opts *opt, int fp64, int rng_mode)
{
	Oracle *o = new Oracle;
	o->opt = *opt;
	o->fp64 = fp64;
	o->rng_mode = rng_mode;
	return o;
}

void orc_destroy(void *h) { delete (Oracle *)h; }

const char *orc_error(void *h) { return ((Oracle *)h)->err.c_str(); }

int orc_load_mem(void *h, const char *xml, size_t len)
{
	Oracle *o = (Oracle *)h;
	o->frame.reset();
	o->frame_msec = LONG_MIN;
	o->loaded = false;
	if(!load_scene(o->sc, o->opt, xml, len, o->err)) return SRAY_ELOAD;
	o->loaded = true;
	return 0;
}

int orc_load(void *h, const char *path)
{
	Oracle *o = (Oracle *)h;
	FILE *fp = fopen(path, "rb");
	if(!fp) { o->err = std::string("failed to open file: ") + path; return SRAY_ELOAD; }
	fseek(fp, 0, SEEK_END);
	long sz = ftell(fp);
	fseek(fp, 0, SEEK_SET);
	std::string buf((size_t)sz, '\0');
	size_t rd = fread(&buf[0], 1, (size_t)sz, fp);
	fclose(fp);
	return orc_load_mem(h, buf.data(), rd);
}

int orc_scene_info(void *h, int *n_obj, int *n_lights, int *n_mat, int64_t *n_tris)
{
	Oracle *o = (Oracle *)h;
	if(n_obj) *n_obj = (int)o->sc.objs.size();
	if(n_lights) *n_lights = (int)o->sc.lights.size();
	if(n_mat) *n_mat = (int)o->sc.mats.size();
	if(n_tris) *n_tris = o->sc.n_tris;
	return 0;
}

int orc_prepare_frame(void *h, long msec) { return prepare((Oracle *)h, msec); }

int orc_photon_info(void *h, int *n_caust, int *n_gi, double *gather_dist)
{
	Oracle *o = (Oracle *)h;
	if(!o->frame) return SRAY_ESTATE;
	o->frame->photon_counts(n_caust, n_gi);
	if(gather_dist) *gather_dist = o->sc.gather_dist;
	return 0;
}

int orc_get_photons(void *h, int which, float *out, int cap)
{
	Oracle *o = (Oracle *)h;
	if(!o->frame) return SRAY_ESTATE;
	return o->frame->photons(which, out, cap);
}

int orc_render_rows(void *h, long msec, int y0, int y1, float *fb, int nthreads, int quirk_sum, int *spp_out)
{
	Oracle *o = (Oracle *)h;
	int r = prepare(o, msec);
	if(r) return r;
	o->frame->pix_base = o->pix_base;
	return o->frame->render_rows(y0, y1, fb, nthreads, quirk_sum, spp_out);
}

int orc_render_row_list(void *h, long msec, int n, const int *rows, float *fb, int nthreads, int quirk_sum, int *spp_out)
{
	Oracle *o = (Oracle *)h;
	int r = prepare(o, msec);
	if(r) return r;
	o->frame->pix_base = o->pix_base;
	return o->frame->render_row_list(n, rows, fb, nthreads, quirk_sum, spp_out);
}

int orc_primary_hits(void *h, long msec, int *obj, int *prim, double *t, unsigned char *tie)
{
	Oracle *o = (Oracle *)h;
	int r = prepare(o, msec);
	if(r) return r;
	o->frame->pix_base = o->pix_base;
	return o->frame->primary_hits(obj, prim, t, tie);
}

int orc_set_opts(void *h, const sray_opts *opt)
{
	Oracle *o = (Oracle *)h;
	if(o->loaded && (opt->meshoct_max_depth != o->opt.meshoct_max_depth || opt->meshoct_max_items != o->opt.meshoct_max_items)) {
		o->err = "mesh octree options change needs a scene reload";
		return SRAY_ESTATE;
	}
	o->opt = *opt;
	o->frame.reset();
	o->frame_msec = LONG_MIN;
	return 0;
}

int orc_set_pixel_base(void *h, int base)
{
	Oracle *o = (Oracle *)h;
	if(base < 0) { o->err = "negative pixel base"; return SRAY_EINVAL; }
	o->pix_base = (uint32_t)base;
	return 0;
}

int orc_phase_ms(void *h, double *ms)
{
	Oracle *o = (Oracle *)h;
	if(!o->frame) { o->err = "no frame prepared"; return SRAY_ESTATE; }
	ms[0] = o->frame->ms_build;
	ms[1] = o->frame->ms_proj;
	ms[2] = o->frame->ms_photons;
	return 0;
}

int orc_cast_rays(void *h, int n, const double *orig, const double *dir, const int *time,
		int *obj, int *prim, double *t, unsigned char *tie)
{
	Oracle *o = (Oracle *)h;
	if(!o->frame) {
		int r = prepare(o, 0);
		if(r) return r;
	}
	return o->frame->cast_rays(n, orig, dir, time, obj, prim, t, tie);
}

int orc_gather(void *h, int which, int n, const double *pos, const double *norm, double *out)
{
	Oracle *o = (Oracle *)h;
	if(!o->frame) return SRAY_ESTATE;
	return o->frame->gather(which, n, pos, norm, out);
}

int orc_counters(void *h, int64_t *rays, int64_t *node_visits, int64_t *prim_tests, int64_t *shadow_rays, int64_t *gathers)
{
	Oracle *o = (Oracle *)h;
	if(!o->frame) return SRAY_ESTATE;
	const Counters &c = o->frame->ctr;
	if(rays) *rays = c.rays;
	if(node_visits) *node_visits = c.nodes;
	if(prim_tests) *prim_tests = c.prims;
	if(shadow_rays) *shadow_rays = c.shadow;
	if(gathers) *gathers = c.gathers;
	return 0;
}

void sray_default_opts(sray_opts *o)
{
	memset(o, 0, sizeof *o);
	o->width = 640; o->height = 480;
	o->min_samples = 1; o->max_samples = 1;
	o->max_var = 0.005f;
	o->min_energy = 0.0001f;
	o->shadow_samples = 1;
	o->diffuse_samples = 1;
	o->threads = 0;
	o->blk_sz = 48;
	o->iter = 7;
	o->fps = 30;
	o->gather_dist = 0.001f;
	o->photon_energy = 300.0f;
	o->scnoct_max_depth = 5; o->scnoct_max_items = 5;
	o->meshoct_max_depth = 7; o->meshoct_max_items = 14;
	o->gather_rcap = 0.5f;
	o->seed = 0x5EED0001ull;
}

} /* extern "C" */
