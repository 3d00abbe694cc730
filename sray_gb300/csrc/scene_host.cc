/* scene_host.cc -- S-ray scene database on the host (see scene_host.h).
 *
 * Reference behaviour reproduced here:
 *   XML attribute typing            src/xmltree.c:51-95
 *   scene loading order             src/scene.cc:93-183
 *   materials and defaults          src/material.cc:68-111
 *   objects / meshes                src/object.cc:28-58, src/meshload.cc:55-157
 *   lights                          src/light.cc:38-63, 255-275, 326-350
 *   cameras                         src/camera.cc:16-66, 161-234
 *   keyframe tracks and transforms  src/anim.inl:70-263, src/anim.cc:68-121, 391-427
 *   octree build                    src/octree.inl:119-191
 *   scene octree                    src/scene.cc:353-390
 *   projection maps                 src/projmap.cc:25-160, src/light.cc:151-200, 392-432
 */
#include <math.h>
#include <float.h>
#include <limits.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <unistd.h>
#include <algorithm>
#include <thread>
#include "scene_host.h"
#include "sray_rng.h"

namespace sray {

/* ------------------------------------------------------------------ */
/* textures                                                             */
/* ------------------------------------------------------------------ */
namespace {

/* a PPM header number: decimal digits after whitespace and '#' comments */
int ppm_number(FILE *fp)
{
	int c, v = 0, any = 0;
	while((c = fgetc(fp)) != EOF) {
		if(c == '#') {
			while((c = fgetc(fp)) != EOF && c != '\n') {}
			continue;
		}
		if(c >= '0' && c <= '9') {
			if(v > 100000000) return -1;
			v = v * 10 + (c - '0');
			any = 1;
		} else if(any) {
			break;
		}
	}
	return any ? v : -1;
}

}  // namespace

bool load_texture(const char *name, Texture &t)
{
	const char *env = getenv("SRAY_DATA_PATH");
	if(!env || !*env || !name) return false;
	std::string path(env, strcspn(env, ":"));
	path += "/";
	path += name;
	if(access(path.c_str(), F_OK) != 0) return false;
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
		for(int k = 0; k < 3; k++) t.pix[i * 4 + k] = (float)rgb[i * 3 + k] / 255.0f;
		t.pix[i * 4 + 3] = 1.0f;
	}
	return true;
}

/* ------------------------------------------------------------------ */
/* flat XML DOM: names and values are views into the document buffer   */
/* ------------------------------------------------------------------ */
namespace {

struct XAttr {
	const char *name;
	const char *val;
	int nlen, vlen;
};

struct XNode {
	const char *name;
	int nlen;
	int attr0, nattr;
	int first_child = -1, last_child = -1, next = -1;
};

struct Typed {
	int type;        /* 0 str, 1 int, 2 flt, 3 vec */
	int ival;
	double fval;
	double vval[4];
	std::string str;
};

enum { T_STR, T_INT, T_FLT, T_VEC };

struct Doc {
	std::vector<XNode> nodes;
	std::vector<XAttr> attrs;
	std::string err;

	static bool eq(const char *s, int n, const char *lit)
	{
		int l = (int)strlen(lit);
		return l == n && memcmp(s, lit, n) == 0;
	}
	bool is(int node, const char *lit) const { return eq(nodes[node].name, nodes[node].nlen, lit); }

	const XAttr *attr(int node, const char *name) const
	{
		const XNode &n = nodes[node];
		for(int i = 0; i < n.nattr; i++) {
			const XAttr &a = attrs[n.attr0 + i];
			if(eq(a.name, a.nlen, name)) return &a;
		}
		return 0;
	}

	static std::string decode(const char *v, int n)
	{
		std::string s(v, n);
		if(s.find('&') == std::string::npos) return s;
		std::string o;
		for(size_t i = 0; i < s.size(); i++) {
			if(s[i] == '&') {
				size_t semi = s.find(';', i);
				if(semi != std::string::npos) {
					std::string e = s.substr(i + 1, semi - i - 1);
					const char *r = e == "lt" ? "<" : e == "gt" ? ">" : e == "amp" ? "&" : e == "quot" ? "\"" : e == "apos" ? "'" : 0;
					if(r) { o += r; i = semi; continue; }
				}
			}
			o += s[i];
		}
		return o;
	}

	/* xml_create_attr typing (src/xmltree.c:75-93); numbers are stored as
	 * float, as struct xml_attr holds them (src/xmltree.h:31-33) */
	static bool typed(const XAttr *a, Typed *t)
	{
		if(!a) return false;
		t->str = decode(a->val, a->vlen);
		const char *val = t->str.c_str();
		t->type = T_STR;
		t->ival = 0;
		t->fval = 0.0;
		t->vval[0] = t->vval[1] = t->vval[2] = t->vval[3] = 0.0;
		if(isdigit((unsigned char)val[0]) || ((val[0] == '+' || val[0] == '-') && isdigit((unsigned char)val[1]))) {
			t->type = strchr(val, '.') ? T_FLT : T_INT;
			t->ival = atoi(val);
			t->fval = (float)strtod(val, 0);
			t->vval[0] = t->vval[1] = t->vval[2] = t->vval[3] = 1.0;
			int i;
			for(i = 0; i < 4; i++) {
				if(!*val) break;
				t->vval[i] = (float)strtod(val, 0);
				while(*val && !isspace((unsigned char)*val)) val++;
				while(*val && isspace((unsigned char)*val)) val++;
			}
			if(i > 1) t->type = T_VEC;
		}
		return true;
	}

	/* fast path for the mesh elements: integer attribute (id / vref indices) */
	static bool int_attr(const XAttr *a, int *out)
	{
		if(!a || a->vlen <= 0) return false;
		const char *v = a->val;
		if(!(isdigit((unsigned char)v[0]) || ((v[0] == '+' || v[0] == '-') && a->vlen > 1 && isdigit((unsigned char)v[1])))) return false;
		for(int i = 0; i < a->vlen; i++) {
			if(v[i] == '.') return false;
			if(isspace((unsigned char)v[i])) {
				/* more than one number makes it a vector */
				for(int j = i; j < a->vlen; j++) if(!isspace((unsigned char)v[j])) return false;
				break;
			}
		}
		*out = atoi(v);
		return true;
	}

	bool skip_mesh = false;   /* leave the children of <mesh> elements unparsed */

	bool parse(const char *p, size_t len)
	{
		const char *end = p + len;
		std::vector<int> stack;
		nodes.reserve(len / 48 + 16);
		attrs.reserve(len / 40 + 16);
		while(p < end) {
			while(p < end && *p != '<') p++;
			if(p >= end) break;
			if(p + 3 < end && p[1] == '!' && p[2] == '-' && p[3] == '-') {
				const char *e = p + 4;
				while(e + 2 < end && !(e[0] == '-' && e[1] == '-' && e[2] == '>')) e++;
				if(e + 2 >= end) { err = "unterminated comment"; return false; }
				p = e + 3;
				continue;
			}
			if(p + 1 < end && (p[1] == '?' || p[1] == '!')) {
				while(p < end && *p != '>') p++;
				p++;
				continue;
			}
			if(p + 1 < end && p[1] == '/') {
				p += 2;
				const char *ns = p;
				while(p < end && *p != '>' && !isspace((unsigned char)*p)) p++;
				if(stack.empty()) { err = "unbalanced closing tag"; return false; }
				const XNode &top = nodes[stack.back()];
				if(top.nlen != (int)(p - ns) || memcmp(top.name, ns, top.nlen) != 0) {
					err = "mismatched closing tag </" + std::string(ns, p - ns) + ">";
					return false;
				}
				while(p < end && *p != '>') p++;
				p++;
				stack.pop_back();
				continue;
			}
			p++;
			XNode n;
			n.name = p;
			while(p < end && !isspace((unsigned char)*p) && *p != '/' && *p != '>') p++;
			n.nlen = (int)(p - n.name);
			n.attr0 = (int)attrs.size();
			n.nattr = 0;
			bool selfclose = false;
			for(;;) {
				while(p < end && isspace((unsigned char)*p)) p++;
				if(p >= end) { err = "unexpected end of document in a tag"; return false; }
				if(*p == '/') {
					if(p + 1 < end && p[1] == '>') { p += 2; selfclose = true; break; }
					err = "malformed tag";
					return false;
				}
				if(*p == '>') { p++; break; }
				XAttr a;
				a.name = p;
				while(p < end && *p != '=' && !isspace((unsigned char)*p)) p++;
				a.nlen = (int)(p - a.name);
				while(p < end && isspace((unsigned char)*p)) p++;
				if(p >= end || *p != '=') { err = "attribute without value"; return false; }
				p++;
				while(p < end && isspace((unsigned char)*p)) p++;
				if(p >= end || (*p != '"' && *p != '\'')) { err = "unquoted attribute value"; return false; }
				char q = *p++;
				a.val = p;
				while(p < end && *p != q) p++;
				if(p >= end) { err = "unterminated attribute value"; return false; }
				a.vlen = (int)(p - a.val);
				p++;
				attrs.push_back(a);
				n.nattr++;
			}
			int id = (int)nodes.size();
			nodes.push_back(n);
			if(!stack.empty()) {
				XNode &par = nodes[stack.back()];
				if(par.last_child < 0) par.first_child = id;
				else nodes[par.last_child].next = id;
				par.last_child = id;
			} else if(id != 0) {
				err = "more than one root element";
				return false;
			}
			if(!selfclose && skip_mesh && eq(n.name, n.nlen, "mesh")) {
				/* the mesh's elements come from the side-car: jump past </mesh> */
				static const char close[] = "</mesh";
				const char *c = std::search(p, end, close, close + 6);
				if(c >= end) { err = "unterminated <mesh>"; return false; }
				p = c + 6;
				while(p < end && *p != '>') p++;
				p++;
				continue;
			}
			if(!selfclose) stack.push_back(id);
		}
		if(nodes.empty()) { err = "no root element"; return false; }
		if(!stack.empty()) { err = "unexpected end of document"; return false; }
		return true;
	}
};

}  // namespace

/* ------------------------------------------------------------------ */
/* keyframe tracks (src/anim.inl:70-263)                                */
/* ------------------------------------------------------------------ */
static_assert(sizeof(Vec3) == 3 * sizeof(double) && sizeof(Quat) == 4 * sizeof(double), "track values are packed doubles");

/* a track as the flat view the shared evaluator reads */
template <class T> static KeyView key_view(const Track<T> &tr)
{
	KeyView k;
	k.time = tr.time.data();
	k.val = reinterpret_cast<const double *>(tr.val.data());
	k.def = reinterpret_cast<const double *>(&tr.def);
	k.n = (int)tr.time.size();
	k.dim = (int)(sizeof(T) / sizeof(double));
	k.interp = tr.interp;
	k.extrap = tr.extrap;
	return k;
}

template <class T> static void set_key(Track<T> &tr, int time, const T &v)
{
	if(!tr.time.empty()) {
		int n = key_nearest(tr.time.data(), 0, (int)tr.time.size() - 1, time);
		if(tr.time[n] == time) { tr.val[n] = v; return; }
	}
	size_t pos = std::upper_bound(tr.time.begin(), tr.time.end(), time) - tr.time.begin();
	tr.time.insert(tr.time.begin() + pos, time);
	tr.val.insert(tr.val.begin() + pos, v);
}

static Vec3 eval_vec(const Track<Vec3> &tr, int t)
{
	double o[3];
	key_eval(key_view(tr), t, o);
	return Vec3(o[0], o[1], o[2]);
}

/* ------------------------------------------------------------------ */
/* 4x4 matrices (row-major, column vectors)                             */
/* ------------------------------------------------------------------ */
void mat_inverse(double out[4][4], const double m[4][4]) { m4_inverse(out, m); }
static Vec3 m_pt(const double m[4][4], const Vec3 &p)
{
	return Vec3(m[0][0] * p.x + m[0][1] * p.y + m[0][2] * p.z + m[0][3],
			m[1][0] * p.x + m[1][1] * p.y + m[1][2] * p.z + m[1][3],
			m[2][0] * p.x + m[2][1] * p.y + m[2][2] * p.z + m[2][3]);
}

XForm::XForm()
{
	pos.def = Vec3(0, 0, 0);
	scale.def = Vec3(1, 1, 1);
	Quat id = {1, 0, 0, 0};
	rot.def = id;
}
Vec3 XForm::position(int t) const { return eval_vec(pos, t); }
Vec3 XForm::scaling(int t) const { return eval_vec(scale, t); }

/* XFormNode::get_xform_matrix: pivot * T * R * S * -pivot (src/anim.cc:391-419) */
void XForm::matrix(int t, double m[4][4]) const
{
	double p[3], q[4], s[3], pv[3] = {pivot.x, pivot.y, pivot.z};
	key_eval(key_view(pos), t, p);
	key_eval(key_view(rot), t, q);
	key_eval(key_view(scale), t, s);
	node_matrix(p, q, s, pv, m);
}

static double v_len(const Vec3 &v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
static Vec3 v_cross(const Vec3 &a, const Vec3 &b)
{
	return Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static Vec3 v_norm(const Vec3 &v) { double l = v_len(v); return Vec3(v.x / l, v.y / l, v.z / l); }

/* TargetCamera::get_matrix (src/camera.cc:216-234) */
void Camera::matrix(int t, double m[4][4]) const
{
	if(!target) {
		xf.matrix(t, m);
		return;
	}
	Vec3 p = xf.position(t), tg = txf.position(t);
	Vec3 up(0, 1, 0);
	Vec3 dir = v_norm(Vec3(tg.x - p.x, tg.y - p.y, tg.z - p.z));
	Vec3 right = v_norm(v_cross(up, dir));
	up = v_cross(dir, right);
	double roll = txf.scaling(t).x;
	double half = roll * 0.5, sn = sin(half);
	double q[4] = {cos(half), dir.x * sn, dir.y * sn, dir.z * sn};
	double rm[4][4];
	m4_quat(rm, q);
	Vec3 u(rm[0][0] * up.x + rm[0][1] * up.y + rm[0][2] * up.z, rm[1][0] * up.x + rm[1][1] * up.y + rm[1][2] * up.z,
			rm[2][0] * up.x + rm[2][1] * up.y + rm[2][2] * up.z);
	Vec3 r(rm[0][0] * right.x + rm[0][1] * right.y + rm[0][2] * right.z, rm[1][0] * right.x + rm[1][1] * right.y + rm[1][2] * right.z,
			rm[2][0] * right.x + rm[2][1] * right.y + rm[2][2] * right.z);
	m4_ident(m);
	m[0][0] = r.x; m[0][1] = u.x; m[0][2] = dir.x; m[0][3] = p.x;
	m[1][0] = r.y; m[1][1] = u.y; m[1][2] = dir.y; m[1][3] = p.y;
	m[2][0] = r.z; m[2][1] = u.z; m[2][2] = dir.z; m[2][3] = p.z;
}

/* ------------------------------------------------------------------ */
/* bounds and octree                                                     */
/* ------------------------------------------------------------------ */
Box Object::bounds(const std::vector<Mesh> &meshes, int t) const
{
	if(is_static) return static_box;
	Box b;
	double m[4][4];
	xf.matrix(t, m);
	if(type == OBJ_SPHERE) {
		Vec3 c = m_pt(m, Vec3(0, 0, 0));
		for(int i = 0; i < 3; i++) { b.mn[i] = c[i] - rad; b.mx[i] = c[i] + rad; }
	} else if(type == OBJ_CYLINDER) {
		Vec3 s1 = m_pt(m, Vec3(0, start, 0)), s2 = m_pt(m, Vec3(0, end, 0));
		for(int i = 0; i < 3; i++) {
			double a0 = s1[i] - rad, a1 = s2[i] - rad, c0 = s1[i] + rad, c1 = s2[i] + rad;
			b.mn[i] = a0 < a1 ? a0 : a1;
			b.mx[i] = c0 > c1 ? c0 : c1;
		}
	} else {
		for(int i = 0; i < 3; i++) { b.mn[i] = FLT_MAX; b.mx[i] = -FLT_MAX; }
		const Mesh &me = meshes[mesh];
		size_t nv = me.posd.size() / 3;
		for(size_t v = 0; v < nv; v++) {
			Vec3 p = m_pt(m, Vec3(me.posd[v * 3], me.posd[v * 3 + 1], me.posd[v * 3 + 2]));
			for(int i = 0; i < 3; i++) {
				if(p[i] < b.mn[i]) b.mn[i] = p[i];
				if(p[i] > b.mx[i]) b.mx[i] = p[i];
			}
		}
	}
	return b;
}

static inline bool overlap(const Box &a, const Box &b)
{
	for(int i = 0; i < 3; i++) if(a.mn[i] > b.mx[i] || b.mn[i] > a.mx[i]) return false;
	return true;
}

namespace {
struct OctBuilder {
	BuildOctree *o;
	const std::vector<Box> *boxes;
	int max_depth, max_items;

	void subdivide(int ni, int lvl)
	{
		if((int)o->nodes[ni].items.size() <= max_items || lvl >= max_depth) return;
		Box b = o->nodes[ni].box;
		double c[3];
		for(int i = 0; i < 3; i++) c[i] = (b.mn[i] + b.mx[i]) * 0.5;
		/* child layout of src/octree.inl:160-168 */
		static const int hi[8][3] = {{0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1}};
		int first = (int)o->nodes.size();
		o->nodes.resize(first + 8);
		o->nodes[ni].child = first;
		for(int k = 0; k < 8; k++) {
			BuildOctree::Node &ch = o->nodes[first + k];
			for(int i = 0; i < 3; i++) {
				ch.box.mn[i] = hi[k][i] ? c[i] : b.mn[i];
				ch.box.mx[i] = hi[k][i] ? b.mx[i] : c[i];
			}
			const std::vector<int> &pit = o->nodes[ni].items;
			std::vector<int> it;
			for(size_t j = 0; j < pit.size(); j++) if(overlap((*boxes)[pit[j]], ch.box)) it.push_back(pit[j]);
			o->nodes[first + k].items.swap(it);
			subdivide(first + k, lvl + 1);
		}
		std::vector<int>().swap(o->nodes[ni].items);
	}
};
}  // namespace

void BuildOctree::build(const std::vector<Box> &boxes, int max_depth, int max_items)
{
	nodes.clear();
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
	OctBuilder b;
	b.o = this;
	b.boxes = &boxes;
	b.max_depth = max_depth;
	b.max_items = max_items;
	if((int)boxes.size() > max_items) b.subdivide(0, 0);
}

/* device child slot of the reference's child k (src/octree.inl:160-168):
 * slot bits are x | y << 1 | z << 2 of the child's half-space */
static const int child_slot[8] = {0, 1, 3, 2, 4, 5, 7, 6};

void flatten_octree(const BuildOctree &oct, std::vector<DevNode> &out, std::vector<int> &slots, std::vector<int> *index_of)
{
	if(oct.nodes.empty()) return;
	/* pad so the root sits at index 7 mod 8: every group of 8 siblings
	 * (384 bytes) then starts on a 128-byte line */
	while((out.size() & 7) != 7) {
		DevNode pad;
		memset(&pad, 0, sizeof pad);
		out.push_back(pad);
	}
	size_t base = out.size();
	/* breadth-first renumbering: children of a node stay consecutive */
	std::vector<int> order;
	order.reserve(oct.nodes.size());
	std::vector<int> newidx(oct.nodes.size(), -1);
	order.push_back(0);
	newidx[0] = 0;
	for(size_t q = 0; q < order.size(); q++) {
		int n = order[q];
		int c = oct.nodes[n].child;
		if(c >= 0) {
			size_t g = order.size();
			order.resize(g + 8);
			for(int k = 0; k < 8; k++) {
				newidx[c + k] = (int)(g + child_slot[k]);
				order[g + child_slot[k]] = c + k;
			}
		}
	}
	out.resize(base + order.size());
	for(size_t q = 0; q < order.size(); q++) {
		const BuildOctree::Node &n = oct.nodes[order[q]];
		DevNode &d = out[base + q];
		for(int i = 0; i < 3; i++) { d.mn[i] = (float)n.box.mn[i]; d.mx[i] = (float)n.box.mx[i]; d.mid[i] = 0.0f; }
		d.mask = 0;
		if(n.child >= 0) {
			d.first = (int)base + newidx[n.child];
			d.count = -1;
			/* the children's bounds are mn/centre/mx of this box, rounded the
			 * same way as the boxes the builder gave them */
			for(int i = 0; i < 3; i++) d.mid[i] = (float)((n.box.mn[i] + n.box.mx[i]) * 0.5);
			for(int k = 0; k < 8; k++) {
				const BuildOctree::Node &c = oct.nodes[n.child + k];
				if(c.child >= 0 || !c.items.empty()) d.mask |= 1u << child_slot[k];
			}
		} else {
			d.first = (int)slots.size();
			d.count = (int)n.items.size();
			slots.insert(slots.end(), n.items.begin(), n.items.end());
		}
	}
	if(index_of) {
		index_of->assign(oct.nodes.size(), -1);
		for(size_t q = 0; q < order.size(); q++) (*index_of)[order[q]] = (int)(base + q);
	}
}

static int octree_home(const BuildOctree &oct, const Box &b, const std::vector<int> &index_of)
{
	/* descend while exactly one child takes the item (the builder's overlap
	 * rule decides which children list it) */
	int n = 0;
	for(;;) {
		int c = oct.nodes[n].child;
		if(c < 0) break;
		int only = -1, hits = 0;
		for(int k = 0; k < 8; k++) {
			if(overlap(b, oct.nodes[c + k].box)) {
				hits++;
				only = c + k;
			}
		}
		if(hits != 1) break;
		n = only;
	}
	return index_of[n];
}

void octree_homes_boxes(const BuildOctree &oct, const std::vector<Box> &boxes, const std::vector<int> &index_of,
		std::vector<int> &home)
{
	home.assign(boxes.size(), -1);
	if(oct.nodes.empty()) return;
	for(size_t i = 0; i < boxes.size(); i++) home[i] = octree_home(oct, boxes[i], index_of);
}

void octree_homes(const BuildOctree &oct, const std::vector<double> &posd, const std::vector<int> &index_of,
		std::vector<int> &home)
{
	size_t nf = posd.size() / 9;
	home.assign(nf, -1);
	if(oct.nodes.empty()) return;
	for(size_t f = 0; f < nf; f++) {
		Box b;
		for(int k = 0; k < 3; k++) { b.mn[k] = FLT_MAX; b.mx[k] = -FLT_MAX; }
		for(int v = 0; v < 3; v++) {
			for(int k = 0; k < 3; k++) {
				double c = posd[f * 9 + v * 3 + k];
				if(c < b.mn[k]) b.mn[k] = c;
				if(c > b.mx[k]) b.mx[k] = c;
			}
		}
		home[f] = octree_home(oct, b, index_of);
	}
}

/* ------------------------------------------------------------------ */
/* projection maps                                                       */
/* ------------------------------------------------------------------ */
ProjMap::ProjMap()
{
	cells.assign(udiv * vdiv, 0);
	cell_area.resize(udiv * vdiv);
	total_area = 0.0;
	for(int i = 0; i < udiv * vdiv; i++) {
		int uc = i % udiv, vc = i / udiv;
		double c[4][3];
		for(int j = 0; j < 4; j++) corner_dir(uc, vc, j, c[j]);
		Vec3 v0(c[0][0], c[0][1], c[0][2]), v1(c[1][0], c[1][1], c[1][2]);
		Vec3 v2(c[2][0], c[2][1], c[2][2]), v3(c[3][0], c[3][1], c[3][2]);
		Vec3 e1(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z), e2(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z);
		Vec3 e3(v3.x - v0.x, v3.y - v0.y, v3.z - v0.z);
		double area = v_len(v_cross(e1, e2)) * 0.5;
		area += v_len(v_cross(e2, e3)) * 0.5;
		cell_area[i] = area;
		total_area += area;
	}
}

/* ProjMap::cell_corner_dir (src/projmap.cc:124-140); the 64x32 grid's corner
 * directions are computed once and reused (same values every call) */
static void corner_dir_eval(int udiv, int vdiv, int uc, int vc, int corner, double out[3])
{
	static const int offs[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
	double du = 1.0 / udiv, dv = 1.0 / vdiv;
	double u = (uc + offs[corner][0]) * du, v = (vc + offs[corner][1]) * dv;
	double theta = u * M_PI * 2.0, phi = v * M_PI;
	out[0] = 1.0 * cos(theta) * sin(phi);
	out[1] = 1.0 * cos(phi);
	out[2] = 1.0 * sin(theta) * sin(phi);
}

struct CornerTable {
	double d[64 * 32][4][3];
	CornerTable()
	{
		for(int i = 0; i < 64 * 32; i++)
			for(int k = 0; k < 4; k++) corner_dir_eval(64, 32, i % 64, i / 64, k, d[i][k]);
	}
};

static const CornerTable &corner_table()
{
	static const CornerTable *t = new CornerTable();
	return *t;
}

void ProjMap::corner_dir(int uc, int vc, int corner, double out[3]) const
{
	if(udiv == 64 && vdiv == 32) {
		const double *c = corner_table().d[vc * 64 + uc][corner];
		out[0] = c[0]; out[1] = c[1]; out[2] = c[2];
		return;
	}
	corner_dir_eval(udiv, vdiv, uc, vc, corner, out);
}

void ProjMap::cell_from_dir(const double d[3], int *uc, int *vc) const
{
	double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
	double theta = atan2(d[2], d[0]);
	double phi = acos(d[1] / r);
	if(theta < 0.0) theta = M_PI * 2.0 + theta;
	double u = theta / (M_PI * 2.0), v = phi / M_PI;
	int a = (int)(u * udiv), b = (int)(v * vdiv);
	*uc = a < 0 ? 0 : (a >= udiv ? udiv - 1 : a);
	*vc = b < 0 ? 0 : (b >= vdiv ? vdiv - 1 : b);
}

void ProjMap::set_cell(int uc, int vc, bool val)
{
	int idx = vc * udiv + uc;
	if((bool)cells[idx] != val) {
		double change = cell_area[idx] / total_area;
		coverage += val ? change : -change;
	}
	cells[idx] = val;
}

void ProjMap::set_all(bool v) { std::fill(cells.begin(), cells.end(), v ? 1 : 0); coverage = v ? 1.0 : 0.0; }
void ProjMap::clear() { set_all(false); }
double ProjMap::get_coverage() const { return coverage < 0.0 ? 0.0 : (coverage > 1.0 ? 1.0 : coverage); }

/* Candidate columns/rows of the 64x32 grid for one box: every cell with a
 * corner inside the box's bounding sphere (seen from the light) lies in the
 * spherical cap of angular radius t around the sphere's direction, since the
 * corner test |lpos + c d - ctr|^2 <= r^2 with |c| = 1, d = |ctr - lpos| is
 * c . v^ >= 1 - r^2 / (2 d^2).  The cap is bounded in colatitude by t and in
 * azimuth by asin(sin t / sin phi); one cell and 0.02 rad of margin are added,
 * and the exact corner test of the reference decides inside the candidates. */
static bool cap_candidates(const double v[3], double objdist, double rad_sq, int *vc0, int *vc1, bool cols[64])
{
	double cos_t = 1.0 - rad_sq / (2.0 * objdist * objdist);
	if(cos_t <= -1.0 + 1e-9) return false;
	double t = acos(cos_t < 1.0 ? cos_t : 1.0) + 0.02;
	double phi0 = acos(v[1] / objdist);
	double theta0 = atan2(v[2], v[0]);
	if(theta0 < 0.0) theta0 += 2.0 * M_PI;
	double dv = M_PI / 32.0, du = 2.0 * M_PI / 64.0;
	double plo = phi0 - t, phi_hi = phi0 + t;
	int a = (int)floor(plo / dv) - 1, b = (int)floor(phi_hi / dv) + 1;
	*vc0 = a < 0 ? 0 : a;
	*vc1 = b > 31 ? 31 : b;
	if(plo <= 0.0 || phi_hi >= M_PI) {
		for(int k = 0; k < 64; k++) cols[k] = true;
		return true;
	}
	double smin = sin(plo) < sin(phi_hi) ? sin(plo) : sin(phi_hi);
	double st = sin(t);
	if(st >= smin) {
		for(int k = 0; k < 64; k++) cols[k] = true;
		return true;
	}
	double dmax = asin(st / smin) + 0.02;
	for(int k = 0; k < 64; k++) cols[k] = false;
	int u0 = (int)floor((theta0 - dmax) / du) - 1, u1 = (int)floor((theta0 + dmax) / du) + 1;
	if(u1 - u0 >= 63) {
		for(int k = 0; k < 64; k++) cols[k] = true;
		return true;
	}
	for(int u = u0; u <= u1; u++) cols[((u % 64) + 64) % 64] = true;
	return true;
}

/* ::build_projmap (src/light.cc:392-432) */
static void project_boxes(ProjMap *map, const Vec3 &lpos, const std::vector<Box> &boxes)
{
	for(size_t i = 0; i < boxes.size(); i++) {
		const Box &b = boxes[i];
		if(lpos.x >= b.mn[0] && lpos.y >= b.mn[1] && lpos.z >= b.mn[2] && lpos.x < b.mx[0] && lpos.y < b.mx[1] && lpos.z < b.mx[2]) {
			map->set_all(true);
			return;
		}
		Vec3 ctr((b.mn[0] + b.mx[0]) / 2.0, (b.mn[1] + b.mx[1]) / 2.0, (b.mn[2] + b.mx[2]) / 2.0);
		Vec3 dm(b.mn[0] - ctr.x, b.mn[1] - ctr.y, b.mn[2] - ctr.z);
		double rad_sq = dm.x * dm.x + dm.y * dm.y + dm.z * dm.z;
		double v[3] = {ctr.x - lpos.x, ctr.y - lpos.y, ctr.z - lpos.z};
		double objdist = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
		int uc, vc;
		map->cell_from_dir(v, &uc, &vc);
		map->set_cell(uc, vc, true);
		int vc0 = 0, vc1 = map->vdiv - 1;
		bool cols[64];
		bool limited = map->udiv == 64 && map->vdiv == 32 && objdist > 0.0 && cap_candidates(v, objdist, rad_sq, &vc0, &vc1, cols);
		for(int row = vc0; row <= vc1; row++) {
			for(int col = 0; col < map->udiv; col++) {
				if(limited && !cols[col]) continue;
				for(int k = 0; k < 4; k++) {
					double cd[3];
					map->corner_dir(col, row, k, cd);
					double px = lpos.x + cd[0] * objdist, py = lpos.y + cd[1] * objdist, pz = lpos.z + cd[2] * objdist;
					double dx = px - ctr.x, dy = py - ctr.y, dz = pz - ctr.z;
					if(dx * dx + dy * dy + dz * dz <= rad_sq) {
						map->set_cell(col, row, true);
						break;
					}
				}
			}
		}
	}
}

/* Light::build_proj_intern (src/light.cc:151-200); light samples on the
 * projection-map stream of the light */
void HostScene::build_projmaps(int t0, int t1, uint64_t seed, int light0, int nlight, int obj0, int nobj)
{
	if(nlight < 0) nlight = (int)lights.size() - light0;
	if(nobj < 0) nobj = (int)objs.size() - obj0;
	/* each light's maps depend only on its own random stream: one thread per light */
	std::vector<std::thread> th;
	for(int k = 0; k < nlight; k++)
		th.push_back(std::thread([this, light0, k, t0, t1, seed, obj0, nobj]() { build_light_projmaps(light0 + k, t0, t1, seed, k, obj0, nobj); }));
	for(auto &t : th) t.join();
}

void HostScene::build_light_projmaps(size_t li, int t0, int t1, uint64_t seed, int key, int obj0, int nobj)
{
	light_projmaps(li, t0, t1, seed, key, obj0, nobj, lights[li].pm, lights[li].spm);
}

void HostScene::light_projmaps(size_t li, int t0, int t1, uint64_t seed, int key, int obj0, int nobj, ProjMap &pm, ProjMap &spm) const
{
	{
		const Light &L = lights[li];
		pm.clear();
		spm.clear();
		if(nobj <= 0) return;
		int tm[3] = {t0, t1, -1};
		if(t0 == t1) tm[1] = -1;
		int samples = L.type == LT_SPHERE ? 8 : 1;
		/* one stream per light, drawn in order over both shutter ends */
		sray_rng s;
		sray_rng_init(&s, seed, SRAY_DOM_PROJMAP, (uint32_t)key, 0);
		for(int ti = 0; ti < 2 && tm[ti] != -1; ti++) {
			std::vector<Box> boxes((size_t)nobj), cboxes;
			for(int j = 0; j < nobj; j++) {
				size_t i = (size_t)(obj0 + j);
				const Material &m = objs[i].mat >= 0 ? mats[objs[i].mat] : defmat;
				boxes[j] = object_bounds(i, tm[ti]);
				if(m.refl > 0.0 || m.refr > 0.0) cboxes.push_back(boxes[j]);
			}
			for(int k = 0; k < samples; k++) {
				Vec3 lp = L.xf.position(tm[ti]);
				if(L.type == LT_SPHERE) {
					double u0 = sray_rng_uniform_d(&s), u1 = sray_rng_uniform_d(&s);
					double z = 2.0 * u1 - 1.0, sxy = sqrt(1.0 - z * z), ang = 2.0 * M_PI * u0;
					double r = (double)L.radius;
					lp = Vec3(lp.x + r * cos(ang) * sxy, lp.y + r * sin(ang) * sxy, lp.z + r * z);
				} else if(L.type == LT_BOX) {
					double m0[4][4];
					L.xf.matrix(0, m0);
					Vec3 v;
					v.x = L.dim.x * sray_rng_uniform_d(&s) - 0.5 * L.dim.x;
					v.y = L.dim.y * sray_rng_uniform_d(&s) - 0.5 * L.dim.y;
					v.z = L.dim.z * sray_rng_uniform_d(&s) - 0.5 * L.dim.z;
					lp = m_pt(m0, v);
				}
				project_boxes(&pm, lp, boxes);
				project_boxes(&spm, lp, cboxes);
			}
		}
	}
}

Box HostScene::object_bounds(size_t i, int t) const
{
	if(t == bt0 && i < box_t0.size()) return box_t0[i];
	if(t == bt1 && i < box_t1.size()) return box_t1[i];
	return objs[i].bounds(meshes, t);
}

/* Scene::build_tree (src/scene.cc:353-390) */
void HostScene::build_tree(int t0, int t1, const sray_opts &opt)
{
	std::vector<Box> boxes(objs.size());
	bt0 = t0;
	bt1 = t1;
	box_t0.resize(objs.size());
	box_t1.resize(objs.size());
	for(size_t i = 0; i < objs.size(); i++) {
		box_t0[i] = objs[i].bounds(meshes, t0);
		box_t1[i] = t1 == t0 ? box_t0[i] : objs[i].bounds(meshes, t1);
	}
	for(size_t i = 0; i < objs.size(); i++) {
		Box s = box_t0[i], e = box_t1[i];
		for(int k = 0; k < 3; k++) {
			boxes[i].mn[k] = s.mn[k] < e.mn[k] ? s.mn[k] : e.mn[k];
			boxes[i].mx[k] = s.mx[k] > e.mx[k] ? s.mx[k] : e.mx[k];
		}
	}
	oct.build(boxes, opt.scnoct_max_depth, opt.scnoct_max_items);
	oct_boxes = boxes;
	const Box &rb = oct.nodes[0].box;
	double dx = rb.mx[0] - rb.mn[0], dy = rb.mx[1] - rb.mn[1], dz = rb.mx[2] - rb.mn[2];
	gather_dist = sqrt(dx * dx + dy * dy + dz * dz) * opt.gather_dist;
}

void HostScene::bound_objects(int t0, int t1, const sray_opts &opt)
{
	bt0 = t0;
	bt1 = t1;
	box_t0.resize(objs.size());
	box_t1.resize(objs.size());
	oct_boxes.resize(objs.size());
	for(size_t i = 0; i < objs.size(); i++) {
		box_t0[i] = objs[i].bounds(meshes, t0);
		box_t1[i] = t1 == t0 ? box_t0[i] : objs[i].bounds(meshes, t1);
		for(int k = 0; k < 3; k++) {
			oct_boxes[i].mn[k] = std::min(box_t0[i].mn[k], box_t1[i].mn[k]);
			oct_boxes[i].mx[k] = std::max(box_t0[i].mx[k], box_t1[i].mx[k]);
		}
	}
	oct.nodes.assign(1, BuildOctree::Node());
	oct.nodes[0].box = box_at(t0, t1);
	const Box &rb = oct.nodes[0].box;
	double dx = rb.mx[0] - rb.mn[0], dy = rb.mx[1] - rb.mn[1], dz = rb.mx[2] - rb.mn[2];
	gather_dist = sqrt(dx * dx + dy * dy + dz * dz) * opt.gather_dist;
}

/* the root box of Scene::build_tree(t0, t1) (src/scene.cc:353-390): the
 * union of every object's bounds at t0 and t1 */
Box HostScene::box_at(int t0, int t1, int obj0, int nobj) const
{
	if(nobj < 0) nobj = (int)objs.size() - obj0;
	Box u;
	for(int k = 0; k < 3; k++) { u.mn[k] = FLT_MAX; u.mx[k] = -FLT_MAX; }
	for(size_t i = (size_t)obj0; i < (size_t)(obj0 + nobj); i++) {
		Box b[2] = {object_bounds(i, t0), t1 == t0 ? object_bounds(i, t0) : object_bounds(i, t1)};
		for(int j = 0; j < 2; j++)
			for(int k = 0; k < 3; k++) {
				if(b[j].mn[k] < u.mn[k]) u.mn[k] = b[j].mn[k];
				if(b[j].mx[k] > u.mx[k]) u.mx[k] = b[j].mx[k];
			}
	}
	return u;
}

/* gather_dist of Scene::build_tree(t0, t1) (src/scene.cc:384-387): the
 * diagonal of the root box times the option */
double HostScene::gather_dist_at(int t0, int t1, const sray_opts &opt, int obj0, int nobj) const
{
	Box b = box_at(t0, t1, obj0, nobj);
	double dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
	return sqrt(dx * dx + dy * dy + dz * dz) * opt.gather_dist;
}

/* ------------------------------------------------------------------ */
/* loading                                                               */
/* ------------------------------------------------------------------ */
static uint64_t fnv(const void *p, size_t n, uint64_t h)
{
	const unsigned char *c = (const unsigned char *)p;
	for(size_t i = 0; i < n; i++) { h ^= c[i]; h *= 0x100000001b3ull; }
	return h;
}

namespace {
struct Loader {
	const Doc &d;
	HostScene &sc;
	const sray_opts &opt;
	std::string &err;
	const std::vector<int> *sidecar_mesh = nullptr;   /* unique mesh of each mesh object, in document order */
	size_t mesh_objects = 0;
	std::vector<int> mesh_of_object;                  /* filled while loading (for writing a side-car) */

	void load_xform(int n, XForm &xf)
	{
		Typed t;
		int msec = 0;
		if(Doc::typed(d.attr(n, "interpolate"), &t)) {
			int v = t.str == "linear" ? INTERP_LINEAR : t.str == "step" ? INTERP_STEP : t.str == "cubic" ? INTERP_CUBIC : -1;
			if(v >= 0) xf.pos.interp = xf.rot.interp = xf.scale.interp = v;
		}
		if(Doc::typed(d.attr(n, "extrapolate"), &t)) {
			int v = t.str == "clamp" ? EXTRAP_CLAMP : t.str == "repeat" ? EXTRAP_REPEAT : t.str == "pingpong" ? EXTRAP_PINGPONG : -1;
			if(v >= 0) xf.pos.extrap = xf.rot.extrap = xf.scale.extrap = v;
		}
		if(Doc::typed(d.attr(n, "time"), &t) && t.type == T_INT) msec = t.ival;
		if(Doc::typed(d.attr(n, "pos"), &t) && t.type == T_VEC) set_key(xf.pos, msec, Vec3(t.vval[0], t.vval[1], t.vval[2]));
		if(Doc::typed(d.attr(n, "rot"), &t) && t.type == T_VEC) {
			Quat q = {t.vval[0], t.vval[1], t.vval[2], t.vval[3]};
			double l = sqrt(q.s * q.s + q.x * q.x + q.y * q.y + q.z * q.z);
			if(l > 0.0) { q.s /= l; q.x /= l; q.y /= l; q.z /= l; }
			set_key(xf.rot, msec, q);
		}
		if(Doc::typed(d.attr(n, "axisrot"), &t) && t.type == T_VEC) {
			double ang = (t.vval[0] * M_PI) / 180.0, half = ang * 0.5, sn = sin(half);
			Quat q = {cos(half), t.vval[1] * sn, t.vval[2] * sn, t.vval[3] * sn};
			set_key(xf.rot, msec, q);
		}
		if(Doc::typed(d.attr(n, "scale"), &t) && t.type == T_VEC) set_key(xf.scale, msec, Vec3(t.vval[0], t.vval[1], t.vval[2]));
		if(Doc::typed(d.attr(n, "pivot"), &t) && t.type == T_VEC) xf.pivot = Vec3(t.vval[0], t.vval[1], t.vval[2]);
	}

	bool load_material(int n)
	{
		Material m;
		Typed t;
		if(!Doc::typed(d.attr(n, "name"), &t)) { err = "invalid material: name attribute not found"; return false; }
		m.name = t.str;
		if(Doc::typed(d.attr(n, "shader"), &t)) m.phong = t.str == "phong";
		for(int c = d.nodes[n].first_child; c >= 0; c = d.nodes[c].next) {
			if(!d.is(c, "mattr")) continue;
			Typed an, av;
			if(!Doc::typed(d.attr(c, "name"), &an) || !Doc::typed(d.attr(c, "value"), &av)) continue;
			double col[4];
			if(av.type == T_VEC) { col[0] = av.vval[0]; col[1] = av.vval[1]; col[2] = av.vval[2]; col[3] = 1.0; }
			else if(av.type == T_FLT || av.type == T_INT) { col[0] = col[1] = col[2] = av.fval; col[3] = 1.0; }
			else continue;
			/* a "map" loads a texture of its own; one that fails to load
			 * leaves the attribute untextured (src/material.cc:64-72) */
			int tex = -1;
			Typed am;
			if(Doc::typed(d.attr(c, "map"), &am)) {
				Texture tx;
				if(load_texture(am.str.c_str(), tx)) {
					tex = (int)sc.texs.size();
					sc.texs.push_back(std::move(tx));
				} else {
					fprintf(stderr, "failed to load texture: %s\n", am.str.c_str());
				}
			}
			/* set_attribute replaces the colour and the texture (src/material.cc:140-151) */
			if(an.str == "diffuse") { memcpy(m.kd, col, sizeof col); m.tex[TA_DIFFUSE] = tex; }
			else if(an.str == "specular") { memcpy(m.ks, col, sizeof col); m.tex[TA_SPECULAR] = tex; }
			else if(an.str == "shininess") { m.shin = col[0]; m.tex[TA_SHININESS] = tex; }
			else if(an.str == "reflect") { m.refl = col[0]; m.tex[TA_REFLECT] = tex; }
			else if(an.str == "refract") { m.refr = col[0]; m.tex[TA_REFRACT] = tex; }
			else if(an.str == "ior") { m.ior = col[0]; m.tex[TA_IOR] = tex; }
			else if(an.str == "normal") { m.have_normal = true; m.nrm_scale = col[0]; m.tex[TA_NORMAL] = tex; }
		}
		sc.mats.push_back(m);
		return true;
	}

	bool read_vec(int n, double v[3])
	{
		const XAttr *a = d.attr(n, "val");
		if(!a) return false;
		/* numeric vector: at least two numbers (src/xmltree.c:75-93) */
		const char *p = a->val, *e = a->val + a->vlen;
		if(!(isdigit((unsigned char)p[0]) || ((p[0] == '+' || p[0] == '-') && isdigit((unsigned char)p[1])))) return false;
		double vv[4] = {1, 1, 1, 1};
		int i;
		char buf[128];
		int len = a->vlen < 127 ? a->vlen : 127;
		memcpy(buf, p, len);
		buf[len] = 0;
		const char *q = buf;
		for(i = 0; i < 4; i++) {
			if(!*q) break;
			vv[i] = (float)strtod(q, 0);
			while(*q && !isspace((unsigned char)*q)) q++;
			while(*q && isspace((unsigned char)*q)) q++;
		}
		(void)e;
		if(i < 2) return false;
		v[0] = vv[0]; v[1] = vv[1]; v[2] = vv[2];
		return true;
	}

	/* Mesh::load_xml (src/meshload.cc:55-157) */
	bool load_mesh(int objn, Object &o)
	{
		if(sidecar_mesh) {
			if(mesh_objects >= sidecar_mesh->size()) { err = "side-car holds fewer meshes than the document"; return false; }
			o.mesh = (*sidecar_mesh)[mesh_objects++];
			sc.n_tris += (int64_t)(sc.meshes[o.mesh].posd.size() / 9);
			return true;
		}
		bool ok = load_mesh_xml(objn, o);
		if(ok) mesh_of_object.push_back(o.mesh);
		return ok;
	}

	bool load_mesh_xml(int objn, Object &o)
	{
		int mn = -1;
		for(int c = d.nodes[objn].first_child; c >= 0; c = d.nodes[c].next) if(d.is(c, "mesh")) { mn = c; break; }
		if(mn < 0) { err = "<mesh> not found in mesh object " + o.name; return false; }
		static const char *ename[4] = {"vertex", "normal", "texcoord", "tangent"};
		struct Elem { double v[3]; int id; };
		std::vector<Elem> el[4];
		bool ordered[4] = {true, true, true, true};
		int cur[4] = {0, 0, 0, 0};
		std::vector<int> fr;   /* 12 ints per face: vertex, normal, tangent, texcoord x3 */
		for(int c = d.nodes[mn].first_child; c >= 0; c = d.nodes[c].next) {
			int e = -1;
			for(int k = 0; k < 4; k++) if(d.is(c, ename[k])) { e = k; break; }
			if(e >= 0) {
				Elem x;
				if(!Doc::int_attr(d.attr(c, "id"), &x.id)) x.id = cur[e];
				x.v[0] = x.v[1] = x.v[2] = 0.0;
				read_vec(c, x.v);
				if(x.id != cur[e]++) ordered[e] = false;
				el[e].push_back(x);
			} else if(d.is(c, "face")) {
				int f[12] = {0};
				int k = 0;
				for(int vr = d.nodes[c].first_child; vr >= 0 && k < 3; vr = d.nodes[vr].next) {
					if(!d.is(vr, "vref")) continue;
					int v;
					f[k * 4 + 0] = Doc::int_attr(d.attr(vr, "vertex"), &v) ? v : 0;
					f[k * 4 + 1] = Doc::int_attr(d.attr(vr, "normal"), &v) ? v : 0;
					f[k * 4 + 2] = Doc::int_attr(d.attr(vr, "tangent"), &v) ? v : 0;
					f[k * 4 + 3] = Doc::int_attr(d.attr(vr, "texcoord"), &v) ? v : 0;
					k++;
				}
				fr.insert(fr.end(), f, f + 12);
			}
		}
		for(int e = 0; e < 4; e++) {
			if(!ordered[e]) std::stable_sort(el[e].begin(), el[e].end(), [](const Elem &a, const Elem &b) { return a.id < b.id; });
			if(!el[e].empty() && el[e].back().id != (int)el[e].size() - 1) {
				err = "error loading mesh " + o.name + ": missing vertex elements";
				return false;
			}
		}
		size_t nf = fr.size() / 12;
		Mesh m;
		m.pos.resize(nf * 9);
		m.posd.resize(nf * 9);
		m.attr.assign(nf * 24, 0.0f);
		for(size_t i = 0; i < nf; i++) {
			for(int j = 0; j < 3; j++) {
				int vi = fr[i * 12 + j * 4], ni = fr[i * 12 + j * 4 + 1], gi = fr[i * 12 + j * 4 + 2], ti = fr[i * 12 + j * 4 + 3];
				if(vi < 0 || vi >= (int)el[0].size()) { err = "face vertex index out of range in " + o.name; return false; }
				for(int k = 0; k < 3; k++) {
					m.posd[i * 9 + j * 3 + k] = el[0][vi].v[k];
					m.pos[i * 9 + j * 3 + k] = (float)el[0][vi].v[k];
				}
				if(!el[1].empty()) {
					if(ni < 0 || ni >= (int)el[1].size()) { err = "normal index out of range in " + o.name; return false; }
					for(int k = 0; k < 3; k++) m.attr[i * 24 + j * 3 + k] = (float)el[1][ni].v[k];
				}
				if(!el[3].empty()) {
					if(gi < 0 || gi >= (int)el[3].size()) { err = "tangent index out of range in " + o.name; return false; }
					for(int k = 0; k < 3; k++) m.attr[i * 24 + 9 + j * 3 + k] = (float)el[3][gi].v[k];
				}
				if(!el[2].empty()) {
					if(ti < 0 || ti >= (int)el[2].size()) { err = "texcoord index out of range in " + o.name; return false; }
					m.attr[i * 24 + 18 + j * 2] = (float)el[2][ti].v[0];
					m.attr[i * 24 + 18 + j * 2 + 1] = (float)el[2][ti].v[1];
				}
			}
		}
		/* identical meshes share one device copy */
		uint64_t h = fnv(m.posd.data(), m.posd.size() * sizeof(double), 0xcbf29ce484222325ull);
		h = fnv(m.attr.data(), m.attr.size() * sizeof(float), h);
		for(size_t u = 0; u < sc.meshes.size(); u++) {
			if(sc.meshes[u].hash == h && sc.meshes[u].posd == m.posd && sc.meshes[u].attr == m.attr) {
				o.mesh = (int)u;
				sc.n_tris += (int64_t)nf;
				return true;
			}
		}
		m.hash = h;
		o.mesh = (int)sc.meshes.size();
		sc.meshes.push_back(std::move(m));
		sc.n_tris += (int64_t)nf;
		return true;
	}

	bool load_object(int n)
	{
		Typed t;
		if(!Doc::typed(d.attr(n, "type"), &t)) { err = "invalid object: no type attribute."; return false; }
		Object o;
		if(t.str == "sphere") o.type = OBJ_SPHERE;
		else if(t.str == "cylinder") o.type = OBJ_CYLINDER;
		else if(t.str == "mesh") o.type = OBJ_MESH;
		else { err = "invalid object: unknown type: " + t.str; return false; }
		if(Doc::typed(d.attr(n, "name"), &t)) o.name = t.str;
		bool have_shape = false;
		for(int c = d.nodes[n].first_child; c >= 0; c = d.nodes[c].next) {
			if(d.is(c, "matref")) {
				if(!Doc::typed(d.attr(c, "name"), &t)) { err = "invalid material reference in object " + o.name; return false; }
				int found = -1;
				for(size_t m = 0; m < sc.mats.size(); m++) if(sc.mats[m].name == t.str) { found = (int)m; break; }
				if(found < 0) { err = "material " + t.str + " referenced by object " + o.name + " does not exist"; return false; }
				o.mat = found;
			} else if(d.is(c, "xform")) {
				load_xform(c, o.xf);
			} else if(o.type == OBJ_SPHERE && d.is(c, "sphere")) {
				if(Doc::typed(d.attr(c, "rad"), &t)) o.rad = t.fval;
				have_shape = true;
			} else if(o.type == OBJ_CYLINDER && d.is(c, "cylinder")) {
				if(Doc::typed(d.attr(c, "rad"), &t)) o.rad = t.fval;
				if(Doc::typed(d.attr(c, "start"), &t)) o.start = t.fval;
				if(Doc::typed(d.attr(c, "end"), &t)) o.end = t.fval;
				have_shape = true;
			}
		}
		if(o.type == OBJ_MESH) {
			if(!load_mesh(n, o)) return false;
		} else if(!have_shape) {
			err = std::string(o.type == OBJ_SPHERE ? "sphere" : "cylinder") + " object " + o.name + " has no shape element";
			return false;
		}
		sc.objs.push_back(o);
		return true;
	}

	bool load_light(int n)
	{
		Typed t;
		if(!Doc::typed(d.attr(n, "type"), &t)) { err = "invalid light: no type attribute."; return false; }
		Light l;
		if(t.str == "point") l.type = LT_POINT;
		else if(t.str == "sphere") l.type = LT_SPHERE;
		else if(t.str == "box") l.type = LT_BOX;
		else { err = "invalid light: unknown type: " + t.str; return false; }
		if(Doc::typed(d.attr(n, "color"), &t)) {
			if(t.type == T_VEC) { l.col[0] = t.vval[0]; l.col[1] = t.vval[1]; l.col[2] = t.vval[2]; l.col[3] = 1.0; }
			else if(t.type == T_INT || t.type == T_FLT) { l.col[0] = l.col[1] = l.col[2] = t.fval; l.col[3] = 1.0; }
		}
		for(int c = d.nodes[n].first_child; c >= 0; c = d.nodes[c].next) {
			if(d.is(c, "xform")) load_xform(c, l.xf);
			else if(l.type == LT_SPHERE && d.is(c, "sphere")) {
				if(!Doc::typed(d.attr(c, "rad"), &t)) { err = "sphere light without rad"; return false; }
				l.radius = (float)t.fval;
			} else if(l.type == LT_BOX && d.is(c, "aabox")) {
				Typed a, b;
				if(!Doc::typed(d.attr(c, "min"), &a) || a.type != T_VEC || !Doc::typed(d.attr(c, "max"), &b) || b.type != T_VEC) {
					err = "invalid aabox in box light";
					return false;
				}
				l.dim = Vec3(b.vval[0] - a.vval[0], b.vval[1] - a.vval[1], b.vval[2] - a.vval[2]);
			}
		}
		sc.lights.push_back(l);
		return true;
	}

	bool load_camera(int n, bool &have)
	{
		Typed t;
		if(!Doc::typed(d.attr(n, "type"), &t)) { err = "invalid camera: no type attribute."; return false; }
		Camera c;
		c.aspect = (double)opt.width / (double)opt.height;
		c.shutter = opt.shutter;
		if(t.str == "free") c.target = 0;
		else if(t.str == "target") {
			c.target = 1;
			set_key(c.xf.pos, 0, Vec3(0, 5, 10));
			set_key(c.txf.pos, 0, Vec3(0, 0, 0));
			set_key(c.txf.scale, 0, Vec3(0, 0, 0));
		} else { err = "invalid camera: unknown type: " + t.str; return false; }
		if(Doc::typed(d.attr(n, "shutter"), &t)) c.shutter = (int)t.fval;
		if(Doc::typed(d.attr(n, "fov"), &t) && (t.type == T_FLT || t.type == T_INT)) c.vfov = (t.fval * M_PI) / 180.0;
		int target = -1;
		for(int ch = d.nodes[n].first_child; ch >= 0; ch = d.nodes[ch].next) {
			if(d.is(ch, "xform")) load_xform(ch, c.xf);
			else if(d.is(ch, "target") && target < 0) target = ch;
		}
		if(c.target) {
			if(target < 0) { err = "failed to load target camera, no <target> child"; return false; }
			for(int ch = d.nodes[target].first_child; ch >= 0; ch = d.nodes[ch].next) if(d.is(ch, "xform")) load_xform(ch, c.txf);
		}
		if(!have) {
			sc.cam = c;
			have = true;
		}
		return true;
	}

	bool run()
	{
		int root = 0;
		for(int n = d.nodes[root].first_child; n >= 0; n = d.nodes[n].next) {
			if(d.is(n, "material") && !load_material(n)) return false;
		}
		bool have_cam = false;
		for(int n = d.nodes[root].first_child; n >= 0; n = d.nodes[n].next) {
			Typed t;
			if(d.is(n, "env")) {
				if(Doc::typed(d.attr(n, "ambient"), &t)) {
					if(t.type == T_VEC) { sc.env_amb[0] = t.vval[0]; sc.env_amb[1] = t.vval[1]; sc.env_amb[2] = t.vval[2]; sc.env_amb[3] = 1.0; }
					else if(t.type == T_INT || t.type == T_FLT) { sc.env_amb[0] = sc.env_amb[1] = sc.env_amb[2] = t.fval; sc.env_amb[3] = 1.0; }
				}
				if(Doc::typed(d.attr(n, "bgcolor"), &t) && t.type == T_VEC) {
					sc.env_col[0] = t.vval[0]; sc.env_col[1] = t.vval[1]; sc.env_col[2] = t.vval[2]; sc.env_col[3] = 1.0;
				}
				if(Doc::typed(d.attr(n, "ior"), &t) && t.type == T_FLT) sc.env_ior = t.fval;
			} else if(d.is(n, "object")) {
				if(!load_object(n)) return false;
			} else if(d.is(n, "light")) {
				if(!load_light(n)) return false;
			} else if(d.is(n, "camera")) {
				if(!load_camera(n, have_cam)) return false;
			}
		}
		if(!have_cam) {
			sc.cam = Camera();
			sc.cam.aspect = (double)opt.width / (double)opt.height;
			sc.cam.shutter = opt.shutter;
		}
		return true;
	}
};
}  // namespace

/* ---- binary side-car of a document's meshes ----
 * header: magic, format version, document size and hash, the mesh octree
 * options; per unique mesh: faces, vertices (double, 9 per face),
 * attributes (float, 24 per face), content hash, octree (per node: box,
 * first child, items), binary hierarchy (nodes, leaf order, depth); then
 * the unique mesh of every mesh object in document order. */
static const char SIDECAR_MAGIC[8] = {'S', 'R', 'A', 'Y', 'M', 'S', 'H', '1'};

static uint64_t text_hash(const char *p, size_t n)
{
	uint64_t h = 0x243f6a8885a308d3ull ^ (uint64_t)n;
	size_t i = 0;
	for(; i + 8 <= n; i += 8) {
		uint64_t w;
		memcpy(&w, p + i, 8);
		h = (h ^ w) * 0x9e3779b97f4a7c15ull;
		h ^= h >> 29;
	}
	uint64_t w = 0;
	memcpy(&w, p + i, n - i);
	h = (h ^ w) * 0x9e3779b97f4a7c15ull;
	return h ^ (h >> 31);
}

namespace {
struct Writer {
	FILE *f;
	bool ok = true;
	void raw(const void *p, size_t n) { if(ok && n && fwrite(p, 1, n, f) != n) ok = false; }
	template <class T> void val(const T &v) { raw(&v, sizeof v); }
	template <class T> void vec(const std::vector<T> &v) { val((uint64_t)v.size()); raw(v.data(), v.size() * sizeof(T)); }
};
struct Reader {
	const char *p, *end;
	bool ok = true;
	void raw(void *dst, size_t n)
	{
		if(!ok || (size_t)(end - p) < n) { ok = false; return; }
		memcpy(dst, p, n);
		p += n;
	}
	template <class T> void val(T &v) { raw(&v, sizeof v); }
	template <class T> void vec(std::vector<T> &v)
	{
		uint64_t n = 0;
		val(n);
		if(!ok || n > (uint64_t)(end - p) / sizeof(T)) { ok = false; return; }
		v.resize(n);
		raw(v.data(), n * sizeof(T));
	}
};
}  // namespace

static bool write_sidecar(const char *path, const HostScene &sc, const std::vector<int> &mesh_of_object, uint64_t doc_size,
		uint64_t doc_hash, const sray_opts &opt)
{
	std::string tmp = std::string(path) + ".tmp";
	FILE *f = fopen(tmp.c_str(), "wb");
	if(!f) return false;
	Writer w{f};
	w.raw(SIDECAR_MAGIC, 8);
	w.val(doc_size);
	w.val(doc_hash);
	w.val((int32_t)opt.meshoct_max_depth);
	w.val((int32_t)opt.meshoct_max_items);
	w.val((uint64_t)sc.meshes.size());
	for(const Mesh &m : sc.meshes) {
		w.vec(m.posd);
		w.vec(m.attr);
		w.val(m.hash);
		w.val((uint64_t)m.oct.nodes.size());
		for(const BuildOctree::Node &n : m.oct.nodes) {
			w.val(n.box);
			w.val((int32_t)n.child);
			w.vec(n.items);
		}
		w.vec(m.bvh.nodes);
		w.vec(m.bvh.order);
		w.val((int32_t)m.bvh.depth);
	}
	w.vec(mesh_of_object);
	bool ok = w.ok && fclose(f) == 0;
	if(!ok) { remove(tmp.c_str()); return false; }
	return rename(tmp.c_str(), path) == 0;
}

/* the side-car's meshes and structures if it belongs to this document and
 * these options, else false */
static bool read_sidecar(const char *path, HostScene &sc, std::vector<int> &mesh_of_object, uint64_t doc_size, uint64_t doc_hash,
		const sray_opts &opt)
{
	FILE *f = fopen(path, "rb");
	if(!f) return false;
	std::vector<char> buf;
	if(fseek(f, 0, SEEK_END) == 0) {
		long sz = ftell(f);
		if(sz > 0) {
			buf.resize((size_t)sz);
			fseek(f, 0, SEEK_SET);
			if(fread(buf.data(), 1, buf.size(), f) != buf.size()) buf.clear();
		}
	}
	fclose(f);
	if(buf.size() < 8 || memcmp(buf.data(), SIDECAR_MAGIC, 8) != 0) return false;
	Reader r{buf.data() + 8, buf.data() + buf.size()};
	uint64_t size = 0, hash = 0, nm = 0;
	int32_t depth = 0, items = 0;
	r.val(size);
	r.val(hash);
	r.val(depth);
	r.val(items);
	if(!r.ok || size != doc_size || hash != doc_hash || depth != opt.meshoct_max_depth || items != opt.meshoct_max_items) return false;
	r.val(nm);
	if(!r.ok || nm > (1u << 24)) return false;
	std::vector<Mesh> meshes(nm);
	for(Mesh &m : meshes) {
		r.vec(m.posd);
		r.vec(m.attr);
		r.val(m.hash);
		uint64_t nn = 0;
		r.val(nn);
		if(!r.ok || nn > (uint64_t)(r.end - r.p)) return false;
		m.oct.nodes.resize(nn);
		for(BuildOctree::Node &n : m.oct.nodes) {
			int32_t child = 0;
			r.val(n.box);
			r.val(child);
			n.child = child;
			r.vec(n.items);
		}
		r.vec(m.bvh.nodes);
		r.vec(m.bvh.order);
		int32_t bd = 0;
		r.val(bd);
		m.bvh.depth = bd;
		if(!r.ok || m.posd.size() % 9 || m.attr.size() != m.posd.size() / 9 * 24) return false;
		m.pos.resize(m.posd.size());
		for(size_t i = 0; i < m.posd.size(); i++) m.pos[i] = (float)m.posd[i];
	}
	r.vec(mesh_of_object);
	if(!r.ok) return false;
	for(int u : mesh_of_object) if(u < 0 || (uint64_t)u >= nm) return false;
	sc.meshes = std::move(meshes);
	return true;
}

bool HostScene::load(const char *text, size_t len, const sray_opts &opt, std::string &err, const char *sidecar, bool *used)
{
	if(used) *used = false;
	uint64_t doc_hash = sidecar ? text_hash(text, len) : 0;
	std::vector<int> cached_map;
	HostScene cached;
	bool have_sidecar = sidecar && read_sidecar(sidecar, cached, cached_map, len, doc_hash, opt);
	Doc d;
	d.skip_mesh = have_sidecar;
	if(!d.parse(text, len)) { err = "xml: " + d.err; return false; }
	*this = HostScene();
	if(have_sidecar) meshes = std::move(cached.meshes);
	Loader ld = {d, *this, opt, err};
	if(have_sidecar) ld.sidecar_mesh = &cached_map;
	if(!ld.run()) return false;
	if(have_sidecar && ld.mesh_objects != cached_map.size()) { err = "side-car holds more meshes than the document"; return false; }
	if(used) *used = have_sidecar;
	finish_load(opt, !have_sidecar);
	if(sidecar && !have_sidecar) write_sidecar(sidecar, *this, ld.mesh_of_object, len, doc_hash, opt);
	return true;
}

/* after the scene's contents are in: the mesh octrees in object space
 * (Mesh::build_tree, src/mesh.cc:210-226) and hierarchies, one per unique
 * mesh, built on all host cores (unless they came from a side-car), and
 * the static objects' bounds */
void HostScene::finish_load(const sray_opts &opt, bool build_meshes)
{
	std::vector<std::thread> th;
	size_t nm = build_meshes ? meshes.size() : 0;
	/* tasks 0 .. nm-1 build octrees, nm .. 2nm-1 hierarchies */
	size_t ntask = 2 * nm;
	unsigned nth = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)ntask));
	for(unsigned w = 0; w < nth; w++) {
		th.push_back(std::thread([this, &opt, w, nth, nm, ntask]() {
			for(size_t task = w; task < ntask; task += nth) {
				if(task >= nm) {
					meshes[task - nm].bvh.build(meshes[task - nm].pos);
					continue;
				}
				size_t u = task;
				Mesh &m = meshes[u];
				size_t nf = m.posd.size() / 9;
				std::vector<Box> boxes(nf);
				for(size_t i = 0; i < nf; i++) {
					Box &b = boxes[i];
					for(int k = 0; k < 3; k++) { b.mn[k] = FLT_MAX; b.mx[k] = -FLT_MAX; }
					for(int v = 0; v < 3; v++) {
						for(int k = 0; k < 3; k++) {
							double c = m.posd[i * 9 + v * 3 + k];
							if(c < b.mn[k]) b.mn[k] = c;
							if(c > b.mx[k]) b.mx[k] = c;
						}
					}
				}
				m.oct.build(boxes, opt.meshoct_max_depth, opt.meshoct_max_items);
			}
		}));
	}
	for(auto &t : th) t.join();
	/* objects with at most one key per transform track have time-independent bounds */
	for(size_t i = 0; i < objs.size(); i++) {
		Object &o = objs[i];
		o.is_static = false;
		if(o.xf.pos.time.size() <= 1 && o.xf.rot.time.size() <= 1 && o.xf.scale.time.size() <= 1) {
			o.static_box = o.bounds(meshes, 0);
			o.is_static = true;
		}
	}
}

/* ---- a scene set ---- */
void HostScene::append_scene(HostScene &&o)
{
	if(ranges.empty()) {
		SceneRange r0;
		r0.nobj = (int)objs.size();
		r0.nlight = (int)lights.size();
		r0.cam = cam;
		r0.env_ior = env_ior;
		memcpy(r0.env_col, env_col, sizeof env_col);
		memcpy(r0.env_amb, env_amb, sizeof env_amb);
		ranges.push_back(r0);
	}
	SceneRange r;
	r.obj0 = (int)objs.size();
	r.nobj = (int)o.objs.size();
	r.light0 = (int)lights.size();
	r.nlight = (int)o.lights.size();
	r.cam = o.cam;
	r.env_ior = o.env_ior;
	memcpy(r.env_col, o.env_col, sizeof env_col);
	memcpy(r.env_amb, o.env_amb, sizeof env_amb);
	int tex0 = (int)texs.size(), mat0 = (int)mats.size(), mesh0 = (int)meshes.size();
	for(Texture &t : o.texs) texs.push_back(std::move(t));
	for(Material m : o.mats) {
		for(int k = 0; k < TA_COUNT; k++) if(m.tex[k] >= 0) m.tex[k] += tex0;
		mats.push_back(m);
	}
	for(Mesh &m : o.meshes) meshes.push_back(std::move(m));
	for(Object ob : o.objs) {
		if(ob.mat >= 0) ob.mat += mat0;
		if(ob.mesh >= 0) ob.mesh += mesh0;
		objs.push_back(ob);
	}
	for(const Light &l : o.lights) lights.push_back(l);
	n_tris += o.n_tris;
	ranges.push_back(r);
}

/* ---- a scene given as tables ---- */
template <class T> static bool desc_track(const sray_track_desc &d, int width, Track<T> &tr, const char *what, std::string &err,
		T (*make)(const double *))
{
	if(d.nkeys < 0 || (d.nkeys > 0 && (!d.time || !d.val))) { err = std::string("bad ") + what + " track"; return false; }
	if(d.interp < INTERP_STEP || d.interp > INTERP_CUBIC || d.extrap < EXTRAP_CLAMP || d.extrap > EXTRAP_PINGPONG) {
		err = std::string("bad interpolation or extrapolation of a ") + what + " track";
		return false;
	}
	tr.interp = d.interp;
	tr.extrap = d.extrap;
	for(int k = 0; k < d.nkeys; k++) set_key(tr, d.time[k], make(d.val + (size_t)k * width));
	return true;
}

static Vec3 make_vec3(const double *v) { return Vec3(v[0], v[1], v[2]); }
static Quat make_quat(const double *v) { Quat q = {v[0], v[1], v[2], v[3]}; return q; }

static bool desc_xform(const sray_xform_desc &d, XForm &xf, std::string &err)
{
	if(!desc_track(d.pos, 3, xf.pos, "position", err, make_vec3)) return false;
	if(!desc_track(d.rot, 4, xf.rot, "rotation", err, make_quat)) return false;
	if(!desc_track(d.scale, 3, xf.scale, "scale", err, make_vec3)) return false;
	xf.pivot = Vec3(d.pivot[0], d.pivot[1], d.pivot[2]);
	return true;
}

bool HostScene::from_desc(const sray_scene_desc &d, const sray_opts &opt, std::string &err)
{
	*this = HostScene();
	if(d.n_materials < 0 || d.n_objects < 0 || d.n_lights < 0 || d.n_textures < 0 ||
			(d.n_materials && !d.materials) || (d.n_objects && !d.objects) || (d.n_lights && !d.lights) ||
			(d.n_textures && !d.textures)) {
		err = "bad scene description: negative count or missing table";
		return false;
	}
	for(int i = 0; i < d.n_textures; i++) {
		const sray_texture_desc &t = d.textures[i];
		if(t.width <= 0 || t.height <= 0 || !t.pixels) { err = "bad texture " + std::to_string(i); return false; }
		Texture tx;
		tx.xsz = t.width;
		tx.ysz = t.height;
		tx.pix.assign(t.pixels, t.pixels + (size_t)t.width * t.height * 4);
		texs.push_back(std::move(tx));
	}
	for(int i = 0; i < d.n_materials; i++) {
		const sray_material_desc &md = d.materials[i];
		Material m;
		m.name = md.name ? md.name : "";
		m.phong = md.phong ? 1 : 0;
		for(int a = 0; a < SRAY_ATTR_COUNT; a++) {
			if(!md.attr[a].present) continue;
			const double *col = md.attr[a].col;
			int tex = md.attr[a].texture;
			if(tex < -1 || tex >= d.n_textures) { err = "material " + m.name + ": texture index out of range"; return false; }
			switch(a) {
			case SRAY_ATTR_DIFFUSE: memcpy(m.kd, col, sizeof m.kd); m.tex[TA_DIFFUSE] = tex; break;
			case SRAY_ATTR_SPECULAR: memcpy(m.ks, col, sizeof m.ks); m.tex[TA_SPECULAR] = tex; break;
			case SRAY_ATTR_SHININESS: m.shin = col[0]; m.tex[TA_SHININESS] = tex; break;
			case SRAY_ATTR_REFLECT: m.refl = col[0]; m.tex[TA_REFLECT] = tex; break;
			case SRAY_ATTR_REFRACT: m.refr = col[0]; m.tex[TA_REFRACT] = tex; break;
			case SRAY_ATTR_IOR: m.ior = col[0]; m.tex[TA_IOR] = tex; break;
			case SRAY_ATTR_NORMAL: m.have_normal = true; m.nrm_scale = col[0]; m.tex[TA_NORMAL] = tex; break;
			}
		}
		mats.push_back(m);
	}
	for(int i = 0; i < d.n_objects; i++) {
		const sray_object_desc &od = d.objects[i];
		Object o;
		o.name = od.name ? od.name : "";
		if(od.type < SRAY_OBJ_SPHERE || od.type > SRAY_OBJ_MESH) { err = "object " + o.name + ": unknown type"; return false; }
		o.type = od.type;
		if(od.material < -1 || od.material >= d.n_materials) { err = "object " + o.name + ": material index out of range"; return false; }
		o.mat = od.material;
		if(!desc_xform(od.xform, o.xf, err)) { err = "object " + o.name + ": " + err; return false; }
		o.rad = od.rad;
		o.start = od.start;
		o.end = od.end;
		if(o.type == OBJ_MESH) {
			if(od.nfaces < 0 || (od.nfaces > 0 && !od.pos)) { err = "mesh " + o.name + ": no vertex data"; return false; }
			size_t nf = (size_t)od.nfaces;
			Mesh m;
			m.posd.assign(od.pos, od.pos + nf * 9);
			m.pos.resize(nf * 9);
			for(size_t k = 0; k < nf * 9; k++) m.pos[k] = (float)m.posd[k];
			m.attr.assign(nf * 24, 0.0f);
			for(size_t f = 0; f < nf; f++) {
				for(int k = 0; k < 9; k++) {
					if(od.normal) m.attr[f * 24 + k] = (float)od.normal[f * 9 + k];
					if(od.tangent) m.attr[f * 24 + 9 + k] = (float)od.tangent[f * 9 + k];
				}
				if(od.texcoord) for(int k = 0; k < 6; k++) m.attr[f * 24 + 18 + k] = (float)od.texcoord[f * 6 + k];
			}
			/* identical meshes share one device copy */
			uint64_t h = fnv(m.posd.data(), m.posd.size() * sizeof(double), 0xcbf29ce484222325ull);
			h = fnv(m.attr.data(), m.attr.size() * sizeof(float), h);
			o.mesh = -1;
			for(size_t u = 0; u < meshes.size(); u++)
				if(meshes[u].hash == h && meshes[u].posd == m.posd && meshes[u].attr == m.attr) { o.mesh = (int)u; break; }
			if(o.mesh < 0) {
				m.hash = h;
				o.mesh = (int)meshes.size();
				meshes.push_back(std::move(m));
			}
			n_tris += (int64_t)nf;
		}
		objs.push_back(o);
	}
	for(int i = 0; i < d.n_lights; i++) {
		const sray_light_desc &ld = d.lights[i];
		Light l;
		if(ld.type < SRAY_LIGHT_POINT || ld.type > SRAY_LIGHT_BOX) { err = "light " + std::to_string(i) + ": unknown type"; return false; }
		l.type = ld.type;
		memcpy(l.col, ld.color, sizeof l.col);
		if(!desc_xform(ld.xform, l.xf, err)) { err = "light " + std::to_string(i) + ": " + err; return false; }
		l.radius = (float)ld.radius;
		l.dim = Vec3(ld.dim[0], ld.dim[1], ld.dim[2]);
		lights.push_back(l);
	}
	cam = Camera();
	cam.aspect = (double)opt.width / (double)opt.height;
	cam.shutter = opt.shutter;
	if(d.camera) {
		cam.target = d.camera->target ? 1 : 0;
		cam.vfov = d.camera->vfov;
		cam.shutter = d.camera->shutter;
		if(!desc_xform(d.camera->xform, cam.xf, err) || !desc_xform(d.camera->target_xform, cam.txf, err)) {
			err = "camera: " + err;
			return false;
		}
	}
	memcpy(env_amb, d.env_ambient, sizeof env_amb);
	memcpy(env_col, d.env_color, sizeof env_col);
	env_ior = d.env_ior;
	finish_load(opt, true);
	return true;
}

}  // namespace sray
