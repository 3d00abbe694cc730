/* Host-side check of sray_gpu_upload_scene's scene tables (no GPU): the
 * scene built from a sray_scene_desc (HostScene::from_desc) must equal the
 * scene the XML loader builds from the same document -- materials, objects,
 * mesh data, lights, environment, and every transform (object, light and
 * camera matrices, light positions) at every integer millisecond of a
 * window.  Built as a shared library by tests/test_scene_desc.py, which
 * calls desc_matches_xml with tables from sray_gb300/scene_desc.py, and
 * linked into tests/adapter_check.cc, which passes the tables the
 * reference-side adapter makes from the reference's own Scene. */
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <string>
#include "scene_host.h"

using namespace sray;

static std::string g_msg;

#define DIFF(cond, ...) do { if(cond) { char b_[512]; snprintf(b_, sizeof b_, __VA_ARGS__); g_msg = b_; return false; } } while(0)

static bool same4(const double *a, const double *b) { return memcmp(a, b, 4 * sizeof(double)) == 0; }

static bool same_xf(const char *what, int idx, const XForm &a, const XForm &b, int lo, int hi, bool light)
{
	for(int t = lo; t <= hi; t++) {
		double ma[4][4], mb[4][4];
		a.matrix(t, ma);
		b.matrix(t, mb);
		DIFF(memcmp(ma, mb, sizeof ma) != 0, "%s %d: matrix differs at %d ms", what, idx, t);
		if(light) {
			Vec3 pa = a.position(t), pb = b.position(t);
			DIFF(pa.x != pb.x || pa.y != pb.y || pa.z != pb.z, "%s %d: position differs at %d ms", what, idx, t);
		}
	}
	return true;
}

static bool same_scene(const HostScene &a, const HostScene &b, int lo, int hi, int check_textures)
{
	DIFF(a.mats.size() != b.mats.size(), "materials: %zu against %zu", a.mats.size(), b.mats.size());
	for(size_t i = 0; i < a.mats.size(); i++) {
		const Material &x = a.mats[i], &y = b.mats[i];
		DIFF(x.name != y.name || x.phong != y.phong, "material %zu: name or shader", i);
		DIFF(!same4(x.kd, y.kd) || !same4(x.ks, y.ks), "material %zu (%s): diffuse or specular", i, x.name.c_str());
		DIFF(x.shin != y.shin || x.refl != y.refl || x.refr != y.refr || x.ior != y.ior, "material %zu (%s): scalars", i, x.name.c_str());
		DIFF(x.have_normal != y.have_normal || x.nrm_scale != y.nrm_scale, "material %zu: normal attribute", i);
		if(check_textures) for(int k = 0; k < TA_COUNT; k++) DIFF(x.tex[k] != y.tex[k], "material %zu: texture of attribute %d", i, k);
	}
	if(check_textures) {
		DIFF(a.texs.size() != b.texs.size(), "textures: %zu against %zu", a.texs.size(), b.texs.size());
		for(size_t i = 0; i < a.texs.size(); i++)
			DIFF(a.texs[i].xsz != b.texs[i].xsz || a.texs[i].ysz != b.texs[i].ysz || a.texs[i].pix != b.texs[i].pix, "texture %zu", i);
	}
	DIFF(a.objs.size() != b.objs.size(), "objects: %zu against %zu", a.objs.size(), b.objs.size());
	DIFF(a.meshes.size() != b.meshes.size(), "unique meshes: %zu against %zu", a.meshes.size(), b.meshes.size());
	DIFF(a.n_tris != b.n_tris, "triangles");
	for(size_t i = 0; i < a.objs.size(); i++) {
		const Object &x = a.objs[i], &y = b.objs[i];
		DIFF(x.type != y.type || x.name != y.name || x.mat != y.mat, "object %zu: type, name or material", i);
		DIFF(x.type != OBJ_MESH && x.rad != y.rad, "object %zu (%s): radius", i, x.name.c_str());
		DIFF(x.type == OBJ_CYLINDER && (x.start != y.start || x.end != y.end), "object %zu (%s): extent", i, x.name.c_str());
		DIFF(x.mesh != y.mesh, "object %zu: mesh", i);
		if(x.mesh >= 0) {
			const Mesh &p = a.meshes[x.mesh], &q = b.meshes[y.mesh];
			DIFF(p.posd != q.posd || p.pos != q.pos, "object %zu (%s): vertices", i, x.name.c_str());
			DIFF(p.attr != q.attr, "object %zu (%s): vertex attributes", i, x.name.c_str());
			DIFF(p.oct.nodes.size() != q.oct.nodes.size() || p.bvh.nodes.size() != q.bvh.nodes.size(), "object %zu: mesh structures", i);
		}
		DIFF(x.is_static != y.is_static, "object %zu (%s): static", i, x.name.c_str());
		if(!same_xf("object", (int)i, x.xf, y.xf, lo, hi, false)) return false;
	}
	DIFF(a.lights.size() != b.lights.size(), "lights: %zu against %zu", a.lights.size(), b.lights.size());
	for(size_t i = 0; i < a.lights.size(); i++) {
		const Light &x = a.lights[i], &y = b.lights[i];
		DIFF(x.type != y.type, "light %zu: type", i);
		DIFF(!same4(x.col, y.col), "light %zu: colour %g %g %g %g against %g %g %g %g", i, x.col[0], x.col[1], x.col[2], x.col[3],
				y.col[0], y.col[1], y.col[2], y.col[3]);
		DIFF(x.type == LT_SPHERE && x.radius != y.radius, "light %zu: radius", i);
		DIFF(x.type == LT_BOX && (x.dim.x != y.dim.x || x.dim.y != y.dim.y || x.dim.z != y.dim.z), "light %zu: box", i);
		if(!same_xf("light", (int)i, x.xf, y.xf, lo, hi, true)) return false;
	}
	DIFF(a.cam.target != b.cam.target || a.cam.vfov != b.cam.vfov || a.cam.shutter != b.cam.shutter || a.cam.aspect != b.cam.aspect,
			"camera: kind, field of view, shutter or aspect");
	for(int t = lo; t <= hi; t++) {
		double ma[4][4], mb[4][4];
		a.cam.matrix(t, ma);
		b.cam.matrix(t, mb);
		DIFF(memcmp(ma, mb, sizeof ma) != 0, "camera matrix differs at %d ms", t);
	}
	DIFF(!same4(a.env_amb, b.env_amb) || !same4(a.env_col, b.env_col) || a.env_ior != b.env_ior, "environment");
	return true;
}

extern "C" int desc_matches_xml(const sray_scene_desc *d, const char *xml, size_t len, const sray_opts *opt, int lo, int hi,
		int check_textures, char *msg, size_t cap)
{
	HostScene a, b;
	std::string err;
	int ok = 1;
	if(!a.from_desc(*d, *opt, err)) { g_msg = "from_desc: " + err; ok = 0; }
	else if(!b.load(xml, len, *opt, err)) { g_msg = "load: " + err; ok = 0; }
	else if(!same_scene(a, b, lo, hi, check_textures)) ok = 0;
	else g_msg = "same";
	snprintf(msg, cap, "%s", g_msg.c_str());
	return ok;
}
