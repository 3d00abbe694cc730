/* render_gpu.cc -- rend_init / render (src/render.h:6-7) on the GPU library.
 *
 * Replaces src/render.cc: the reference's frame (build_accel, shoot_photons
 * and render_frame on the tpool, src/render.cc:34-244) becomes one call of
 * sray_gpu_render, after the scene that main loaded (src/sray.cc:99-131)
 * has been handed over with sray_gpu_upload_scene.  Link:
 *   g++ -o sray <the reference's objects but render.o, tpool.o, block.o>
 *       render_gpu.o -L<dir of libsray_gpu.so> -lsray_gpu
 */
#include <stdio.h>
#include <string.h>
#include <math.h>
#include "render_gpu.h"
#include "render.h"
#include "opt.h"
#include "img.h"
#include "object.h"
#include "sphere.h"
#include "cylinder.h"
#include "mesh.h"
#include "material.h"
#include "light.h"
#include "camera.h"
#include "shader.h"

/* S-ray's options as the library's (src/opt.h:38-62) */
static void to_sray_opts(sray_opts *o)
{
	sray_default_opts(o);
	o->width = opt.width;
	o->height = opt.height;
	o->min_samples = opt.min_samples;
	o->max_samples = opt.max_samples;
	o->max_var = opt.max_var;
	o->min_energy = opt.min_energy;
	o->shadow_samples = opt.shadow_samples;
	o->diffuse_samples = opt.diffuse_samples;
	o->threads = opt.threads;
	o->blk_sz = opt.blk_sz;
	o->iter = opt.iter;
	o->fps = opt.fps;
	o->mblur = opt.mblur;
	o->shutter = opt.shutter;
	o->time_start = opt.time_start;
	o->time_end = opt.time_end;
	o->caust_photons = opt.caust_photons;
	o->gi_photons = opt.gi_photons;
	o->gather_dist = opt.gather_dist;
	o->photon_energy = opt.photon_energy;
	o->scnoct_max_depth = opt.scnoct_max_depth;
	o->scnoct_max_items = opt.scnoct_max_items;
	o->meshoct_max_depth = opt.meshoct_max_depth;
	o->meshoct_max_items = opt.meshoct_max_items;
}

/* one sampled track: step keys where the value changes */
static void sample_track(SceneTables *T, sray_track_desc *tr, int width, long t_lo, long t_hi,
		void (*get)(const void *node, int t, double *v), const void *node)
{
	std::vector<int> times;
	std::vector<double> vals;
	double prev[4] = {0, 0, 0, 0}, cur[4];
	for(long t = t_lo; t <= t_hi; t++) {
		get(node, (int)t, cur);
		if(times.empty() || memcmp(prev, cur, width * sizeof(double)) != 0) {
			times.push_back((int)t);
			vals.insert(vals.end(), cur, cur + width);
			memcpy(prev, cur, sizeof prev);
		}
	}
	T->times.push_back(times);
	T->values.push_back(vals);
	tr->nkeys = (int)times.size();
	tr->interp = 0;   /* step */
	tr->extrap = 0;   /* clamp */
	tr->time = T->times.back().data();
	tr->val = T->values.back().data();
}

static void get_pos(const void *n, int t, double *v)
{
	Vector3 p = ((const XFormNode *)n)->get_local_position(t);
	v[0] = p.x; v[1] = p.y; v[2] = p.z;
}
static void get_rot(const void *n, int t, double *v)
{
	Quaternion q = ((const XFormNode *)n)->get_local_rotation(t);
	v[0] = q.s; v[1] = q.v.x; v[2] = q.v.y; v[3] = q.v.z;
}
static void get_scale(const void *n, int t, double *v)
{
	Vector3 s = ((const XFormNode *)n)->get_local_scaling(t);
	v[0] = s.x; v[1] = s.y; v[2] = s.z;
}
/* a target camera's aim point and roll (src/camera.cc:198-214) */
static void get_target(const void *n, int t, double *v)
{
	Vector3 p = ((const TargetCamera *)n)->get_target(t);
	v[0] = p.x; v[1] = p.y; v[2] = p.z;
}
static void get_roll(const void *n, int t, double *v)
{
	double r = ((const TargetCamera *)n)->get_roll(t);
	v[0] = v[1] = v[2] = r;
}

static void sample_xform(SceneTables *T, sray_xform_desc *xf, const XFormNode *node, long t_lo, long t_hi)
{
	memset(xf, 0, sizeof *xf);
	sample_track(T, &xf->pos, 3, t_lo, t_hi, get_pos, node);
	sample_track(T, &xf->rot, 4, t_lo, t_hi, get_rot, node);
	sample_track(T, &xf->scale, 3, t_lo, t_hi, get_scale, node);
	const Vector3 &pv = node->get_pivot();
	xf->pivot[0] = pv.x; xf->pivot[1] = pv.y; xf->pivot[2] = pv.z;
}

static void color4(const Color &c, double *out)
{
	out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
}

bool sray_tables_from_scene(const Scene *scn, long t_lo, long t_hi, SceneTables *T, std::string *err)
{
	static const char *attr_name[SRAY_ATTR_COUNT] = {"diffuse", "specular", "shininess", "reflect", "refract", "ior", "normal"};
	/* the tables are referenced by address: reserve so nothing moves */
	int nmat = scn->get_material_count(), nobj = scn->get_object_count(), nlt = scn->get_light_count();
	T->times.reserve(3 * (nobj + nlt + 2));
	T->values.reserve(3 * (nobj + nlt + 2));
	T->meshdata.reserve(4 * nobj);
	T->mats.resize(nmat);
	ShaderFunc phong = get_shader("phong");
	for(int i = 0; i < nmat; i++) {
		const Material *m = scn->get_material(i);
		sray_material_desc &md = T->mats[i];
		memset(&md, 0, sizeof md);
		md.name = m->get_name();
		md.phong = m->get_shader() == phong;
		for(int a = 0; a < SRAY_ATTR_COUNT; a++) {
			const MatAttrib *at = m->find_attribute(attr_name[a]);
			md.attr[a].texture = -1;
			if(!at) continue;
			md.attr[a].present = 1;
			color4(at->col, md.attr[a].col);
			/* Texture keeps its image private (src/texture.h:37-40): a
			 * textured attribute goes over with its colour alone */
			if(at->tex) T->textured_attributes++;
		}
	}
	Material *const *mats = scn->get_materials();
	T->objs.resize(nobj);
	for(int i = 0; i < nobj; i++) {
		const Object *o = scn->get_object(i);
		sray_object_desc &od = T->objs[i];
		memset(&od, 0, sizeof od);
		od.name = o->get_name();
		od.material = -1;
		for(int k = 0; k < nmat; k++) if(mats[k] == o->get_material()) { od.material = k; break; }
		sample_xform(T, &od.xform, o, t_lo, t_hi);
		if(const Sphere *s = dynamic_cast<const Sphere *>(o)) {
			od.type = SRAY_OBJ_SPHERE;
			od.rad = s->get_radius();
		} else if(const Cylinder *c = dynamic_cast<const Cylinder *>(o)) {
			od.type = SRAY_OBJ_CYLINDER;
			od.rad = c->get_radius();
			od.start = c->get_start();
			od.end = c->get_end();
		} else if(const Mesh *me = dynamic_cast<const Mesh *>(o)) {
			od.type = SRAY_OBJ_MESH;
			int nf = me->get_face_count();
			std::vector<double> pos(9 * (size_t)nf), nrm(9 * (size_t)nf), tng(9 * (size_t)nf), tex(6 * (size_t)nf);
			for(int f = 0; f < nf; f++) {
				const Triangle *tr = me->get_face(f);
				for(int j = 0; j < 3; j++) {
					const Vertex &v = tr->v[j];
					double *p = &pos[f * 9 + j * 3], *n = &nrm[f * 9 + j * 3], *g = &tng[f * 9 + j * 3];
					p[0] = v.pos.x; p[1] = v.pos.y; p[2] = v.pos.z;
					n[0] = v.norm.x; n[1] = v.norm.y; n[2] = v.norm.z;
					g[0] = v.tang.x; g[1] = v.tang.y; g[2] = v.tang.z;
					tex[f * 6 + j * 2] = v.tex.x;
					tex[f * 6 + j * 2 + 1] = v.tex.y;
				}
			}
			T->meshdata.push_back(std::move(pos));
			od.pos = T->meshdata.back().data();
			T->meshdata.push_back(std::move(nrm));
			od.normal = T->meshdata.back().data();
			T->meshdata.push_back(std::move(tng));
			od.tangent = T->meshdata.back().data();
			T->meshdata.push_back(std::move(tex));
			od.texcoord = T->meshdata.back().data();
			od.nfaces = nf;
		} else {
			*err = std::string("object ") + (o->get_name() ? o->get_name() : "?") + " is of a type the GPU library does not know";
			return false;
		}
	}
	T->lights.resize(nlt);
	for(int i = 0; i < nlt; i++) {
		const Light *l = scn->get_light(i);
		sray_light_desc &ld = T->lights[i];
		memset(&ld, 0, sizeof ld);
		ld.type = SRAY_LIGHT_POINT;
		if(const SphLight *s = dynamic_cast<const SphLight *>(l)) {
			ld.type = SRAY_LIGHT_SPHERE;
			ld.radius = s->get_radius();
		} else if(const BoxLight *b = dynamic_cast<const BoxLight *>(l)) {
			ld.type = SRAY_LIGHT_BOX;
			Vector3 d = b->get_dimensions();
			ld.dim[0] = d.x; ld.dim[1] = d.y; ld.dim[2] = d.z;
		}
		color4(l->get_color(), ld.color);
		sample_xform(T, &ld.xform, l, t_lo, t_hi);
	}
	const Camera *cam = scn->get_camera();
	memset(&T->cam, 0, sizeof T->cam);
	if(cam) {
		T->cam.vfov = cam->get_vertical_fov();
		T->cam.shutter = cam->get_shutter();
		sample_xform(T, &T->cam.xform, cam, t_lo, t_hi);
		if(const TargetCamera *tc = dynamic_cast<const TargetCamera *>(cam)) {
			T->cam.target = 1;
			sray_xform_desc &tx = T->cam.target_xform;
			sample_track(T, &tx.pos, 3, t_lo, t_hi, get_target, tc);
			sample_track(T, &tx.scale, 3, t_lo, t_hi, get_roll, tc);
		}
	}
	memset(&T->desc, 0, sizeof T->desc);
	T->desc.n_materials = nmat;
	T->desc.n_objects = nobj;
	T->desc.n_lights = nlt;
	T->desc.materials = T->mats.data();
	T->desc.objects = T->objs.data();
	T->desc.lights = T->lights.data();
	T->desc.camera = cam ? &T->cam : nullptr;
	color4(scn->get_env_ambient(), T->desc.env_ambient);
	color4(scn->get_env_color(), T->desc.env_color);
	T->desc.env_ior = scn->get_env_ior();
	return true;
}

/* ---- the entry points ---- */
static Image *framebuffer;
static const Scene *uploaded;

static bool gpu_error(const char *what)
{
	char msg[512];
	sray_gpu_last_error(msg, sizeof msg);
	fprintf(stderr, "%s: %s\n", what, msg);
	return false;
}

bool rend_init(Image *fb)
{
	sray_opts o;
	to_sray_opts(&o);
	if(sray_gpu_init(&o) != 0) return gpu_error("GPU renderer");
	framebuffer = fb;
	uploaded = nullptr;
	return true;
}

void render(long msec)
{
	Scene *scn = get_scene();
	if(scn != uploaded) {
		/* the whole animation's transforms, with the shutter on either side */
		long sh = scn->get_camera() ? scn->get_camera()->get_shutter() : opt.shutter;
		long lo = (opt.time_start < msec ? opt.time_start : msec) - 2 * sh - 4;
		long hi = (opt.time_end > msec ? opt.time_end : msec) + 2 * sh + 4;
		SceneTables T;
		std::string err;
		if(!sray_tables_from_scene(scn, lo, hi, &T, &err)) {
			fprintf(stderr, "GPU renderer: %s\n", err.c_str());
			return;
		}
		if(T.textured_attributes) fprintf(stderr, "GPU renderer: %d textured attributes rendered with their colour\n", T.textured_attributes);
		if(sray_gpu_upload_scene(&T.desc) != 0) {
			gpu_error("GPU scene upload");
			return;
		}
		uploaded = scn;
	}
	/* octree build, photon maps and every pixel of the frame, into the
	 * row-major RGBA float image the reference writes (src/render.cc:210-243) */
	if(sray_gpu_render(msec, framebuffer->get_pixels(), 0, 0) != 0) gpu_error("GPU render");
}
