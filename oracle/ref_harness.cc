/* ref_harness.cc -- TEST INFRASTRUCTURE: runs the reference's own rendering
 * code (compiled unmodified from its sources) with a Philox stream selected
 * per photon and per pixel sample, and writes what the oracle is checked
 * against: primary-hit ids, stored photons and the rendered image.
 *
 * The loops that select streams restate the reference's drivers:
 * shoot_photons (src/render.cc:67-122), build_caustics_map /
 * build_global_map (src/scene.cc:445-534) and render_block
 * (src/render.cc:194-244); everything they call is the reference's code.
 *
 * usage: ref_harness scene.xml out_prefix seed y0 y1 [reference options...]
 *        ref_harness --time scene.xml reps [reference options...]
 *        ref_harness --restore dump.txt out.bin [reference options...]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <vector>
#define private public
#define protected public
#include "scene.h"
#include "mesh.h"
#include "camera.h"
#include "light.h"
#include "opt.h"
#include "img.h"
#include "render.h"
#include "timer.h"
#undef private
#undef protected
#include "sray_rng.h"

void shim_rng_select(sray_rng *s);
extern "C" int shim_rand(void);   /* rand() of the reference's sources */

static uint64_t g_seed;

static void dump_photons(const char *fname, PhotonMap &pm)
{
	FILE *fp = fopen(fname, "wb");
	if(!fp) return;
	for(size_t i = 0; i < pm.photons.size(); i++) {
		const Photon *p = pm.photons[i];
		float f[16] = {(float)p->pos.x, (float)p->pos.y, (float)p->pos.z, (float)p->dir.x, (float)p->dir.y, (float)p->dir.z,
			(float)p->norm.x, (float)p->norm.y, (float)p->norm.z, (float)p->col.x, (float)p->col.y, (float)p->col.z,
			(float)p->col.w, (float)p->type, 0.0f, 0.0f};
		fwrite(f, sizeof f, 1, fp);
	}
	fclose(fp);
}

/* --time scene.xml reps [reference options...]: the reference's own frame
 * entry point, rend_init + render(msec) (src/render.cc:22-55: build_accel,
 * shoot_photons and render_frame on its pthread tpool), timed with its own
 * get_msec (src/timer.c:13-25), reps times.  Prints one JSON line. */
static int time_render(int argc, char **argv)
{
	const char *scene_path = argv[2];
	int reps = atoi(argv[3]);
	std::vector<char *> av;
	av.push_back(argv[0]);
	for(int i = 4; i < argc; i++) av.push_back(argv[i]);
	av.push_back((char *)scene_path);
	av.push_back(0);
	if(parse_opt((int)av.size() - 1, av.data()) == -1) return 1;
	opt.verb = -1;
	Scene *scn = new Scene;
	if(!scn->load(scene_path)) return 1;
	if(!scn->get_camera()) scn->set_camera(new Camera);
	set_scene(scn);
	Image fb;
	if(!fb.create(opt.width, opt.height)) return 1;
	if(!rend_init(&fb)) return 1;
	const char *ms_env = getenv("SRAY_REF_MSEC");
	long msec = ms_env ? atol(ms_env) : 0;
	std::vector<unsigned long> ms;
	for(int i = 0; i < reps; i++) {
		unsigned long t0 = get_msec();
		render(msec);
		ms.push_back(get_msec() - t0);
	}
	double sum = 0.0;
	for(int i = 0; i < opt.width * opt.height * 4; i++) sum += fb.pixels[i];
	/* on a line of its own: render() prints debug lines on stdout */
	printf("\n{\"threads\": %d, \"width\": %d, \"height\": %d, \"render_ms\": [", opt.threads, opt.width, opt.height);
	for(size_t i = 0; i < ms.size(); i++) printf("%s%lu", i ? ", " : "", ms[i]);
	printf("], \"pixel_sum\": %.6g}\n", sum);
	return 0;
}

/* --restore dump.txt out.bin [reference options...]: PhotonMap::restore
 * (src/pmap.cc:207-251) of a dump file, its photons written as 16 floats
 * each (pos, dir, norm, col, type) -- the reference reading a dump another
 * program wrote. */
static int restore_dump(int argc, char **argv)
{
	std::vector<char *> av;
	av.push_back(argv[0]);
	for(int i = 4; i < argc; i++) av.push_back(argv[i]);
	av.push_back((char *)"none.xml");
	av.push_back(0);
	if(parse_opt((int)av.size() - 1, av.data()) == -1) return 1;
	opt.verb = -1;
	PhotonMap pm;
	if(!pm.restore(argv[2])) return 1;
	dump_photons(argv[3], pm);
	return 0;
}

int main(int argc, char **argv)
{
	if(argc >= 4 && strcmp(argv[1], "--time") == 0) return time_render(argc, argv);
	if(argc >= 4 && strcmp(argv[1], "--restore") == 0) return restore_dump(argc, argv);
	if(argc < 6) {
		fprintf(stderr, "usage: %s scene.xml out_prefix seed y0 y1 [options]\n", argv[0]);
		return 1;
	}
	const char *scene_path = argv[1], *prefix = argv[2];
	g_seed = strtoull(argv[3], 0, 0);
	int y0 = atoi(argv[4]), y1 = atoi(argv[5]);
	std::vector<char *> av;
	av.push_back(argv[0]);
	for(int i = 6; i < argc; i++) av.push_back(argv[i]);
	av.push_back((char *)scene_path);
	av.push_back(0);
	if(parse_opt((int)av.size() - 1, av.data()) == -1) return 1;
	opt.verb = -1;

	Scene *scn = new Scene;
	if(!scn->load(scene_path)) return 1;
	if(!scn->get_camera()) scn->set_camera(new Camera);
	Camera *cam = scn->get_camera();
	/* the frame time (default 0): SRAY_REF_MSEC */
	const char *ms_env = getenv("SRAY_REF_MSEC");
	long msec = ms_env ? atol(ms_env) : 0;
	long shutter = cam->get_shutter();
	long t0 = msec - shutter / 2, t1 = t0 + shutter;

	/* build_accel */
	scn->build_tree(t0, t1);

	/* shoot_photons with one stream per light (projection maps) and per photon */
	int num_lights = scn->get_light_count();
	if((opt.caust_photons || opt.gi_photons) && num_lights) {
		std::vector<LightPower> ltpow(num_lights);
		double acc_power = 0.0;
		Light **lights = (Light **)scn->get_lights();
		for(int i = 0; i < num_lights; i++) {
			Color col = lights[i]->get_color();
			ltpow[i].intensity = (col.x + col.y + col.z) / 3.0;
			acc_power += ltpow[i].intensity;
			int num_obj = scn->get_object_count();
			if(num_obj) {
				sray_rng s;
				sray_rng_init(&s, g_seed, SRAY_DOM_PROJMAP, (uint32_t)i, 0);
				shim_rng_select(&s);
				lights[i]->build_projmap((const Object **)scn->get_objects(), num_obj, t0, t1);
				shim_rng_select(0);
			}
		}
		for(int i = 0; i < num_lights; i++) ltpow[i].photon_power = ltpow[i].intensity / acc_power;
		for(int global = 0; global < 2; global++) {
			PhotonMap &map = global ? scn->gi_map : scn->caust_map;
			int num = global ? opt.gi_photons : opt.caust_photons;
			map.clear();
			for(int li = 0; li < num_lights; li++) {
				int nphot = (int)ceil((double)num * ltpow[li].photon_power);
				for(int j = 0; j < nphot; j++) {
					sray_rng s;
					sray_rng_init(&s, g_seed, global ? SRAY_DOM_GLOBAL : SRAY_DOM_CAUST, (uint32_t)j, (uint32_t)li);
					shim_rng_select(&s);
					int ms = t0 == t1 ? (int)t0 : (int)(shim_rand() % (t1 - t0) + t0);
					Photon p = lights[li]->gen_photon(ms, global ? SAMPLE_OBJ : SAMPLE_SPEC_OBJ);
					Ray ray;
					ray.origin = p.pos;
					ray.dir = p.dir;
					ray.time = ms;
					ray.iter = opt.iter;
					if(global) {
						if(scn->trace_global_photon(ray, &p)) map.add_photon(p.pos, p.dir, p.norm, p.col);
					} else {
						if(scn->trace_caustics_photon(ray, &p) && p.type == CAUST_PHOTON) map.add_photon(p.pos, p.dir, p.norm, p.col);
					}
					shim_rng_select(0);
				}
				if(nphot) map.scale_photon_power(1.0 / (double)nphot);
			}
		}
	}
	char fname[1024];
	snprintf(fname, sizeof fname, "%s.caust", prefix);
	dump_photons(fname, scn->caust_map);
	snprintf(fname, sizeof fname, "%s.gi", prefix);
	dump_photons(fname, scn->gi_map);
	/* the maps in the reference's own text format (PhotonMap::dump,
	 * src/pmap.cc:180-205) */
	snprintf(fname, sizeof fname, "%s.caust.dump", prefix);
	scn->caust_map.dump(fname);
	snprintf(fname, sizeof fname, "%s.gi.dump", prefix);
	scn->gi_map.dump(fname);

	/* primary hits: object index, triangle index of meshes, t */
	int W = opt.width, H = opt.height;
	snprintf(fname, sizeof fname, "%s.hits", prefix);
	FILE *fh = fopen(fname, "wb");
	for(int y = y0; y < y1; y++) {
		for(int x = 0; x < W; x++) {
			uint32_t pix = (uint32_t)(y * W + x);
			sray_rng s;
			sray_rng_init(&s, g_seed, SRAY_DOM_PIXEL, pix, 0);
			shim_rng_select(&s);
			Ray ray = cam->get_primary_ray(x, y, 0, t0);
			shim_rng_select(0);
			SurfPoint sp;
			Object *o = scn->cast_ray(ray, &sp);
			int oi = -1, prim = -1;
			double t = 0.0;
			if(o) {
				for(int k = 0; k < scn->get_object_count(); k++) if(scn->get_object(k) == o) oi = k;
				t = sp.dist;
				prim = 0;
				Mesh *m = dynamic_cast<Mesh *>(o);
				if(m) {
					Ray lr = ray.transformed(m->get_inv_xform_matrix(ray.time));
					SurfPoint sp2;
					OctItem<Triangle *> *it = m->octree.intersect(lr, &sp2);
					prim = it ? (int)(it->data - &m->faces[0]) : -2;
				}
			}
			fwrite(&oi, 4, 1, fh);
			fwrite(&prim, 4, 1, fh);
			fwrite(&t, 8, 1, fh);
		}
	}
	fclose(fh);

	/* render_block's per-pixel loop; the framebuffer keeps the mean and the
	 * sample count (the reference's own buffer arithmetic differs for spp > 1) */
	snprintf(fname, sizeof fname, "%s.img", prefix);
	FILE *fi = fopen(fname, "wb");
	std::vector<Color> subpix(opt.max_samples > 0 ? opt.max_samples : 1);
	for(int y = y0; y < y1; y++) {
		for(int x = 0; x < W; x++) {
			uint32_t pix = (uint32_t)(y * W + x);
			float img[4] = {0, 0, 0, 0};
			int i = 0;
			while(i < opt.max_samples) {
				sray_rng s;
				sray_rng_init(&s, g_seed, SRAY_DOM_PIXEL, pix, (uint32_t)i);
				shim_rng_select(&s);
				Ray ray = cam->get_primary_ray(x, y, i, t0);
				ray.iter = opt.iter;
				subpix[i] = scn->trace_ray(ray);
				shim_rng_select(0);
				Color pixel;
				pixel.x = img[0] += subpix[i].x;
				pixel.y = img[1] += subpix[i].y;
				pixel.z = img[2] += subpix[i].z;
				pixel.w = img[3] += subpix[i].w;
				i++;
				if(i >= opt.min_samples && i > 1) {
					float rcp = (float)(1.0 / (double)i);
					Color mean = pixel * rcp;
					float sqdist = 0.0f;
					for(int k = 0; k < i; k++) sqdist += (mean - subpix[k]).length_sq();
					if(sqdist * rcp < opt.max_var) break;
				}
			}
			double rcp = 1.0 / (double)i;
			float out[5] = {(float)(img[0] * rcp), (float)(img[1] * rcp), (float)(img[2] * rcp), (float)(img[3] * rcp), (float)i};
			fwrite(out, sizeof out, 1, fi);
		}
	}
	fclose(fi);
	return 0;
}
