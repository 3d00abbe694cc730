/* render_gpu.h -- S-ray's renderer entry points on top of libsray_gpu.so.
 *
 * render_gpu.cc is linked into S-ray in place of src/render.cc (and of
 * src/tpool.cc and src/block.c, which it no longer needs): it implements
 * rend_init(Image*) and render(long msec) (src/render.h:6-7) by handing the
 * in-memory Scene (get_scene(), src/scene.h:32-33) to the GPU library as
 * tables and rendering each frame there.  It builds against the reference's
 * own headers; nothing of the GPU library's C++ crosses into it.
 */
#ifndef SRAY_RENDER_GPU_H_
#define SRAY_RENDER_GPU_H_

#include <string>
#include <vector>
#include "scene.h"
#include "sray_gpu.h"

/* The tables of one scene and the description that points into them. */
struct SceneTables {
	sray_scene_desc desc;
	std::vector<sray_material_desc> mats;
	std::vector<sray_object_desc> objs;
	std::vector<sray_light_desc> lights;
	sray_camera_desc cam;
	std::vector<std::vector<int> > times;        /* key times of every track */
	std::vector<std::vector<double> > values;    /* key values of every track */
	std::vector<std::vector<double> > meshdata;  /* per mesh: positions, normals, tangents, texcoords */
	int textured_attributes = 0;                 /* attributes whose texture could not be passed */
};

/* Flatten `scn` for sray_gpu_upload_scene.  Transform tracks are sampled at
 * every millisecond of [t_lo, t_hi] from the nodes' local position,
 * rotation and scale (XFormNode::get_local_*, src/anim.cc:359-373) and kept
 * as step keys where the value changes, so the GPU's matrices at any
 * integer time of the window are the reference's; outside the window the
 * end keys hold. */
bool sray_tables_from_scene(const Scene *scn, long t_lo, long t_hi, SceneTables *out, std::string *err);

#endif
