/* sray_oracle.h -- C API of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++ restatement of S-ray's rendering path, used by
 * the test suite as the checker of the GPU library, by bench.py as the
 * timed CPU baseline, and by __graft_entry__.smoke().  Nothing in the
 * product links or calls it.  It runs in two precisions:
 *   fp64 = 1: every per-ray quantity in double, as the reference computes it;
 *   fp64 = 0: per-ray arithmetic in float with the operation order of the
 *             CUDA kernels, scene set-up (matrices, octree boxes, projection
 *             maps) in double and rounded to float, as the GPU library does.
 */
#ifndef SRAY_ORACLE_H_
#define SRAY_ORACLE_H_

#include <stdint.h>
#include "sray_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* rng_mode: 0 = one sequential stream per pixel sample consumed in the
 * reference's depth-first shading order (what the compiled reference sees
 * through its RNG shim); 1 = draws keyed by the ray's path in the shading
 * tree (what the GPU wavefront uses). */
void *orc_create(const sray_opts *opt, int fp64, int rng_mode);
void orc_destroy(void *h);
int orc_load(void *h, const char *xml_path);
int orc_load_mem(void *h, const char *xml, size_t len);
const char *orc_error(void *h);

int orc_scene_info(void *h, int *n_obj, int *n_lights, int *n_mat, int64_t *n_tris);

/* Scene::build_tree + shoot_photons for frame msec (t0/t1 from the camera shutter) */
int orc_prepare_frame(void *h, long msec);
/* caustic / global photons stored, and the gather radius */
int orc_photon_info(void *h, int *n_caust, int *n_gi, double *gather_dist);
/* 16 floats per photon: pos xyz, dir xyz, norm xyz, col rgba, 3 unused */
int orc_get_photons(void *h, int which, float *out, int cap);

/* Render pixel rows [y0, y1) of the prepared frame into fb (width*height*4
 * floats; rows outside the range untouched).  nthreads = 0: all cores.
 * quirk_sum = 1 keeps the reference's framebuffer arithmetic for
 * spp > 1 (sum of samples, one float rescaled, src/render.cc:220-240);
 * 0 writes the mean.  spp_out (optional, width*height ints) receives the
 * number of samples taken per pixel. */
int orc_render_rows(void *h, long msec, int y0, int y1, float *fb, int nthreads,
		int quirk_sum, int *spp_out);

/* The same for the n listed rows (any order, each in [0, height)). */
int orc_render_row_list(void *h, long msec, int n, const int *rows, float *fb, int nthreads,
		int quirk_sum, int *spp_out);

/* Primary ray (sample 0) closest hits of the prepared frame. */
int orc_primary_hits(void *h, long msec, int *obj, int *prim, double *t, unsigned char *tie);

/* Closest hits of arbitrary world rays (dir carries the segment length). */
int orc_cast_rays(void *h, int n, const double *orig, const double *dir, const int *time,
		int *obj, int *prim, double *t, unsigned char *tie);

/* Gathers at arbitrary points of the prepared frame: which = 0 caustic
 * irradiance_est, 1 global radiance_est.  out: n*4 doubles. */
int orc_gather(void *h, int which, int n, const double *pos, const double *norm, double *out);

/* Replace the options of a loaded oracle (photon counts, samples, ...; not
 * the mesh octree options, which shape the loaded meshes).  The next call
 * prepares the frame again. */
int orc_set_opts(void *h, const sray_opts *opt);

/* Offset added to every pixel index in the pixel sample streams' keys of
 * later orc_render_rows / orc_primary_hits calls (a job of a GPU batch keys
 * its pixels by their place in the batch).  Default 0. */
int orc_set_pixel_base(void *h, int base);

/* Wall time of the last frame preparation's phases, ms: ms[0] scene tree and
 * frame tables, ms[1] projection maps, ms[2] photon tracing and map build. */
int orc_phase_ms(void *h, double *ms);

/* Work counters of the last orc_render_rows / orc_primary_hits call. */
int orc_counters(void *h, int64_t *rays, int64_t *node_visits, int64_t *prim_tests,
		int64_t *shadow_rays, int64_t *gathers);

#ifdef __cplusplus
}
#endif

#endif
