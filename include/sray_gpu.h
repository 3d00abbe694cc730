/* sray_gpu.h -- C-ABI of the GB300 rendering path (libsray_gpu.so).
 *
 * This library replaces the rendering hot path of S-ray: the per-frame
 * entry point render() and everything below it (octree traversal, the
 * triangle/sphere/cylinder intersectors, photon emission and tracing, the
 * photon-map gathers, Phong shading with reflection/refraction and the
 * final gather, adaptive supersampling and the tpool block scheduler).
 * The scene stays in S-ray's XML format and its meaning is unchanged.
 *
 * Conventions: every entry point returns 0 on success and a negative
 * SRAY_E* code on failure; sray_gpu_last_error() then returns a message.
 * No C++ types or exceptions cross this boundary.  One renderer context
 * per process, bound to the CUDA device current at sray_gpu_init(); a call
 * made while another device is current returns SRAY_ESTATE.
 * Functions that take a `stream` argument enqueue on that CUDA stream
 * (NULL = the legacy default stream) and return once the result is
 * available unless stated otherwise.
 */
#ifndef SRAY_GPU_H_
#define SRAY_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SRAY_RAY_MAGNITUDE 10000.0   /* src/opt.h:21 */

enum {
	SRAY_OK = 0,
	SRAY_EINVAL = -1,      /* bad argument */
	SRAY_ELOAD = -2,       /* scene file missing or malformed */
	SRAY_ECUDA = -3,       /* CUDA runtime error */
	SRAY_ESTATE = -4,      /* call out of order (e.g. render before load) */
	SRAY_EDEVICE = -5,     /* a kernel raised its error word (queue overflow, bounded wait expired) */
	SRAY_ENOMEM = -6,
	SRAY_EIO = -7          /* a file could not be opened or written */
};

/* Render options.  Field meanings and defaults follow the reference's
 * struct options (src/opt.h:38-62, defaults src/opt.c:357-388); fields
 * after `meshoct_max_items` are extensions of this library. */
typedef struct sray_opts {
	int width, height;             /* -s WxH                  (640x480) */
	int min_samples, max_samples;  /* -r min[-max]            (1-1) */
	float max_var;                 /* -d max sample variance  (0.005) */
	float min_energy;              /* -e ray energy cut-off   (0.0001) */
	int shadow_samples;            /* -shadowrays             (1) */
	int diffuse_samples;           /* -diffuserays            (1) */
	int threads;                   /* -t host threads of the CPU path (0 = all) */
	int blk_sz;                    /* -b tile size            (48) */
	int iter;                      /* -i max recursion depth  (7) */
	int fps;                       /* -f                      (30) */
	int mblur;                     /* -m motion blur          (0) */
	int shutter;                   /* -u shutter ms           (0) */
	int time_start, time_end;      /* -a range                (0-0) */
	int caust_photons, gi_photons; /* -c, -g                  (0, 0) */
	float gather_dist;             /* -gatherdisc, fraction of the scene diagonal (0.001) */
	float photon_energy;           /* -photonenergy           (300) */
	int scnoct_max_depth, scnoct_max_items;   /* -soctdepth/-soctitems (5/5) */
	int meshoct_max_depth, meshoct_max_items; /* -moctdepth/-moctitems (7/14) */
	/* ---- extensions ---- */
	int caust_k;                   /* >0: k-nearest caustic gather instead of the fixed-radius range */
	int gi_k;                      /* >0: k-nearest global gather */
	float gather_rcap;             /* radius cap of the k-nearest gathers (scene units) */
	int rng_paths;                 /* 1: shading draws keyed by the ray's path in the shading tree */
	uint64_t seed;                 /* Philox key of every random stream */
	/* radiance cache (no reference counterpart): the final gather's indirect
	 * light from the network instead of diffuse rays + photon gathers */
	int nrc;                       /* 0 plain final gather; 1 cache with per-region
	                                  fallback to the plain gather; 2 cache everywhere */
	int nrc_train_samples;         /* training vertices per frame (65536) */
	float nrc_max_rel_err;         /* validation relative error above which a region
	                                  falls back to the plain gather (0.05) */
	int nrc_train_steps;           /* Adam steps per frame over the training vertices (4) */
	int nrc_fallback_samples;      /* final-gather rays per vertex in a fallback region
	                                  (0: diffuse_samples) */
	int reserved[3];
} sray_opts;

/* Fill `o` with the reference defaults (src/opt.c:357-388). */
void sray_default_opts(sray_opts *o);

/* Create the renderer context on the current CUDA device.
 * Replaces rend_init(Image*) (src/render.cc:22-32): the framebuffer is
 * passed to sray_gpu_render() instead of being bound here. */
int sray_gpu_init(const sray_opts *opt);

/* Change options after init (e.g. photon counts, sample counts). */
int sray_gpu_set_opts(const sray_opts *opt);

/* Load an S-ray XML scene.  Replaces Scene::load(const char*)
 * (src/scene.cc:93-183): materials first, then env/object/light/camera,
 * meshes built with the mesh octree options (src/meshload.cc:55-157). */
int sray_gpu_load_scene(const char *xml_path);

/* Same, from an in-memory XML document of `len` bytes. */
int sray_gpu_load_scene_mem(const char *xml, size_t len);

/* Load an XML scene with a binary side-car of its meshes (extension; the
 * reference parses every mesh element, src/meshload.cc:55-157).  When the
 * file at `sidecar` was written for this exact document and the same mesh
 * octree options, the meshes, their octrees and hierarchies are read from
 * it and the document's <mesh> elements are skipped; otherwise the document
 * is loaded in full and the side-car is written.  *used (optional) = 1 when
 * the side-car was used. */
int sray_gpu_load_scene_sidecar(const char *xml_path, const char *sidecar, int *used);

/* ---- A scene given as tables (instead of an XML document) ----
 * The scene classes of the reference -- Scene (src/scene.h:36-130), Object
 * with Sphere / Cylinder / Mesh (src/object.h:40-85, src/sphere.h,
 * src/cylinder.h, src/mesh.h:25-62), Material with its attributes
 * (src/material.h:29-101), Light with SphLight / BoxLight (src/light.h:42-121),
 * Camera / TargetCamera (src/camera.h:26-90) and the keyframe tracks of
 * XFormNode (src/anim.h) -- flattened into plain arrays, so that a scene built
 * or changed in memory reaches the GPU without an XML round trip.  All
 * pointers are host memory, read during the call only. */

/* One keyframe track (src/anim.h Track<T>): key times (ms, ascending) and
 * values (3 doubles per key for position and scale, 4 for rotation as a
 * quaternion s, x, y, z); interpolation 0 step, 1 linear, 2 cubic;
 * extrapolation 0 clamp, 1 repeat.  nkeys = 0: the track's default
 * (position 0, identity rotation, unit scale). */
typedef struct sray_track_desc {
	int nkeys;
	int interp, extrap;
	const int *time;
	const double *val;
} sray_track_desc;

/* An XFormNode: position, rotation and scale tracks and the pivot
 * (src/anim.cc:391-419 builds pivot * T * R * S * -pivot from them). */
typedef struct sray_xform_desc {
	sray_track_desc pos, rot, scale;
	double pivot[3];
} sray_xform_desc;

/* material attributes, in the order of sray_material_desc.attr */
enum { SRAY_ATTR_DIFFUSE, SRAY_ATTR_SPECULAR, SRAY_ATTR_SHININESS, SRAY_ATTR_REFLECT, SRAY_ATTR_REFRACT,
	SRAY_ATTR_IOR, SRAY_ATTR_NORMAL, SRAY_ATTR_COUNT };

/* A texture image: RGBA floats, rows top first (src/img.h Image). */
typedef struct sray_texture_desc {
	int width, height;
	const float *pixels;
} sray_texture_desc;

typedef struct sray_material_desc {
	const char *name;
	int phong;                      /* 1: shade_phong; 0: shade_undef (src/shader.cc:36-73) */
	struct {
		int present;                /* the material has this attribute (Material::have_attribute) */
		double col[4];              /* its colour (MatAttrib::col; scalars in x) */
		int texture;                /* index into sray_scene_desc.textures, -1: none */
	} attr[SRAY_ATTR_COUNT];
} sray_material_desc;

enum { SRAY_OBJ_SPHERE = 0, SRAY_OBJ_CYLINDER = 1, SRAY_OBJ_MESH = 2 };

typedef struct sray_object_desc {
	const char *name;
	int type;                       /* SRAY_OBJ_* */
	int material;                   /* index into sray_scene_desc.materials, -1: the default */
	sray_xform_desc xform;
	double rad, start, end;         /* sphere radius; cylinder radius and y range [start, end) */
	int nfaces;                     /* mesh: triangles, each with its own three vertices
	                                   (src/mesh.h:30-41 Triangle::v) in object space */
	const double *pos;              /* nfaces * 9 */
	const double *normal;           /* nfaces * 9, NULL: zero */
	const double *tangent;          /* nfaces * 9, NULL: zero */
	const double *texcoord;         /* nfaces * 6, NULL: zero */
} sray_object_desc;

enum { SRAY_LIGHT_POINT = 0, SRAY_LIGHT_SPHERE = 1, SRAY_LIGHT_BOX = 2 };

typedef struct sray_light_desc {
	int type;                       /* SRAY_LIGHT_* */
	double color[4];
	sray_xform_desc xform;
	double radius;                  /* sphere light */
	double dim[3];                  /* box light: extent of its box */
} sray_light_desc;

typedef struct sray_camera_desc {
	int target;                     /* 1: TargetCamera, aimed at target_xform's position,
	                                   rolled by its scale track's x (src/camera.cc:216-234) */
	double vfov;                    /* vertical field of view, radians */
	int shutter;                    /* ms */
	sray_xform_desc xform, target_xform;
} sray_camera_desc;

typedef struct sray_scene_desc {
	int n_materials, n_objects, n_lights, n_textures;
	const sray_material_desc *materials;
	const sray_object_desc *objects;
	const sray_light_desc *lights;
	const sray_texture_desc *textures;
	const sray_camera_desc *camera;    /* NULL: the default camera */
	double env_ambient[4], env_color[4], env_ior;
	int reserved[4];
} sray_scene_desc;

/* Load a scene given as tables.  Replaces Scene::load (src/scene.cc:93-183)
 * for a scene that exists in memory: the meshes get their octrees
 * (src/mesh.cc:210-226) and hierarchies, identical meshes share one device
 * copy, and everything after it (sray_gpu_build, _render, ...) is as for
 * sray_gpu_load_scene.  Returns SRAY_EINVAL with a message for a malformed
 * description (bad type, material, texture or face data). */
int sray_gpu_upload_scene(const sray_scene_desc *desc);

/* Prepend a directory to the texture search path SRAY_DATA_PATH, as
 * add_path does (src/datapath.c:40-51); sray prepends the scene file's
 * directory before loading it (src/sray.cc:101-112).  Textures named by a
 * material attribute's "map" are searched in the FIRST directory of the
 * list only, as the reference's find_file does (src/datapath.c:57-113); a
 * texture that is not found leaves its attribute untextured
 * (src/material.cc:64-72).  Binary PPM (P6) files are read.  Affects the
 * next scene load. */
int sray_gpu_add_data_path(const char *dir);

/* Scene summary: counts of objects, lights, materials, triangles (summed
 * over mesh objects), unique device meshes. */
int sray_gpu_scene_info(int *n_objects, int *n_lights, int *n_materials,
		int64_t *n_triangles, int *n_unique_meshes);

/* Build the acceleration structures for the shutter interval [t0, t1]
 * (ms).  Replaces Scene::build_tree (src/scene.cc:353-390). */
int sray_gpu_build(long t0, long t1);

/* Shoot the caustic and global photon maps for [t0, t1] and build the
 * device photon maps.  Replaces shoot_photons (src/render.cc:67-122),
 * Scene::build_caustics_map/build_global_map (src/scene.cc:445-534) and
 * PhotonMap::add_photon/scale_photon_power (src/pmap.cc:73-100).
 * The stored counts are returned through the optional pointers. */
int sray_gpu_shoot_photons(long t0, long t1, int *caust_stored, int *gi_stored, void *stream);

/* Render frame `msec` into an RGBA float32 framebuffer of width*height*4
 * floats (row-major, as the reference's Image, src/render.cc:210-243).
 * `fb_is_device` = 0: `fb` is host memory and is written on return;
 * 1: `fb` is device memory on this context's device.
 * Replaces render(long msec) (src/render.cc:34-55) including the accel
 * build and photon shooting of that frame. */
int sray_gpu_render(long msec, float *fb, int fb_is_device, void *stream);

/* Render only (acceleration structures and photon maps already built by
 * sray_gpu_build / sray_gpu_shoot_photons for the frame containing `msec`):
 * the block loop of render_frame (src/render.cc:124-244). */
int sray_gpu_render_pixels(long msec, float *fb, int fb_is_device, void *stream);

/* Closest hit of `n` rays given in world space (origin xyz, dir xyz with
 * the segment parameter t in [eps, 1], integer time) -- the GPU form of
 * Scene::cast_ray (src/scene.cc:764-794).  All arrays are device pointers.
 * Outputs: object index (-1 = miss), primitive index (triangle index of the
 * object's mesh, 0 for spheres/cylinders), the hit parameter t, and a flag
 * byte that is 1 when another primitive was found at exactly the same t. */
int sray_gpu_cast_rays(int n, const float *orig, const float *dir, const int *time,
		int *obj, int *prim, float *t, unsigned char *tie, void *stream);

/* Primary rays of frame `msec`, sample 0, and their closest hits: per pixel
 * object index, primitive index, t and tie flag (device pointers of
 * width*height entries).  Parity probe for src/camera.cc:119-142 + cast_ray. */
int sray_gpu_primary_hits(long msec, int *obj, int *prim, float *t, unsigned char *tie, void *stream);

/* Photon-map estimates at `n` caller-given points of the current frame's
 * maps: which = 0 is PhotonMap::irradiance_est on the caustic map
 * (src/pmap.cc:109-139), 1 is PhotonMap::radiance_est on the global map
 * (src/pmap.cc:143-178), with the gather radius / k-nearest options of the
 * frame.  pos and norm are device arrays of n*3 floats, out receives n*3
 * floats (rgb).  The maps must have been built (sray_gpu_shoot_photons). */
int sray_gpu_photon_gather(int which, int n, const float *pos, const float *norm, float *out, void *stream);

/* Allocation-free form of sray_gpu_photon_gather.  This entry point has no
 * counterpart in the reference.  It is for callers that must not allocate
 * device memory while they run: an application that hands all device memory
 * to its own pooling allocator (a cudaMalloc from inside the frame can fail
 * or fragment that pool), or an interactive loop that cannot afford the
 * device-wide synchronisation a cudaMalloc or cudaFree implies.  The request
 * staging that sray_gpu_photon_gather allocates lives instead in a fixed
 * array compiled into the library: SRAY_NOALLOC_MAX_POINTS requests (3 MiB,
 * held on every GPU that loads the library until the process exits).
 *  - n > SRAY_NOALLOC_MAX_POINTS is rejected with SRAY_EINVAL.
 *  - The first call on a device looks up the array's device address on that
 *    device (the renderer's, which must be current).  No call may be made
 *    while a stream is being captured into a graph: every call waits for its
 *    stream (below).
 *  - All calls share the one array and it keeps the previous call's
 *    requests; each call writes all the requests it reads, so nothing needs
 *    clearing, but calls that overlap on the GPU (several host threads or
 *    streams at once) race on it.
 * Arguments, results and errors are those of sray_gpu_photon_gather.  Like
 * it, the call waits for `stream` to finish its work (cudaStreamSynchronize)
 * before it returns, so `out` is written on return. */
#define SRAY_NOALLOC_MAX_POINTS 65536
int sray_gpu_photon_gather_noalloc(int which, int n, const float *pos, const float *norm, float *out, void *stream);

/* Copy the stored photons of map `which` (0 = caustic, 1 = global) to host
 * memory as 16 floats each: pos xyz, dir xyz, norm xyz, power rgba, and
 * three unused.  `cap` is the capacity in photons; returns the count through
 * `n_out`.  Photons are in Morton order. */
int sray_gpu_get_photons(int which, float *out, int cap, int *n_out);

/* PhotonMap::dump / restore (src/pmap.cc:180-251), in the reference's text
 * format ("energy %f", then "<pos> <dir> <norm> <col>" per photon).  Restore
 * scales the powers by this renderer's photon_energy over the dump's and
 * builds the map on the device over the current frame's scene bounds
 * (after sray_gpu_build); sray_gpu_render_pixels then gathers from it.
 * The photon count goes through n_out. */
int sray_gpu_dump_photons(int which, const char *path);
int sray_gpu_restore_photons(int which, const char *path, int *n_out);

/* Device-side statistics of the last render: rays traced per kind. */
typedef struct sray_stats {
	int64_t primary_rays, shadow_rays, secondary_rays, gather_rays;
	int64_t photons_emitted, photons_stored, gathers;
	int64_t samples;               /* pixel samples taken (adaptive) */
	int64_t node_visits, prim_tests;  /* traversal work (when counting is on): octree
	                                     node records read, primitive tests */
	int kernel_launches;           /* kernels launched by the last render */
	int pad;
	int64_t h2d_bytes, d2h_bytes;  /* host<->device bytes copied by the last render */
	int64_t gather_tested;         /* photons whose distance a gather computed */
	int64_t gather_candidates;     /* of those, photons within the gather radius */
	int64_t gather_selects;        /* gathers with more candidates than k */
	int64_t gather_spills;         /* gathers whose candidates overflowed the on-chip cache */
	int64_t bvh_fallbacks;         /* mesh hits found through the hierarchy that the
	                                  octree did not confirm (traced by the octree) */
	int64_t shadow_node_visits;    /* the same traversal work of the light samples' */
	int64_t shadow_prim_tests;     /* any-hit passes (when counting is on) */
} sray_stats;

int sray_gpu_get_stats(sray_stats *st);

/* Radiance-cache state of the renderer (opts.nrc != 0). */
typedef struct sray_nrc_stats {
	int64_t frames;                /* frames that trained the cache */
	int64_t vertices;              /* final-gather vertices of the last frame */
	int64_t cached;                /* of those, shaded from the network */
	int64_t train_samples;         /* training vertices of the last frame */
	int64_t val_samples;           /* validation vertices of the last frame */
	int regions;                   /* spatial regions (grid cells over the scene box) */
	int regions_validated;         /* regions with enough validation vertices */
	int regions_cached;            /* regions the network serves (error <= threshold) */
	float val_rel_err;             /* |sum prediction - sum target| / sum target over
	                                  the validated regions (running sums) */
	float loss;                    /* training loss of the last step */
	int pad;
	int64_t reserved[4];
} sray_nrc_stats;

int sray_gpu_nrc_stats(sray_nrc_stats *st);
/* forget the validation history (every region back to the plain gather) and
 * re-initialise the network from `seed` */
int sray_gpu_nrc_reset(uint64_t seed);

/* ---- Radiance cache (extension, no reference counterpart) ----
 * A small MLP standing in for the final gather of indirect light
 * (shade_phong's diffuse rays + PhotonMap::radiance_est, src/shader.cc:154-187,
 * src/pmap.cc:143-178).  Inputs x[n][9]: position scaled to the scene box,
 * unit normal, unit direction (each within [-4096, 4096]); outputs y[n][3].  12-band sin/cos encoding,
 * 216 -> 64 -> 64 -> 64 -> 64 -> 3 (ReLU), BF16 weights on tensor cores with
 * FP32 accumulation, relative L2 loss, Adam (lr 1e-3).  Parameters are
 * exchanged as SRAY_NRC_PARAMS floats in the order W1 (64x216, row-major),
 * b1, W2, b2, W3, b3, W4, b4, W5 (3x64), b5.  Pointers to x, y, targets,
 * gradient and loss are device pointers. */
#define SRAY_NRC_PARAMS 26563

int sray_nrc_reset(uint64_t seed);
int sray_nrc_set_params(const float *params, int n);
int sray_nrc_get_params(float *params, int n);
int sray_nrc_infer(int n, const float *x, float *y, void *stream);
/* the same inference enqueued on `stream` without waiting for it; a
 * tensor-core wait that ran out (SRAY_EDEVICE) is reported by the next
 * sray_nrc_check or sray_nrc_infer */
int sray_nrc_infer_async(int n, const float *x, float *y, void *stream);
/* waits for `stream`; SRAY_EDEVICE when an inference's bounded wait ran out
 * since the last check */
int sray_nrc_check(void *stream);
/* gradient of the loss over the batch (no update) */
int sray_nrc_gradients(int n, const float *x, const float *targets, float *grad, float *loss, void *stream);
/* one Adam step on the batch; *loss (device, optional) = the batch loss before the step */
int sray_nrc_train(int n, const float *x, const float *targets, float *loss, void *stream);
int sray_nrc_last_error(char *buf, size_t len);

/* Profiling (extension, no reference counterpart).  flags bit 0: time every
 * kernel launch with CUDA events recorded on the launch stream; bit 1: count
 * octree node records read and primitive tests in the closest-hit kernel (slower;
 * reported through sray_stats.node_visits / prim_tests). */
int sray_gpu_set_profiling(int flags);

/* Accumulated kernel times since the last call with reset = 1: for up to
 * `max` kernel kinds, the name (NUL-separated in `names`), total ms and
 * launch count.  Returns the number of kinds through `n_out`.  Kinds named
 * "host.<phase>" are host wall-clock phases timed beside the kernels (a
 * batch's frame build, the photon thread, waits for the photon maps and for
 * each bounce's queue count); their count is the times the phase ran. */
int sray_gpu_kernel_times(char *names, size_t names_cap, double *ms, int64_t *launches, int max,
		int *n_out, int reset);

/* Scheduler tuning (extension, no reference counterpart; the reference's
 * scheduler is a thread pool over 48x48 tiles, src/tpool.cc:48-225).  The
 * queue depths at which a wavefront's tail is handed to a persistent launch,
 * that launch's size, thread- or warp-per-ray traversal by pass size, the
 * any-hit child order and the streams' priorities.  The defaults are the
 * autotuner's choice on the 1080p production frame. */
typedef struct sray_tuning {
	int render_tail;          /* rays in flight below which the rest of the shading tree
	                             runs in the persistent pool launch (0: none) */
	int pool_blocks_per_sm;   /* 128-thread blocks per SM of the pool launch (4) */
	int photon_tail;          /* photons in flight below which the photon tail runs in one
	                             persistent launch (65536) */
	int shadow_order;         /* any-hit traversal of light samples: 0 visits a node's hit
	                             children nearest first, 1 in the node's order (0) */
	int stream_priority;      /* which of the two concurrent streams gets the device's
	                             greatest priority: 0 neither, 1 the photon stream, 2 the
	                             render work (on an internal stream ordered after and
	                             before the caller's) (2) */
	int warp_rays;            /* closest-hit passes of at most this many rays trace one
	                             ray per warp instead of one per thread (0: never) (16384) */
	int warp_segments;        /* the same for light-sample passes of at most this many
	                             segments (16384) */
	int queue_depth;          /* primary rays per wave: a sample batch's pixels go through
	                             the shading tree in waves of at most this many primary
	                             rays, each wave finished before the next (0: one wave) (0) */
	int side_gather;          /* 1: the first sample batch's photon-map gathers start as
	                             soon as the maps exist, on a stream of their own beside
	                             the remaining bounces; 2: the same, the render loop
	                             waiting for the maps at the second bounce (a check of
	                             that path independent of timing) (0) */
	int sort_rays;            /* secondary closest-hit passes of at least this many rays are
	                             first sorted by direction octant and origin cell, so that a
	                             warp's rays start close together and head the same way
	                             (0: never) (0) */
	int side_shadow;          /* 1: a bounce's light samples and photon-map gathers run on a
	                             stream of their own beside the next bounce's closest hits
	                             and shading (1) */
} sray_tuning;

typedef struct sray_tune_trial {
	sray_tuning tuning;
	float ms_per_frame;       /* mean over the trial's timed frames */
	int pad;
} sray_tune_trial;

int sray_gpu_get_tuning(sray_tuning *t);
int sray_gpu_set_tuning(const sray_tuning *t);

/* The autotuner: renders frame `msec` into the device framebuffer `fb` on
 * `stream` under candidate tunings (coordinate descent over the fields of
 * sray_tuning, one warm-up and two groups of `frames` timed frames each,
 * CUDA-event timing, the slower group counting), keeps the fastest and
 * returns it with its time.  Every trial goes into `log` (up to `log_cap`,
 * count through `n_log`). */
int sray_gpu_autotune(long msec, float *fb, int frames, void *stream, sray_tuning *best, float *best_ms,
		sray_tune_trial *log, int log_cap, int *n_log);

/* Host-side fault injection for tests (extension, no reference
 * counterpart; the reference's only failure handling is its signal
 * handlers, src/sray.cc:85-89).  Nothing here makes a kernel fault, trap or
 * hang: the injected conditions are ones the library already detects and
 * reports, made to happen on demand.  Settings hold until changed (all zero
 * but fail_alloc_after = -1 turns injection off).
 *  - fail_alloc_after >= 0: that many more device allocations succeed, then
 *    every one fails as out of memory; the call that needed it returns
 *    SRAY_ENOMEM and the context stays usable.
 *  - queue_cap > 0: the shading tree's child ray queue takes at most that
 *    many rays; a frame that makes more returns SRAY_EDEVICE.
 *  - pool_spin_limit > 0: polls of a slot before the persistent shading
 *    pool (sray_tuning.render_tail) gives up waiting for work (default
 *    about half a second); a frame whose wait runs out returns
 *    SRAY_EDEVICE.
 *  - photon_group > 0: a batch's photon maps are traced in wavefronts of
 *    at most about that many photons (whole jobs; default 2^26), each
 *    group's maps copied out of the wavefront's buffers before the next;
 *    the images do not change. */
typedef struct sray_faults {
	int fail_alloc_after;
	int queue_cap;
	int pool_spin_limit;
	int photon_group;
	int reserved[4];
} sray_faults;

int sray_gpu_set_faults(const sray_faults *f);

/* Copy the last error message (NUL-terminated, truncated to `cap`). */
int sray_gpu_last_error(char *buf, size_t cap);

/* The autotuner for batches (sray_gpu_render_batch): the queue depth
 * (65,536, 262,144, 1,048,576, 4,194,304 or 16,777,216 primary rays per
 * wave; device memory grows with it) against the
 * traversal mode (thread per ray; one warp per ray in passes of at most
 * 16,384 rays or segments; one warp per ray in every pass), then the best
 * pair with the shading tree's tail in the persistent pool launch (below
 * 32,768 and 131,072 rays in flight); each trial timed over `frames`
 * batches after one warm-up.  Keeps and returns the fastest; trials go into
 * `log` as for sray_gpu_autotune. */
struct sray_job;
int sray_gpu_autotune_batch(const struct sray_job *jobs, int n, int frames, void *stream, sray_tuning *best, float *best_ms,
		sray_tune_trial *log, int log_cap, int *n_log);

/* A batch of frames of the loaded scene in one wavefront (extension; the
 * reference renders one frame per render() call, src/render.cc:34-55).
 * Each job has its own frame time, resolution and device framebuffer
 * (width * height * 4 floats), its scene (in a scene set) and optionally its
 * own photon counts; the jobs share the other options (samples, depth) and
 * use their scene's camera (its aspect is the one set at load, as for a
 * single frame).  The acceleration structures are built once over the union of
 * the jobs' shutter intervals, each job gets its own photon maps (shot over
 * its own interval), and all jobs' pixels go through the same camera,
 * closest-hit, shading, shadow and gather launches and the same adaptive
 * sample batches.  A job's image equals the one sray_gpu_render gives for
 * it alone, except that its random streams are keyed by its pixel's index
 * in the batch (job j's pixels follow those of jobs 0..j-1): job 0 matches
 * exactly. */
typedef struct sray_job {
	long msec;
	int width, height;
	float *fb;                /* device framebuffer */
	int scene;                /* its scene in a scene set (sray_gpu_load_scene_set); 0 otherwise */
	int caust_photons;        /* its photon counts (0: the options') */
	int gi_photons;
	int reserved;
} sray_job;

int sray_gpu_render_batch(const sray_job *jobs, int n, void *stream);

/* Load several scene documents as one scene set (extension; the reference
 * holds one scene, src/scene.h:32-33): batches can then mix jobs of
 * different scenes (sray_job.scene = the index into xml_paths), each
 * rendered as sray_gpu_render would render it alone with the same random
 * streams, keyed by its pixels' place in the batch.  The scenes' meshes,
 * materials, lights and cameras live side by side in one set of device
 * tables; each frame builds every scene's octree and object hierarchy, and
 * a ray finds its scene through its job.  A scene set renders through
 * sray_gpu_render_batch only (nrc = 0); one document makes an ordinary
 * scene. */
int sray_gpu_load_scene_set(const char *const *xml_paths, int n);

/* Release every device buffer and the context. */
void sray_gpu_shutdown(void);

#ifdef __cplusplus
}
#endif

#endif /* SRAY_GPU_H_ */
