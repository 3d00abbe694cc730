/* renderer.h -- host-side state of the GPU renderer behind the C-ABI. */
#ifndef SRAY_RENDERER_H_
#define SRAY_RENDERER_H_

#include <string>
#include <vector>
#include <atomic>
#include <mutex>
#include <thread>
#include <chrono>
#include <cuda_runtime.h>
#include "sray_gpu.h"
#include "scene_host.h"
#include "dev_common.cuh"

namespace sray {

/* Host-side fault injection (sray_gpu_set_faults): the device allocations
 * left before they fail as out of memory (-1: off), a cap on the shading
 * tree's child queue, and the persistent pool's wait limit.  Nothing here
 * makes a kernel fault, trap or hang. */
struct FaultState {
	std::atomic<int> alloc_left{-1};
	std::atomic<int> queue_cap{0};
	std::atomic<int> spin_limit{0};
	std::atomic<int> photon_group{0};
};
extern FaultState g_faults;

/* one device allocation under the injected failure count */
static inline bool fault_alloc_fails()
{
	int left = g_faults.alloc_left.load();
	while(left > 0 && !g_faults.alloc_left.compare_exchange_weak(left, left - 1)) {}
	return left == 0;
}

/* a device allocation that only grows */
struct DevBuf {
	void *p = nullptr;
	size_t bytes = 0;
	cudaError_t ensure(size_t n)
	{
		if(n <= bytes) return cudaSuccess;
		if(p) cudaFree(p);
		p = nullptr;
		bytes = 0;
		if(fault_alloc_fails()) return cudaErrorMemoryAllocation;
		cudaError_t e = cudaMalloc(&p, n < 256 ? 256 : n);
		if(e == cudaSuccess) bytes = n < 256 ? 256 : n;
		return e;
	}
	template <class T> cudaError_t upload(const std::vector<T> &v, cudaStream_t s)
	{
		cudaError_t e = ensure(v.size() * sizeof(T) + 16);
		if(e != cudaSuccess || v.empty()) return e;
		return cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
	}
	void release()
	{
		if(p) cudaFree(p);
		p = nullptr;
		bytes = 0;
	}
	template <class T> T *as() const { return (T *)p; }
};

/* structure-of-arrays ray queue */
struct RayQueue {
	float4 *o;      /* origin xyz, energy */
	float4 *d;      /* direction xyz, current ior */
	float4 *w;      /* throughput weight rgb, unused */
	int4 *meta;     /* pixel, iter, path, time */
	float4 *stk;    /* ior stack */
	int2 *ext;      /* sample | diffuse index << 16, stack depth */
	int *count;
	int cap;
};

/* a pending photon-map gather: pos + kind, normal + pixel, weight */
struct GatherReq {
	float4 a;
	float4 b;
	float4 w;
};

/* a shadow ray: origin + time, direction + pixel, contribution if unoccluded */
struct ShadowReq {
	float4 a;
	float4 b;
	float4 w;
};

/* device-side error and work counters */
struct DevCounters {
	int overflow;        /* traversal stack or queue overflow */
	int gen_dir_fail;    /* projection-map rejection sampling gave up */
	int pad[2];
	unsigned long long rays[4];   /* primary, secondary, shadow, gather */
	unsigned long long nodes, prims;
	unsigned long long g_tested, g_cand, g_select, g_spill;   /* gather work */
	unsigned long long bvh_fallbacks;   /* hierarchy hits the octree did not confirm */
	unsigned long long snodes, sprims;  /* node records read and primitive tests of light samples */
	unsigned long long nrc[4];          /* final-gather vertices, cached: sample batch 0, batch 1 */
};

/* per-region validation of the radiance cache: the frame's sums of
 * prediction and target (channel sums), the record count and the squared
 * prediction - target differences, their running
 * (exponentially decayed) totals, the fallback flags the shading kernels
 * read, and a summary [validated regions, cached regions, relative error] */
struct NrcRegionStats {
	float sy[NRC_REGIONS], st[NRC_REGIONS], sn[NRC_REGIONS], sq[NRC_REGIONS];
	float ey[NRC_REGIONS], et[NRC_REGIONS], en[NRC_REGIONS], eq[NRC_REGIONS];
	float summary[4];
	unsigned char fallback[NRC_REGIONS];
};

struct PhotonBufs {
	DevBuf ph, cells, tmp_ph, keys, keys2, vals, vals2, lin, hist, scan;
	DPhotonMap map;
	int n = 0;
};

struct Renderer {
	sray_opts opt;
	int device = 0;
	HostScene sc;
	bool loaded = false;
	std::string err;

	/* scene tables (per load) */
	DevBuf mnodes, mtris, mprim, tri_pos, tri_attr, objs, mats, texs, texels, lights, bnodes, btris, bprim, bhome;
	DevBuf anims, key_t, key_v;   /* keyframe tracks of the objects, then the lights */
	/* frame tables (per build) */
	DevBuf snodes, sslots, xf, light_pos, cam_m, tnodes, ohome;
	bool built = false;
	bool has_tlas = false;
	int t0 = 0, t1 = 0, tlo = 0, nt = 1;
	int scene_root = 0;
	long frame_msec = 0;
	bool photons_ready = false;
	PhotonBufs caust, gi;
	DScene S = {};                /* S.nrc is set per sample batch (nrc_setup) */

	/* render buffers */
	DevBuf qbuf[2], hits, gq, sq, acc, hist, sums, active[2], spp, fbdev, ctr, counts, fbl, pool_ready;
	RayQueue q[2];
	int qcap[2] = {0, 0};
	/* a pass sorted before it is traced (sray_tuning.sort_rays): the sorted
	 * copy's queue (swapped with the pass's), keys and values, scratch */
	DevBuf qsbuf, rs_keys, rs_hist, rs_part;
	/* pinned host words the per-pass counts are read into (a read into
	 * pageable memory is staged and waits inside the copy call): [0..7] the
	 * render loop's, [8..15] the photon thread's */
	int *pin = nullptr;
	RayQueue qs = {};
	int qscap = 0;
	int sort_pass(int cur, int n, cudaStream_t s);
	/* queue Q's first n entries in the order of the top `bits` of their
	 * 24-bit keys (direction octant over the Morton code of the origin's cell
	 * in a 128^3 grid), through the scratch queue T (swapped with Q) and the
	 * key, histogram and partial-sum buffers */
	int sort_queue(RayQueue &Q, DevBuf &Qbuf, int &Qcap, RayQueue &T, DevBuf &Tbuf, int &Tcap, DevBuf &keysb, DevBuf &hist,
			DevBuf &part, int n, int bits, const char *name, cudaStream_t s);
	/* photon tracing has buffers and a stream of its own, so that it can run
	 * beside the first bounce of a frame */
	DevBuf pqbuf[2], phits, pfbl, pcounts, pctr;
	RayQueue pq[2];
	int pqcap[2] = {0, 0};
	/* an emission pass of at least PHOTON_SORT_MIN photons is sorted before
	 * it is traced, with scratch of its own (the photon stream runs beside
	 * the frame's) */
	DevBuf pqsbuf, ps_keys, ps_hist, ps_part;
	RayQueue pqs = {};
	int pqscap = 0;
	int sort_photon_pass(int cur, int n, cudaStream_t s);
	cudaStream_t ps = nullptr;
	int ps_priority = -1;      /* 1 when ps has the greatest priority */
	cudaStream_t hs = nullptr; /* the frame's stream under stream_priority 2 */
	cudaStream_t gs = nullptr; /* the gather stream under side_gather */
	cudaEvent_t gs_fork = nullptr, gs_done = nullptr;
	/* side_shadow: the light-sample stream, its requests double-buffered
	 * by bounce parity (sq / gq for even bounces, sq2 / gq2 for odd), its
	 * fallback lists */
	cudaStream_t xs = nullptr;
	int xs_priority = -1;      /* 1 when xs has the greatest priority */
	cudaEvent_t xs_fork = nullptr, xs_done[2] = {nullptr, nullptr};
	DevBuf sq2, gq2, fbs[2];
	int side_stream();
	int shadow_rays_on(const ShadowReq *q, int *count, int cap, DevBuf &fb, cudaStream_t st);
	DevBuf gq_side;            /* its copy of the accumulated gather requests */
	std::atomic<bool> photon_finished{false};   /* the photon thread has returned */
	int gather_stream();
	cudaEvent_t hs_fork = nullptr, hs_join = nullptr;
	int priority_stream();
	int shadow_rays(int cap, cudaStream_t s);

	cudaEvent_t ps_done = nullptr;
	sray_stats stats;
	/* the autotuner's choice on the production frame */
	sray_tuning tune = {0, 4, 65536, 0, 2, 16384, 16384, 0, 0, 0, 1};
	int nsm = 0;                  /* multiprocessors of the device */
	/* Octree retraces follow every hierarchy pass and nearly always find no
	 * ray listed (a couple a frame).  Their grid-stride launches are sized
	 * from the last frame's count: one block when it was small, so that an
	 * empty launch needs a single free slot instead of one on every SM
	 * (beside the photon stream's blocks, a full-width launch waited for
	 * SMs to drain).  Any count is traced correctly, only more slowly. */
	std::atomic<int64_t> retrace_hint{0};   /* also read by the photon thread */
	int retrace_grid() const
	{
		int64_t b = (retrace_hint.load(std::memory_order_relaxed) + 127) / 128;
		return b < 1 ? 1 : (b > nsm ? nsm : (int)b);
	}

	/* radiance cache: queries (inputs, weight + slot), training and
	 * validation records (inputs, targets, predictions), region statistics */
	DevBuf nrc_qx, nrc_qw, nrc_rx, nrc_rt, nrc_ry, nrc_regions;
	int nrc_qcap = 0, nrc_rcap = 0;
	bool nrc_regions_ready = false;
	int64_t nrc_frames = 0;
	int64_t nrc_expect = 0;       /* final-gather vertices of the last frame's first sample batch */
	int nrc_last_train = 0, nrc_last_val = 0;
	int64_t nrc_last_vertices = 0, nrc_last_cached = 0;
	/* a batch of jobs (render_batch): their pixel count, job table, photon
	 * maps (caustic and global per job) */
	struct JobMaps { PhotonBufs caust, gi; };
	int batch_npix = 0;
	std::vector<int> batch_t0, batch_t1;   /* jobs' shutter intervals: the photon job shoots one map pair each */
	double map_gather_dist = -1.0;         /* >= 0: the range radius of the maps being built (a batch job's) */
	bool map_has_box = false;              /* the grid box of the maps being built (a batch job's scene */
	Box map_box;                           /* over its own interval), else the frame octree's root box */
	void batch_projmaps(std::vector<std::vector<uint32_t>> &bits, std::vector<std::vector<float>> &cov);
	/* the photon wavefront's tables (photon.cu): jobs, per-light prefix sums
	 * and scales, projection maps and coverages, the photons' job table for
	 * the traversal, stored photons and their flags by global index */
	DevBuf pw_jobs, pw_prefix, pw_scale, pw_bits, pw_cov, pw_pix, pw_out, pw_valid;
	/* a batch's maps built together (photon_finalize_jobs): scan scratch,
	 * segment bounds and offsets, compacted and sorted photons, grids, keys,
	 * cell tables */
	DevBuf pw_part, pw_tiles, pw_bounds, pw_offs, pw_ph, pw_sorted, pw_grids, pw_morton, pw_cellbase, pw_keys, pw_lin, pw_cells, pw_hist;
	std::vector<int> batch_scene, batch_caust, batch_gi;   /* jobs' scenes and photon counts (0: the options') */
	/* a scene set: its scene descriptors on the device */
	DevBuf dscenes;
	std::vector<DevSceneRef> scene_refs;
	bool in_batch = false;
	int build_frame_set(long t0, long t1, cudaStream_t s);
	DevBuf djobs, dmaps;
	std::vector<JobMaps> job_maps;
	int render_batch(const sray_job *jobs, int n, cudaStream_t s);
	int nrc_setup(int batch, int n_prim, int wave_rays, cudaStream_t s);
	int nrc_wave_done(cudaStream_t s);
	int nrc_batch_done(int batch, cudaStream_t s);
	int nrc_reset_regions(cudaStream_t s);

	/* profiling: event pairs per launch, resolved after each synchronisation.
	 * The photon maps are traced by a host thread of their own beside the
	 * render loop, so the bookkeeping is locked and the byte counters are
	 * atomic. */
	int prof_flags = 0;
	long long launch_count = 0;
	std::atomic<int64_t> h2d{0}, d2h{0};   /* host<->device bytes since the last reset */
	struct KTime { std::string name; double ms = 0.0; long long launches = 0; };
	std::vector<KTime> ktimes;
	struct Pending { int kind; cudaEvent_t a, b; };
	std::vector<Pending> pending;
	std::vector<cudaEvent_t> event_pool;
	std::mutex prof_mu;
	int kind_of(const char *name);
	/* host time of a phase since t0 (host_now_ms), kept beside the kernels'
	 * under its name ("host.<phase>") while kernel timing is on */
	void host_time(const char *name, double t0);
	static double host_now_ms()
	{
		return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
	}
	void prof_begin(const char *name, int *kind_cache, cudaStream_t s, Pending *p);
	void prof_end(Pending *p, cudaStream_t s);
	void prof_collect();

	/* the photon maps of a frame, traced by a host thread on the photon
	 * stream while the render loop goes on; the photon-map gathers wait */
	std::thread photon_thread;
	int photon_rc = 0;
	int start_photon_job(cudaStream_t s);
	int finish_photon_job();
	int photon_job(DScene base);
	int shoot_maps(const DScene &base, cudaStream_t s, int *nc, int *ng);

	int fail(int code, const std::string &msg) { err = msg; return code; }
	int cuda_fail(cudaError_t e, const char *where)
	{
		err = std::string(where) + ": " + cudaGetErrorString(e);
		return e == cudaErrorMemoryAllocation ? SRAY_ENOMEM : SRAY_ECUDA;
	}

	int upload_scene(cudaStream_t s);
	int build_frame(long t0, long t1, cudaStream_t s);
	int shoot(cudaStream_t s, int *nc, int *ng);
	/* overlap_photons: shoot the photon maps on the photon stream while the
	 * first bounce's closest hits, shading and shadow rays run, the gathers
	 * waiting for them */
	int render_pixels(long msec, float *fb, int fb_is_device, cudaStream_t s, bool overlap_photons = false);
	int ensure_queue(int which, int cap);
	int child_cap(int cap) const;
	int queue_overflow(int count, int cap);
	int ensure_pqueue(int which, int cap);
	int queue_alloc(DevBuf &buf, RayQueue &Q, int &qc, int cap);
	/* coherent: a pass of camera rays (traced as warp packets when it is large) */
	int trace_rays(const RayQueue &q, int n, const char *name, bool count, cudaStream_t s, bool coherent = false);
	int trace_rays_with(const DScene &D, const RayQueue &q, int n, const char *name, bool count, cudaStream_t s, int4 *hit_out,
			DevBuf &fb, DevCounters *c, bool short_blocks = false, bool coherent = false);
	int photon_stream();
	void fill_scene_desc();
};

#define LAUNCH(R_, kname_, s_, ...) do { \
		static thread_local int kind_ = -1; \
		Renderer::Pending pend_; (R_).prof_begin(kname_, &kind_, s_, &pend_); \
		__VA_ARGS__; \
		(R_).prof_end(&pend_, s_); \
	} while(0)

/* render.cu: closest hits of the first n rays of q into R.hits */
int launch_trace(Renderer &R, const DScene &D, const RayQueue &q, int n, const char *name, cudaStream_t s);

/* photon.cu: both maps traced with the scene view `base` */
/* a frame's photon maps as a job of the photon wavefront (photon.cu) */
struct PhotonJobSpec {
	int num[2] = {0, 0};          /* photons asked for: caustic, global map */
	int light0 = 0, nlights = 0;  /* its scene's lights */
	int t0 = 0, t1 = 0;           /* its interval */
	int scene = -1;               /* its scene in a scene set (-1: the view's own) */
	const std::vector<uint32_t> *bits = nullptr;   /* its projection maps, 128 words per light */
	const std::vector<float> *cov = nullptr;       /* their coverages, 2 per light */
};
struct PJobOut { int base = 0; int total[2] = {0, 0}; };   /* a job's photons: first global index, counts per map */
int photon_trace_jobs(Renderer &R, const DScene &base, const std::vector<PhotonJobSpec> &spec, std::vector<PJobOut> &out,
		cudaStream_t s);
int photon_finalize(Renderer &R, int global, const int *valid, const DevPhoton *in, int total, cudaStream_t s, int *stored);
int sort_pairs(Renderer &R, unsigned *keys, unsigned *vals, unsigned *keys2, unsigned *vals2, int n, int bits, DevBuf &hist,
		DevBuf &part, const char *name, cudaStream_t s, unsigned **vals_out);
int photon_finalize_jobs(Renderer &R, const std::vector<PJobOut> &jobs, const std::vector<Box> &boxes,
		const std::vector<double> &gather_dist, std::vector<DPhotonMap> &maps, cudaStream_t s);
int photon_shoot_maps(Renderer &R, const DScene &base, const std::vector<uint32_t> &bits, const std::vector<float> &cov,
		cudaStream_t s, int *caust_stored, int *gi_stored);
/* photon.cu: map `global` (0 caustic, 1 global) over the n photons in its buffer / from host photons */
int photon_map_build(Renderer &R, int global, int n, cudaStream_t s);
int photon_map_restore(Renderer &R, int global, const std::vector<DevPhoton> &h, cudaStream_t s);

}  // namespace sray

#endif
