/* photon.cu -- photon emission and tracing, and the device photon map.
 *
 *   k_photon_emit   Light::gen_photon (src/light.cc:111-148) with ProjMap::gen_dir
 *                   (src/projmap.cc:193-209), one thread per photon, each on its
 *                   own Philox stream, so photon j of light i is the same photon
 *                   the CPU oracle shoots
 *   k_photon_bounce Scene::trace_caustics_photon / trace_global_photon
 *                   (src/scene.cc:571-760), one interaction per pass; the
 *                   renderer's k_trace finds the hits in between
 *   compaction      keeps stored photons in emission order
 *   k_rs_*          stable LSD radix sort of the photons by the Morton code of
 *                   their grid cell
 *   k_cells         (first, end) of every occupied cell
 * PhotonMap::add_photon / scale_photon_power (src/pmap.cc:73-100) become the
 * per-light power scale applied at store time.  The kd-tree of the reference
 * (kd_insert3f, kd_nearest_range3f) is replaced by the Morton-ordered grid:
 * a range query visits the cells overlapping the query cube and tests every
 * photon in them with the kd-tree's distance rule, so the photon set of each
 * gather is the same.
 */
#include <math.h>
#include <string.h>
#include <algorithm>
#include <cooperative_groups.h>
#include "renderer.h"

namespace cg = cooperative_groups;

namespace sray {

enum { CAUST_PHOTON = 1, GI_PHOTON = 2, DIRECT_PHOTON = 0 };

struct PRay {
	V3 o, d;
	int time, iter;
	IorStack st;
};

struct PState {
	float col[3];
	int type;
	V3 pos, dir, norm;
};

/* outcome of one photon-surface interaction */
enum { P_DROP = 0, P_STORE = 1, P_CONT = 2, P_TO_CAUST = 3 };

__device__ __forceinline__ void refract_ray(PRay &r, V3 n, float mat_ior, bool entering, float ray_mag)
{
	float ior = r.st.calc_ior(entering, mat_ior);
	if(entering) r.st.enter(mat_ior);
	else r.st.leave();
	r.d = refraction(r.d / ray_mag, n, ior) * ray_mag;
	if(dot(r.d, n) > 0.0f) {
		if(entering) r.st.leave();
		else r.st.enter(mat_ior);
	}
}

/* one iteration of Scene::trace_caustics_photon (src/scene.cc:571-647) at
 * the hit h: reflect or refract (P_CONT) or absorb and store (P_STORE) */
__device__ int caust_step(const DScene &S, PRay &r, PState &ph, const Hit &h, sray_rng *s)
{
	const DevMat &m = mat_of(S, h.obj);
	Surf sp;
	surface_point(S, h, r.o, r.d, r.time, sp, m.textured, m.textured && m.tex[TA_NORMAL] >= 0);
	MatVals mv;
	mat_values(S, m, sp.tex, mv);
	float refl = mv.refl, refr = mv.refr, mat_ior = mv.ior;
	bool entering;
	V3 normal;
	float ray_mag = len(r.d);
	if(dot(r.d, sp.normal) > 0.0f) { normal = -sp.normal; entering = false; }
	else { normal = sp.normal; entering = true; }
	float ior = r.st.calc_ior(entering, mat_ior);
	/* a normal map replaces the normal after the index of refraction is
	 * known (src/scene.cc:600-605) */
	if(m.have_normal) normal = bump_normal(S, m, sp);
	float ray_dot_n = dot(-r.d / ray_mag, normal);
	float sf0 = refr > 0.0f ? (ior - 1.0f) / (ior + 1.0f) : 1.0f;
	float fres = fresnel(sf0 * sf0, ray_dot_n);
	refl = fres * refl;
	refr = (1.0f - fres) * refr;
	float rnum = frand(s, 1.0f);
	if(rnum < refl) {
		r.d = reflection(r.d, normal);
		r.iter--;
		r.o = sp.pos;
		ph.type = CAUST_PHOTON;
		for(int k = 0; k < 3; k++) ph.col[k] = ph.col[k] * mv.ks[k];
		return P_CONT;
	}
	if(rnum < refr) {
		refract_ray(r, normal, mat_ior, entering, ray_mag);
		r.o = sp.pos;
		ph.type = CAUST_PHOTON;
		for(int k = 0; k < 3; k++) ph.col[k] = ph.col[k] * mv.ks[k];
		return P_CONT;
	}
	ph.dir = normalized(r.d);
	ph.pos = sp.pos;
	ph.norm = normal;
	return P_STORE;
}

/* one iteration of Scene::trace_global_photon (src/scene.cc:650-760) at the
 * hit h: diffuse bounce (P_CONT), specular bounce that hands the photon to
 * the caustic rules (P_TO_CAUST), absorption (P_DROP) or storage (P_STORE) */
__device__ int global_step(const DScene &S, PRay &r, PState &ph, const Hit &h, sray_rng *s)
{
	V3 incident = normalized(r.d);
	const DevMat &m = mat_of(S, h.obj);
	Surf sp;
	surface_point(S, h, r.o, r.d, r.time, sp, m.textured);
	V3 normal;
	bool entering;
	float ray_mag = len(r.d);
	if(dot(r.d, sp.normal) > 0.0f) { normal = -sp.normal; entering = false; }
	else { normal = sp.normal; entering = true; }
	MatVals mv;
	mat_values(S, m, sp.tex, mv);
	float diff_avg = (mv.kd[0] + mv.kd[1] + mv.kd[2]) / 3.0f;
	float spec_avg = (mv.ks[0] + mv.ks[1] + mv.ks[2]) / 3.0f;
	float rnum = frand(s, 1.0f);
	if(rnum < diff_avg) {
		V3 dir = sphrand(s, 1.0f);
		if(dot(dir, normal) < 0.0f) dir = -dir;
		float ndotl = dot(-incident, normal);
		r.d = dir * (float)SRAY_RAY_MAGNITUDE;
		r.iter--;
		r.o = sp.pos;
		ph.type = GI_PHOTON;
		for(int k = 0; k < 3; k++) ph.col[k] = ph.col[k] * (ndotl * (mv.kd[k] / diff_avg));
		return P_CONT;
	}
	if(rnum < diff_avg + spec_avg) {
		float refl = mv.refl, refr = mv.refr, mat_ior = mv.ior;
		float ior = r.st.calc_ior(entering, mat_ior);
		float ray_dot_n = dot(-r.d / ray_mag, normal);
		float sf0 = refr > 0.0f ? (ior - 1.0f) / (ior + 1.0f) : 1.0f;
		float fres = fresnel(sf0 * sf0, ray_dot_n);
		refl = fres * refl;
		refr = (1.0f - fres) * refr;
		float rn2 = frand(s, 1.0f);
		if(rn2 < refl) {
			r.d = reflection(r.d, normal);
			r.iter--;
			r.o = sp.pos;
			ph.type = CAUST_PHOTON;
			for(int k = 0; k < 3; k++) ph.col[k] = ph.col[k] * mv.ks[k];
			return P_TO_CAUST;
		}
		if(rn2 < refr) {
			refract_ray(r, normal, mat_ior, entering, ray_mag);
			r.o = sp.pos;
			ph.type = CAUST_PHOTON;
			for(int k = 0; k < 3; k++) ph.col[k] = ph.col[k] * mv.ks[k];
			return P_TO_CAUST;
		}
		return P_DROP;
	}
	ph.dir = incident;
	ph.pos = sp.pos;
	ph.norm = normal;
	return P_STORE;
}

/* ProjMap::gen_dir(true) with cell_from_dir in deterministic float math;
 * gives up (photon lost, error word set) after a bounded number of tries */
__device__ bool gen_dir(const uint32_t *bits, sray_rng *s, V3 *out)
{
	for(int it = 0; it < (1 << 20); it++) {
		V3 v = sphrand(s, 1.0f);
		float theta = sray_atan2_f(v.z, v.x);
		float phi = sray_atan2_f(sqrtf(v.x * v.x + v.z * v.z), v.y);
		if(theta < 0.0f) theta = SRAY_TWO_PI_F + theta;
		float u = theta / SRAY_TWO_PI_F, w = phi / SRAY_PI_F;
		int uc = (int)(u * 64.0f), vc = (int)(w * 32.0f);
		uc = uc < 0 ? 0 : (uc > 63 ? 63 : uc);
		vc = vc < 0 ? 0 : (vc > 31 ? 31 : vc);
		int idx = vc * 64 + uc;
		if(bits[idx >> 5] & (1u << (idx & 31))) { *out = v; return true; }
	}
	return false;
}

/* The reference traces one photon to its end with recursive calls, one map
 * after the other.  Here the photons of both maps advance together, one
 * surface interaction per pass, over ray queues that the renderer's
 * closest-hit kernel traces:
 *   k_photon_emit    Light::gen_photon (src/light.cc:111-148) with
 *                    ProjMap::gen_dir (src/projmap.cc:193-209) -> queue
 *   k_trace          closest hits of the queue (render.cu)
 *   k_photon_bounce  one trace_caustics_photon / trace_global_photon step
 *                    per photon -> stored photon, next queue, or loss
 *   k_photon_finish  the last photons, each traced to its end
 * A photon keeps its own Philox stream: the queue carries its stream address
 * (map, light, index) and draw count, so photon j of light i takes the same
 * draws and the same path as the CPU oracle's recursive tracer.
 *
 * Photon queue entry (RayQueue fields):
 *   o = origin, colour r     d = direction, colour g
 *   w = colour b, ior, interactions in this phase, photon index in its map
 *   meta = light, iter, phase | type << 4 | map << 8, time
 *   stk = ior stack          ext = draws taken, stack depth
 * Phase 0 follows the global rules, phase 1 the caustic rules; map 0 is the
 * caustic map, map 1 the global one. */

#define PHOTON_GUARD 4096   /* interactions per phase (loop bound of the oracle's tracer) */
#define PHOTON_SORT_MIN (1 << 20)   /* an emission pass of at least this many photons is sorted before it is traced */

/* A job of the photon wavefront: one frame's two maps (a batch traces the
 * maps of all its jobs in one wavefront).  Its photons are the global
 * indices [base, base + total[0]) (caustic map) and then total[1] more
 * (global map); each keeps the stream address of its frame's own photon
 * (map, light within the scene, index within the light). */
struct PJob {
	int base;
	int total[2];
	int light0, nlights;  /* its scene's lights in the light table */
	int prefix0;          /* per-light prefix sums at prefix + prefix0: the caustic
	                         map's nlights + 1, then the global map's */
	int scale0;           /* per-light power scales at scale + scale0: caustic, then global */
	int proj0;            /* its first light's projection maps (128 words) and coverages (2) */
	int t0, t1;           /* the frame's interval */
};

struct PhotonSet {
	int njobs, total;
	const PJob *jobs;
	const int *prefix;
	const float *scale;
	const uint32_t *projbits;
	const float *coverage;
	DevPhoton *out;       /* per global index: the stored photon and its flag */
	int *valid;
};

__device__ __forceinline__ int pjob_of(const PhotonSet &P, int id)
{
	int lo = 0, hi = P.njobs - 1;
	while(lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if(P.jobs[mid].base <= id) lo = mid;
		else hi = mid - 1;
	}
	return lo;
}

__device__ __forceinline__ void push_photon(const RayQueue &q, int slot, const PRay &r, const PState &ph, int guard, int gid,
		int li, int job, int phase, int map, uint32_t draws)
{
	q.o[slot] = make_float4(r.o.x, r.o.y, r.o.z, ph.col[0]);
	q.d[slot] = make_float4(r.d.x, r.d.y, r.d.z, ph.col[1]);
	q.w[slot] = make_float4(ph.col[2], r.st.ior, __int_as_float(guard), __int_as_float(gid));
	q.meta[slot] = make_int4(li | (job << 16), r.iter, phase | (ph.type << 4) | (map << 8), r.time);
	q.stk[slot] = make_float4(r.st.stk[0], r.st.stk[1], r.st.stk[2], r.st.stk[3]);
	q.ext[slot] = make_int2((int)draws, r.st.sp);
}

static __device__ __forceinline__ int photon_slot(int *counter)
{
	cg::coalesced_group g = cg::coalesced_threads();
	int base = 0;
	if(g.thread_rank() == 0) base = atomicAdd(counter, (int)g.size());
	return g.shfl(base, 0) + (int)g.thread_rank();
}

__global__ void __launch_bounds__(128) k_photon_emit(DScene S, PhotonSet P, RayQueue q, DevCounters *ctr)
{
	int gfail = 0;
	for(int id = blockIdx.x * blockDim.x + threadIdx.x; id < P.total; id += gridDim.x * blockDim.x) {
		int job = pjob_of(P, id);
		const PJob &J = P.jobs[job];
		int local = id - J.base;
		int map = local >= J.total[0] ? 1 : 0;
		int gid = map ? local - J.total[0] : local;
		int global = map;
		const int *prefix = P.prefix + J.prefix0 + map * (J.nlights + 1);
		int li = 0;
		while(li + 1 < J.nlights && prefix[li + 1] <= gid) li++;
		int j = gid - prefix[li];
		sray_rng s;
		sray_rng_init(&s, S.seed, global ? SRAY_DOM_GLOBAL : SRAY_DOM_CAUST, (uint32_t)j, (uint32_t)li);
		int ms = J.t0 == J.t1 ? J.t0 : (sray_rng_int(&s) % (J.t1 - J.t0) + J.t0);
		int lg = J.light0 + li;
		const DevLight &L = S.lights[lg];
		PState ph;
		V3 pos = light_point(S, lg, ms, &s);
		float cov = P.coverage[(J.proj0 + li) * 2 + (global ? 0 : 1)];
		const uint32_t *bits = P.projbits + (size_t)(J.proj0 + li) * 128 + (global ? 0 : 64);
		for(int k = 0; k < 3; k++) ph.col[k] = L.col[k] * S.photon_energy;
		for(int k = 0; k < 3; k++) ph.col[k] = ph.col[k] * cov;
		ph.type = DIRECT_PHOTON;
		bool proj = true;
		if(cov == 0.0f) {
			proj = false;
			for(int k = 0; k < 3; k++) ph.col[k] = L.col[k] * S.photon_energy;
		}
		V3 dir;
		bool ok = true;
		if(proj) {
			ok = gen_dir(bits, &s, &dir);
			if(!ok) gfail = 1;
		} else {
			dir = sphrand(&s, 1.0f);
		}
		P.valid[id] = 0;
		if(ok && S.iter > 0) {
			PRay r;
			r.o = pos;
			r.d = dir * (float)SRAY_RAY_MAGNITUDE;
			r.time = ms;
			r.iter = S.iter;
			r.st.ior = 1.0f;
			r.st.sp = 0;
			for(int k = 0; k < 4; k++) r.st.stk[k] = 0.0f;
			int slot = photon_slot(q.count);
			push_photon(q, slot, r, ph, 0, id, li, job, global ? 0 : 1, map, s.n);
		}
	}
	if(gfail) atomicOr(&ctr->gen_dir_fail, 1);
}

/* a photon in flight, as the queue entry holds it */
struct PFlight {
	PRay r;
	PState ph;
	int li, job, gid, phase, guard, map;   /* gid: the photon's global index */
	uint32_t draws;
};

__device__ __forceinline__ void load_photon(const RayQueue &q, int i, PFlight &f)
{
	float4 o4 = q.o[i], d4 = q.d[i], w4 = q.w[i], k4 = q.stk[i];
	int4 meta = q.meta[i];
	int2 ext = q.ext[i];
	f.li = meta.x & 0xffff;
	f.job = meta.x >> 16;
	f.phase = meta.z & 15;
	f.map = (meta.z >> 8) & 1;
	f.guard = __float_as_int(w4.z);
	f.gid = __float_as_int(w4.w);
	f.r.o = mk(o4.x, o4.y, o4.z);
	f.r.d = mk(d4.x, d4.y, d4.z);
	f.r.time = meta.w;
	f.r.iter = meta.y;
	f.r.st.ior = w4.y;
	f.r.st.stk[0] = k4.x; f.r.st.stk[1] = k4.y; f.r.st.stk[2] = k4.z; f.r.st.stk[3] = k4.w;
	f.r.st.sp = ext.y;
	f.ph.col[0] = o4.w; f.ph.col[1] = d4.w; f.ph.col[2] = w4.x;
	f.ph.type = (meta.z >> 4) & 15;
	f.draws = (uint32_t)ext.x;
}

/* one surface interaction of a photon at hit h (h.obj >= 0): stores it
 * (returns 1), loses it (0) or leaves it ready for its next trace (2) */
__device__ __forceinline__ int photon_interact(const DScene &S, const PhotonSet &P, PFlight &f, const Hit &h)
{
	int global = f.map;
	const PJob &J = P.jobs[f.job];
	int gid = f.gid - J.base - (f.map ? J.total[0] : 0);   /* within its frame's map */
	sray_rng s;
	sray_rng_init(&s, S.seed, global ? SRAY_DOM_GLOBAL : SRAY_DOM_CAUST,
			(uint32_t)(gid - P.prefix[J.prefix0 + f.map * (J.nlights + 1) + f.li]), (uint32_t)f.li);
	sray_rng_seek(&s, f.draws);
	int res = f.phase == 0 ? global_step(S, f.r, f.ph, h, &s) : caust_step(S, f.r, f.ph, h, &s);
	f.draws = s.n;
	if(res == P_STORE) {
		if(!global && f.ph.type != CAUST_PHOTON) return 0;
		float sc = P.scale[J.scale0 + f.map * J.nlights + f.li];
		DevPhoton p;
		p.p[0] = f.ph.pos.x; p.p[1] = f.ph.pos.y; p.p[2] = f.ph.pos.z; p.p[3] = f.ph.col[0] * sc;
		p.d[0] = f.ph.dir.x; p.d[1] = f.ph.dir.y; p.d[2] = f.ph.dir.z; p.d[3] = f.ph.col[1] * sc;
		p.n[0] = f.ph.norm.x; p.n[1] = f.ph.norm.y; p.n[2] = f.ph.norm.z; p.n[3] = f.ph.col[2] * sc;
		P.out[f.gid] = p;
		P.valid[f.gid] = 1;
		return 1;
	}
	if(res == P_DROP) return 0;
	if(res == P_TO_CAUST) {
		f.phase = 1;
		f.guard = 0;
	} else if(++f.guard >= PHOTON_GUARD) {
		return 0;
	}
	return f.r.iter <= 0 ? 0 : 2;
}

__global__ void __launch_bounds__(128) k_photon_bounce(DScene S, PhotonSet P, RayQueue qi, const int4 *hits, RayQueue qo)
{
	int n = *qi.count;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int4 hv = hits[i];
		if(hv.y < 0) continue;                       /* photon left the scene */
		Hit h;
		h.t = __int_as_float(hv.x);
		h.obj = hv.y;
		h.prim = hv.z;
		h.tie = hv.w;
		PFlight f;
		load_photon(qi, i, f);
		if(photon_interact(S, P, f, h) != 2) continue;
		int slot = photon_slot(qo.count);
		if(slot >= qo.cap) continue;                 /* cannot happen: a photon has one successor */
		push_photon(qo, slot, f.r, f.ph, f.guard, f.gid, f.li, f.job, f.phase, f.map, f.draws);
	}
}

/* The tail of the photon maps: once few photons are left, each thread takes
 * photons from the queue (through a shared counter) and traces every one to
 * its end, instead of one interaction per pass; a pass costs as much as its
 * slowest ray, and the tail is made of few photons on long paths.  Photons
 * whose hit the octrees must decide are handed back, before that trace, to
 * the pending queue, which the pass-wise loop finishes. */
__global__ void __launch_bounds__(128) k_photon_finish(DScene S, PhotonSet P, RayQueue qi, int *next, RayQueue qpend,
		DevCounters *ctr)
{
	int n = *qi.count;
	int overflow = 0;
	for(;;) {
		int i = atomicAdd(next, 1);
		if(i >= n) break;
		PFlight f;
		load_photon(qi, i, f);
		for(int step = 0; step < 2 * PHOTON_GUARD + 2; step++) {
			Hit h;
			if(!trace_two_level<false, false>(S, f.r.o, f.r.d, f.r.time, h, nullptr, &overflow, pixel_scene(S, f.gid))) {
				int slot = photon_slot(qpend.count);
				if(slot < qpend.cap) push_photon(qpend, slot, f.r, f.ph, f.guard, f.gid, f.li, f.job, f.phase, f.map, f.draws);
				break;
			}
			if(h.obj < 0) break;
			if(photon_interact(S, P, f, h) != 2) break;
		}
	}
	if(overflow) atomicOr(&ctr->overflow, 1);
}

/* ---------------- scan / compaction ---------------- */
#define TILE 2048

__global__ void k_count_valid(const int *valid, int n, unsigned *bcount)
{
	__shared__ int s;
	if(threadIdx.x == 0) s = 0;
	__syncthreads();
	int base = blockIdx.x * TILE, c = 0;
	for(int i = base + threadIdx.x; i < base + TILE && i < n; i += blockDim.x) c += valid[i];
	atomicAdd(&s, c);
	__syncthreads();
	if(threadIdx.x == 0) bcount[blockIdx.x] = s;
}

/* exclusive scan of m entries by one block of 1024 threads; total -> *total */
__global__ void k_scan_excl(unsigned *data, int m, unsigned *total)
{
	__shared__ unsigned part[1024];
	int t = threadIdx.x;
	int chunk = (m + 1023) / 1024;
	int b = t * chunk, e = min(b + chunk, m);
	unsigned s = 0;
	for(int i = b; i < e; i++) s += data[i];
	part[t] = s;
	__syncthreads();
	for(int off = 1; off < 1024; off <<= 1) {
		unsigned v = t >= off ? part[t - off] : 0;
		__syncthreads();
		part[t] += v;
		__syncthreads();
	}
	unsigned run = part[t] - s;
	for(int i = b; i < e; i++) {
		unsigned v = data[i];
		data[i] = run;
		run += v;
	}
	if(t == 1023 && total) *total = part[1023];
}

/* order-preserving compaction of one tile per block */
__global__ void k_compact(const int *valid, const DevPhoton *in, int n, const unsigned *boffs, DevPhoton *out)
{
	__shared__ int wsum[8];
	__shared__ int run;
	int base = blockIdx.x * TILE;
	int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	if(threadIdx.x == 0) run = (int)boffs[blockIdx.x];
	__syncthreads();
	for(int r = 0; r < TILE / 256; r++) {
		int i = base + r * 256 + threadIdx.x;
		int v = (i < n) ? valid[i] : 0;
		unsigned bal = __ballot_sync(0xffffffffu, v);
		int wpre = __popc(bal & ((1u << lane) - 1u));
		if(lane == 0) wsum[w] = __popc(bal);
		__syncthreads();
		int off = run;
		for(int k = 0; k < w; k++) off += wsum[k];
		if(v) out[off + wpre] = in[i];
		__syncthreads();
		if(threadIdx.x == 0) {
			int t = 0;
			for(int k = 0; k < 8; k++) t += wsum[k];
			run += t;
		}
		__syncthreads();
	}
}

/* ---------------- grid keys and radix sort ---------------- */
__device__ __forceinline__ unsigned spread3(unsigned v)
{
	v &= 0x3ff;
	v = (v | (v << 16)) & 0x030000FF;
	v = (v | (v << 8)) & 0x0300F00F;
	v = (v | (v << 4)) & 0x030C30C3;
	v = (v | (v << 2)) & 0x09249249;
	return v;
}

__global__ void k_keys(const DevPhoton *ph, int n, DPhotonMap M, int morton, unsigned *keys, unsigned *vals, unsigned *lin)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int c[3];
		for(int a = 0; a < 3; a++) {
			double v = floor(((double)ph[i].p[a] - (double)M.org[a]) / (double)M.cell);
			c[a] = v < 0.0 ? 0 : (v > (double)(M.dims[a] - 1) ? M.dims[a] - 1 : (int)v);
		}
		unsigned l = (unsigned)(((size_t)c[2] * M.dims[1] + c[1]) * M.dims[0] + c[0]);
		keys[i] = morton ? (spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2)) : l;
		vals[i] = (unsigned)i;
		lin[i] = l;
	}
}

#define RS_THREADS 256

__global__ void k_rs_hist(const unsigned *keys, int n, int shift, unsigned *hist, int nblocks)
{
	__shared__ unsigned h[256];
	h[threadIdx.x] = 0;
	__syncthreads();
	int base = blockIdx.x * TILE;
	for(int i = base + threadIdx.x; i < base + TILE && i < n; i += RS_THREADS) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
	__syncthreads();
	hist[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

/* stable scatter: tile items in order, ranks within a round from warp match masks */
__global__ void k_rs_scatter(const unsigned *keys, const unsigned *vals, int n, int shift, const unsigned *offs, int nblocks,
		unsigned *okeys, unsigned *ovals)
{
	__shared__ unsigned base[256];
	__shared__ unsigned wcnt[RS_THREADS / 32][257];
	int t = threadIdx.x, lane = t & 31, w = t >> 5;
	base[t] = offs[(size_t)t * nblocks + blockIdx.x];
	int tile = blockIdx.x * TILE;
	for(int r = 0; r < TILE / RS_THREADS; r++) {
		for(int k = 0; k < RS_THREADS / 32; k++) wcnt[k][t] = 0;
		if(t == 0) for(int k = 0; k < RS_THREADS / 32; k++) wcnt[k][256] = 0;
		__syncthreads();
		int i = tile + r * RS_THREADS + t;
		bool v = i < n;
		unsigned key = v ? keys[i] : 0u;
		unsigned d = v ? ((key >> shift) & 255u) : 256u;
		unsigned peers = __match_any_sync(0xffffffffu, d);
		int rank = __popc(peers & ((1u << lane) - 1u));
		if(lane == __ffs(peers) - 1) wcnt[w][d] = __popc(peers);
		__syncthreads();
		if(v) {
			unsigned pos = base[d] + rank;
			for(int k = 0; k < w; k++) pos += wcnt[k][d];
			okeys[pos] = key;
			ovals[pos] = vals[i];
		}
		__syncthreads();
		unsigned add = 0;
		for(int k = 0; k < RS_THREADS / 32; k++) add += wcnt[k][t];
		base[t] += add;
		__syncthreads();
	}
}

__global__ void k_permute(const DevPhoton *in, const unsigned *vals, const unsigned *lin_in, int n, DevPhoton *out, unsigned *lin_out)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		unsigned v = vals[i];
		out[i] = in[v];
		lin_out[i] = lin_in[v];
	}
}

__global__ void k_cells(const unsigned *lin, int n, uint2 *cells)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		unsigned l = lin[i];
		if(i == 0 || lin[i - 1] != l) cells[l].x = (unsigned)i;
		if(i == n - 1 || lin[i + 1] != l) cells[l].y = (unsigned)(i + 1);
	}
}

/* Photon launches run beside the frame's higher-priority stream: a block
 * per `block` items, so that blocks are short-lived and the frame's kernels
 * get SMs as they free, instead of a capped grid whose blocks stride over
 * the whole launch and hold their SMs until it ends. */
static int grid_n(int n, int block)
{
	int g = (n + block - 1) / block;
	return g < 1 ? 1 : g;
}

#define PCK(call, where) do { cudaError_t e_ = (call); if(e_ != cudaSuccess) return R.cuda_fail(e_, where); } while(0)

/* emission counts of one map of a frame: photons split by mean light
 * intensity (src/render.cc:87-110); appends the per-light prefix sums
 * (nl + 1) and power scales (nl), returns the map's total */
static int split_photons(const Renderer &R, int light0, int nl, int num, std::vector<int> &prefix, std::vector<float> &scale)
{
	size_t p0 = prefix.size();
	prefix.resize(p0 + nl + 1, 0);
	scale.resize(scale.size() + nl, 0.0f);
	size_t s0 = scale.size() - nl;
	if(num <= 0 || nl <= 0) return 0;
	std::vector<double> inten(nl);
	double accp = 0.0;
	for(int i = 0; i < nl; i++) {
		const double *c = R.sc.lights[light0 + i].col;
		inten[i] = (c[0] + c[1] + c[2]) / 3.0;
		accp += inten[i];
	}
	for(int i = 0; i < nl; i++) {
		int nphot = (int)ceil((double)num * (inten[i] / accp));
		prefix[p0 + i + 1] = prefix[p0 + i] + nphot;
		scale[s0 + i] = nphot ? (float)(1.0 / (double)nphot) : 0.0f;
	}
	return prefix[p0 + nl];
}

/* Both photon maps of every job, traced as one wavefront on stream s: the
 * emission of all jobs' photons in one launch, then passes of closest hits
 * and interactions over one queue (each photon finds its job, and through
 * it its scene, lights, interval and projection maps), then the tail.  The
 * stored photons and their flags stay in R.pw_out / R.pw_valid by global
 * index; jobs[j].base and total[] locate each job's two segments. */
int photon_trace_jobs(Renderer &R, const DScene &base, const std::vector<PhotonJobSpec> &spec, std::vector<PJobOut> &out,
		cudaStream_t s)
{
	int n = (int)spec.size();
	out.assign(n, PJobOut());
	std::vector<PJob> jobs(n);
	std::vector<int> prefix;
	std::vector<float> scale, cov;
	std::vector<uint32_t> bits;
	std::vector<DevJob> pj(n);
	int64_t all = 0;
	for(int j = 0; j < n; j++) {
		const PhotonJobSpec &J = spec[j];
		PJob &d = jobs[j];
		memset(&d, 0, sizeof d);
		d.base = (int)all;
		d.light0 = J.light0;
		d.nlights = J.nlights;
		d.prefix0 = (int)prefix.size();
		d.scale0 = (int)scale.size();
		d.proj0 = (int)(cov.size() / 2);
		d.t0 = J.t0;
		d.t1 = J.t1;
		for(int m = 0; m < 2; m++) d.total[m] = split_photons(R, J.light0, J.nlights, J.num[m], prefix, scale);
		if(J.nlights > 0) {
			if(!J.bits || !J.cov || J.bits->size() < (size_t)J.nlights * 128 || J.cov->size() < (size_t)J.nlights * 2)
				return R.fail(SRAY_ESTATE, "photon job without its projection maps");
			bits.insert(bits.end(), J.bits->begin(), J.bits->begin() + (size_t)J.nlights * 128);
			cov.insert(cov.end(), J.cov->begin(), J.cov->begin() + (size_t)J.nlights * 2);
		}
		memset(&pj[j], 0, sizeof pj[j]);
		pj[j].pix0 = d.base;
		pj[j].scene = J.scene;
		out[j].base = d.base;
		out[j].total[0] = d.total[0];
		out[j].total[1] = d.total[1];
		all += (int64_t)d.total[0] + d.total[1];
		if(all > INT_MAX / 2) return R.fail(SRAY_EINVAL, "too many photons in one wavefront");
	}
	if(all == 0) return 0;
	PCK(R.pw_jobs.upload(jobs, s), "photon jobs");
	PCK(R.pw_prefix.upload(prefix, s), "photon prefix");
	PCK(R.pw_scale.upload(scale, s), "photon scale");
	PCK(R.pw_bits.upload(bits, s), "projection maps");
	PCK(R.pw_cov.upload(cov, s), "coverage");
	PCK(R.pw_pix.upload(pj, s), "photon job table");
	R.h2d += (int64_t)(jobs.size() * sizeof(PJob) + prefix.size() * 4 + scale.size() * 4 + bits.size() * 4 + cov.size() * 4 +
			pj.size() * sizeof(DevJob));
	PCK(R.pw_out.ensure((size_t)all * sizeof(DevPhoton)), "photon buffer");
	PCK(R.pw_valid.ensure((size_t)all * sizeof(int)), "photon flags");
	PhotonSet PSet;
	PSet.njobs = n;
	PSet.total = (int)all;
	PSet.jobs = R.pw_jobs.as<PJob>();
	PSet.prefix = R.pw_prefix.as<int>();
	PSet.scale = R.pw_scale.as<float>();
	PSet.projbits = R.pw_bits.as<uint32_t>();
	PSet.coverage = R.pw_cov.as<float>();
	PSet.out = R.pw_out.as<DevPhoton>();
	PSet.valid = R.pw_valid.as<int>();
	PCK(R.pctr.ensure(sizeof(DevCounters)), "counters");
	PCK(R.pcounts.ensure(64 * sizeof(int)), "counts");
	PCK(cudaMemsetAsync(R.pctr.p, 0, sizeof(DevCounters), s), "counters");
	PCK(cudaMemsetAsync(R.pcounts.p, 0, 4 * sizeof(int), s), "photon queue counts");
	int *cnt = R.pcounts.as<int>();
	R.pq[0].count = cnt + 0;
	R.pq[1].count = cnt + 1;
	if(R.ensure_pqueue(0, (int)all) || R.ensure_pqueue(1, (int)all)) return SRAY_ECUDA;
	PCK(R.phits.ensure((size_t)all * 16), "photon hits");
	/* the scene as the photon kernels see it: their counters, and in a scene
	 * set the photon job table, through which a photon's global index finds
	 * its scene (the render's pixel table is not theirs) */
	DScene PS = base;
	PS.bvh_fallbacks = &R.pctr.as<DevCounters>()->bvh_fallbacks;
	PS.jobs = PS.nscenes > 1 ? R.pw_pix.as<DevJob>() : nullptr;
	PS.njobs = PS.nscenes > 1 ? n : 0;
	DevCounters *pctr = R.pctr.as<DevCounters>();
	LAUNCH(R, "photon_emit", s, k_photon_emit<<<grid_n((int)all, 128), 128, 0, s>>>(PS, PSet, R.pq[0], pctr));
	/* the emitted count (a photon whose direction sampling fails is not queued) */
	PCK(cudaMemcpyAsync(R.pin + 8, R.pq[0].count, sizeof(int), cudaMemcpyDeviceToHost, s), "photon queue count");
	PCK(cudaStreamSynchronize(s), "photon emission");
	int cur = 0;
	int n_live = R.pin[8];
	R.d2h += sizeof(int);
	R.prof_collect();
	bool finished = false;
	for(int pass = 0; n_live > 0; pass++) {
		if(pass >= 2 * PHOTON_GUARD + 4) return R.fail(SRAY_EDEVICE, "photon paths did not terminate");
		PCK(cudaMemsetAsync(R.pq[cur ^ 1].count, 0, sizeof(int), s), "reset photon queue");
		if(!finished && pass > 0 && n_live <= R.tune.photon_tail) {
			/* the tail in one launch; what it hands back continues pass-wise */
			finished = true;
			PCK(cudaMemsetAsync(cnt + 2, 0, sizeof(int), s), "reset photon tail counter");
			LAUNCH(R, "photon_finish", s, k_photon_finish<<<grid_n(n_live, 128), 128, 0, s>>>(PS, PSet, R.pq[cur], cnt + 2,
					R.pq[cur ^ 1], pctr));
			PCK(cudaMemcpyAsync(R.pin + 8, R.pq[cur ^ 1].count, sizeof(int), cudaMemcpyDeviceToHost, s), "photon queue count");
			PCK(cudaStreamSynchronize(s), "photon tail");
			n_live = R.pin[8];
			R.d2h += sizeof(int);
			R.prof_collect();
			cur ^= 1;
			continue;
		}
		/* a large emission pass in the order of direction octant and origin
		 * cell: the photons of a warp then leave one light into one octant
		 * (the queue's order is arbitrary anyway: its slots come from
		 * atomics, and each entry carries its photon's identity); the
		 * bounced passes gain less than their sort costs */
		if(pass == 0 && n_live >= PHOTON_SORT_MIN)
			if(int r = R.sort_photon_pass(cur, n_live, s)) return r;
		if(launch_trace(R, PS, R.pq[cur], n_live, "photon_trace", s)) return SRAY_ECUDA;
		LAUNCH(R, "photon_bounce", s, k_photon_bounce<<<grid_n(n_live, 128), 128, 0, s>>>(PS, PSet, R.pq[cur], R.phits.as<int4>(),
				R.pq[cur ^ 1]));
		PCK(cudaMemcpyAsync(R.pin + 8, R.pq[cur ^ 1].count, sizeof(int), cudaMemcpyDeviceToHost, s), "photon queue count");
		PCK(cudaStreamSynchronize(s), "photon pass");
		n_live = R.pin[8];
		R.d2h += sizeof(int);
		R.prof_collect();
		cur ^= 1;
	}
	DevCounters hc;
	PCK(cudaMemcpyAsync(&hc, pctr, sizeof hc, cudaMemcpyDeviceToHost, s), "counters");
	PCK(cudaStreamSynchronize(s), "photon trace");
	R.d2h += sizeof(DevCounters);
	if(hc.overflow) return R.fail(SRAY_EDEVICE, "traversal stack overflow while tracing photons");
	if(hc.gen_dir_fail) return R.fail(SRAY_EDEVICE, "projection-map sampling found no covered cell");
	return 0;
}

/* a map's stored photons from its segment of the wavefront's output
 * (flags `valid`, photons `in`, `total` of them): compacted in emission
 * order, sorted by grid cell, with the cell table */
int photon_finalize(Renderer &R, int global, const int *valid, const DevPhoton *in, int total, cudaStream_t s, int *stored)
{
	PhotonBufs &P = global ? R.gi : R.caust;
	*stored = 0;
	P.map.n = 0;
	if(total <= 0) return 0;
	/* compaction in emission order */
	int nb = (total + TILE - 1) / TILE;
	PCK(P.scan.ensure((size_t)(nb + 4) * sizeof(unsigned)), "scan");
	unsigned *bc = P.scan.as<unsigned>();
	LAUNCH(R, "photon_compact", s, k_count_valid<<<nb, 256, 0, s>>>(valid, total, bc));
	LAUNCH(R, "photon_compact", s, k_scan_excl<<<1, 1024, 0, s>>>(bc, nb, bc + nb));
	unsigned h_n = 0;
	PCK(cudaMemcpyAsync(&h_n, bc + nb, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "stored count");
	PCK(cudaStreamSynchronize(s), "photon compaction");
	R.d2h += sizeof(unsigned);
	R.prof_collect();
	int n = (int)h_n;
	*stored = n;
	if(n == 0) return 0;
	PCK(P.ph.ensure((size_t)n * sizeof(DevPhoton)), "photon map");
	LAUNCH(R, "photon_compact", s, k_compact<<<nb, 256, 0, s>>>(valid, in, total, bc, P.ph.as<DevPhoton>()));
	return photon_map_build(R, global, n, s);
}

/* both photon maps of the frame (one job): the wavefront, then each map from
 * its segment */
int photon_shoot_maps(Renderer &R, const DScene &base, const std::vector<uint32_t> &bits, const std::vector<float> &cov,
		cudaStream_t s, int *nc, int *ng)
{
	*nc = *ng = 0;
	R.caust.map.n = 0;
	R.gi.map.n = 0;
	std::vector<PhotonJobSpec> spec(1);
	PhotonJobSpec &J = spec[0];
	J.num[0] = R.opt.caust_photons;
	J.num[1] = R.opt.gi_photons;
	J.light0 = 0;
	J.nlights = (int)R.sc.lights.size();
	J.t0 = base.t0;
	J.t1 = base.t1;
	J.scene = -1;
	J.bits = &bits;
	J.cov = &cov;
	std::vector<PJobOut> out;
	int r = photon_trace_jobs(R, base, spec, out, s);
	if(r) return r;
	const DevPhoton *ph = R.pw_out.as<DevPhoton>();
	const int *valid = R.pw_valid.as<int>();
	if((r = photon_finalize(R, 0, valid, ph, out[0].total[0], s, nc))) return r;
	int o1 = out[0].total[0];
	return photon_finalize(R, 1, valid + o1, ph + o1, out[0].total[1], s, ng);
}

/* A map's grid over box rb for gathers of radius rad (k nearest, or all
 * within rad when k = 0): cells twice the radius, so that a query cube
 * overlaps at most 2x2x2, at most 2^26 of them; the map's range constants.
 * Morton keys when every dimension fits 10 bits. */
static void map_grid(int k, double rad, const Box &rb, DPhotonMap &M, bool *morton, size_t *ncells)
{
	double cell = rad > 0.0 ? 2.0 * rad : 1.0;
	double ext[3];
	for(int a = 0; a < 3; a++) ext[a] = rb.mx[a] - rb.mn[a];
	int dims[3];
	for(;;) {
		double total_cells = 1.0;
		for(int a = 0; a < 3; a++) {
			dims[a] = (int)floor(ext[a] / cell) + 1;
			total_cells *= dims[a];
		}
		if(total_cells <= (double)(1 << 26)) break;
		cell *= 1.25;
	}
	M.k = k;
	M.cell = (float)cell;
	while((double)M.cell < cell) M.cell = nextafterf(M.cell, INFINITY);
	for(int a = 0; a < 3; a++) { M.dims[a] = dims[a]; M.org[a] = (float)rb.mn[a]; }
	for(int a = 0; a < 3; a++) while((double)M.org[a] > rb.mn[a]) M.org[a] = nextafterf(M.org[a], -INFINITY);
	M.range = (double)(float)rad;
	M.inv_area = (float)(1.0 / (M_PI * (rad * rad)));
	M.range_f = (float)rad;
	{
		double r2 = (double)M.range_f * (double)M.range_f;   /* exact: 48 significant bits */
		M.r2_hi = (float)r2;
		M.r2_lo = (float)(r2 - (double)M.r2_hi);
		M.screen = (float)(r2 * (1.0 + 1.0 / 1048576.0));
	}
	*morton = dims[0] <= 1024 && dims[1] <= 1024 && dims[2] <= 1024;
	*ncells = (size_t)dims[0] * dims[1] * dims[2];
}

/* the map over the n photons in P.ph: grid, Morton sort, cell table */
int photon_map_build(Renderer &R, int global, int n, cudaStream_t s)
{
	PhotonBufs &P = global ? R.gi : R.caust;
	const sray_opts &opt = R.opt;
	if(R.sc.oct.nodes.empty()) return R.fail(SRAY_ESTATE, "no scene bounds (build the frame first)");
	/* grid over the scene bounds (a batch job's: its scene over its own
	 * interval, the box its frame alone would have) */
	const Box &rb = R.map_has_box ? R.map_box : R.sc.oct.nodes[0].box;
	int k = global ? opt.gi_k : opt.caust_k;
	/* a job of a batch gathers with the radius of its own interval */
	double rad = k > 0 ? (double)opt.gather_rcap : (R.map_gather_dist >= 0.0 ? R.map_gather_dist : R.sc.gather_dist);
	DPhotonMap &M = P.map;
	bool morton;
	size_t ncells;
	map_grid(k, rad, rb, M, &morton, &ncells);
	M.n = n;
	PCK(P.keys.ensure((size_t)n * 4), "keys");
	PCK(P.keys2.ensure((size_t)n * 4), "keys");
	PCK(P.vals.ensure((size_t)n * 4), "vals");
	PCK(P.vals2.ensure((size_t)n * 4), "vals");
	PCK(P.lin.ensure((size_t)n * 8), "cell ids");
	PCK(P.cells.ensure(ncells * sizeof(uint2)), "cell table");
	unsigned *keys = P.keys.as<unsigned>(), *keys2 = P.keys2.as<unsigned>();
	unsigned *vals = P.vals.as<unsigned>(), *vals2 = P.vals2.as<unsigned>();
	unsigned *lin = P.lin.as<unsigned>(), *lin2 = lin + n;
	LAUNCH(R, "photon_sort", s, k_keys<<<grid_n(n, 256), 256, 0, s>>>(P.ph.as<DevPhoton>(), n, M, morton ? 1 : 0, keys, vals, lin));
	unsigned maxkey = morton ? (1u << 30) - 1u : (unsigned)(ncells - 1);
	int bits = 0;
	while(bits < 32 && (maxkey >> bits)) bits++;
	int passes = (bits + 7) / 8;
	int nbr = (n + TILE - 1) / TILE;
	PCK(P.hist.ensure((size_t)256 * nbr * sizeof(unsigned) + 16), "radix histogram");
	for(int ps = 0; ps < passes; ps++) {
		int shift = ps * 8;
		LAUNCH(R, "photon_sort", s, k_rs_hist<<<nbr, RS_THREADS, 0, s>>>(keys, n, shift, P.hist.as<unsigned>(), nbr));
		LAUNCH(R, "photon_sort", s, k_scan_excl<<<1, 1024, 0, s>>>(P.hist.as<unsigned>(), 256 * nbr, nullptr));
		LAUNCH(R, "photon_sort", s, k_rs_scatter<<<nbr, RS_THREADS, 0, s>>>(keys, vals, n, shift, P.hist.as<unsigned>(), nbr, keys2, vals2));
		std::swap(keys, keys2);
		std::swap(vals, vals2);
	}
	PCK(P.tmp_ph.ensure((size_t)n * sizeof(DevPhoton)), "photon buffer");
	LAUNCH(R, "photon_sort", s, k_permute<<<grid_n(n, 256), 256, 0, s>>>(P.ph.as<DevPhoton>(), vals, lin, n, P.tmp_ph.as<DevPhoton>(), lin2));
	PCK(cudaMemsetAsync(P.cells.p, 0, ncells * sizeof(uint2), s), "cell table");
	LAUNCH(R, "photon_sort", s, k_cells<<<grid_n(n, 256), 256, 0, s>>>(lin2, n, P.cells.as<uint2>()));
	std::swap(P.ph, P.tmp_ph);
	M.ph = P.ph.as<DevPhoton>();
	M.cells = P.cells.as<uint2>();
	PCK(cudaStreamSynchronize(s), "photon map build");
	R.prof_collect();
	return 0;
}

/* ---------------- the maps of many jobs at once (a batch) ----------------
 * The wavefront's output holds every job's two maps as segments (job-major,
 * caustic then global).  One compaction keeps the stored photons of all
 * segments in emission order; each photon's key is its cell in its own
 * map's grid; a stable LSD radix sort by key and then by segment leaves the
 * segments in order, each sorted by cell with ties in emission order -- the
 * order a map sorted alone gets -- and each segment's cell table indexes
 * its own photons. */

#define SCAN_PART 8192   /* entries per block of the long scan */

/* exclusive scan of each SCAN_PART-entry part in place (1024 threads, 8
 * entries each); the part's total into sums */
__global__ void k_scan_part(unsigned *data, int m, unsigned *sums)
{
	__shared__ unsigned part[1024];
	int t = threadIdx.x;
	int b = blockIdx.x * SCAN_PART + t * 8;
	unsigned v[8], sum = 0;
	#pragma unroll
	for(int k = 0; k < 8; k++) {
		v[k] = b + k < m ? data[b + k] : 0u;
		sum += v[k];
	}
	part[t] = sum;
	__syncthreads();
	for(int off = 1; off < 1024; off <<= 1) {
		unsigned u = t >= off ? part[t - off] : 0u;
		__syncthreads();
		part[t] += u;
		__syncthreads();
	}
	unsigned run = part[t] - sum;
	#pragma unroll
	for(int k = 0; k < 8; k++) {
		if(b + k < m) data[b + k] = run;
		run += v[k];
	}
	if(t == 1023) sums[blockIdx.x] = part[1023];
}

__global__ void k_scan_add(unsigned *data, int m, const unsigned *offs)
{
	unsigned o = offs[blockIdx.x];
	int b = blockIdx.x * SCAN_PART;
	for(int i = b + threadIdx.x; i < b + SCAN_PART && i < m; i += blockDim.x) data[i] += o;
}

/* the segment holding compacted index i: the last s with offs[s] <= i */
__device__ __forceinline__ int seg_of(const unsigned *offs, int nseg, unsigned i)
{
	int lo = 0, hi = nseg - 1;
	while(lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if(offs[mid] <= i) lo = mid;
		else hi = mid - 1;
	}
	return lo;
}

/* compacted index of each segment boundary: the tile's offset plus the
 * stored photons of the tile before it (one block per boundary) */
__global__ void k_seg_offsets(const int *valid, const unsigned *tile_offs, const int *bounds, unsigned *offs)
{
	__shared__ int red[256];
	int b = bounds[blockIdx.x], tile = b / TILE, c = 0;
	for(int i = tile * TILE + threadIdx.x; i < b; i += blockDim.x) c += valid[i];
	red[threadIdx.x] = c;
	__syncthreads();
	for(int off = 128; off > 0; off >>= 1) {
		if(threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
		__syncthreads();
	}
	if(threadIdx.x == 0) offs[blockIdx.x] = tile_offs[tile] + (unsigned)red[0];
}

/* cell keys of the compacted photons, each in its segment's grid */
__global__ void k_keys_seg(const DevPhoton *ph, int n, const DPhotonMap *grids, const int *morton, const unsigned *offs, int nseg,
		unsigned *keys, unsigned *vals, unsigned *lin)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		const DPhotonMap &M = grids[seg_of(offs, nseg, (unsigned)i)];
		int c[3];
		for(int a = 0; a < 3; a++) {
			double v = floor(((double)ph[i].p[a] - (double)M.org[a]) / (double)M.cell);
			c[a] = v < 0.0 ? 0 : (v > (double)(M.dims[a] - 1) ? M.dims[a] - 1 : (int)v);
		}
		unsigned l = (unsigned)(((size_t)c[2] * M.dims[1] + c[1]) * M.dims[0] + c[0]);
		keys[i] = morton[seg_of(offs, nseg, (unsigned)i)] ? (spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2)) : l;
		vals[i] = (unsigned)i;
		lin[i] = l;
	}
}

/* the segment of each entry (by its compacted index) as the next pass's key */
__global__ void k_seg_keys(const unsigned *vals, int n, const unsigned *offs, int nseg, unsigned *keys)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) keys[i] = (unsigned)seg_of(offs, nseg, vals[i]);
}

/* (first, end) of every occupied cell of every segment, relative to the
 * segment's first photon, in the segment's own cell table */
__global__ void k_cells_seg(const unsigned *lin, int n, const unsigned *offs, int nseg, const unsigned long long *cell_base, uint2 *cells)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int sg = seg_of(offs, nseg, (unsigned)i);
		unsigned i0 = offs[sg], i1 = offs[sg + 1];
		unsigned l = lin[i];
		uint2 *c = cells + cell_base[sg];
		if((unsigned)i == i0 || lin[i - 1] != l) c[l].x = (unsigned)i - i0;
		if((unsigned)i + 1 == i1 || lin[i + 1] != l) c[l].y = (unsigned)i + 1 - i0;
	}
}

/* exclusive scan of m entries (scratch `part` for the parts' totals); the
 * total into *total when given */
static int scan_long(Renderer &R, unsigned *data, int m, unsigned *total, DevBuf &part, const char *name, cudaStream_t s)
{
	if(m <= 65536) {
		LAUNCH(R, name, s, k_scan_excl<<<1, 1024, 0, s>>>(data, m, total));
		return 0;
	}
	int parts = (m + SCAN_PART - 1) / SCAN_PART;
	PCK(part.ensure((size_t)(parts + 4) * sizeof(unsigned)), "scan parts");
	unsigned *sums = part.as<unsigned>();
	LAUNCH(R, name, s, k_scan_part<<<parts, 1024, 0, s>>>(data, m, sums));
	LAUNCH(R, name, s, k_scan_excl<<<1, 1024, 0, s>>>(sums, parts, total));
	LAUNCH(R, name, s, k_scan_add<<<parts, 256, 0, s>>>(data, m, sums));
	return 0;
}

/* stable LSD radix sort of n (key, value) pairs over the low `bits` bits of
 * the keys, ping-ponging with keys2 / vals2; *vals_out is the buffer that
 * holds the sorted values (scratch: hist, part) */
int sort_pairs(Renderer &R, unsigned *keys, unsigned *vals, unsigned *keys2, unsigned *vals2, int n, int bits, DevBuf &hist,
		DevBuf &part, const char *name, cudaStream_t s, unsigned **vals_out)
{
	int nbr = (n + TILE - 1) / TILE;
	PCK(hist.ensure((size_t)256 * nbr * sizeof(unsigned) + 16), "radix histogram");
	unsigned *h = hist.as<unsigned>();
	for(int shift = 0; shift < bits; shift += 8) {
		LAUNCH(R, name, s, k_rs_hist<<<nbr, RS_THREADS, 0, s>>>(keys, n, shift, h, nbr));
		if(scan_long(R, h, 256 * nbr, nullptr, part, name, s)) return SRAY_ECUDA;
		LAUNCH(R, name, s, k_rs_scatter<<<nbr, RS_THREADS, 0, s>>>(keys, vals, n, shift, h, nbr, keys2, vals2));
		std::swap(keys, keys2);
		std::swap(vals, vals2);
	}
	*vals_out = vals;
	return 0;
}

/* every job's two maps from the wavefront's output: maps[2j] caustic,
 * maps[2j + 1] global, over the boxes and range radii of the jobs' own
 * frames.  Returns 1 (nothing done) when the maps' cell tables together
 * would pass 2^28 cells, for the map-by-map build to take over. */
int photon_finalize_jobs(Renderer &R, const std::vector<PJobOut> &jobs, const std::vector<Box> &boxes,
		const std::vector<double> &gather_dist, std::vector<DPhotonMap> &maps, cudaStream_t s)
{
	const sray_opts &opt = R.opt;
	int nj = (int)jobs.size(), nseg = 2 * nj;
	maps.assign(nseg, DPhotonMap());
	std::vector<int> morton(nseg);
	std::vector<unsigned long long> cell_base(nseg + 1, 0);
	for(int sg = 0; sg < nseg; sg++) {
		int k = (sg & 1) ? opt.gi_k : opt.caust_k;
		double rad = k > 0 ? (double)opt.gather_rcap : gather_dist[sg >> 1];
		bool mo;
		size_t nc;
		map_grid(k, rad, boxes[sg >> 1], maps[sg], &mo, &nc);
		morton[sg] = mo ? 1 : 0;
		cell_base[sg + 1] = cell_base[sg] + nc;
	}
	if(cell_base[nseg] > (1ull << 28)) return 1;
	const PJobOut &last = jobs[nj - 1];
	int total = last.base + last.total[0] + last.total[1];
	if(total == 0) return 0;
	const int *valid = R.pw_valid.as<int>();
	int nb = (total + TILE - 1) / TILE;
	PCK(R.pw_tiles.ensure((size_t)(nb + 4) * sizeof(unsigned)), "scan");
	unsigned *bc = R.pw_tiles.as<unsigned>();
	LAUNCH(R, "photon_compact", s, k_count_valid<<<nb, 256, 0, s>>>(valid, total, bc));
	if(scan_long(R, bc, nb, bc + nb, R.pw_part, "photon_compact", s)) return SRAY_ECUDA;
	std::vector<int> bounds(nseg + 1);
	for(int j = 0; j < nj; j++) {
		bounds[2 * j] = jobs[j].base;
		bounds[2 * j + 1] = jobs[j].base + jobs[j].total[0];
	}
	bounds[nseg] = total;
	PCK(R.pw_bounds.upload(bounds, s), "segment bounds");
	PCK(R.pw_offs.ensure((size_t)(nseg + 1) * sizeof(unsigned)), "segment offsets");
	unsigned *offs = R.pw_offs.as<unsigned>();
	LAUNCH(R, "photon_compact", s, k_seg_offsets<<<nseg + 1, 256, 0, s>>>(valid, bc, R.pw_bounds.as<int>(), offs));
	std::vector<unsigned> h_offs(nseg + 1);
	PCK(cudaMemcpyAsync(h_offs.data(), offs, (nseg + 1) * sizeof(unsigned), cudaMemcpyDeviceToHost, s), "segment offsets");
	PCK(cudaStreamSynchronize(s), "photon compaction");
	R.d2h += (int64_t)(nseg + 1) * sizeof(unsigned);
	R.h2d += (int64_t)bounds.size() * sizeof(int);
	R.prof_collect();
	int n = (int)h_offs[nseg];
	for(int sg = 0; sg < nseg; sg++) maps[sg].n = (int)(h_offs[sg + 1] - h_offs[sg]);
	if(n == 0) return 0;
	PCK(R.pw_ph.ensure((size_t)n * sizeof(DevPhoton)), "photon maps");
	PCK(R.pw_sorted.ensure((size_t)n * sizeof(DevPhoton)), "photon maps");
	LAUNCH(R, "photon_compact", s, k_compact<<<nb, 256, 0, s>>>(valid, R.pw_out.as<DevPhoton>(), total, bc, R.pw_ph.as<DevPhoton>()));
	PCK(R.pw_grids.upload(maps, s), "map grids");
	PCK(R.pw_morton.upload(morton, s), "map keys");
	PCK(R.pw_cellbase.upload(cell_base, s), "cell tables");
	R.h2d += (int64_t)(maps.size() * sizeof(DPhotonMap) + morton.size() * 4 + cell_base.size() * 8);
	PCK(R.pw_keys.ensure((size_t)n * 16), "keys");
	PCK(R.pw_lin.ensure((size_t)n * 8), "cell ids");
	PCK(R.pw_cells.ensure((size_t)cell_base[nseg] * sizeof(uint2) + 16), "cell tables");
	unsigned *keys = R.pw_keys.as<unsigned>(), *vals = keys + n, *keys2 = keys + 2 * (size_t)n, *vals2 = keys + 3 * (size_t)n;
	unsigned *lin = R.pw_lin.as<unsigned>(), *lin2 = lin + n;
	LAUNCH(R, "photon_sort", s, k_keys_seg<<<grid_n(n, 256), 256, 0, s>>>(R.pw_ph.as<DevPhoton>(), n, R.pw_grids.as<DPhotonMap>(),
			R.pw_morton.as<int>(), offs, nseg, keys, vals, lin));
	int key_bits = 0;
	for(int sg = 0; sg < nseg; sg++) {
		unsigned long long maxkey = morton[sg] ? (1ull << 30) - 1ull : cell_base[sg + 1] - cell_base[sg] - 1ull;
		int b = 0;
		while(b < 32 && (maxkey >> b)) b++;
		key_bits = std::max(key_bits, b);
	}
	int seg_bits = 0;
	while(seg_bits < 32 && ((unsigned)(nseg - 1) >> seg_bits)) seg_bits++;
	int nbr = (n + TILE - 1) / TILE;
	PCK(R.pw_hist.ensure((size_t)256 * nbr * sizeof(unsigned) + 16), "radix histogram");
	unsigned *hist = R.pw_hist.as<unsigned>();
	int key_passes = (key_bits + 7) / 8, seg_passes = (seg_bits + 7) / 8;
	for(int ps = 0; ps < key_passes + seg_passes; ps++) {
		if(ps == key_passes)
			LAUNCH(R, "photon_sort", s, k_seg_keys<<<grid_n(n, 256), 256, 0, s>>>(vals, n, offs, nseg, keys));
		int shift = (ps < key_passes ? ps : ps - key_passes) * 8;
		LAUNCH(R, "photon_sort", s, k_rs_hist<<<nbr, RS_THREADS, 0, s>>>(keys, n, shift, hist, nbr));
		if(scan_long(R, hist, 256 * nbr, nullptr, R.pw_part, "photon_sort", s)) return SRAY_ECUDA;
		LAUNCH(R, "photon_sort", s, k_rs_scatter<<<nbr, RS_THREADS, 0, s>>>(keys, vals, n, shift, hist, nbr, keys2, vals2));
		std::swap(keys, keys2);
		std::swap(vals, vals2);
	}
	LAUNCH(R, "photon_sort", s, k_permute<<<grid_n(n, 256), 256, 0, s>>>(R.pw_ph.as<DevPhoton>(), vals, lin, n, R.pw_sorted.as<DevPhoton>(),
			lin2));
	PCK(cudaMemsetAsync(R.pw_cells.p, 0, (size_t)cell_base[nseg] * sizeof(uint2), s), "cell tables");
	LAUNCH(R, "photon_sort", s, k_cells_seg<<<grid_n(n, 256), 256, 0, s>>>(lin2, n, offs, nseg, R.pw_cellbase.as<unsigned long long>(),
			R.pw_cells.as<uint2>()));
	for(int sg = 0; sg < nseg; sg++) {
		maps[sg].ph = R.pw_sorted.as<DevPhoton>() + h_offs[sg];
		maps[sg].cells = R.pw_cells.as<uint2>() + cell_base[sg];
	}
	PCK(cudaStreamSynchronize(s), "photon map build");
	R.prof_collect();
	return 0;
}

/* map `global` from host photons (a restored dump) */
int photon_map_restore(Renderer &R, int global, const std::vector<DevPhoton> &h, cudaStream_t s)
{
	PhotonBufs &P = global ? R.gi : R.caust;
	int n = (int)h.size();
	P.map.n = 0;
	if(n == 0) return 0;
	PCK(P.ph.ensure((size_t)n * sizeof(DevPhoton)), "photon map");
	PCK(P.tmp_ph.ensure((size_t)n * sizeof(DevPhoton)), "photon buffer");
	PCK(cudaMemcpyAsync(P.ph.p, h.data(), (size_t)n * sizeof(DevPhoton), cudaMemcpyHostToDevice, s), "upload photons");
	R.h2d += (int64_t)n * sizeof(DevPhoton);
	return photon_map_build(R, global, n, s);
}

}  // namespace sray
