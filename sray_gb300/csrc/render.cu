/* render.cu -- wavefront rendering kernels, the frame driver and the C-ABI.
 *
 * One pixel sample of every active pixel is rendered per pass:
 *   k_camera    primary rays            Camera::get_primary_ray (src/camera.cc:119-142)
 *   k_trace     closest hits            Scene::cast_ray / Octree::intersect (src/scene.cc:764,
 *                                        src/octree.inl:201-241) with the intersectors;
 *                                        camera rays by k_trace_packet, a warp per 8 x 4 patch
 *   k_shade     Phong + shadows + spawn shade_phong / calc_lighting / shade_undef
 *                                        (src/shader.cc:36-283)
 *   k_gather    photon-map estimates    PhotonMap::irradiance_est / radiance_est (src/pmap.cc:109-178)
 *   k_finish    adaptive supersampling  render_block / variance (src/render.cc:194-270)
 * The recursion of trace_ray is unrolled into bounces over SoA ray queues:
 * every ray carries the product of the weights that the reference's nested
 * return expression (src/shader.cc:246) applies to its radiance, and adds
 * its local terms to the pixel sample directly.
 */
#include <math.h>
#include <cmath>
#include <float.h>
#include <limits.h>
#include <string.h>
#include <stddef.h>
#include <stdio.h>
#include <algorithm>
#include <mutex>
#include <cooperative_groups.h>
#include <cooperative_groups/scan.h>
#include "renderer.h"
#include "nrc.h"
#include "range_ff.h"
#include "slot_order.h"

namespace cg = cooperative_groups;

namespace sray {

#define DIFFUSE_ITER 0x7fffffff   /* INT_MAX marks a final-gather ray (src/shader.cc:78-81) */

static __device__ __forceinline__ int warp_alloc(int *counter, int n)
{
	cg::coalesced_group g = cg::coalesced_threads();
	int excl = cg::exclusive_scan(g, n);
	int base = 0;
	if(g.thread_rank() == g.size() - 1) base = atomicAdd(counter, excl + n);
	base = g.shfl(base, g.size() - 1);
	return base + excl;
}

/* ---------------------------------------------------------------- */
/* primary rays of samples [s0, s0 + width) of every active pixel; the ray's
 * accumulator slot is (active index * width + sample - s0) */
__global__ void k_camera(DScene S, const int *active, int a0, int na, int s0, int width, RayQueue q, float4 *acc,
		DevCounters *ctr)
{
	/* a wave: active pixels [a0, a0 + na); queue entry i is accumulator slot a0 * width + i */
	int n = na * width;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int a = a0 + i / width, j = i - (i / width) * width;
		int slot = a0 * width + i;
		int p = slot_pixel(active, a, S.njobs > 0 ? 0 : S.width, S.height);
		int sample = s0 + j;
		int W = S.width, Hh = S.height, lp = p, t0 = S.t0, cam_base = 0;
		float cam_f = S.cam_f, xsz = S.cam_xsz, ysz = S.cam_ysz;
		if(S.njobs > 0) {
			/* a batch: the job's resolution, camera (its scene's) and frame time */
			const DevJob &J = S.jobs[job_of(S, p)];
			W = J.width; Hh = J.height; lp = p - J.pix0; t0 = J.t0;
			cam_f = J.cam_f; xsz = J.cam_xsz; ysz = J.cam_ysz;
			cam_base = J.cam_base;
		}
		int x = lp % W, y = lp / W;
		sray_rng s;
		sray_rng_init(&s, S.seed, SRAY_DOM_PIXEL, (uint32_t)p, (uint32_t)sample);
		float px = ((float)x / (float)W) * xsz - xsz / 2.0f;
		float py = 1.0f - ((float)y / (float)Hh) * ysz;
		if(sample > 0) {
			px = px + xsz * (frand(&s, 1.0f) - 0.5f) / (float)W;
			py = py + ysz * (frand(&s, 1.0f) - 0.5f) / (float)Hh;
		}
		V3 d = mk(px, py, cam_f) * S.cam_maxd;
		int time = t0;
		if(S.mblur && sample > 0 && S.shutter > 0) time += sray_rng_int(&s) % S.shutter - S.shutter / 2;
		const float *m = S.cam_m + ((size_t)cam_base + time_index(S, time)) * 12;
		V3 o = mul_pt(m, mk(0.0f, 0.0f, 0.0f));
		d = mul_dir(m, d);
		q.o[i] = make_float4(o.x, o.y, o.z, 1.0f);
		q.d[i] = make_float4(d.x, d.y, d.z, 1.0f);
		q.w[i] = make_float4(1.0f, 1.0f, 1.0f, __int_as_float(p));
		q.meta[i] = make_int4(slot, S.iter, 1, time);
		q.stk[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
		q.ext[i] = make_int2(sample, 0);
		acc[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) {
		*q.count = n;
		atomicAdd(&ctr->rays[0], (unsigned long long)n);
	}
}

/* ---------------------------------------------------------------- */
/* sorting a pass before it is traced: key = direction octant over the
 * Morton code of the origin's cell in a 128^3 grid over the scene box */
__device__ __forceinline__ unsigned spread7(unsigned v)
{
	v &= 0x7f;
	v = (v | (v << 8)) & 0x0000F00Fu;
	v = (v | (v << 4)) & 0x000C30C3u;
	v = (v | (v << 2)) & 0x00249249u;
	return v;
}

__global__ void k_ray_keys(RayQueue q, int n, float lx, float ly, float lz, float sx, float sy, float sz, int kshift, unsigned *keys,
		unsigned *vals)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		float4 o = q.o[i], d = q.d[i];
		int cx = (int)((o.x - lx) * sx), cy = (int)((o.y - ly) * sy), cz = (int)((o.z - lz) * sz);
		cx = cx < 0 ? 0 : (cx > 127 ? 127 : cx);
		cy = cy < 0 ? 0 : (cy > 127 ? 127 : cy);
		cz = cz < 0 ? 0 : (cz > 127 ? 127 : cz);
		unsigned oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
		keys[i] = ((oct << 21) | spread7((unsigned)cx) | (spread7((unsigned)cy) << 1) | (spread7((unsigned)cz) << 2)) >> kshift;
		vals[i] = (unsigned)i;
	}
}

/* the pass's entries in sorted order */
__global__ void k_ray_permute(RayQueue in, const unsigned *vals, int n, RayQueue out)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		unsigned v = vals[i];
		out.o[i] = in.o[v];
		out.d[i] = in.d[v];
		out.w[i] = in.w[v];
		out.meta[i] = in.meta[v];
		out.stk[i] = in.stk[v];
		out.ext[i] = in.ext[v];
	}
}

/* Closest hits.  HYB = true traces through the mesh hierarchies and lists
 * the rays whose result the octree must decide in fb (count in fb[0], ray
 * indices from fb + 1); HYB = false traces the listed rays with the octree
 * alone.  Keeping the two in separate kernels keeps the octree code out of
 * the hierarchy traversal's register allocation. */
template <bool COUNT, bool HYB>
__global__ void __launch_bounds__(SRAY_TRACE_THREADS, 8) k_trace(DScene S, RayQueue q, int4 *hits, DevCounters *ctr, int *fb)
{
	int n = HYB ? *q.count : fb[0];
	TraceCounters tc = {0, 0};
	int overflow = 0;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int ri = HYB ? i : fb[1 + i];
		float4 o = q.o[ri], d = q.d[ri];
		int time = q.meta[ri].w;
		int scene = S.nscenes > 1 ? pixel_scene(S, __float_as_int(q.w[ri].w)) : -1;
		Hit h;
		bool sure = true;
		if(HYB) sure = trace_two_level<COUNT, false>(S, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), time, h, &tc, &overflow, scene) != 0;
		else trace_closest_octree_impl<COUNT>(S, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), time, h, &tc, &overflow, scene);
		if(HYB && !sure) {
			fb[1 + atomicAdd(fb, 1)] = ri;
			continue;
		}
		hits[ri] = make_int4(__float_as_int(h.t), h.obj, h.prim, h.tie);
	}
	if(overflow) atomicOr(&ctr->overflow, 1);
	if(COUNT) {
		atomicAdd(&ctr->nodes, tc.nodes);
		atomicAdd(&ctr->prims, tc.prims);
	}
	if(!HYB && n > 0 && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr->bvh_fallbacks, (unsigned long long)n);
}

/* Closest hits of coherent rays -- a pass of camera rays, the 32 of a warp
 * from an 8 x 4 pixel patch -- by one traversal per warp: the warp walks the
 * two-level hierarchy together, opening a node when any lane's widened box
 * test reaches one of its children and taking the reached children nearest
 * first by their smallest entry distance over the lanes; each lane tests its
 * own ray against the boxes, objects and faces the warp visits, and enters
 * an instance only when its own ray enters the instance's mesh box within
 * its best distance.  A lane's result equals the thread-per-ray
 * traversal's: a box, object or face its own traversal would not have
 * reached holds no candidate within the lane's best distance (the box tests
 * are conservative and bounded by the best so far), so the candidates at
 * the final distance, the tie flag and the octree confirmation are the
 * same; a ray that traversal hands to the octrees (a tie, an unconfirmed
 * hit, a mesh without a hierarchy) goes to the octree retrace here too.  The
 * warp's stack (entries and their smallest entry distance) is in shared
 * memory; every branch around a warp vote is the same for all lanes.
 * Returns 0 when the octrees must decide, else 1 with the closest hit in h
 * (h.obj -1: none). */
__device__ __forceinline__ int ford(float x)
{
	int b = __float_as_int(x);
	return b >= 0 ? b : b ^ 0x7fffffff;
}

__device__ __forceinline__ float ford_inv(int b) { return __int_as_float(b >= 0 ? b : b ^ 0x7fffffff); }

__device__ __forceinline__ int packet_trace(const DScene &S, bool valid, V3 wo, V3 wd, int time, int *st_node, float *st_te,
		Hit &h, int *overflow)
{
	const unsigned FULL = 0xffffffffu;
	const int lane = threadIdx.x & 31;
	h.t = FLT_MAX;
	h.obj = -1;
	h.prim = -1;
	h.tie = 0;
	const int2 roots = scene_roots(S, -1);
	if(roots.x < 0) return 1;
	if(roots.y < 0) return 0;
	const int ti = time_index(S, time);
	const RayT wr = make_ray(wo, wd);
	const DevNode &sroot = S.snodes[roots.x];
	const RayC wc = make_rayc(wr, box_bound(sroot.mn, sroot.mx));
	RayT r = wr;
	RayC rc = wc;
	float best = FLT_MAX;
	int bobj = -1, bprim = -1, bslot = -1;
	bool eq = false, undecided = false;
	bool live = valid;     /* the lane takes part in the current instance (or the object level) */
	int sp = 0, inst_base = 0, iobj = -1;
	bool inst = false;
	int cur = roots.y;
	for(;;) {
		if(cur == BVH_NONE) {
			bool found = false;
			while(sp > 0) {
				const int k = sp - 1;
				if(inst && k < inst_base) {   /* the instance's entries are done */
					inst = false;
					iobj = -1;
					r = wr;
					rc = wc;
					live = valid;
				}
				sp = k;
				if(__any_sync(FULL, live && st_te[k] <= best)) {
					cur = st_node[k];
					found = true;
					break;
				}
			}
			if(!found) break;
		}
		if(!inst && cur < 0) {
			/* object ~cur */
			const int o = ~cur;
			cur = BVH_NONE;
			const DevObj ob = S.objs[o];
			const RayT orr = object_ray(S, o, ti, wo, wd);
			if(ob.type != 2) {
				float t;
				if(valid && (ob.type == 0 ? sphere_hit(orr, ob.rad, S.eps, t) : cylinder_hit(orr, ob.rad, ob.start, ob.end, S.eps, t))
						&& t <= best) {
					if(t < best) {
						best = t;
						bobj = o;
						bprim = 0;
						bslot = -1;
						eq = false;
					} else if(o != bobj || bprim != 0) {
						eq = true;
					}
				}
				continue;
			}
			if(ob.mesh_root < 0) continue;
			if(ob.bvh_root < 0) {
				undecided = undecided || valid;
				continue;
			}
			float te = 0.0f;
			const DevNode &rn = S.mnodes[ob.mesh_root];
			const bool enter = valid && box_hit(rn.mn, rn.mx, orr, te) && !SRAY_PRUNE(te, best);
			if(!__any_sync(FULL, enter)) continue;
			r = orr;
			rc = make_rayc(orr, box_bound(rn.mn, rn.mx));
			inst = true;
			inst_base = sp;
			iobj = o;
			live = enter;
			cur = ob.bvh_root;
			continue;
		}
		if(inst && cur < 0) {
			/* a leaf of the mesh hierarchy: its faces, for the lanes in the instance */
			const unsigned v = ~(unsigned)cur;
			cur = BVH_NONE;
			const int start = (int)(v >> 4), cnt = (int)(v & 15u);
			const float4 *tp = reinterpret_cast<const float4 *>(S.btris + start);
			for(int k = 0; k < cnt; k++) {
				const float4 a = __ldg(tp + 3 * k), b = __ldg(tp + 3 * k + 1), c = __ldg(tp + 3 * k + 2);
				float t;
				if(!live || !tri_hit(a, b, c, r, S.eps, best, t)) continue;
				const int prim = __ldg(S.bprim + start + k);
				if(t < best) {
					best = t;
					bobj = iobj;
					bprim = prim;
					bslot = start + k;
					eq = false;
				} else if(iobj != bobj || prim != bprim) {
					eq = true;
				}
			}
			continue;
		}
		/* a node: the lanes' box tests, then the warp's smallest entry distance per child */
		const float4 *np = reinterpret_cast<const float4 *>((inst ? S.bnodes : S.tnodes) + cur);
		const NodePlanes pl = node_planes(np, rc);
		const int4 ch = __ldg(reinterpret_cast<const int4 *>(np) + 6);
		const float lim = fminf(best, 1.0f);
		int ref[4] = {ch.x, ch.y, ch.z, ch.w};
		float tn;
		float key[4];
		key[0] = (live && ref[0] != BVH_NONE && wide_box(rc, pl.nx.x, pl.ny.x, pl.nz.x, pl.fx.x, pl.fy.x, pl.fz.x, lim, tn)) ? tn : INFINITY;
		key[1] = (live && ref[1] != BVH_NONE && wide_box(rc, pl.nx.y, pl.ny.y, pl.nz.y, pl.fx.y, pl.fy.y, pl.fz.y, lim, tn)) ? tn : INFINITY;
		key[2] = (live && ref[2] != BVH_NONE && wide_box(rc, pl.nx.z, pl.ny.z, pl.nz.z, pl.fx.z, pl.fy.z, pl.fz.z, lim, tn)) ? tn : INFINITY;
		key[3] = (live && ref[3] != BVH_NONE && wide_box(rc, pl.nx.w, pl.ny.w, pl.nz.w, pl.fx.w, pl.fy.w, pl.fz.w, lim, tn)) ? tn : INFINITY;
		#pragma unroll
		for(int k = 0; k < 4; k++) key[k] = ford_inv(__reduce_min_sync(FULL, ford(key[k])));
#define SRAY_CSWAP(i, j) do { if(key[j] < key[i]) { float tk = key[i]; key[i] = key[j]; key[j] = tk; int tr_ = ref[i]; ref[i] = ref[j]; ref[j] = tr_; } } while(0)
		SRAY_CSWAP(0, 1);
		SRAY_CSWAP(2, 3);
		SRAY_CSWAP(0, 2);
		SRAY_CSWAP(1, 3);
		SRAY_CSWAP(1, 2);
#undef SRAY_CSWAP
		if(key[0] == INFINITY) {
			cur = BVH_NONE;
			continue;
		}
		#pragma unroll
		for(int k = 3; k >= 1; k--) {
			if(key[k] == INFINITY) continue;
			if(sp >= SRAY_STACK) {
				*overflow = 1;
				return 1;
			}
			if(lane == 0) {
				st_node[sp] = ref[k];
				st_te[sp] = key[k];
			}
			sp++;
		}
		__syncwarp(FULL);
		cur = ref[0];
	}
	if(!valid) return 1;
	if(undecided) return 0;
	if(bobj < 0) return 1;
	if(eq) return 0;
	/* confirm against the octrees */
	if(bslot >= 0 && !octree_reaches(S.mnodes, S.mprim, __ldg(S.bhome + bslot), object_ray(S, bobj, ti, wo, wd), bprim, best, true))
		return 0;
	if(!octree_reaches(S.snodes, S.sslots, __ldg(S.ohome + bobj), wr, bobj, best, true)) return 0;
	h.t = best;
	h.obj = bobj;
	h.prim = bprim;
	h.tie = 0;
	return 1;
}

/* a pass of coherent closest-hit rays (one scene), a warp per 32 rays; the
 * rays the octrees must decide are listed in fb as by k_trace */
#ifndef SRAY_PACKET_BLOCKS
#define SRAY_PACKET_BLOCKS 6     /* resident blocks per SM: 80 registers */
#endif
__global__ void __launch_bounds__(SRAY_TRACE_THREADS, SRAY_PACKET_BLOCKS) k_trace_packet(DScene S, RayQueue q, int4 *hits, DevCounters *ctr, int *fb)
{
	__shared__ int st_node[SRAY_TRACE_THREADS / 32][SRAY_STACK];
	__shared__ float st_te[SRAY_TRACE_THREADS / 32][SRAY_STACK];
	const int n = *q.count;
	const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
	int overflow = 0;
	for(int base = (blockIdx.x * (SRAY_TRACE_THREADS / 32) + w) * 32; base < n; base += gridDim.x * SRAY_TRACE_THREADS) {
		const int ri = base + lane;
		const bool valid = ri < n;
		float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f), d = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
		int time = S.t0;
		if(valid) {
			o = q.o[ri];
			d = q.d[ri];
			time = q.meta[ri].w;
		}
		Hit h;
		const int res = packet_trace(S, valid, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), time, st_node[w], st_te[w], h, &overflow);
		if(!valid) continue;
		if(res == 0) {
			fb[1 + atomicAdd(fb, 1)] = ri;
			continue;
		}
		hits[ri] = make_int4(__float_as_int(h.t), h.obj, h.prim, h.tie);
	}
	if(overflow) atomicOr(&ctr->overflow, 1);
}

/* Closest hits with one warp per ray, for passes of few rays (the tails of
 * the shading tree: long mirror and glass chains, grazing rays), whose
 * launches otherwise last as long as one thread's chain of dependent node
 * fetches.  The warp keeps the ray's stack in shared memory and takes up to
 * eight entries per step: four lanes per entry test a node's four children,
 * a leaf's faces, or an object.  The hit children are sorted across the
 * warp and stacked nearest on top.  The result is the thread-per-ray
 * traversal's: the closest candidate over every entry whose box is reached
 * within the best distance so far, with a tie where two different faces or
 * objects share it (the candidates at the final distance are reached in any
 * order), confirmed against the octrees; a ray it cannot decide (a tie, an
 * unconfirmed hit, a full stack) goes to the octree retrace. */
#define WR_CAP 512
#define WR_POP 8


/* One ray's two-level traversal by the calling warp (all 32 lanes, the
 * same arguments), with the warp's stack st_*.  ANY = false: returns 1 with
 * the closest hit in best / bobj / bprim (bobj -1: none), 0 when the
 * octrees must decide.  ANY = true (a light sample, segment [eps, 1]):
 * returns 1 when a hit the octrees reach exists, 0 when none exists, 2 when
 * the octrees must decide. */
template <bool ANY>
__device__ __forceinline__ int warp_trace(const DScene &S, V3 wo, V3 wd, int time, int *st_ref, int *st_obj, float *st_te, float &best,
		int &bobj, int &bprim, int scene)
{
	const unsigned FULL = 0xffffffffu;
	int lane = threadIdx.x & 31;
	int g = lane >> 2, sub = lane & 3;
	best = ANY ? 1.0f : FLT_MAX;
	bobj = -1;
	bprim = -1;
	const int2 roots = scene_roots(S, scene);
	if(roots.x < 0) return ANY ? 0 : 1;
	if(roots.y < 0) return ANY ? 2 : 0;
	int bslot = -1;
	int ti = time_index(S, time);
	RayT wr = make_ray(wo, wd);
	const DevNode &sroot = S.snodes[roots.x];
	RayC wc = make_rayc(wr, box_bound(sroot.mn, sroot.mx));
	bool eq = false;
	if(lane == 0) {
		st_ref[0] = roots.y;   /* the object hierarchy's root */
		st_obj[0] = -1;
		st_te[0] = -INFINITY;
	}
	int sp = 1;
	__syncwarp();
	while(sp > 0) {
		int npop = sp < WR_POP ? sp : WR_POP;
		int base = sp - npop;
		bool active = g < npop;
		int eref = 0, eobj = -1;
		if(active) {
			eref = st_ref[base + g];
			eobj = st_obj[base + g];
			active = ANY || st_te[base + g] <= best;
		}
		__syncwarp();
		sp = base;
		float ct = INFINITY;
		int cobj = -1, cprim = -1, cslot = -1;
		bool ceq = false, push = false, lbail = false;
		int pref = 0, pobj = -1;
		float pte = 0.0f;
		if(active) {
			if(eobj < 0 && eref < 0) {
				/* an object of the object hierarchy */
				if(sub == 0) {
					int o = ~eref;
					const DevObj ob = S.objs[o];
					RayT orr = object_ray(S, o, ti, wo, wd);
					if(ob.type != 2) {
						float t;
						bool hit = ob.type == 0 ? sphere_hit(orr, ob.rad, S.eps, t) : cylinder_hit(orr, ob.rad, ob.start, ob.end, S.eps, t);
						if(hit && t <= best) { ct = t; cobj = o; cprim = 0; cslot = -1; }
					} else if(ob.mesh_root >= 0) {
						if(ob.bvh_root < 0) {
							lbail = true;
						} else {
							float te;
							const DevNode &rn = S.mnodes[ob.mesh_root];
							if(box_hit(rn.mn, rn.mx, orr, te) && (ANY || !SRAY_PRUNE(te, best))) {
								push = true;
								pref = ob.bvh_root;
								pobj = o;
								pte = te;
							}
						}
					}
				}
			} else if(eref < 0) {
				/* a leaf of object eobj's mesh hierarchy: faces sub, sub + 4, ... */
				unsigned v = ~(unsigned)eref;
				int start = (int)(v >> 4), cnt = (int)(v & 15u);
				RayT orr = object_ray(S, eobj, ti, wo, wd);
				const float4 *tp = reinterpret_cast<const float4 *>(S.btris + start);
				for(int k = sub; k < cnt; k += 4) {
					float4 a = __ldg(tp + 3 * k), b = __ldg(tp + 3 * k + 1), c = __ldg(tp + 3 * k + 2);
					float t;
					if(!tri_hit(a, b, c, orr, S.eps, best, t)) continue;
					int prim = __ldg(S.bprim + start + k);
					if(t < ct) { ct = t; cobj = eobj; cprim = prim; cslot = start + k; ceq = false; }
					else if(t == ct) ceq = true;
				}
			} else {
				/* a node: child `sub` */
				const float4 *np = reinterpret_cast<const float4 *>((eobj >= 0 ? S.bnodes : S.tnodes) + eref);
				RayC rc = wc;
				if(eobj >= 0) {
					const DevNode &rn = S.mnodes[S.objs[eobj].mesh_root];
					rc = make_rayc(object_ray(S, eobj, ti, wo, wd), box_bound(rn.mn, rn.mx));
				}
				int ch = __ldg(reinterpret_cast<const int *>(np + 6) + sub);
				float tn;
				/* this lane's child in each bound vector, entry and exit planes by the direction's signs */
				const float *nf = reinterpret_cast<const float *>(np) + sub;
				int sx = (rc.neg & 1u) ? 12 : 0, sy = (rc.neg & 2u) ? 12 : 0, sz = (rc.neg & 4u) ? 12 : 0;
				if(ch != BVH_NONE && wide_box(rc, __ldg(nf + sx), __ldg(nf + 4 + sy), __ldg(nf + 8 + sz), __ldg(nf + 12 - sx),
						__ldg(nf + 16 - sy), __ldg(nf + 20 - sz), fminf(best, 1.0f), tn)) {
					push = true;
					pref = ch;
					pobj = eobj;
					pte = tn;
				}
			}
		}
		if(__any_sync(FULL, lbail)) return ANY ? 2 : 0;
		/* the step's closest candidate */
		float m = ct;
		for(int off = 16; off > 0; off >>= 1) m = fminf(m, __shfl_xor_sync(FULL, m, off));
		if(m < INFINITY && m <= best) {
			unsigned at = __ballot_sync(FULL, ct == m);
			int src = __ffs(at) - 1;
			int mobj = __shfl_sync(FULL, cobj, src), mprim = __shfl_sync(FULL, cprim, src), mslot = __shfl_sync(FULL, cslot, src);
			if(ANY) {
				best = m;
				bobj = mobj;
				bprim = mprim;
				bslot = mslot;
				break;
			}
			bool other = __any_sync(FULL, ct == m && (ceq || cobj != mobj || cprim != mprim));
			if(m < best) {
				best = m;
				bobj = mobj;
				bprim = mprim;
				bslot = mslot;
				eq = other;
			} else if(other || mobj != bobj || mprim != bprim) {
				eq = true;
			}
		}
		/* stack the hit children, farthest first so that the nearest pop first */
		unsigned pm = __ballot_sync(FULL, push);
		int cnt = __popc(pm);
		if(sp + cnt > WR_CAP) return ANY ? 2 : 0;
		float key = push ? pte : -INFINITY;
		int idx = lane;
		for(int k = 2; k <= 32; k <<= 1) {
			for(int j = k >> 1; j > 0; j >>= 1) {
				float ok = __shfl_xor_sync(FULL, key, j);
				int oi = __shfl_xor_sync(FULL, idx, j);
				bool desc = (lane & k) == 0;         /* descending runs first: a descending sort overall */
				bool lower = (lane & j) == 0;
				bool take = lower == desc ? (ok > key || (ok == key && oi < idx)) : (ok < key || (ok == key && oi > idx));
				if(take) { key = ok; idx = oi; }
			}
		}
		int sref = __shfl_sync(FULL, pref, idx), sobj = __shfl_sync(FULL, pobj, idx);
		float ste = __shfl_sync(FULL, pte, idx);
		if(lane < cnt) {
			st_ref[sp + lane] = sref;
			st_obj[sp + lane] = sobj;
			st_te[sp + lane] = ste;
		}
		sp += cnt;
		__syncwarp();
	}
	if(bobj < 0) return ANY ? 0 : 1;
	if(!ANY && eq) return 0;
	int ok = 1;
	if(lane == 0) {
		if(bslot >= 0 && !octree_reaches(S.mnodes, S.mprim, __ldg(S.bhome + bslot), object_ray(S, bobj, ti, wo, wd), bprim, best, !ANY))
			ok = 0;
		else if(!octree_reaches(S.snodes, S.sslots, __ldg(S.ohome + bobj), wr, bobj, best, !ANY))
			ok = 0;
	}
	ok = __shfl_sync(FULL, ok, 0);
	if(ANY) return ok ? 1 : 2;
	return ok;
}

__global__ void __launch_bounds__(128) k_trace_warp(DScene S, RayQueue q, int4 *hits, int *fb)
{
	__shared__ int s_ref[4][WR_CAP];
	__shared__ int s_obj[4][WR_CAP];
	__shared__ float s_te[4][WR_CAP];
	int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	int n = *q.count;
	for(int ri = blockIdx.x * 4 + w; ri < n; ri += gridDim.x * 4) {
		float4 o4 = q.o[ri], d4 = q.d[ri];
		float best;
		int bobj, bprim;
		int scene = S.nscenes > 1 ? pixel_scene(S, __float_as_int(q.w[ri].w)) : -1;
		int res = warp_trace<false>(S, mk(o4.x, o4.y, o4.z), mk(d4.x, d4.y, d4.z), q.meta[ri].w, s_ref[w], s_obj[w], s_te[w], best, bobj,
				bprim, scene);
		if(lane == 0) {
			if(!res) fb[1 + atomicAdd(fb, 1)] = ri;
			else if(bobj >= 0) hits[ri] = make_int4(__float_as_int(best), bobj, bprim, 0);
			else hits[ri] = make_int4(__float_as_int(FLT_MAX), -1, -1, 0);
		}
		__syncwarp();
	}
}

__device__ __forceinline__ void acc_add(float4 *acc, int p, float r, float g, float b)
{
	atomicAdd(&acc[p].x, r);
	atomicAdd(&acc[p].y, g);
	atomicAdd(&acc[p].z, b);
}

__device__ __forceinline__ float maxf_ref(float a, float b) { return a > b ? a : b; }

#define MAX_DS 128

struct ShadeOut {
	RayQueue qo;
	GatherReq *gq;
	int *gq_count;
	int gq_cap;
	ShadowReq *sq;
	int *sq_count;
	int sq_cap;
};

__device__ __forceinline__ void push_child(ShadeOut &out, V3 o, V3 d, float energy, int iter, int path, int dsub,
		const IorStack &st, float wr, float wg, float wb, int pixel, int aslot, int sample, int time, int *overflow)
{
	int slot = warp_alloc(out.qo.count, 1);
	if(slot >= out.qo.cap) { *overflow = 1; return; }
	RayQueue &q = out.qo;
	q.o[slot] = make_float4(o.x, o.y, o.z, energy);
	q.d[slot] = make_float4(d.x, d.y, d.z, st.ior);
	q.w[slot] = make_float4(wr, wg, wb, __int_as_float(pixel));
	q.meta[slot] = make_int4(aslot, iter, path, time);
	q.stk[slot] = make_float4(st.stk[0], st.stk[1], st.stk[2], st.stk[3]);
	q.ext[slot] = make_int2(sample | (dsub << 16), st.sp);
}

__device__ __forceinline__ void push_gather(ShadeOut &out, V3 pos, V3 n, int kind, int pixel, float wr, float wg, float wb,
		int *overflow)
{
	int slot = warp_alloc(out.gq_count, 1);
	if(slot >= out.gq_cap) { *overflow = 1; return; }
	GatherReq g;
	g.a = make_float4(pos.x, pos.y, pos.z, __int_as_float(kind));
	g.b = make_float4(n.x, n.y, n.z, __int_as_float(pixel));
	g.w = make_float4(wr, wg, wb, 0.0f);
	out.gq[slot] = g;
}

/* a shadow ray and the light contribution it carries if unoccluded */
__device__ __forceinline__ void push_shadow(ShadeOut &out, V3 o, V3 d, int time, int pixel, float wr, float wg, float wb,
		int *overflow, int scene = -1)
{
	int slot = warp_alloc(out.sq_count, 1);
	if(slot >= out.sq_cap) { *overflow = 1; return; }
	ShadowReq r;
	r.a = make_float4(o.x, o.y, o.z, __int_as_float(time));
	r.b = make_float4(d.x, d.y, d.z, __int_as_float(pixel));
	r.w = make_float4(wr, wg, wb, __int_as_float(scene));
	out.sq[slot] = r;
}

/* a ray of the shading tree, as a queue entry holds it */
struct RayRec {
	V3 o, d;
	float energy;
	IorStack st;
	float w[3];
	int pixel, aslot, iter, path, time, sample, dsub;
};

__device__ __forceinline__ void load_ray(const RayQueue &q, int i, RayRec &r)
{
	float4 o4 = q.o[i], d4 = q.d[i], w4 = q.w[i], st4 = q.stk[i];
	int4 meta = q.meta[i];
	int2 ext = q.ext[i];
	r.o = mk(o4.x, o4.y, o4.z);
	r.d = mk(d4.x, d4.y, d4.z);
	r.energy = o4.w;
	r.st.ior = d4.w;
	r.st.stk[0] = st4.x; r.st.stk[1] = st4.y; r.st.stk[2] = st4.z; r.st.stk[3] = st4.w;
	r.st.sp = ext.y;
	r.w[0] = w4.x; r.w[1] = w4.y; r.w[2] = w4.z;
	r.pixel = __float_as_int(w4.w);
	r.aslot = meta.x;
	r.iter = meta.y;
	r.path = meta.z;
	r.time = meta.w;
	r.sample = ext.x & 0xffff;
	r.dsub = ext.x >> 16;
}

__device__ __forceinline__ void store_ray(const RayQueue &q, int slot, const RayRec &r)
{
	q.o[slot] = make_float4(r.o.x, r.o.y, r.o.z, r.energy);
	q.d[slot] = make_float4(r.d.x, r.d.y, r.d.z, r.st.ior);
	q.w[slot] = make_float4(r.w[0], r.w[1], r.w[2], __int_as_float(r.pixel));
	q.meta[slot] = make_int4(r.aslot, r.iter, r.path, r.time);
	q.stk[slot] = make_float4(r.st.stk[0], r.st.stk[1], r.st.stk[2], r.st.stk[3]);
	q.ext[slot] = make_int2(r.sample | (r.dsub << 16), r.st.sp);
}

__device__ __forceinline__ RayRec make_child(const RayRec &p, V3 o, V3 d, float energy, int iter, int path, int dsub, const IorStack &st,
		float wr, float wg, float wb)
{
	RayRec c;
	c.o = o;
	c.d = d;
	c.energy = energy;
	c.st = st;
	c.w[0] = wr; c.w[1] = wg; c.w[2] = wb;
	c.pixel = p.pixel;
	c.aslot = p.aslot;
	c.iter = iter;
	c.path = path;
	c.time = p.time;
	c.sample = p.sample;
	c.dsub = dsub;
	return c;
}

/* ---- radiance cache at a final-gather vertex ---- */

/* 32-bit integer hash: the "lowbias32" finaliser of C. Wellons' hash
 * prospector (xorshift-multiply, two rounds) */
__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
	x ^= x >> 16;
	x *= 0x7feb352du;
	x ^= x >> 15;
	x *= 0x846ca68bu;
	x ^= x >> 16;
	return x;
}

/* network inputs of a vertex: position in the scene box, normal and
 * incident direction, all mapped to [0, 1] */
__device__ __forceinline__ void nrc_inputs(const DNrc &N, V3 pos, V3 n, V3 d, float *x)
{
	x[0] = (pos.x - N.lo[0]) * N.sc[0];
	x[1] = (pos.y - N.lo[1]) * N.sc[1];
	x[2] = (pos.z - N.lo[2]) * N.sc[2];
	x[3] = 0.5f * (n.x + 1.0f);
	x[4] = 0.5f * (n.y + 1.0f);
	x[5] = 0.5f * (n.z + 1.0f);
	x[6] = 0.5f * (d.x + 1.0f);
	x[7] = 0.5f * (d.y + 1.0f);
	x[8] = 0.5f * (d.z + 1.0f);
}

__device__ __forceinline__ int nrc_region(const float *x)
{
	int c[3];
	#pragma unroll
	for(int a = 0; a < 3; a++) {
		float v = x[a] * (float)NRC_GRID;
		int k = v > 0.0f ? (int)v : 0;
		c[a] = k < NRC_GRID ? k : NRC_GRID - 1;
	}
	return (c[2] * NRC_GRID + c[1]) * NRC_GRID + c[0];
}

/* warp-aggregated count of the threads for which pred holds */
__device__ __forceinline__ void warp_count(unsigned long long *p, bool pred)
{
	cg::coalesced_group g = cg::coalesced_threads();
	unsigned int n = __popc(g.ballot(pred));
	if(g.thread_rank() == 0 && n) atomicAdd(p, (unsigned long long)n);
}

__device__ __forceinline__ void store_x(float *dst, const float *x)
{
	#pragma unroll
	for(int k = 0; k < 9; k++) dst[k] = x[k];
}

/* shade one hit: env colour for misses, shade_phong / shade_undef
 * (src/shader.cc:36-283) for hits.  Light samples, children (reflection,
 * refraction, final-gather rays) and photon gathers go to the emitter `em`:
 * em.shadow(origin, dir, time, slot, contribution rgb) for a light sample
 * whose contribution counts when the segment is unoccluded,
 * em.gather(pos, normal, kind, slot, weight rgb), em.child(ray). */
template <class E>
__device__ __forceinline__ void shade_one(const DScene &S, const RayRec &ray, const Hit &h, int depth, float4 *acc, E &em)
{
	int aslot = ray.aslot;
	int pixel = ray.pixel;
	int iter = ray.iter, path = ray.path, time = ray.time;
	int sample = ray.sample;
	int dsub = ray.dsub;
	V3 rd = ray.d;
	const float *w = ray.w;
	/* the ray's scene: its lights and environment (a scene set's, or the view's) */
	const int scene = pixel_scene(S, pixel);
	int l0 = 0, nl = S.nlights;
	/* (values, not pointers: the address of a kernel parameter would copy
	 * the scene view to local memory) */
	float4 env_col = make_float4(S.env_col[0], S.env_col[1], S.env_col[2], S.env_col[3]);
	float4 env_amb = make_float4(S.env_amb[0], S.env_amb[1], S.env_amb[2], S.env_amb[3]);
	if(scene >= 0) {
		const DevSceneRef &SR = S.scenes[scene];
		l0 = SR.light0;
		nl = SR.nlights;
		env_col = make_float4(SR.env_col[0], SR.env_col[1], SR.env_col[2], SR.env_col[3]);
		env_amb = make_float4(SR.env_amb[0], SR.env_amb[1], SR.env_amb[2], SR.env_amb[3]);
	}
	if(h.obj < 0) {
		acc_add(acc, aslot, w[0] * env_col.x, w[1] * env_col.y, w[2] * env_col.z);
		if(depth == 0) acc[aslot].w = env_col.w;
		return;
	}
	if(depth == 0) acc[aslot].w = 1.0f;
	const DevMat &mat = mat_of(S, h.obj);
	Surf sp;
	surface_point(S, h, ray.o, rd, time, sp, !mat.phong || mat.textured, mat.textured && mat.tex[TA_NORMAL] >= 0);
	if(!mat.phong) {
		/* shade_undef (src/shader.cc:36-73) */
		sray_rng rng;
		sray_rng_init(&rng, S.seed, SRAY_DOM_PIXEL | ((uint32_t)path << 4), (uint32_t)pixel, (uint32_t)(sample | (dsub << 16)));
		int tx = (int)(sp.tex[0] * 20.0f), ty = (int)(sp.tex[1] * 10.0f);
		bool even = (tx % 2) == (ty % 2);
		float tc[3] = {even ? 1.0f : 0.2f, 0.3f, even ? 0.2f : 1.0f};
		acc_add(acc, aslot, w[0] * (0.1f * tc[0]), w[1] * (0.1f * tc[1]), w[2] * (0.1f * tc[2]));
		for(int li = l0; li < l0 + nl; li++) {
			const DevLight &L = S.lights[li];
			V3 lpos = light_point(S, li, time, &rng);
			V3 ldir = lpos - sp.pos;
			float ldist = len(ldir);
			V3 sdir = ldir;
			ldir = ldir / ldist;
			V3 vdir = -normalized(rd);
			V3 hdir = normalized(ldir + vdir);
			float ndotl = maxf_ref(dot(sp.normal, ldir), 0.0f);
			float ndoth = maxf_ref(dot(sp.normal, hdir), 0.0f);
			float pw = powf(ndoth, 50.0f);
			em.shadow(shadow_origin(sp, sdir), sdir, time, aslot, w[0] * (ndotl * L.col[0] * tc[0] + pw * L.col[0]),
					w[1] * (ndotl * L.col[1] * tc[1] + pw * L.col[1]), w[2] * (ndotl * L.col[2] * tc[2] + pw * L.col[2]), scene);
		}
		return;
	}
	/* shade_phong (src/shader.cc:83-247) */
	bool entering;
	V3 normal;
	if(dot(rd, sp.normal) > 0.0f) { normal = -sp.normal; entering = false; }
	else { normal = sp.normal; entering = true; }
	float ray_mag = len(rd);
	V3 incident = rd / ray_mag;
	MatVals mv;
	mat_values(S, mat, sp.tex, mv);
	const float *kd = mv.kd, *ks = mv.ks;
	if(iter == DIFFUSE_ITER) {
		/* final-gather ray: radiance_est(...) * kd */
		em.gather(sp.pos, normal, S.njobs > 0 ? 2 * job_of(S, pixel) + 1 : 1, aslot, w[0] * kd[0], w[1] * kd[1], w[2] * kd[2]);
		return;
	}
	float energy = ray.energy;
	const IorStack &st = ray.st;
	sray_rng rng;
	sray_rng_init(&rng, S.seed, SRAY_DOM_PIXEL | ((uint32_t)path << 4), (uint32_t)pixel, (uint32_t)sample);
	float refl_fact = mv.refl, trans_fact = mv.refr, mat_ior = mv.ior;
	float ior = st.calc_ior(entering, mat_ior);
	/* a normal map replaces the (flipped) normal after the index of
	 * refraction is known (src/shader.cc:133-139) */
	if(mat.have_normal) normal = bump_normal(S, mat, sp);
	/* ambient: (env_ambient * kd) * kd */
	acc_add(acc, aslot, w[0] * (env_amb.x * kd[0] * kd[0]), w[1] * (env_amb.y * kd[1] * kd[1]),
			w[2] * (env_amb.z * kd[2] * kd[2]));
	V3 vref = reflection(incident, normal);
	for(int li = l0; li < l0 + nl; li++) {
		const DevLight &L = S.lights[li];
		int ns = L.type != 0 ? S.shadow_samples : 1;
		float scale = ns > 1 ? 1.0f / (float)ns : 1.0f;
		for(int si = 0; si < ns; si++) {
			V3 lpos = light_point(S, li, time, &rng);
			V3 ldir = lpos - sp.pos;
			float ldist = len(ldir);
			V3 sdir = ldir;
			ldir = ldir / ldist;
			float ndotl = maxf_ref(dot(normal, ldir), 0.0f);
			float rdotl = maxf_ref(dot(vref, ldir), 0.0f);
			float pw = powf(rdotl, mv.shin);
			float c[3];
			for(int k = 0; k < 3; k++) {
				float lc = L.col[k] * 1.0f;
				c[k] = ((ndotl * lc) * scale) * kd[k] + ((pw * lc) * scale) * ks[k];
			}
			if(c[0] != 0.0f || c[1] != 0.0f || c[2] != 0.0f)
				em.shadow(shadow_origin(sp, sdir), sdir, time, aslot, w[0] * c[0], w[1] * c[1], w[2] * c[2], scene);
		}
	}
	/* final gather: diffuse rays end at their next hit (src/shader.cc:154-187) */
	if(S.gi_on) {
		int ds = S.diffuse_samples < MAX_DS ? S.diffuse_samples : MAX_DS;
		bool cached = false;
		int rec = -1;
		if(S.nrc.mode) {
			/* the radiance cache: a query in a region the network serves;
			 * a training or validation record where the frame's hash
			 * selects the vertex (its diffuse rays carry weight g alone, so
			 * that the record's slot receives the plain estimate / (w kd)) */
			const DNrc &N = S.nrc;
			float x[9];
			nrc_inputs(N, sp.pos, normal, incident, x);
			cached = N.mode == 2 || !N.fallback[nrc_region(x)];
			uint32_t hsel = hash32(N.key ^ hash32((uint32_t)pixel * 0x9e3779b9u ^ hash32((uint32_t)path + 0x632be5abu * (uint32_t)sample)));
			if(hsel < N.p_train) {
				int j = warp_alloc(N.tcount, 1);
				if(j < N.tcap) rec = j;
			} else if(hsel - N.p_train < N.p_val) {
				int j = warp_alloc(N.tcount + 1, 1);
				if(j < N.vcap) rec = N.tcap + j;
			}
			if(rec >= 0) store_x(N.tx + (size_t)rec * 9, x);
			if(cached) {
				int j = warp_alloc(N.qcount, 1);
				if(j < N.qcap) {
					store_x(N.qx + (size_t)j * 9, x);
					N.qw[j] = make_float4(w[0] * kd[0], w[1] * kd[1], w[2] * kd[2], __int_as_float(aslot));
				} else {
					cached = false;   /* query queue full: the plain gather */
				}
			}
			warp_count(N.counters, true);
			warp_count(N.counters + 1, cached);
		}
		/* rays of the image's plain gather: ds, or the fallback count in a
		 * fallback region; of a record: ds for training, NRC_VAL_RAYS (at
		 * least) for validation, whose targets judge the network */
		int nimg = cached ? 0 : (S.nrc.mode && S.nrc.fb_samples > 0 ? S.nrc.fb_samples : ds);
		int nrec = rec < 0 ? 0 : (rec < S.nrc.tcap ? ds : (ds > NRC_VAL_RAYS ? ds : NRC_VAL_RAYS));
		for(int k = 0; k < nimg; k++) {
			V3 dir = sphrand(&rng, 1.0f);
			float ndotl;
			if((ndotl = dot(dir, normal)) < 0.0f) dir = -dir;
			float diff_energy = ndotl * energy;
			if(diff_energy > S.min_energy) {
				float g = nimg > 1 ? ndotl / (float)nimg : ndotl;
				em.child(make_child(ray, sp.pos, dir * ray_mag, diff_energy, DIFFUSE_ITER, path * 4 + 2, k, st, w[0] * kd[0] * g,
						w[1] * kd[1] * g, w[2] * kd[2] * g));
			}
		}
		if(nrec) {
			/* a record's directions come from a stream keyed by the frame, so
			 * that a vertex trained again sees a new estimate */
			sray_rng rr;
			sray_rng_init(&rr, S.seed ^ ((uint64_t)S.nrc.key << 32), SRAY_DOM_NRC | ((uint32_t)path << 4), (uint32_t)pixel,
					(uint32_t)sample);
			for(int k = 0; k < nrec; k++) {
				V3 dir = sphrand(&rr, 1.0f);
				float ndotl;
				if((ndotl = dot(dir, normal)) < 0.0f) dir = -dir;
				float diff_energy = ndotl * energy;
				if(diff_energy > S.min_energy) {
					float g = nrec > 1 ? ndotl / (float)nrec : ndotl;
					RayRec c = make_child(ray, sp.pos, dir * ray_mag, diff_energy, DIFFUSE_ITER, path * 4 + 2, k, st, g, g, g);
					c.aslot = S.nrc.t0 + rec;
					em.child(c);
				}
			}
		}
	}
	float ray_dot_n = dot(-rd / ray_mag, normal);
	float sf0 = trans_fact > 0.0f ? (ior - 1.0f) / (ior + 1.0f) : 1.0f;
	float fres = fresnel(sf0 * sf0, ray_dot_n);
	float refl_energy = refl_fact * energy;
	if(refl_energy > S.min_energy && iter > 0) {
		float g = refl_fact * fres;
		em.child(make_child(ray, sp.pos, reflection(rd, normal), refl_energy, iter - 1, path * 4, 0, st, w[0] * ks[0] * g,
				w[1] * ks[1] * g, w[2] * ks[2] * g));
	}
	float trans_energy = trans_fact * energy;
	if(trans_energy > S.min_energy && iter > 0) {
		IorStack cs = st;
		if(entering) cs.enter(mat_ior);
		else cs.leave();
		V3 td = refraction(rd / ray_mag, normal, ior) * ray_mag;
		if(dot(td, normal) > 0.0f) {
			if(entering) cs.leave();
			else cs.enter(mat_ior);
		}
		float g = trans_fact * (1.0f - fres);
		em.child(make_child(ray, sp.pos, td, trans_energy, iter - 1, path * 4 + 1, 0, cs, w[0] * ks[0] * g, w[1] * ks[1] * g,
				w[2] * ks[2] * g));
	}
	if(S.caust_on) em.gather(sp.pos, normal, S.njobs > 0 ? 2 * job_of(S, pixel) : 0, aslot, w[0], w[1], w[2]);
}

/* the wavefront emitter: everything goes to the next pass's queues */
struct QueueEmitter {
	ShadeOut *out;
	int *overflow;
	__device__ void shadow(V3 o, V3 d, int time, int slot, float r, float g, float b, int scene)
	{
		push_shadow(*out, o, d, time, slot, r, g, b, overflow, scene);
	}
	__device__ void gather(V3 pos, V3 n, int kind, int slot, float r, float g, float b) { push_gather(*out, pos, n, kind, slot, r, g, b, overflow); }
	__device__ void child(const RayRec &c)
	{
		int slot = warp_alloc(out->qo.count, 1);
		if(slot >= out->qo.cap) { *overflow = 1; return; }
		store_ray(out->qo, slot, c);
	}
};

__global__ void __launch_bounds__(128) k_shade(DScene S, RayQueue qi, const int4 *hits, ShadeOut out, float4 *acc, int depth,
		DevCounters *ctr)
{
	int n = *qi.count;
	int overflow = 0;
	QueueEmitter em;
	em.out = &out;
	em.overflow = &overflow;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		RayRec r;
		load_ray(qi, i, r);
		int4 hv = hits[i];
		Hit h;
		h.t = __int_as_float(hv.x);
		h.obj = hv.y;
		h.prim = hv.z;
		h.tie = hv.w;
		shade_one(S, r, h, depth, acc, em);
	}
	if(overflow) atomicOr(&ctr->overflow, 1);
}

/* The tail of the shading tree (below tune.render_tail rays in flight).
 * Past the first bounces few rays are left,
 * on long and branching paths (chains through glass and mirrors), and a
 * pass costs as much as its slowest ray.  k_render_pool runs the rest of the
 * tree in one launch over a shared pool of rays: the queue's rays occupy
 * the first slots, every thread claims the next slot, waits until a ray is
 * there, traces and shades it and appends its children to the pool.  Light
 * samples are traced on the spot (their contribution added when the
 * hierarchies confirm the segment unoccluded, queued for the octree pass
 * when they cannot decide); photon gathers are queued for the warp-per-query
 * kernel; a ray whose closest hit the octrees must decide goes to the
 * pending queue unshaded.
 *
 * Pool control words: [0] next slot to claim, [1] slots filled or reserved,
 * [2] rays in flight (in the pool and not yet shaded), [3] error.  A slot's
 * ready flag is set after its record is written (with a fence); records are
 * read through L2 (__ldcg), never from a possibly stale L1 line.  A thread
 * whose slot is beyond every reservation leaves once no ray is in flight
 * (no more can come); every wait is bounded and sets the error word when
 * it runs out. */
#define POOL_SPIN_LIMIT (1 << 22) /* polls of a slot before the pool gives up (about 0.5 s; a
                                     sray_gpu_set_faults test lowers it) */
#define POOL_HEADROOM 64          /* pool slots per ray it starts with */
#define POOL_SHADOW (-0x7ffffff0)   /* iter of a pool item that is a light sample's shadow ray */

__device__ __forceinline__ void load_ray_l2(const RayQueue &q, int i, RayRec &r)
{
	float4 o4 = __ldcg(q.o + i), d4 = __ldcg(q.d + i), w4 = __ldcg(q.w + i), st4 = __ldcg(q.stk + i);
	int4 meta = __ldcg(q.meta + i);
	int2 ext = __ldcg(q.ext + i);
	r.o = mk(o4.x, o4.y, o4.z);
	r.d = mk(d4.x, d4.y, d4.z);
	r.energy = o4.w;
	r.st.ior = d4.w;
	r.st.stk[0] = st4.x; r.st.stk[1] = st4.y; r.st.stk[2] = st4.z; r.st.stk[3] = st4.w;
	r.st.sp = ext.y;
	r.w[0] = w4.x; r.w[1] = w4.y; r.w[2] = w4.z;
	r.pixel = __float_as_int(w4.w);
	r.aslot = meta.x;
	r.iter = meta.y;
	r.path = meta.z;
	r.time = meta.w;
	r.sample = ext.x & 0xffff;
	r.dsub = ext.x >> 16;
}

struct PoolEmitter {
	const DScene *S;
	ShadeOut *out;
	RayQueue *pool;
	int *ready, *ctl;
	float4 *acc;
	int *overflow;
	unsigned long long shadows;
	/* a light sample becomes a pool item of its own (iter = POOL_SHADOW, its
	 * scene in path), traced by whichever thread claims it */
	__device__ void shadow(V3 o, V3 d, int time, int slot, float r, float g, float b, int scene)
	{
		RayRec c;
		c.o = o;
		c.d = d;
		c.energy = 0.0f;
		c.st.ior = 1.0f;
		c.st.stk[0] = c.st.stk[1] = c.st.stk[2] = c.st.stk[3] = 0.0f;
		c.st.sp = 0;
		c.w[0] = r; c.w[1] = g; c.w[2] = b;
		c.pixel = 0;
		c.aslot = slot;
		c.iter = POOL_SHADOW;
		c.path = scene;
		c.time = time;
		c.sample = 0;
		c.dsub = 0;
		child(c);
	}
	__device__ void gather(V3 pos, V3 n, int kind, int slot, float r, float g, float b) { push_gather(*out, pos, n, kind, slot, r, g, b, overflow); }
	__device__ void child(const RayRec &c)
	{
		atomicAdd(&ctl[2], 1);                 /* in flight before it can be claimed */
		int j = atomicAdd(&ctl[1], 1);
		if(j >= pool->cap) {
			*overflow = 1;
			atomicSub(&ctl[2], 1);
			return;
		}
		store_ray(*pool, j, c);
		__threadfence();
		atomicExch(&ready[j], 1);
	}
};

__global__ void __launch_bounds__(128) k_render_pool(DScene S, RayQueue pool, int *ready, int *ctl, ShadeOut out, float4 *acc,
		DevCounters *ctr, int spin_limit)
{
	int overflow = 0;
	PoolEmitter em;
	em.S = &S;
	em.out = &out;
	em.pool = &pool;
	em.ready = ready;
	em.ctl = ctl;
	em.acc = acc;
	em.overflow = &overflow;
	em.shadows = 0;
	unsigned long long traced = 0;
	volatile int *vready = ready;
	volatile int *vctl = ctl;
	for(;;) {
		int i = atomicAdd(&ctl[0], 1);
		if(i >= pool.cap) break;
		bool have = false;
		for(int spin = 0; spin < spin_limit; spin++) {
			if(vready[i]) { have = true; break; }
			if(vctl[2] == 0) {
				__threadfence();
				if(vctl[1] <= i) break;   /* nothing in flight and no reservation reaches slot i */
			}
			__nanosleep(128);
		}
		if(!have) {
			if(!(vctl[2] == 0 && vctl[1] <= i)) atomicOr(&ctl[3], 1);   /* gave up waiting */
			break;
		}
		__threadfence();
		RayRec r;
		load_ray_l2(pool, i, r);
		Hit h;
		if(r.iter == POOL_SHADOW) {
			int res = trace_two_level<false, true>(S, r.o, r.d, r.time, h, nullptr, &overflow, r.path);
			if(res == 0) acc_add(acc, r.aslot, r.w[0], r.w[1], r.w[2]);
			else if(res == 2) push_shadow(out, r.o, r.d, r.time, r.aslot, r.w[0], r.w[1], r.w[2], &overflow, r.path);
			if(res != 2) em.shadows++;
		} else if(!trace_two_level<false, false>(S, r.o, r.d, r.time, h, nullptr, &overflow, pixel_scene(S, r.pixel))) {
			int slot = atomicAdd(out.qo.count, 1);
			if(slot >= out.qo.cap) overflow = 1;
			else store_ray(out.qo, slot, r);
		} else {
			traced++;
			shade_one(S, r, h, 1, acc, em);
		}
		atomicSub(&ctl[2], 1);   /* after its children were counted in flight */
	}
	if(overflow) atomicOr(&ctr->overflow, 1);
	if(traced) atomicAdd(&ctr->rays[1], traced);
	if(em.shadows) atomicAdd(&ctr->rays[2], em.shadows);
}

/* shadow rays: the reference tests visibility with cast_ray(shadow_ray)
 * (src/shader.cc:266), a hit anywhere on the segment [eps, 1] blocks */
/* shadow rays; HYB and fb as for k_trace */
template <bool HYB, bool SORT = true, bool COUNT = false>
__global__ void __launch_bounds__(SRAY_TRACE_THREADS, 8) k_shadow(DScene S, const ShadowReq *sq, const int *sq_count, float4 *acc,
		DevCounters *ctr, int *fb)
{
	int n = HYB ? *sq_count : fb[0];
	int overflow = 0;
	TraceCounters tc = {0, 0};
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int ri = HYB ? i : fb[1 + i];
		ShadowReq r = sq[ri];
		int time = __float_as_int(r.a.w), pixel = __float_as_int(r.b.w);
		int res;
		int scene = S.nscenes > 1 ? __float_as_int(r.w.w) : -1;
		if(HYB) {
			Hit h;
			res = trace_two_level<COUNT, true, SORT>(S, mk(r.a.x, r.a.y, r.a.z), mk(r.b.x, r.b.y, r.b.z), time, h, &tc, &overflow,
					scene);
		} else {
			res = trace_any_octree_impl(S, mk(r.a.x, r.a.y, r.a.z), mk(r.b.x, r.b.y, r.b.z), time, &overflow, scene) ? 1 : 0;
		}
		if(HYB && res == 2) {
			fb[1 + atomicAdd(fb, 1)] = ri;
			continue;
		}
		if(res == 0) acc_add(acc, pixel, r.w.x, r.w.y, r.w.z);
	}
	if(overflow) atomicOr(&ctr->overflow, 1);
	if(COUNT) {
		atomicAdd(&ctr->snodes, tc.nodes);
		atomicAdd(&ctr->sprims, tc.prims);
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) {
		if(HYB) atomicAdd(&ctr->rays[2], (unsigned long long)n);
		else if(n > 0) atomicAdd(&ctr->bvh_fallbacks, (unsigned long long)n);
	}
}

/* light samples with one warp per segment (as k_trace_warp), for passes of
 * few samples */
__global__ void __launch_bounds__(128) k_shadow_warp(DScene S, const ShadowReq *sq, const int *sq_count, float4 *acc, DevCounters *ctr,
		int *fb)
{
	__shared__ int s_ref[4][WR_CAP];
	__shared__ int s_obj[4][WR_CAP];
	__shared__ float s_te[4][WR_CAP];
	int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	int n = *sq_count;
	for(int ri = blockIdx.x * 4 + w; ri < n; ri += gridDim.x * 4) {
		ShadowReq r = sq[ri];
		float best;
		int bobj, bprim;
		int res = warp_trace<true>(S, mk(r.a.x, r.a.y, r.a.z), mk(r.b.x, r.b.y, r.b.z), __float_as_int(r.a.w), s_ref[w], s_obj[w], s_te[w],
				best, bobj, bprim, S.nscenes > 1 ? __float_as_int(r.w.w) : -1);
		if(lane == 0) {
			if(res == 2) fb[1 + atomicAdd(fb, 1)] = ri;
			else if(res == 0) acc_add(acc, __float_as_int(r.b.w), r.w.x, r.w.y, r.w.z);
		}
		__syncwarp();
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr->rays[2], (unsigned long long)n);
}

/* ---------------------------------------------------------------- */
/* photon-map gathers, one warp per query                             */
/* ---------------------------------------------------------------- */
#define GATHER_WARPS 8
#define KEY_CAP 512

__device__ __forceinline__ float warp_sum(float v)
{
	for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}
__device__ __forceinline__ int warp_sumi(int v)
{
	for(int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}
__device__ __forceinline__ unsigned warp_maxu(unsigned v)
{
	for(int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

struct GatherCells {
	int lo[3], hi[3];
};

/* The grid cells a query must visit: every cell that can hold a photon
 * within the radius.  Photons were binned with floor((p - org) / cell) in
 * double; the window is computed in float and widened by a slack that covers
 * the float rounding (three operations, each within 2^-24 of its operands),
 * so it always contains the exact window and at most grows by one cell where
 * the query's edge lies within the slack of a cell boundary. */
__device__ __forceinline__ void gather_cells(const DPhotonMap &M, V3 q, GatherCells &gc)
{
	float qa[3] = {q.x, q.y, q.z};
	for(int a = 0; a < 3; a++) {
		float base = qa[a] - M.org[a];
		float lo = (base - M.range_f) / M.cell, hi = (base + M.range_f) / M.cell;
		float slack = 1e-3f + (fabsf(base) + M.range_f) / M.cell * 1e-6f;
		lo = floorf(lo - slack);
		hi = floorf(hi + slack);
		float top = (float)(M.dims[a] - 1);
		gc.lo[a] = lo >= 0.0f ? (lo > top ? M.dims[a] - 1 : (int)lo) : 0;
		gc.hi[a] = hi >= 0.0f ? (hi > top ? M.dims[a] - 1 : (int)hi) : 0;
	}
}

/* squared distance in double between a float photon position and the
 * float query point (kd_nearest_range3f semantics) */
__device__ __forceinline__ double dist2(const float4 &p, V3 q)
{
	double dx = (double)p.x - (double)q.x, dy = (double)p.y - (double)q.y, dz = (double)p.z - (double)q.z;
	return dx * dx + dy * dy + dz * dz;
}

/* exact range decisions without double arithmetic (range_ff.h) */
__device__ __forceinline__ bool range_ff(const DPhotonMap &M, float4 p, V3 q, bool &in, unsigned &key)
{
	int inr = 0;
	uint32_t k = 0;
	if(!sray_range_ff(p.x, p.y, p.z, q.x, q.y, q.z, M.r2_hi, M.r2_lo, &inr, &k)) return false;
	in = inr != 0;
	key = k;
	return true;
}

/* The cells overlapping the query cube (at most 2x2x2: cells are twice the
 * gather radius) are looked up by the first lanes; the warp then strides
 * over the concatenation of their photon runs, so every lane tests one
 * photon per step whatever the cell occupancy.  f(in, photon, key) is called
 * by every lane at every step (so it may use warp collectives); `in` tells
 * whether the lane holds a photon within range, key the bits of its squared
 * distance rounded to float. */
template <class F>
__device__ __forceinline__ void for_range(const DPhotonMap &M, const GatherCells &gc, V3 q, int lane, F f)
{
	int nx = gc.hi[0] - gc.lo[0] + 1, ny = gc.hi[1] - gc.lo[1] + 1, nz = gc.hi[2] - gc.lo[2] + 1;
	int ncell = nx * ny * nz;
	float thr = M.screen;
	for(int c0 = 0; c0 < ncell; c0 += 32) {
		int c = c0 + lane;
		unsigned first = 0, cnt = 0;
		if(c < ncell) {
			int cx = c % nx, t = c / nx;
			int cy = t % ny, cz = t / ny;
			uint2 cr = __ldg(reinterpret_cast<const uint2 *>(M.cells) +
					((size_t)(gc.lo[2] + cz) * M.dims[1] + (gc.lo[1] + cy)) * M.dims[0] + (gc.lo[0] + cx));
			first = cr.x;
			cnt = cr.y - cr.x;
		}
		/* inclusive prefix of the run lengths over the lanes */
		unsigned incl = cnt;
		for(int o = 1; o < 32; o <<= 1) {
			unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
			if(lane >= o) incl += v;
		}
		unsigned total = __shfl_sync(0xffffffffu, incl, 31);
		unsigned excl = incl - cnt;
		int nl = min(32, ncell - c0);
		for(unsigned base = 0; base < total; base += 32) {
			unsigned v = base + lane;
			/* run holding virtual index v: the last lane whose exclusive prefix <= v
			 * (all lanes take part in the shuffles, so the loop stays uniform) */
			int owner = 0;
			for(int k = 1; k < nl; k++) {
				unsigned ek = __shfl_sync(0xffffffffu, excl, k);
				if(ek <= v) owner = k;
			}
			unsigned fo = __shfl_sync(0xffffffffu, first, owner);
			unsigned eo = __shfl_sync(0xffffffffu, excl, owner);
			bool in = false;
			unsigned j = 0, key = 0;
			if(v < total) {
				j = fo + (v - eo);
				float4 p = __ldg(reinterpret_cast<const float4 *>(M.ph + j));
				float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
				float d2f = dx * dx + dy * dy + dz * dz;
				/* screen: d2f is within 6 ulp of the exact sum of squares, so
				 * above range^2 (1 + 2^-20) the photon is out of range */
				if(!(d2f > thr) && !range_ff(M, p, q, in, key)) {
					double d2 = dist2(p, q);
					in = d2 <= M.range * M.range;
					key = __float_as_uint((float)d2);
				}
			}
			f(in, (int)j, key);
		}
	}
}

__device__ __forceinline__ void photon_term(const DevPhoton *ph, int j, int kind, V3 n, float max_cos, float *sum)
{
	const float4 *pp = reinterpret_cast<const float4 *>(ph + j);
	float4 p = __ldg(pp), d = __ldg(pp + 1), nn = __ldg(pp + 2);
	V3 dir = mk(d.x, d.y, d.z);
	if(kind == 0) {
		if(dot(dir, n) < 0.0f) { sum[0] += p.w; sum[1] += d.w; sum[2] += nn.w; }
	} else {
		float ndotl = dot(-dir, n);
		if(ndotl > 0.0f && dot(mk(nn.x, nn.y, nn.z), n) > max_cos) {
			sum[0] += p.w * ndotl; sum[1] += d.w * ndotl; sum[2] += nn.w * ndotl;
		}
	}
}

/* estimate of one query by one full warp; returns the rgb estimate in all
 * lanes.  keys/idx: KEY_CAP entries of this warp's shared memory, holding the
 * candidates (photons within range) in the order the warp visits them. */
struct GatherWork {
	unsigned long long tested, cand, select, spill;
};

/* More candidates than the on-chip list holds (a dense caustic inside the
 * radius cap): a histogram of the candidates' keys in GATHER_BINS
 * logarithmic bins (8 per octave of the squared distance, the top bin
 * holding the largest key) finds the bin of the k-th nearest; a second pass
 * lists the candidates of that bin and below, which hold the k nearest, in
 * keys/idx.  Returns the number listed, or -1 if they do not fit either. */
#define GATHER_BINS 256
__device__ __noinline__ int gather_narrow(const DPhotonMap &M, const GatherCells &gc, V3 pos, int lane, unsigned &maxkey,
		unsigned *keys, int *idx, int *hist)
{
	for(int i = lane; i < GATHER_BINS; i += 32) hist[i] = 0;
	__syncwarp();
	int base = (int)(maxkey >> 20) - (GATHER_BINS - 1);
	for_range(M, gc, pos, lane, [&](bool in, int, unsigned key) {
		if(in) {
			int b = (int)(key >> 20) - base;
			atomicAdd(&hist[b > 0 ? b : 0], 1);
		}
	});
	__syncwarp();
	/* the bin of the k-th smallest key: each lane sums 8 bins, a warp scan
	 * finds the lane, the lane its bin */
	int loc[GATHER_BINS / 32];
	int ls = 0;
	#pragma unroll
	for(int i = 0; i < GATHER_BINS / 32; i++) {
		loc[i] = hist[lane * (GATHER_BINS / 32) + i];
		ls += loc[i];
	}
	int incl = ls;
	for(int o = 1; o < 32; o <<= 1) {
		int v = __shfl_up_sync(0xffffffffu, incl, o);
		if(lane >= o) incl += v;
	}
	int excl = incl - ls;
	unsigned m = __ballot_sync(0xffffffffu, excl < M.k && M.k <= incl);
	int owner = m ? __ffs(m) - 1 : 31;
	int bstar = GATHER_BINS - 1;
	if(lane == owner) {
		int c = excl;
		#pragma unroll
		for(int i = 0; i < GATHER_BINS / 32; i++) {
			if(c + loc[i] >= M.k) { bstar = lane * (GATHER_BINS / 32) + i; break; }
			c += loc[i];
		}
	}
	bstar = __shfl_sync(0xffffffffu, bstar, owner);
	int nlist = 0;
	unsigned lt_mask = (1u << lane) - 1u;
	unsigned kmax = 0;
	for_range(M, gc, pos, lane, [&](bool in, int j, unsigned key) {
		bool take = in && (int)(key >> 20) - base <= bstar;
		unsigned b = __ballot_sync(0xffffffffu, take);
		int slot = nlist + __popc(b & lt_mask);
		if(take) {
			kmax = key > kmax ? key : kmax;
			if(slot < KEY_CAP) { keys[slot] = key; idx[slot] = j; }
		}
		nlist += __popc(b);
	});
	__syncwarp();
	if(nlist > KEY_CAP) return -1;
	/* the largest listed key: the k-th nearest when exactly k are listed */
	maxkey = warp_maxu(kmax);
	return nlist;
}

__device__ void gather_one(const DScene &S, int kind, V3 pos, V3 n, unsigned *keys, int *idx, int *hist, float out[3],
		GatherWork &gw)
{
	/* in a batch the request's kind is the index of its job's map */
	const DPhotonMap &M = S.maps ? S.maps[kind] : (kind == 0 ? S.caust : S.gi);
	kind &= 1;
	int lane = threadIdx.x & 31;
	unsigned lt_mask = (1u << lane) - 1u;
	out[0] = out[1] = out[2] = 0.0f;
	if(M.n == 0) return;
	GatherCells gc;
	gather_cells(M, pos, gc);
	float sum[3] = {0.0f, 0.0f, 0.0f};
	int cnt = 0;
	float inv_area = M.inv_area;
	if(M.k <= 0) {
		for_range(M, gc, pos, lane, [&](bool in, int j, unsigned) {
			if(in) {
				cnt++;
				photon_term(M.ph, j, kind, n, S.max_cos, sum);
			}
		});
		cnt = warp_sumi(cnt);
	} else {
		/* k nearest within the radius cap: the k-th smallest float-rounded
		 * squared distance, found by a bitwise radix search over the
		 * candidates' keys */
		unsigned maxkey = 0;
		int ncand = 0;
		for_range(M, gc, pos, lane, [&](bool in, int j, unsigned key) {
			gw.tested += 32;
			unsigned b = __ballot_sync(0xffffffffu, in);
			int slot = ncand + __popc(b & lt_mask);
			if(in) {
				maxkey = key > maxkey ? key : maxkey;
				if(slot < KEY_CAP) { keys[slot] = key; idx[slot] = j; }
			}
			ncand += __popc(b);
		});
		__syncwarp();
		maxkey = warp_maxu(maxkey);
		bool cached = ncand <= KEY_CAP;
		gw.cand += (unsigned)ncand;
		gw.spill += cached ? 0u : 1u;
		gw.select += ncand > M.k ? 1u : 0u;
		if(!cached && ncand > M.k) {
			int nl = gather_narrow(M, gc, pos, lane, maxkey, keys, idx, hist);
			if(nl >= 0) {
				ncand = nl;
				cached = true;
			}
		}
		unsigned kth = maxkey;
		if(ncand > M.k) {
			unsigned prefix = 0;
			int remaining = M.k;
			for(int bit = 31; bit >= 0; bit--) {
				unsigned hmask = bit == 31 ? 0x80000000u : (~((1u << bit) - 1u));
				int c0 = 0;
				if(cached) {
					for(int c = lane; c < ncand; c += 32) if((keys[c] & hmask) == prefix) c0++;
				} else {
					for_range(M, gc, pos, lane, [&](bool in, int, unsigned key) {
						if(in && (key & hmask) == prefix) c0++;
					});
				}
				c0 = warp_sumi(c0);
				if(c0 < remaining) {
					remaining -= c0;
					prefix |= (1u << bit);
				}
			}
			kth = prefix;
		}
		if(cached) {
			for(int c = lane; c < ncand; c += 32) {
				if(keys[c] <= kth) {
					cnt++;
					photon_term(M.ph, idx[c], kind, n, S.max_cos, sum);
				}
			}
		} else {
			for_range(M, gc, pos, lane, [&](bool in, int j, unsigned key) {
				if(in && key <= kth) {
					cnt++;
					photon_term(M.ph, j, kind, n, S.max_cos, sum);
				}
			});
		}
		cnt = warp_sumi(cnt);
		/* 1 / (pi d2_k) in float (the reference rounds the double quotient;
		 * the two differ by at most two units in the last place) */
		inv_area = 1.0f / (3.14159265358979323846f * __uint_as_float(kth));
	}
	sum[0] = warp_sum(sum[0]);
	sum[1] = warp_sum(sum[1]);
	sum[2] = warp_sum(sum[2]);
	if(kind == 0 && cnt < 8) return;
	if(kind == 1 && cnt <= 0) return;
	out[0] = sum[0] * inv_area;
	out[1] = sum[1] * inv_area;
	out[2] = sum[2] * inv_area;
}

__global__ void __launch_bounds__(GATHER_WARPS * 32, 4) k_gather(DScene S, const GatherReq *gq, const int *gq_count,
		float4 *acc, DevCounters *ctr)
{
	__shared__ unsigned keys[GATHER_WARPS][KEY_CAP];
	__shared__ int idx[GATHER_WARPS][KEY_CAP];
	__shared__ int hist[GATHER_WARPS][GATHER_BINS];
	int n = *gq_count;
	int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
	int gw = blockIdx.x * GATHER_WARPS + w, nw = gridDim.x * GATHER_WARPS;
	GatherWork work = {0, 0, 0, 0};
	for(int r = gw; r < n; r += nw) {
		GatherReq g = gq[r];
		int kind = __float_as_int(g.a.w);
		int pixel = __float_as_int(g.b.w);
		float est[3];
		gather_one(S, kind, mk(g.a.x, g.a.y, g.a.z), mk(g.b.x, g.b.y, g.b.z), keys[w], idx[w], hist[w], est, work);
		if(lane == 0) acc_add(acc, pixel, g.w.x * est[0], g.w.y * est[1], g.w.z * est[2]);
		__syncwarp();
	}
	if(lane == 0 && work.tested) {
		atomicAdd(&ctr->g_tested, work.tested);
		atomicAdd(&ctr->g_cand, work.cand);
		atomicAdd(&ctr->g_select, work.select);
		atomicAdd(&ctr->g_spill, work.spill);
	}
	if(blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&ctr->rays[3], (unsigned long long)n);
}

/* gathers at caller-given points: requests packed from the caller's arrays,
 * one warp per request, the estimate written to out[3 * i] */
__global__ void k_pack_gather(int kind, int n, const float *pos, const float *norm, GatherReq *gq)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		GatherReq g;
		g.a = make_float4(pos[i * 3], pos[i * 3 + 1], pos[i * 3 + 2], __int_as_float(kind));
		g.b = make_float4(norm[i * 3], norm[i * 3 + 1], norm[i * 3 + 2], __int_as_float(i));
		g.w = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
		gq[i] = g;
	}
}

__global__ void __launch_bounds__(GATHER_WARPS * 32, 3) k_gather_points(DScene S, const GatherReq *gq, int n, float *out)
{
	__shared__ unsigned keys[GATHER_WARPS][KEY_CAP];
	__shared__ int idx[GATHER_WARPS][KEY_CAP];
	__shared__ int hist[GATHER_WARPS][GATHER_BINS];
	int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
	int gw = blockIdx.x * GATHER_WARPS + w, nw = gridDim.x * GATHER_WARPS;
	GatherWork work = {0, 0, 0, 0};
	for(int r = gw; r < n; r += nw) {
		GatherReq g = gq[r];
		int kind = __float_as_int(g.a.w);
		int pt = __float_as_int(g.b.w);
		float est[3];
		gather_one(S, kind, mk(g.a.x, g.a.y, g.a.z), mk(g.b.x, g.b.y, g.b.z), keys[w], idx[w], hist[w], est, work);
		if(lane == 0) {
			out[pt * 3] = est[0];
			out[pt * 3 + 1] = est[1];
			out[pt * 3 + 2] = est[2];
		}
		__syncwarp();
	}
}

/* end of a sample batch: the reference's stop rule applied sample by sample
 * (src/render.cc:199-244): after sample i (counting from 1), if i >= min
 * and i > 1 and the sample variance is below max_var the pixel stops; later
 * samples of the batch were speculative and are discarded */
__global__ void k_finish(const int *active, int tw, int th, const int *n_active_p, int s0, int width, const float4 *acc, float4 *hist,
		float4 *sums, int max_samples, int min_samples, float max_var, int *next, int *next_count, float4 *fb, int *spp)
{
	int n = *n_active_p;
	for(int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
		int p = slot_pixel(active, a, tw, th);
		float4 sum = s0 == 0 ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : sums[p];
		bool done = false;
		int i1 = s0;
		for(int j = 0; j < width && !done; j++) {
			int sample = s0 + j;
			float4 s = acc[(size_t)a * width + j];
			sum.x = sum.x + s.x;
			sum.y = sum.y + s.y;
			sum.z = sum.z + s.z;
			sum.w = sum.w + s.w;
			i1 = sample + 1;
			if(max_samples > 1) hist[(size_t)p * max_samples + sample] = s;
			if(i1 >= max_samples) { done = true; break; }
			if(i1 >= min_samples && i1 > 1) {
				float rcp = (float)(1.0 / (double)i1);
				float4 mean = make_float4(sum.x * rcp, sum.y * rcp, sum.z * rcp, sum.w * rcp);
				float sq = 0.0f;
				for(int k = 0; k < i1; k++) {
					float4 h = hist[(size_t)p * max_samples + k];
					float dx = mean.x - h.x, dy = mean.y - h.y, dz = mean.z - h.z, dw = mean.w - h.w;
					sq = sq + (dx * dx + dy * dy + dz * dz + dw * dw);
				}
				float v = sq * rcp;
				if(v < max_var) done = true;
			}
		}
		if(done) {
			double r = 1.0 / (double)i1;
			fb[p] = make_float4((float)((double)sum.x * r), (float)((double)sum.y * r), (float)((double)sum.z * r),
					(float)((double)sum.w * r));
			if(spp) spp[p] = i1;
		} else {
			sums[p] = sum;
			int slot = warp_alloc(next_count, 1);
			next[slot] = p;
		}
	}
}

/* closest hits of caller-supplied world rays (sray_gpu_cast_rays) */
__global__ void __launch_bounds__(SRAY_TRACE_THREADS) k_cast(DScene S, int n, const float *orig, const float *dir, const int *time, int *obj, int *prim, float *t,
		unsigned char *tie, DevCounters *ctr)
{
	int overflow = 0;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		Hit h;
		trace_closest<false>(S, mk(orig[i * 3], orig[i * 3 + 1], orig[i * 3 + 2]), mk(dir[i * 3], dir[i * 3 + 1], dir[i * 3 + 2]),
				time ? time[i] : S.t0, h, nullptr, &overflow);
		obj[i] = h.obj;
		prim[i] = h.obj >= 0 ? h.prim : -1;
		t[i] = h.obj >= 0 ? h.t : 0.0f;
		tie[i] = (unsigned char)h.tie;
	}
	if(overflow) atomicOr(&ctr->overflow, 1);
}

__global__ void k_primary_hits(DScene S, RayQueue q, const int4 *hits, int *obj, int *prim, float *t, unsigned char *tie)
{
	int n = *q.count;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int4 h = hits[i];
		int p = __float_as_int(q.w[i].w);
		obj[p] = h.y;
		prim[p] = h.y >= 0 ? h.z : -1;
		t[p] = h.y >= 0 ? __int_as_float(h.x) : 0.0f;
		tie[p] = (unsigned char)h.w;
	}
}

/* ================================================================ */
/* host side                                                          */
/* ================================================================ */
/* photons of one wavefront of a batch's photon maps (jobs beyond it go to the next) */
#define PW_MAX_PHOTONS ((int64_t)1 << 26)

/* at most this many gather requests wait for the photon maps across waves */
#define DEFER_MAX_REQS ((int64_t)1 << 28)

static int grid_for(int n, int block)
{
	int sms = 152;
	int g = (n + block - 1) / block;
	int cap = sms * 16;
	if(g > cap) g = cap;
	return g < 1 ? 1 : g;
}

int Renderer::kind_of(const char *name)
{
	for(size_t i = 0; i < ktimes.size(); i++) if(ktimes[i].name == name) return (int)i;
	KTime k;
	k.name = name;
	ktimes.push_back(k);
	return (int)ktimes.size() - 1;
}

void Renderer::host_time(const char *name, double t0)
{
	if(!(prof_flags & 1)) return;
	double ms = host_now_ms() - t0;
	std::lock_guard<std::mutex> lk(prof_mu);
	KTime &k = ktimes[kind_of(name)];
	k.ms += ms;
	k.launches++;
}

void Renderer::prof_begin(const char *name, int *kind_cache, cudaStream_t s, Pending *p)
{
	std::lock_guard<std::mutex> lk(prof_mu);
	int k = *kind_cache;
	if(k < 0 || k >= (int)ktimes.size() || ktimes[k].name != name) *kind_cache = k = kind_of(name);
	p->kind = k;
	p->a = p->b = nullptr;
	launch_count++;
	if(!(prof_flags & 1)) return;
	for(int i = 0; i < 2; i++) {
		cudaEvent_t e;
		if(!event_pool.empty()) { e = event_pool.back(); event_pool.pop_back(); }
		else cudaEventCreate(&e);
		(i ? p->b : p->a) = e;
	}
	cudaEventRecord(p->a, s);
}

void Renderer::prof_end(Pending *p, cudaStream_t s)
{
	if(!p->b) return;
	cudaEventRecord(p->b, s);
	std::lock_guard<std::mutex> lk(prof_mu);
	pending.push_back(*p);
}

/* called after a stream synchronisation: every pending pair has completed */
void Renderer::prof_collect()
{
	std::lock_guard<std::mutex> lk(prof_mu);
	/* pairs on a stream that has not got there yet (the photon stream runs
	 * beside the render stream) stay pending */
	size_t keep = 0;
	for(size_t i = 0; i < pending.size(); i++) {
		if(cudaEventQuery(pending[i].b) != cudaSuccess) {
			pending[keep++] = pending[i];
			continue;
		}
		float ms = 0.0f;
		if(cudaEventElapsedTime(&ms, pending[i].a, pending[i].b) == cudaSuccess) {
			ktimes[pending[i].kind].ms += ms;
			ktimes[pending[i].kind].launches++;
		}
		event_pool.push_back(pending[i].a);
		event_pool.push_back(pending[i].b);
	}
	pending.resize(keep);
}

#define CK(call, where) do { cudaError_t e_ = (call); if(e_ != cudaSuccess) return cuda_fail(e_, where); } while(0)

/* a material's device form; Material::get_value returns float
 * (src/material.cc:193-196) */
static DevMat dev_material(const Material &m)
{
	DevMat d;
	memset(&d, 0, sizeof d);
	for(int k = 0; k < 4; k++) { d.kd[k] = (float)m.kd[k]; d.ks[k] = (float)m.ks[k]; }
	d.shin = (float)m.shin;
	d.refl = (float)m.refl;
	d.refr = (float)m.refr;
	d.ior = (float)m.ior;
	d.phong = m.phong;
	d.have_normal = m.have_normal ? 1 : 0;
	const double scal[TA_COUNT] = {m.kd[0], m.ks[0], m.shin, m.refl, m.refr, m.ior, m.nrm_scale};
	for(int k = 0; k < 8; k++) d.tex[k] = -1;
	for(int k = 0; k < TA_COUNT; k++) {
		d.tex[k] = m.tex[k];
		d.scol[k] = (float)scal[k];
		if(m.tex[k] >= 0) d.textured = 1;
	}
	return d;
}

void Renderer::fill_scene_desc()
{
	DScene &D = S;
	D.snodes = snodes.as<DevNode>();
	D.sslots = sslots.as<int>();
	D.has_scene = built && !sc.oct.nodes.empty() && !sc.objs.empty();
	D.sroot = scene_root;
	D.troot = 0;
	D.nscenes = (int)scene_refs.size();
	D.scenes = scene_refs.empty() ? nullptr : dscenes.as<DevSceneRef>();
	D.mnodes = mnodes.as<DevNode>();
	D.mtris = mtris.as<DevTri>();
	D.mprim = mprim.as<int>();
	D.bnodes = bnodes.as<DevBvh4>();
	D.btris = btris.as<DevTri>();
	D.bprim = bprim.as<int>();
	D.bhome = bhome.as<int>();
	D.tnodes = has_tlas ? tnodes.as<DevBvh4>() : nullptr;
	D.ohome = ohome.as<int>();
	D.bvh_fallbacks = ctr.p ? &ctr.as<DevCounters>()->bvh_fallbacks : nullptr;
	D.objs = objs.as<DevObj>();
	D.nobj = (int)sc.objs.size();
	D.xf = xf.as<float>();
	D.tlo = tlo;
	D.nt = nt;
	D.tri_pos = tri_pos.as<float>();
	D.tri_attr = tri_attr.as<float>();
	D.mats = mats.as<DevMat>();
	D.defmat = dev_material(sc.defmat);
	D.defmat.phong = 0;
	D.texs = texs.as<DevTex>();
	D.texels = texels.as<float4>();
	D.lights = lights.as<DevLight>();
	D.nlights = (int)sc.lights.size();
	D.light_pos = light_pos.as<float>();
	D.cam_m = cam_m.as<float>();
	D.cam_f = (float)(1.0 / tan(0.5 * sc.cam.vfov));
	D.cam_xsz = (float)(sc.cam.aspect * 2.0);
	D.cam_ysz = 2.0f;
	D.cam_maxd = (float)sc.cam.max_dist;
	for(int k = 0; k < 4; k++) { D.env_col[k] = (float)sc.env_col[k]; D.env_amb[k] = (float)sc.env_amb[k]; }
	D.eps = (float)1e-6;
	D.xsmall = (float)1e-8;
	D.min_energy = opt.min_energy;
	D.iter = opt.iter;
	D.diffuse_samples = opt.diffuse_samples;
	D.shadow_samples = opt.shadow_samples;
	D.gi_on = opt.gi_photons != 0;
	D.caust_on = opt.caust_photons != 0;
	D.width = opt.width;
	D.height = opt.height;
	D.mblur = opt.mblur;
	D.shutter = sc.cam.shutter;
	D.t0 = t0;
	D.t1 = t1;
	D.seed = opt.seed;
	D.photon_energy = opt.photon_energy;
	D.max_cos = (float)cos(M_PI / 2.5);
	D.caust = caust.map;
	D.gi = gi.map;
}


/* The frame's transform table on the device: thread (i, t) evaluates the
 * keyframe tracks of object i at time tlo + t and writes its record
 * (forward, inverse, inverse transpose; XF_STRIDE floats), or, past the
 * objects, light i's position (4 floats).  The evaluation is anim_eval.h's,
 * the same code the host runs for object bounds and projection maps. */
__global__ void k_xforms(const DevAnim *anims, const int *kt, const double *kv, int nobj, int nlights, int tlo, int nt, float *xf,
		float *lpos)
{
	long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
	if(i >= (long long)(nobj + nlights) * nt) return;
	int ai = (int)(i / nt), t = (int)(i % nt);
	const DevAnim &a = anims[ai];
	KeyView kp = {kt + a.toff[0], kv + a.voff[0], a.def, a.n[0], 3, a.interp[0], a.extrap[0]};
	double p[3];
	key_eval(kp, tlo + t, p);
	if(ai >= nobj) {
		float *d = lpos + ((size_t)(ai - nobj) * nt + t) * 4;
		d[0] = (float)p[0];
		d[1] = (float)p[1];
		d[2] = (float)p[2];
		d[3] = 0.0f;
		return;
	}
	KeyView kr = {kt + a.toff[1], kv + a.voff[1], a.def + 3, a.n[1], 4, a.interp[1], a.extrap[1]};
	KeyView ks = {kt + a.toff[2], kv + a.voff[2], a.def + 7, a.n[2], 3, a.interp[2], a.extrap[2]};
	double q[4], sc[3], m[4][4];
	key_eval(kr, tlo + t, q);
	key_eval(ks, tlo + t, sc);
	node_matrix(p, q, sc, a.pivot, m);
	pack_transform(m, xf + ((size_t)ai * nt + t) * XF_STRIDE, XF_STRIDE);
}

/* a node's tracks appended to the key tables */
template <class T> static void add_track(const Track<T> &tr, int k, DevAnim &a, std::vector<int> &kt, std::vector<double> &kv)
{
	a.toff[k] = (int)kt.size();
	a.voff[k] = (int)kv.size();
	a.n[k] = (int)tr.time.size();
	a.interp[k] = tr.interp;
	a.extrap[k] = tr.extrap;
	kt.insert(kt.end(), tr.time.begin(), tr.time.end());
	const double *v = reinterpret_cast<const double *>(tr.val.data());
	kv.insert(kv.end(), v, v + tr.val.size() * (sizeof(T) / sizeof(double)));
}
static DevAnim dev_anim(const XForm &xf, bool position_only, std::vector<int> &kt, std::vector<double> &kv)
{
	DevAnim a;
	memset(&a, 0, sizeof a);
	add_track(xf.pos, 0, a, kt, kv);
	if(!position_only) {
		add_track(xf.rot, 1, a, kt, kv);
		add_track(xf.scale, 2, a, kt, kv);
	}
	a.pivot[0] = xf.pivot.x; a.pivot[1] = xf.pivot.y; a.pivot[2] = xf.pivot.z;
	a.def[0] = xf.pos.def.x; a.def[1] = xf.pos.def.y; a.def[2] = xf.pos.def.z;
	a.def[3] = xf.rot.def.s; a.def[4] = xf.rot.def.x; a.def[5] = xf.rot.def.y; a.def[6] = xf.rot.def.z;
	a.def[7] = xf.scale.def.x; a.def[8] = xf.scale.def.y; a.def[9] = xf.scale.def.z;
	return a;
}

int Renderer::upload_scene(cudaStream_t s)
{
	std::vector<DevNode> nodes;
	std::vector<int> slots;
	std::vector<DevTri> tris;
	std::vector<int> prim;
	std::vector<float> tp, ta;
	std::vector<DevBvh4> bn;
	std::vector<DevTri> bt;
	std::vector<int> bp, bh;
	int tri_cursor = 0;
	/* the triangle record the intersection test reads */
	auto record = [](const float *P) {
		DevTri t;
		/* unnormalised face normal cross(v1 - v0, v2 - v0), float ops as the test computes it */
		float e1[3] = {P[3] - P[0], P[4] - P[1], P[5] - P[2]};
		float e2[3] = {P[6] - P[0], P[7] - P[1], P[8] - P[2]};
		float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
		for(int c = 0; c < 3; c++) { t.a[c] = P[c]; t.b[c] = P[3 + c]; t.c[c] = P[6 + c]; }
		t.a[3] = n[0]; t.b[3] = n[1]; t.c[3] = n[2];
		return t;
	};
	for(size_t u = 0; u < sc.meshes.size(); u++) {
		Mesh &m = sc.meshes[u];
		m.tri_base = tri_cursor;
		size_t s0 = slots.size();
		std::vector<int> index_of;
		flatten_octree(m.oct, nodes, slots, &index_of);
		m.node_base = m.oct.nodes.empty() ? -1 : (int)(nodes.size() - m.oct.nodes.size());
		size_t nf = m.pos.size() / 9;
		for(size_t k = s0; k < slots.size(); k++) {
			int f = slots[k];
			tris.push_back(record(&m.pos[(size_t)f * 9]));
			prim.push_back(f);
		}
		/* the hierarchy, with references made absolute */
		m.bvh_base = -1;
		if(!m.bvh.nodes.empty() && bt.size() + m.bvh.order.size() < ((size_t)1 << 27)) {
			int noff = (int)bn.size(), toff = (int)bt.size();
			m.bvh_base = noff;
			std::vector<DevBvh4> n4;
			m.bvh.collapse4(n4);
			for(const DevBvh4 &src : n4) {
				DevBvh4 d = src;
				for(int k = 0; k < 4; k++) {
					int ref = d.child[k];
					if(ref == BVH_NONE) continue;
					if(ref >= 0) d.child[k] = ref + noff;
					else {
						unsigned v = ~(unsigned)ref;
						unsigned start = (v >> 4) + (unsigned)toff, cnt = v & 15u;
						d.child[k] = (int)~((start << 4) | cnt);
					}
				}
				bn.push_back(d);
			}
			std::vector<int> home;
			octree_homes(m.oct, m.posd, index_of, home);
			for(int f : m.bvh.order) {
				bt.push_back(record(&m.pos[(size_t)f * 9]));
				bp.push_back(f);
				bh.push_back(home[f]);
			}
		}
		std::vector<DevBvhNode>().swap(m.bvh.nodes);
		std::vector<int>().swap(m.bvh.order);
		/* leaf slot indices become positions in the triangle-record array */
		tp.insert(tp.end(), m.pos.begin(), m.pos.end());
		ta.insert(ta.end(), m.attr.begin(), m.attr.end());
		tri_cursor += (int)nf;
		std::vector<BuildOctree::Node>().swap(m.oct.nodes);   /* build form no longer needed */
	}
	/* the leaf 'first' fields index `slots`, which coincide with the record array */
	std::vector<DevObj> dobj(sc.objs.size());
	for(size_t i = 0; i < sc.objs.size(); i++) {
		const Object &o = sc.objs[i];
		DevObj &d = dobj[i];
		memset(&d, 0, sizeof d);
		d.type = o.type;
		d.mat = o.mat;
		d.rad = (float)o.rad;
		d.start = (float)o.start;
		d.end = (float)o.end;
		d.mesh_root = -1;
		d.bvh_root = -1;
		if(o.type == OBJ_MESH) {
			const Mesh &m = sc.meshes[o.mesh];
			d.mesh_root = (m.pos.empty() || m.node_base < 0) ? -1 : m.node_base;
			d.tri_base = m.tri_base;
			d.bvh_root = d.mesh_root >= 0 ? m.bvh_base : -1;
		}
	}
	std::vector<DevMat> dm(sc.mats.size());
	for(size_t i = 0; i < sc.mats.size(); i++) dm[i] = dev_material(sc.mats[i]);
	/* the texel table: every texture's RGBA texels, back to back */
	std::vector<DevTex> dtex(sc.texs.size());
	std::vector<float> texel;
	for(size_t i = 0; i < sc.texs.size(); i++) {
		dtex[i].off = (long long)(texel.size() / 4);
		dtex[i].xsz = sc.texs[i].xsz;
		dtex[i].ysz = sc.texs[i].ysz;
		texel.insert(texel.end(), sc.texs[i].pix.begin(), sc.texs[i].pix.end());
	}
	CK(texs.upload(dtex, s), "upload textures");
	CK(texels.upload(texel, s), "upload texels");
	std::vector<DevLight> dl(sc.lights.size());
	for(size_t i = 0; i < sc.lights.size(); i++) {
		const Light &l = sc.lights[i];
		DevLight &d = dl[i];
		memset(&d, 0, sizeof d);
		d.type = l.type;
		d.radius = l.radius;
		for(int k = 0; k < 4; k++) d.col[k] = (float)l.col[k];
		d.dim[0] = (float)l.dim.x; d.dim[1] = (float)l.dim.y; d.dim[2] = (float)l.dim.z;
		double m0[4][4];
		l.xf.matrix(0, m0);
		for(int r = 0; r < 3; r++) for(int c = 0; c < 4; c++) d.box_m[r * 4 + c] = (float)m0[r][c];
	}
	CK(mnodes.upload(nodes, s), "upload mesh nodes");
	CK(mtris.upload(tris, s), "upload mesh triangles");
	CK(mprim.upload(prim, s), "upload mesh primitive ids");
	CK(tri_pos.upload(tp, s), "upload triangle positions");
	CK(tri_attr.upload(ta, s), "upload triangle attributes");
	CK(objs.upload(dobj, s), "upload objects");
	CK(mats.upload(dm, s), "upload materials");
	CK(lights.upload(dl, s), "upload lights");
	/* keyframe tracks: the objects', then the lights' positions */
	std::vector<DevAnim> da;
	std::vector<int> kt;
	std::vector<double> kv;
	for(const Object &o : sc.objs) da.push_back(dev_anim(o.xf, false, kt, kv));
	for(const Light &l : sc.lights) da.push_back(dev_anim(l.xf, true, kt, kv));
	CK(anims.upload(da, s), "upload keyframe tracks");
	CK(key_t.upload(kt, s), "upload key times");
	CK(key_v.upload(kv, s), "upload key values");
	CK(bnodes.upload(bn, s), "upload mesh hierarchies");
	CK(btris.upload(bt, s), "upload hierarchy triangles");
	CK(bprim.upload(bp, s), "upload hierarchy face ids");
	CK(bhome.upload(bh, s), "upload hierarchy home nodes");
	CK(ctr.ensure(sizeof(DevCounters)), "counters");
	CK(cudaStreamSynchronize(s), "upload scene");
	return 0;
}

/* the object hierarchy over items [0, n): each boxed by the union of the
 * octree leaves that list it (so that it is entered whenever the octree
 * would test it), one item per leaf; node references offset by tbase, an
 * item i becomes object ~(obj0 + i) */
static void object_hierarchy(const BuildOctree &oct, size_t no, int obj0, int tbase, std::vector<DevBvh4> &tn)
{
	std::vector<Box> ub(no);
	for(size_t i = 0; i < no; i++) for(int k = 0; k < 3; k++) { ub[i].mn[k] = DBL_MAX; ub[i].mx[k] = -DBL_MAX; }
	for(const BuildOctree::Node &n : oct.nodes) {
		if(n.child >= 0) continue;
		for(int it : n.items) {
			for(int k = 0; k < 3; k++) {
				ub[it].mn[k] = std::min(ub[it].mn[k], n.box.mn[k]);
				ub[it].mx[k] = std::max(ub[it].mx[k], n.box.mx[k]);
			}
		}
	}
	std::vector<float> mn(no * 3), mx(no * 3);
	for(size_t i = 0; i < no; i++) {
		for(int k = 0; k < 3; k++) {
			float lo = (float)ub[i].mn[k], hi = (float)ub[i].mx[k];
			if((double)lo > ub[i].mn[k]) lo = nextafterf(lo, -INFINITY);
			if((double)hi < ub[i].mx[k]) hi = nextafterf(hi, INFINITY);
			if(!(ub[i].mn[k] <= ub[i].mx[k])) { lo = FLT_MAX; hi = -FLT_MAX; }   /* listed in no leaf */
			mn[i * 3 + k] = lo;
			mx[i * 3 + k] = hi;
		}
	}
	MeshBvh tl;
	tl.build_items(mn.data(), mx.data(), no, 1);
	std::vector<DevBvh4> part;
	tl.collapse4(part);
	for(DevBvh4 &d : part) {
		for(int k = 0; k < 4; k++) {
			int ref = d.child[k];
			if(ref == BVH_NONE) continue;
			if(ref >= 0) {
				d.child[k] = ref + tbase;
				continue;
			}
			unsigned v = ~(unsigned)ref;
			d.child[k] = ~(obj0 + tl.order[v >> 4]);   /* leaf: the object itself */
		}
	}
	tn.insert(tn.end(), part.begin(), part.end());
}

/* A scene set's frame: every scene's octree over its own objects (the
 * reference's Scene::build_tree, src/scene.cc:353-390, per scene) and object
 * hierarchy, side by side in one node table; their roots, lights and
 * environments in the scene descriptors; the cameras' matrices per scene */
int Renderer::build_frame_set(long bt0, long bt1, cudaStream_t s)
{
	t0 = (int)bt0;
	t1 = (int)bt1;
	sc.bound_objects(t0, t1, opt);   /* the object bounds cache and the union's box; the scenes' octrees follow */
	int ns = (int)sc.ranges.size();
	std::vector<DevNode> nodes;
	std::vector<int> slots, ohome_h(sc.objs.size(), 0);
	std::vector<DevBvh4> tn;
	scene_refs.assign(ns, DevSceneRef());
	int shutter = 0;
	for(int k = 0; k < ns; k++) {
		const SceneRange &rg = sc.ranges[k];
		DevSceneRef &R = scene_refs[k];
		memset(&R, 0, sizeof R);
		R.sroot = R.troot = -1;
		R.light0 = rg.light0;
		R.nlights = rg.nlight;
		for(int c = 0; c < 4; c++) { R.env_col[c] = (float)rg.env_col[c]; R.env_amb[c] = (float)rg.env_amb[c]; }
		if(rg.cam.shutter > shutter) shutter = rg.cam.shutter;
		if(rg.nobj == 0) continue;
		std::vector<Box> boxes(rg.nobj);
		for(int i = 0; i < rg.nobj; i++) {
			Box a = sc.object_bounds(rg.obj0 + i, t0), b = t1 == t0 ? a : sc.object_bounds(rg.obj0 + i, t1);
			for(int c = 0; c < 3; c++) {
				boxes[i].mn[c] = a.mn[c] < b.mn[c] ? a.mn[c] : b.mn[c];
				boxes[i].mx[c] = a.mx[c] > b.mx[c] ? a.mx[c] : b.mx[c];
			}
		}
		BuildOctree oct;
		oct.build(boxes, opt.scnoct_max_depth, opt.scnoct_max_items);
		size_t slot0 = slots.size();
		std::vector<int> index_of, hm;
		flatten_octree(oct, nodes, slots, &index_of);
		for(size_t q = slot0; q < slots.size(); q++) slots[q] += rg.obj0;
		R.sroot = (int)(nodes.size() - oct.nodes.size());
		R.troot = (int)tn.size();
		object_hierarchy(oct, (size_t)rg.nobj, rg.obj0, R.troot, tn);
		octree_homes_boxes(oct, boxes, index_of, hm);
		for(int i = 0; i < rg.nobj; i++) ohome_h[rg.obj0 + i] = hm[i];
	}
	scene_root = ns > 0 ? scene_refs[0].sroot : 0;
	tlo = t0 - shutter - 2;
	int thi = t1 + shutter + 2;
	nt = thi - tlo + 1;
	size_t nobj = sc.objs.size(), nlt = sc.lights.size();
	CK(xf.ensure(nobj * nt * XF_STRIDE * sizeof(float) + 16), "transform table");
	CK(light_pos.ensure(nlt * nt * 4 * sizeof(float) + 16), "light positions");
	size_t nthr = (nobj + nlt) * (size_t)nt;
	if(nthr) {
		LAUNCH(*this, "xforms", s, k_xforms<<<(unsigned)((nthr + 127) / 128), 128, 0, s>>>(anims.as<DevAnim>(), key_t.as<int>(),
				key_v.as<double>(), (int)nobj, (int)nlt, tlo, nt, xf.as<float>(), light_pos.as<float>()));
		CK(cudaGetLastError(), "transform table");
	}
	std::vector<float> cm((size_t)ns * nt * 12);
	for(int k = 0; k < ns; k++) {
		for(int t = 0; t < nt; t++) {
			double m[4][4];
			sc.ranges[k].cam.matrix(tlo + t, m);
			for(int r = 0; r < 3; r++) for(int c = 0; c < 4; c++) cm[((size_t)k * nt + t) * 12 + r * 4 + c] = (float)m[r][c];
		}
	}
	CK(snodes.upload(nodes, s), "upload scene nodes");
	CK(sslots.upload(slots, s), "upload scene slots");
	CK(tnodes.upload(tn, s), "upload object hierarchies");
	CK(ohome.upload(ohome_h, s), "upload object home nodes");
	CK(dscenes.upload(scene_refs, s), "upload scene descriptors");
	has_tlas = !tn.empty();
	CK(cam_m.upload(cm, s), "upload cameras");
	h2d += (int64_t)(nodes.size() * sizeof(DevNode) + slots.size() * 4 + cm.size() * 4 + tn.size() * sizeof(DevBvh4));
	CK(cudaStreamSynchronize(s), "build frame");
	built = true;
	photons_ready = false;
	caust.map.n = 0;
	gi.map.n = 0;
	fill_scene_desc();
	return 0;
}

int Renderer::build_frame(long bt0, long bt1, cudaStream_t s)
{
	if(!loaded) return fail(SRAY_ESTATE, "no scene loaded");
	if(sc.ranges.size() > 1) {
		if(!in_batch) return fail(SRAY_ESTATE, "a scene set renders through sray_gpu_render_batch");
		return build_frame_set(bt0, bt1, s);
	}
	scene_refs.clear();
	t0 = (int)bt0;
	t1 = (int)bt1;
	sc.build_tree(t0, t1, opt);
	std::vector<DevNode> nodes;
	std::vector<int> slots;
	std::vector<int> index_of;
	flatten_octree(sc.oct, nodes, slots, &index_of);
	scene_root = sc.oct.nodes.empty() ? 0 : (int)(nodes.size() - sc.oct.nodes.size());
	/* the object hierarchy: each object boxed by the union of the octree
	 * leaves that list it (so that it is entered whenever the octree would
	 * test the object), one object per leaf */
	std::vector<DevBvh4> tn;
	std::vector<int> ohome_h;
	if(!sc.oct.nodes.empty() && !sc.objs.empty()) {
		size_t no = sc.objs.size();
		std::vector<Box> ub(no);
		for(size_t i = 0; i < no; i++) for(int k = 0; k < 3; k++) { ub[i].mn[k] = DBL_MAX; ub[i].mx[k] = -DBL_MAX; }
		for(const BuildOctree::Node &n : sc.oct.nodes) {
			if(n.child >= 0) continue;
			for(int it : n.items) {
				for(int k = 0; k < 3; k++) {
					ub[it].mn[k] = std::min(ub[it].mn[k], n.box.mn[k]);
					ub[it].mx[k] = std::max(ub[it].mx[k], n.box.mx[k]);
				}
			}
		}
		std::vector<float> mn(no * 3), mx(no * 3);
		for(size_t i = 0; i < no; i++) {
			for(int k = 0; k < 3; k++) {
				float lo = (float)ub[i].mn[k], hi = (float)ub[i].mx[k];
				if((double)lo > ub[i].mn[k]) lo = nextafterf(lo, -INFINITY);
				if((double)hi < ub[i].mx[k]) hi = nextafterf(hi, INFINITY);
				if(!(ub[i].mn[k] <= ub[i].mx[k])) { lo = FLT_MAX; hi = -FLT_MAX; }   /* listed in no leaf */
				mn[i * 3 + k] = lo;
				mx[i * 3 + k] = hi;
			}
		}
		MeshBvh tl;
		tl.build_items(mn.data(), mx.data(), no, 1);
		tl.collapse4(tn);
		for(DevBvh4 &d : tn) {
			for(int k = 0; k < 4; k++) {
				int ref = d.child[k];
				if(ref == BVH_NONE || ref >= 0) continue;
				unsigned v = ~(unsigned)ref;
				d.child[k] = ~tl.order[v >> 4];   /* leaf: the object itself */
			}
		}
		octree_homes_boxes(sc.oct, sc.oct_boxes, index_of, ohome_h);
	}
	int shutter = sc.cam.shutter;
	tlo = t0 - shutter - 2;
	int thi = t1 + shutter + 2;
	nt = thi - tlo + 1;
	/* object transforms and light positions for every time the frame can
	 * touch, evaluated from the keyframe tracks on the device */
	size_t nobj = sc.objs.size(), nlt = sc.lights.size();
	CK(xf.ensure(nobj * nt * XF_STRIDE * sizeof(float) + 16), "transform table");
	CK(light_pos.ensure(nlt * nt * 4 * sizeof(float) + 16), "light positions");
	size_t nthr = (nobj + nlt) * (size_t)nt;
	if(nthr) {
		LAUNCH(*this, "xforms", s, k_xforms<<<(unsigned)((nthr + 127) / 128), 128, 0, s>>>(anims.as<DevAnim>(), key_t.as<int>(),
				key_v.as<double>(), (int)nobj, (int)nlt, tlo, nt, xf.as<float>(), light_pos.as<float>()));
		CK(cudaGetLastError(), "transform table");
	}
	std::vector<float> cm((size_t)nt * 12);
	for(int t = 0; t < nt; t++) {
		double m[4][4];
		sc.cam.matrix(tlo + t, m);
		for(int r = 0; r < 3; r++) for(int c = 0; c < 4; c++) cm[(size_t)t * 12 + r * 4 + c] = (float)m[r][c];
	}
	CK(snodes.upload(nodes, s), "upload scene nodes");
	CK(sslots.upload(slots, s), "upload scene slots");
	CK(tnodes.upload(tn, s), "upload object hierarchy");
	CK(ohome.upload(ohome_h, s), "upload object home nodes");
	has_tlas = !tn.empty();
	CK(cam_m.upload(cm, s), "upload camera");
	h2d += (int64_t)(nodes.size() * sizeof(DevNode) + slots.size() * 4 + cm.size() * 4);
	CK(cudaStreamSynchronize(s), "build frame");
	built = true;
	photons_ready = false;
	caust.map.n = 0;
	gi.map.n = 0;
	fill_scene_desc();
	return 0;
}

/* a light's projection maps as the photon kernels read them: 2048 cell bits
 * of the map, then of the caustic map; their coverages */
static void pack_projmaps(const ProjMap &pm, const ProjMap &spm, uint32_t *bits, float *cov)
{
	for(int k = 0; k < 128; k++) bits[k] = 0u;
	for(int k = 0; k < 2048; k++) {
		if(pm.cells[k]) bits[k >> 5] |= 1u << (k & 31);
		if(spm.cells[k]) bits[64 + (k >> 5)] |= 1u << (k & 31);
	}
	cov[0] = (float)pm.get_coverage();
	cov[1] = (float)spm.get_coverage();
}

/* every job's projection maps of a batch, on all host cores: each light of a
 * job is one task (its own random stream, its own output) */
void Renderer::batch_projmaps(std::vector<std::vector<uint32_t>> &bits, std::vector<std::vector<float>> &cov)
{
	size_t n = batch_t0.size();
	bits.assign(n, std::vector<uint32_t>());
	cov.assign(n, std::vector<float>());
	struct Task { size_t job; int light; };
	std::vector<Task> tasks;
	std::vector<int> l0(n, 0), o0(n, 0), no(n, (int)sc.objs.size());
	for(size_t j = 0; j < n; j++) {
		int nl = (int)sc.lights.size();
		if(!scene_refs.empty()) {
			const SceneRange &rg = sc.ranges[batch_scene[j]];
			l0[j] = rg.light0;
			nl = rg.nlight;
			o0[j] = rg.obj0;
			no[j] = rg.nobj;
		}
		bits[j].assign((size_t)nl * 128, 0u);
		cov[j].assign((size_t)nl * 2, 0.0f);
		for(int k = 0; k < nl; k++) tasks.push_back(Task{j, k});
	}
	std::atomic<size_t> next{0};
	auto work = [&]() {
		for(size_t i; (i = next.fetch_add(1)) < tasks.size();) {
			const Task &T = tasks[i];
			ProjMap pm, spm;
			sc.light_projmaps((size_t)(l0[T.job] + T.light), (int)batch_t0[T.job], (int)batch_t1[T.job], opt.seed, T.light, o0[T.job],
					no[T.job], pm, spm);
			pack_projmaps(pm, spm, &bits[T.job][(size_t)T.light * 128], &cov[T.job][(size_t)T.light * 2]);
		}
	};
	unsigned hw = std::thread::hardware_concurrency();
	size_t nth = std::min<size_t>(tasks.size(), hw ? hw : 4);
	std::vector<std::thread> th;
	for(size_t t = 1; t < nth; t++) th.push_back(std::thread(work));
	work();
	for(auto &t : th) t.join();
}

/* projection maps and both photon maps on stream s, with the scene view
 * `base` (the projection-map tables are set in a copy of it); the map
 * descriptors land in caust.map / gi.map, which fill_scene_desc() copies
 * into S */
int Renderer::shoot_maps(const DScene &base, cudaStream_t s, int *nc, int *ng)
{
	caust.map.n = 0;
	gi.map.n = 0;
	*nc = *ng = 0;
	int nl = (int)sc.lights.size();
	if(!(opt.caust_photons || opt.gi_photons) || nl == 0) return 0;
	/* projection maps (src/render.cc:87-103) over the photons' interval */
	double tp = host_now_ms();
	sc.build_projmaps(base.t0, base.t1, opt.seed);
	std::vector<uint32_t> bits((size_t)nl * 128, 0u);
	std::vector<float> cov((size_t)nl * 2, 0.0f);
	for(size_t i = 0; i < (size_t)nl; i++) pack_projmaps(sc.lights[i].pm, sc.lights[i].spm, &bits[i * 128], &cov[i * 2]);
	host_time("host.projmaps", tp);
	return photon_shoot_maps(*this, base, bits, cov, s, nc, ng);
}

int Renderer::photon_job(DScene base)
{
	int c = 0, g = 0;
	if(batch_t0.empty()) return shoot_maps(base, ps, &c, &g);
	/* a batch: every job's two maps over its own interval, with its own
	 * photon counts and its scene's lights, in one photon wavefront; then
	 * each map from its segment, and their table */
	size_t n = batch_t0.size();
	std::vector<DPhotonMap> hm(2 * n);
	std::vector<std::vector<uint32_t>> jbits;
	std::vector<std::vector<float>> jcov;
	double tp = host_now_ms();
	batch_projmaps(jbits, jcov);
	host_time("host.projmaps", tp);
	std::vector<PhotonJobSpec> spec(n);
	std::vector<int> o0(n, 0), no(n, (int)sc.objs.size());
	for(size_t j = 0; j < n; j++) {
		PhotonJobSpec &J = spec[j];
		J.light0 = 0;
		J.nlights = (int)sc.lights.size();
		if(!scene_refs.empty()) {
			const SceneRange &rg = sc.ranges[batch_scene[j]];
			J.light0 = rg.light0;
			J.nlights = rg.nlight;
			J.scene = batch_scene[j];
			o0[j] = rg.obj0;
			no[j] = rg.nobj;
		}
		J.num[0] = batch_caust[j] > 0 ? batch_caust[j] : opt.caust_photons;
		J.num[1] = batch_gi[j] > 0 ? batch_gi[j] : opt.gi_photons;
		J.t0 = (int)batch_t0[j];
		J.t1 = (int)batch_t1[j];
		J.bits = &jbits[j];
		J.cov = &jcov[j];
	}
	/* the grids of the jobs' own frames: boxes and range radii over their
	 * own intervals (the batch's tree spans every job's interval) */
	std::vector<Box> boxes(n);
	std::vector<double> gdist(n);
	for(size_t j = 0; j < n; j++) {
		boxes[j] = sc.box_at(batch_t0[j], batch_t1[j], o0[j], no[j]);
		gdist[j] = sc.gather_dist_at(batch_t0[j], batch_t1[j], opt, o0[j], no[j]);
	}
	/* jobs in groups of at most PW_MAX_PHOTONS photons per wavefront, so that
	 * the wavefront's memory follows the group and not the batch; when the
	 * batch takes more than one group, each map is copied out to its job's
	 * own buffers before the next group reuses the wavefront's */
	const int64_t gcap = g_faults.photon_group.load() > 0 ? (int64_t)g_faults.photon_group.load() : PW_MAX_PHOTONS;
	std::vector<size_t> group0(1, 0);
	int64_t acc = 0;
	for(size_t j = 0; j < n; j++) {
		int64_t pj = (int64_t)spec[j].num[0] + spec[j].num[1] + 2 * spec[j].nlights;
		if(j > group0.back() && acc + pj > gcap) {
			group0.push_back(j);
			acc = 0;
		}
		acc += pj;
	}
	group0.push_back(n);
	bool copy_out = group0.size() > 2;
	for(size_t gi0 = 0; gi0 + 1 < group0.size(); gi0++) {
		size_t a = group0[gi0], b = group0[gi0 + 1];
		std::vector<PhotonJobSpec> gspec(spec.begin() + a, spec.begin() + b);
		std::vector<Box> gbox(boxes.begin() + a, boxes.begin() + b);
		std::vector<double> gd(gdist.begin() + a, gdist.begin() + b);
		std::vector<PJobOut> out;
		int r = photon_trace_jobs(*this, base, gspec, out, ps);
		if(r) return r;
		std::vector<DPhotonMap> gm;
		r = photon_finalize_jobs(*this, out, gbox, gd, gm, ps);
		if(r == 0) {
			for(size_t k = 0; k < gm.size(); k++) {
				DPhotonMap &M = gm[k];
				if(copy_out && M.n > 0) {
					/* out of the wavefront's buffers into the job's own */
					PhotonBufs &P = (k & 1) ? job_maps[a + k / 2].gi : job_maps[a + k / 2].caust;
					size_t ncells = (size_t)M.dims[0] * M.dims[1] * M.dims[2];
					CK(P.ph.ensure((size_t)M.n * sizeof(DevPhoton)), "job photon map");
					CK(P.cells.ensure(ncells * sizeof(uint2)), "job cell table");
					CK(cudaMemcpyAsync(P.ph.p, M.ph, (size_t)M.n * sizeof(DevPhoton), cudaMemcpyDeviceToDevice, ps), "job photon map");
					CK(cudaMemcpyAsync(P.cells.p, M.cells, ncells * sizeof(uint2), cudaMemcpyDeviceToDevice, ps), "job cell table");
					M.ph = P.ph.as<DevPhoton>();
					M.cells = P.cells.as<uint2>();
				}
				hm[2 * a + k] = M;
			}
			continue;
		}
		if(r != 1) return r;
		/* cell tables too large to hold together: map by map, into the
		 * jobs' own buffers */
		const DevPhoton *ph = pw_out.as<DevPhoton>();
		const int *valid = pw_valid.as<int>();
		for(size_t j = a; j < b; j++) {
			map_gather_dist = gdist[j];
			map_box = boxes[j];
			map_has_box = true;
			std::swap(caust, job_maps[j].caust);
			std::swap(gi, job_maps[j].gi);
			const PJobOut &o = out[j - a];
			int t0 = o.total[0];
			r = photon_finalize(*this, 0, valid + o.base, ph + o.base, t0, ps, &c);
			if(!r) r = photon_finalize(*this, 1, valid + o.base + t0, ph + o.base + t0, o.total[1], ps, &g);
			std::swap(caust, job_maps[j].caust);
			std::swap(gi, job_maps[j].gi);
			map_gather_dist = -1.0;
			map_has_box = false;
			if(r) return r;
			hm[2 * j] = job_maps[j].caust.map;
			hm[2 * j + 1] = job_maps[j].gi.map;
		}
	}
	caust.map.n = 0;
	gi.map.n = 0;
	CK(dmaps.upload(hm, ps), "job photon maps");
	CK(cudaStreamSynchronize(ps), "job photon maps");
	h2d += (int64_t)(hm.size() * sizeof(DPhotonMap));
	return 0;
}

/* start tracing the photon maps on the photon stream from a host thread of
 * their own; the render stream s has uploaded the frame's tables (build_frame
 * synchronised it) */
int Renderer::start_photon_job(cudaStream_t s)
{
	(void)s;
	int r = photon_stream();
	if(r) return r;
	if(photon_thread.joinable()) return fail(SRAY_ESTATE, "photon maps already being traced");
	photon_rc = 0;
	DScene base = S;
	photon_finished.store(false);
	photon_thread = std::thread([this, base]() {
		double t0 = host_now_ms();
		photon_rc = photon_job(base);
		host_time("host.photon_thread", t0);
		photon_finished.store(true);
	});
	return 0;
}

/* wait for the photon maps; the scene view then carries them */
int Renderer::finish_photon_job()
{
	if(!photon_thread.joinable()) return 0;
	double t0 = host_now_ms();
	photon_thread.join();
	host_time("host.photon_wait", t0);
	if(photon_rc) return photon_rc;
	photons_ready = true;
	fill_scene_desc();
	if(!batch_t0.empty()) S.maps = dmaps.as<DPhotonMap>();   /* the batch's map table */
	return 0;
}

int Renderer::shoot(cudaStream_t s, int *nc, int *ng)
{
	if(!built) return fail(SRAY_ESTATE, "acceleration structures not built");
	int c = 0, g = 0;
	int r = shoot_maps(S, s, &c, &g);
	if(r) return r;
	photons_ready = true;
	fill_scene_desc();
	if(nc) *nc = c;
	if(ng) *ng = g;
	return 0;
}

int Renderer::queue_alloc(DevBuf &buf, RayQueue &Q, int &qc, int cap)
{
	if(cap <= qc) return 0;
	size_t per = 16 * 5 + 8;
	size_t bytes = (size_t)cap * per + 1024;
	CK(buf.ensure(bytes), "allocate ray queue");
	char *b = buf.as<char>();
	int *count = Q.count;
	Q.o = (float4 *)b; b += (size_t)cap * 16;
	Q.d = (float4 *)b; b += (size_t)cap * 16;
	Q.w = (float4 *)b; b += (size_t)cap * 16;
	Q.meta = (int4 *)b; b += (size_t)cap * 16;
	Q.stk = (float4 *)b; b += (size_t)cap * 16;
	Q.ext = (int2 *)b; b += (size_t)cap * 8;
	Q.count = count;
	Q.cap = cap;
	qc = cap;
	return 0;
}

int Renderer::ensure_queue(int which, int cap)
{
	return queue_alloc(qbuf[which], q[which], qcap[which], cap);
}

int Renderer::ensure_pqueue(int which, int cap)
{
	return queue_alloc(pqbuf[which], pq[which], pqcap[which], cap);
}

/* the n rays of q[cur], sorted by direction octant and origin cell into the
 * spare queue, which then becomes q[cur] (the pass's queue and its
 * allocation swapped with the spare's) */
int Renderer::sort_queue(RayQueue &Q, DevBuf &Qbuf, int &Qcap, RayQueue &T, DevBuf &Tbuf, int &Tcap, DevBuf &keysb, DevBuf &hist,
		DevBuf &part, int n, int bits, const char *name, cudaStream_t s)
{
	if(n < 2 || sc.oct.nodes.empty()) return 0;
	if(int r = queue_alloc(Tbuf, T, Tcap, Q.cap)) return r;
	CK(keysb.ensure((size_t)n * 16), "ray sort keys");
	unsigned *keys = keysb.as<unsigned>(), *vals = keys + n, *keys2 = keys + 2 * (size_t)n, *vals2 = keys + 3 * (size_t)n;
	const Box &b = sc.oct.nodes[0].box;
	float ext[3], lo[3];
	for(int a = 0; a < 3; a++) {
		lo[a] = (float)b.mn[a];
		double e = b.mx[a] - b.mn[a];
		ext[a] = e > 0.0 ? (float)(128.0 / e) : 0.0f;
	}
	LAUNCH(*this, name, s, k_ray_keys<<<grid_for(n, 256), 256, 0, s>>>(Q, n, lo[0], lo[1], lo[2], ext[0], ext[1], ext[2],
			24 - bits, keys, vals));
	unsigned *sorted = nullptr;
	if(int r = sort_pairs(*this, keys, vals, keys2, vals2, n, bits, hist, part, name, s, &sorted)) return r;
	LAUNCH(*this, name, s, k_ray_permute<<<grid_for(n, 256), 256, 0, s>>>(Q, sorted, n, T));
	int *count = Q.count;
	std::swap(Q, T);
	std::swap(Qbuf, Tbuf);
	std::swap(Qcap, Tcap);
	Q.count = count;
	return 0;
}

int Renderer::sort_pass(int cur, int n, cudaStream_t s)
{
	return sort_queue(q[cur], qbuf[cur], qcap[cur], qs, qsbuf, qscap, rs_keys, rs_hist, rs_part, n, 24, "ray_sort", s);
}

int Renderer::sort_photon_pass(int cur, int n, cudaStream_t s)
{
	/* one radix pass: the direction octant and the origin's cell in a coarse
	 * grid (the first pass's photons leave from the lights) */
	return sort_queue(pq[cur], pqbuf[cur], pqcap[cur], pqs, pqsbuf, pqscap, ps_keys, ps_hist, ps_part, n, 8, "photon_ray_sort", s);
}

/* ---------------------------------------------------------------- */
/* radiance cache: records, validation and training (host driver below) */

#define NRC_VAL_DECAY 0.98f   /* per-frame decay of a region's running validation sums */
#define NRC_VAL_MIN 64.0f     /* running record count a region needs before it is judged */
#define NRC_LR 1e-3f

/* targets of the training records [0, n_t) and the validation records
 * [tcap, tcap + n_v): the channels their slots accumulated */
__global__ void k_nrc_harvest(const float4 *acc_rec, int n_t, int tcap, int n_v, float *tgt)
{
	int n = tcap + n_v;
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		if(i >= n_t && i < tcap) continue;
		float4 a = acc_rec[i];
		tgt[(size_t)i * 3 + 0] = a.x;
		tgt[(size_t)i * 3 + 1] = a.y;
		tgt[(size_t)i * 3 + 2] = a.z;
	}
}

/* the frame's validation records into their regions' sums */
__global__ void k_nrc_validate(int n, const float *x, const float *y, const float *t, NrcRegionStats *rs)
{
	for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
		int r = nrc_region(x + (size_t)i * 9);
		const float *yi = y + (size_t)i * 3, *ti = t + (size_t)i * 3;
		float ly = fmaxf(yi[0], 0.0f) + fmaxf(yi[1], 0.0f) + fmaxf(yi[2], 0.0f);
		float lt = ti[0] + ti[1] + ti[2];
		atomicAdd(&rs->sy[r], ly);
		atomicAdd(&rs->st[r], lt);
		atomicAdd(&rs->sn[r], 1.0f);
		atomicAdd(&rs->sq[r], (ly - lt) * (ly - lt));
	}
}

__device__ __forceinline__ float block_sum_regions(float v, float *red)
{
	int r = threadIdx.x;
	red[r] = v;
	__syncthreads();
	for(int h = NRC_REGIONS / 2; h > 0; h >>= 1) {
		if(r < h) red[r] += red[r + h];
		__syncthreads();
	}
	float out = red[0];
	__syncthreads();
	return out;
}

/* one block, a thread per region: fold the frame's sums into the running
 * sums and judge each region.  Its validation relative error is
 * |sum prediction - sum target| / sum target over the running sums (the
 * denominator floored at 1% of the mean target, so that dark regions are
 * not judged on noise).  A region is judged once it has NRC_VAL_MIN records
 * and the standard error of that estimate (from the squared differences) is
 * at most half the threshold; the network serves it when judged and the
 * error is at most the threshold, else the plain gather does. */
__global__ void __launch_bounds__(NRC_REGIONS) k_nrc_regions(NrcRegionStats *rs, float decay, float max_rel, float min_n, int mode)
{
	__shared__ float red[NRC_REGIONS];
	int r = threadIdx.x;
	float ey = rs->ey[r] * decay + rs->sy[r];
	float et = rs->et[r] * decay + rs->st[r];
	float en = rs->en[r] * decay + rs->sn[r];
	float eq = rs->eq[r] * decay + rs->sq[r];
	rs->ey[r] = ey;
	rs->et[r] = et;
	rs->en[r] = en;
	rs->eq[r] = eq;
	rs->sy[r] = 0.0f;
	rs->st[r] = 0.0f;
	rs->sn[r] = 0.0f;
	rs->sq[r] = 0.0f;
	float tot_t = block_sum_regions(et, red);
	float tot_n = block_sum_regions(en, red);
	float mean = tot_n > 0.0f ? tot_t / tot_n : 0.0f;
	float den = fmaxf(et, 0.01f * mean * en);
	float err = fabsf(ey - et);
	float var = en > 0.0f ? fmaxf(eq - (ey - et) * (ey - et) / en, 0.0f) : 0.0f;
	bool judged = en >= min_n && den > 0.0f && sqrtf(var) <= 0.5f * max_rel * den;
	bool ok = judged && err <= max_rel * den;
	rs->fallback[r] = (mode == 2 || ok) ? 0 : 1;
	float nj = block_sum_regions(judged ? 1.0f : 0.0f, red);
	float nok = block_sum_regions(ok ? 1.0f : 0.0f, red);
	float se = block_sum_regions(judged ? err : 0.0f, red);
	float stt = block_sum_regions(judged ? et : 0.0f, red);
	if(r == 0) {
		rs->summary[0] = nj;
		rs->summary[1] = nok;
		rs->summary[2] = stt > 0.0f ? se / stt : 0.0f;
		rs->summary[3] = 0.0f;
	}
}

__global__ void k_nrc_reset_regions(NrcRegionStats *rs)
{
	int r = threadIdx.x;
	rs->sy[r] = rs->st[r] = rs->sn[r] = rs->sq[r] = 0.0f;
	rs->ey[r] = rs->et[r] = rs->en[r] = rs->eq[r] = 0.0f;
	rs->fallback[r] = 1;
	if(r < 4) rs->summary[r] = 0.0f;
}

int Renderer::nrc_reset_regions(cudaStream_t s)
{
	CK(nrc_regions.ensure(sizeof(NrcRegionStats)), "radiance cache regions");
	k_nrc_reset_regions<<<1, NRC_REGIONS, 0, s>>>(nrc_regions.as<NrcRegionStats>());
	CK(cudaGetLastError(), "radiance cache regions");
	nrc_regions_ready = true;
	return 0;
}

/* training / validation records wanted per frame and the room for them */
static void nrc_record_caps(const sray_opts &opt, int *ntrain, int *nval, int *tcap, int *vcap)
{
	*ntrain = opt.nrc_train_samples > 0 ? opt.nrc_train_samples : 65536;
	*nval = *ntrain / 4 > 1024 ? *ntrain / 4 : 1024;
	*tcap = *ntrain + *ntrain / 8 + 1024;
	*vcap = *nval + *nval / 8 + 1024;
}

static uint32_t nrc_prob(double f)
{
	if(!(f > 0.0)) return 0u;
	if(f >= 1.0) return 0xffffffffu;
	return (uint32_t)(f * 4294967296.0);
}

static uint32_t nrc_mix(uint64_t v)
{
	v ^= v >> 33;
	v *= 0xff51afd7ed558ccdull;
	v ^= v >> 33;
	v *= 0xc4ceb9fe1a85ec53ull;
	v ^= v >> 33;
	return (uint32_t)v;
}

/* the radiance cache's view of sample batch `batch` (n_prim primary rays):
 * query and record buffers, the record slots past the batch's accumulator
 * slots, and (first batch only) the selection of training and validation
 * vertices, sized from the last frame's vertex count */
int Renderer::nrc_setup(int batch, int n_prim, int wave_rays, cudaStream_t s)
{
	DNrc &N = S.nrc;
	N.mode = S.gi_on ? opt.nrc : 0;
	if(!N.mode) return 0;
	int r = nrc_ensure_ready(opt.seed, s);
	if(r) return fail(r, std::string("radiance cache: ") + nrc_error());
	if(!nrc_regions_ready && (r = nrc_reset_regions(s))) return r;
	int ntrain, nval, tcap, vcap;
	nrc_record_caps(opt, &ntrain, &nval, &tcap, &vcap);
	nrc_rcap = tcap + vcap;
	CK(nrc_rx.ensure((size_t)nrc_rcap * 9 * sizeof(float)), "radiance cache records");
	CK(nrc_rt.ensure((size_t)nrc_rcap * 3 * sizeof(float)), "radiance cache targets");
	CK(nrc_ry.ensure((size_t)vcap * 3 * sizeof(float)), "radiance cache predictions");
	/* queries are answered after each wave (nrc_wave_done) */
	int64_t qc = (int64_t)wave_rays * 2 + 65536;
	if(qc > INT_MAX / 2) qc = INT_MAX / 2;
	nrc_qcap = (int)qc;
	CK(nrc_qx.ensure((size_t)nrc_qcap * 9 * sizeof(float)), "radiance cache queries");
	CK(nrc_qw.ensure((size_t)nrc_qcap * sizeof(float4)), "radiance cache queries");
	CK(acc.ensure(((size_t)n_prim + nrc_rcap) * 16), "accumulator");
	CK(cudaMemsetAsync(acc.as<float4>() + n_prim, 0, (size_t)nrc_rcap * 16, s), "reset record slots");
	int *cnt = counts.as<int>();
	CK(cudaMemsetAsync(cnt + 16, 0, 3 * sizeof(int), s), "reset radiance cache counts");
	N.qx = nrc_qx.as<float>();
	N.qw = nrc_qw.as<float4>();
	N.qcount = cnt + 16;
	N.qcap = nrc_qcap;
	N.tx = nrc_rx.as<float>();
	N.tcount = cnt + 17;
	N.tcap = tcap;
	N.vcap = vcap;
	N.t0 = n_prim;
	N.fallback = nrc_regions.as<NrcRegionStats>()->fallback;
	double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {1.0, 1.0, 1.0};
	if(!sc.oct.nodes.empty()) {
		for(int k = 0; k < 3; k++) {
			lo[k] = sc.oct.nodes[0].box.mn[k];
			hi[k] = sc.oct.nodes[0].box.mx[k];
		}
	}
	for(int k = 0; k < 3; k++) {
		double ext = hi[k] - lo[k];
		N.lo[k] = (float)lo[k];
		N.sc[k] = ext > 0.0 ? (float)(1.0 / ext) : 1.0f;
	}
	if(batch == 0) {
		double expect = nrc_expect > 0 ? (double)nrc_expect : (double)n_prim;
		/* 2 % more training vertices than the batch takes, so that a frame
		 * almost always has the full batch (and replays the training graph) */
		double ft = ntrain * 1.02 / expect, fv = nval / expect;
		if(ft + fv > 1.0) {
			/* fewer vertices than records wanted: every vertex is one, in proportion */
			double sum = ft + fv;
			ft /= sum;
			fv /= sum;
		}
		N.p_train = nrc_prob(ft);
		N.p_val = nrc_prob(fv);
		if((uint64_t)N.p_train + N.p_val > 0xffffffffull) N.p_val = 0xffffffffu - N.p_train;
	} else {
		N.p_train = N.p_val = 0;
	}
	N.key = nrc_mix(opt.seed ^ ((uint64_t)nrc_frames * 0x9e3779b97f4a7c15ull) ^ 0x4e5243ull);
	N.fb_samples = opt.nrc_fallback_samples;
	N.counters = (unsigned long long *)(ctr.as<char>() + offsetof(DevCounters, nrc)) + 2 * (batch > 0);
	return 0;
}

/* the wave's queries: the network's outputs into their accumulators, the
 * query queue emptied for the next wave */
int Renderer::nrc_wave_done(cudaStream_t s)
{
	if(!S.nrc.mode) return 0;
	int *cnt = counts.as<int>();
	int r = 0;
	LAUNCH(*this, "nrc_query", s, r = nrc_query(cnt + 16, nrc_qcap, nrc_qx.as<float>(), nrc_qw.as<float4>(), acc.as<float4>(), s));
	if(r) return fail(r, std::string("radiance cache: ") + nrc_error());
	CK(cudaMemsetAsync(cnt + 16, 0, sizeof(int), s), "reset radiance cache queries");
	return 0;
}

/* after the first sample batch: the records' targets, the validation of
 * the network on the validation records (before it trains on this frame),
 * the regions' fallback flags for the next frame, and the training steps */
int Renderer::nrc_batch_done(int batch, cudaStream_t s)
{
	if(!S.nrc.mode) return 0;
	int *cnt = counts.as<int>();
	int r = 0;
	if(batch != 0) return 0;
	int h[2] = {0, 0};
	CK(cudaMemcpyAsync(h, cnt + 17, sizeof h, cudaMemcpyDeviceToHost, s), "read record counts");
	CK(cudaStreamSynchronize(s), "record counts");
	d2h += sizeof h;
	prof_collect();
	const DNrc &N = S.nrc;
	int n_t = h[0] < N.tcap ? h[0] : N.tcap;
	int n_v = h[1] < N.vcap ? h[1] : N.vcap;
	float *rx = nrc_rx.as<float>(), *rt = nrc_rt.as<float>();
	NrcRegionStats *rs = nrc_regions.as<NrcRegionStats>();
	if(n_t + n_v > 0)
		LAUNCH(*this, "nrc_records", s, k_nrc_harvest<<<grid_for(N.tcap + n_v, 256), 256, 0, s>>>(acc.as<float4>() + N.t0, n_t, N.tcap,
				n_v, rt));
	if(n_v > 0) {
		LAUNCH(*this, "nrc_validate", s, r = nrc_infer(n_v, rx + (size_t)N.tcap * 9, nrc_ry.as<float>(), s));
		if(r) return fail(r, std::string("radiance cache: ") + nrc_error());
		LAUNCH(*this, "nrc_validate", s, k_nrc_validate<<<grid_for(n_v, 256), 256, 0, s>>>(n_v, rx + (size_t)N.tcap * 9,
				nrc_ry.as<float>(), rt + (size_t)N.tcap * 3, rs));
	}
	float max_rel = opt.nrc_max_rel_err;
	LAUNCH(*this, "nrc_validate", s, k_nrc_regions<<<1, NRC_REGIONS, 0, s>>>(rs, NRC_VAL_DECAY, max_rel, NRC_VAL_MIN, N.mode));
	int steps = opt.nrc_train_steps > 0 ? opt.nrc_train_steps : 4;
	int ntrain = opt.nrc_train_samples > 0 ? opt.nrc_train_samples : 65536;
	int use = n_t < ntrain ? n_t : ntrain;
	int per = use / steps;
	if(per < 16) {
		steps = use >= 16 ? 1 : 0;
		per = use;
	}
	if(steps > 0) {
		/* the frame's training steps: one graph launch (steps x NRC_TRAIN_KERNELS kernels) */
		LAUNCH(*this, "nrc_train", s, r = nrc_train_steps(steps, per, rx, rt, NRC_LR, s));
		if(r) return fail(r, std::string("radiance cache: ") + nrc_error());
		launch_count += (long long)steps * NRC_TRAIN_KERNELS - 1;
	}
	nrc_last_train = steps * per;
	nrc_last_val = n_v;
	nrc_frames++;
	return 0;
}

int Renderer::render_pixels(long msec, float *fb, int fb_is_device, cudaStream_t s, bool overlap_photons)
{
	(void)msec;
	if(!built || (!photons_ready && !overlap_photons)) return fail(SRAY_ESTATE, "frame not prepared (build and shoot photons first)");
	bool photons_pending = overlap_photons;
	int npix = batch_npix > 0 ? batch_npix : opt.width * opt.height;
	int ds = opt.diffuse_samples < 0 ? 0 : (opt.diffuse_samples > MAX_DS ? MAX_DS : opt.diffuse_samples);
	int maxs = opt.max_samples < 1 ? 1 : opt.max_samples;
	CK(ctr.ensure(sizeof(DevCounters)), "counters");
	CK(counts.ensure(64 * sizeof(int)), "counts");
	CK(acc.ensure((size_t)npix * 16), "accumulator");
	CK(sums.ensure((size_t)npix * 16), "sums");
	CK(spp.ensure((size_t)npix * 4), "spp");
	if(maxs > 1) {
		CK(hist.ensure((size_t)npix * maxs * 16), "sample history");
		CK(active[0].ensure((size_t)npix * 4), "active list");
		CK(active[1].ensure((size_t)npix * 4), "active list");
	}
	float4 *fbd;
	if(fb_is_device) fbd = (float4 *)fb;
	else {
		CK(fbdev.ensure((size_t)npix * 16), "framebuffer");
		fbd = fbdev.as<float4>();
	}
	/* a vertex sends its image's diffuse rays (the fallback count in a
	 * fallback region); the records' rays come on top, bounded by the record
	 * count of a frame */
	int img_rays = ds;
	int64_t rec_extra = 0;
	if(opt.nrc && opt.gi_photons) {
		int fb = opt.nrc_fallback_samples > MAX_DS ? MAX_DS : opt.nrc_fallback_samples;
		img_rays = fb > ds ? fb : ds;
		int rec_rays = ds > NRC_VAL_RAYS ? ds : NRC_VAL_RAYS;
		int ntrain, nval, tcap, vcap;
		nrc_record_caps(opt, &ntrain, &nval, &tcap, &vcap);
		rec_extra = (int64_t)(tcap + vcap) * rec_rays;
	}
	int per_ray_children = 2 + (opt.gi_photons ? img_rays : 0);
	int shadow_per_ray = 0;
	for(size_t li = 0; li < sc.lights.size(); li++) shadow_per_ray += sc.lights[li].type != LT_POINT ? opt.shadow_samples : 1;
	if(shadow_per_ray < 1) shadow_per_ray = 1;
	if(ensure_queue(0, npix)) return SRAY_ECUDA;
	CK(hits.ensure((size_t)npix * 16), "hits");
	CK(gq.ensure((size_t)npix * sizeof(GatherReq)), "gather queue");
	int *cnt = counts.as<int>();
	/* cnt[0]/cnt[1]: ray queue counts, cnt[2]: gather count, cnt[3]: pixels of the first batch,
	 * cnt[5]: shadow count, cnt[6]: pixels still running after the first batch */
	CK(cudaMemsetAsync(ctr.p, 0, sizeof(DevCounters), s), "reset counters");
	CK(cudaMemsetAsync(counts.p, 0, 64 * sizeof(int), s), "reset counts");
	int h_n = npix;
	CK(cudaMemcpyAsync(cnt + 3, &h_n, sizeof(int), cudaMemcpyHostToDevice, s), "active count");
	h2d += sizeof(int);
	long long l0 = launch_count;
	memset(&stats, 0, sizeof stats);
	int n_active = npix;
	/* the photon thread is always joined before this returns */
	struct PhotonJoin {
		Renderer *R;
		~PhotonJoin() { if(R->photon_thread.joinable()) R->photon_thread.join(); }
	} photon_join{this};
	/* While the photon maps are traced (on the photon stream, from a host
	 * thread of their own), the first sample batch's bounces go on and their
	 * photon-map gathers accumulate in gq; they run in one launch once the
	 * maps exist (before the shading tail, at the latest at the end of the
	 * batch).  gq_upper bounds the gathers queued so far (a shaded ray asks
	 * for at most one). */
	bool deferring = false;
	int64_t gq_upper = 0, gq_defer_cap = 0;
	/* side_gather: the accumulated gathers run on the gather stream from a
	 * copy of their requests, beside the batch's remaining bounces, and the
	 * batch waits for them before its accumulators are read */
	bool side_pending = false;
	struct SideJoin {
		Renderer *R;
		bool *pending;
		~SideJoin() { if(*pending) cudaStreamSynchronize(R->gs); }
	} side_join{this, &side_pending};
	auto flush_gathers = [&]() -> int {
		if(!deferring) return 0;
		deferring = false;
		int r = finish_photon_job();
		if(r) return r;
		if(gq_upper > 0 && tune.side_gather) {
			if(int r2 = gather_stream()) return r2;
			CK(gq_side.ensure((size_t)gq_upper * sizeof(GatherReq)), "side gather queue");
			CK(cudaMemcpyAsync(gq_side.p, gq.p, (size_t)gq_upper * sizeof(GatherReq), cudaMemcpyDeviceToDevice, s), "side gathers");
			CK(cudaMemcpyAsync(cnt + 24, cnt + 2, sizeof(int), cudaMemcpyDeviceToDevice, s), "side gather count");
			CK(cudaEventRecord(gs_fork, s), "side gather fork");
			CK(cudaStreamWaitEvent(gs, gs_fork, 0), "side gather fork");
			LAUNCH(*this, "gather", gs, k_gather<<<grid_for((int)gq_upper, GATHER_WARPS), GATHER_WARPS * 32, 0, gs>>>(S,
					gq_side.as<GatherReq>(), cnt + 24, acc.as<float4>(), ctr.as<DevCounters>()));
			CK(cudaEventRecord(gs_done, gs), "side gather done");
			side_pending = true;
		} else if(gq_upper > 0) {
			LAUNCH(*this, "gather", s, k_gather<<<grid_for((int)gq_upper, GATHER_WARPS), GATHER_WARPS * 32, 0, s>>>(S,
					gq.as<GatherReq>(), cnt + 2, acc.as<float4>(), ctr.as<DevCounters>()));
		}
		gq_upper = 0;
		CK(cudaMemsetAsync(cnt + 2, 0, sizeof(int), s), "reset gather queue");
		return 0;
	};
	/* While the photon maps are still being traced the accumulated gathers
	 * outlive a wave: their queue grows (its requests copied over) up to a
	 * quarter of the free device memory and DEFER_MAX_REQS requests, rather
	 * than the render stream waiting for the maps.  The queues it grew out of
	 * are freed once the stream has passed them. */
	struct Retired {
		std::vector<DevBuf> bufs;
		cudaStream_t s;
		~Retired()
		{
			if(bufs.empty()) return;
			cudaStreamSynchronize(s);
			for(DevBuf &b : bufs) b.release();
		}
	} retired{{}, s};
	auto grow_deferred = [&](int64_t need) -> bool {
		int64_t cap = std::max<int64_t>(need, 2 * gq_defer_cap);
		if(cap > DEFER_MAX_REQS) cap = DEFER_MAX_REQS;
		if(cap < need) return false;
		size_t fr = 0, tot = 0;
		if(cudaMemGetInfo(&fr, &tot) != cudaSuccess || (size_t)cap * sizeof(GatherReq) > fr / 4) return false;
		DevBuf nb;
		if(nb.ensure((size_t)cap * sizeof(GatherReq)) != cudaSuccess) {
			cudaGetLastError();
			return false;
		}
		if(gq_upper > 0 && cudaMemcpyAsync(nb.p, gq.p, (size_t)gq_upper * sizeof(GatherReq), cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
			nb.release();
			return false;
		}
		retired.bufs.push_back(gq);
		gq = nb;
		gq_defer_cap = cap;
		return true;
	};
	/* side_shadow: light samples on their own stream (not in the counting
	 * pass, whose kernels count on the frame's stream); the render loop
	 * joins it at a wave's end, before the persistent pool, and, whatever
	 * the return, before this function's buffers are touched again */
	const bool sides = tune.side_shadow != 0 && !(prof_flags & 2);
	if(sides && side_stream()) return SRAY_ECUDA;
	bool side_busy[2] = {false, false};
	struct ShadowJoin {
		Renderer *R;
		bool *busy;
		~ShadowJoin() { if(busy[0] || busy[1]) cudaStreamSynchronize(R->xs); }
	} shadow_join{this, side_busy};
	auto join_shadows = [&]() -> int {
		for(int k = 0; k < 2; k++) {
			if(!side_busy[k]) continue;
			CK(cudaStreamWaitEvent(s, xs_done[k], 0), "light-sample join");
			side_busy[k] = false;
		}
		return 0;
	};
	auto join_side = [&]() -> int {
		if(!side_pending) return 0;
		side_pending = false;
		CK(cudaStreamWaitEvent(s, gs_done, 0), "side gather join");
		return 0;
	};
	/* sample batches: the first covers the samples every pixel takes before
	 * its first variance test, the second all the remaining samples of the
	 * pixels still running (rendered speculatively, cut by k_finish) */
	int w0 = opt.min_samples > 2 ? opt.min_samples : 2;
	if(w0 > maxs) w0 = maxs;
	int batch_s0[2] = {0, w0};
	int batch_w[2] = {w0, maxs - w0};
	for(int b = 0; b < 2 && n_active > 0 && batch_w[b] > 0; b++) {
		int s0 = batch_s0[b], width = batch_w[b];
		const int *act = b > 0 ? active[0].as<int>() : nullptr;
		int *act_count = b == 0 ? cnt + 3 : cnt + 6;
		int *next_count = b == 0 ? cnt + 6 : cnt + 7;
		int *next_list = active[b].as<int>();
		int n_prim = n_active * width;
		/* waves: at most tune.queue_depth primary rays (whole pixels) per
		 * wave, each traced to the end of its shading tree before the next
		 * starts; the queues are sized for a wave, the accumulators for the
		 * batch */
		int wave_pix = n_active;
		if(tune.queue_depth > 0) {
			wave_pix = tune.queue_depth / width;
			if(wave_pix < 1) wave_pix = 1;
			if(wave_pix > n_active) wave_pix = n_active;
		}
		int wave_rays = wave_pix * width;
		if(ensure_queue(0, wave_rays)) return SRAY_ECUDA;
		CK(acc.ensure((size_t)n_prim * 16), "accumulator");
		if(int r = nrc_setup(b, n_prim, wave_rays, s)) return r;
		if(photons_pending) {
			photons_pending = false;
			int64_t cap = (int64_t)wave_rays * 3 + 65536;
			if(cap > INT_MAX / 2) cap = INT_MAX / 2;
			CK(gq.ensure((size_t)cap * sizeof(GatherReq)), "gather queue");
			CK(cudaMemsetAsync(cnt + 2, 0, sizeof(int), s), "reset gather queue");
			if(int r = start_photon_job(s)) return r;
			deferring = true;
			gq_defer_cap = cap;
			gq_upper = 0;
		}
		for(int a0 = 0; a0 < n_active; a0 += wave_pix) {
		int na = n_active - a0 < wave_pix ? n_active - a0 : wave_pix;
		int n_wave = na * width;
		q[0].count = cnt + 0;
		q[1].count = cnt + 1;
		LAUNCH(*this, "camera", s, k_camera<<<grid_for(n_wave, 256), 256, 0, s>>>(S, act, a0, na, s0, width, q[0], acc.as<float4>(),
				ctr.as<DevCounters>()));
		int n_rays = n_wave;
		int cur = 0;
		bool tail_done = false;
		for(int depth = 0; n_rays > 0; depth++) {
			/* side_gather: once the photon maps exist, the gathers queued so
			 * far go out at the next bounce instead of the batch's end;
			 * side_gather 2 waits for the maps at the second bounce, so that
			 * this mid-batch path runs whatever the timing */
			if(deferring && tune.side_gather && (photon_finished.load() || (tune.side_gather == 2 && depth >= 1)))
				if(int r = flush_gathers()) return r;
			/* the pool holds every ray of the rest of the tree: enter it only
			 * with POOL_HEADROOM times the rays' room in the queue */
			if(depth >= 1 && !tail_done && n_rays <= tune.render_tail && (int64_t)n_rays * POOL_HEADROOM <= q[cur].cap) {
				/* the rest of the shading tree in one launch (k_render_pool) */
				tail_done = true;
				if(int r = join_shadows()) return r;
				if(int r = flush_gathers()) return r;
				q[0].count = cnt + 0;
				q[1].count = cnt + 1;
				CK(cudaMemsetAsync(q[cur ^ 1].count, 0, sizeof(int), s), "reset queue");
				CK(cudaMemsetAsync(cnt + 2, 0, sizeof(int), s), "reset gather queue");
				CK(cudaMemsetAsync(cnt + 5, 0, sizeof(int), s), "reset shadow queue");
				int *ctl = cnt + 8;
				int cap = q[cur].cap;
				CK(pool_ready.ensure((size_t)cap * sizeof(int)), "pool flags");
				CK(cudaMemsetAsync(pool_ready.p, 1, (size_t)n_rays * sizeof(int), s), "pool flags");
				CK(cudaMemsetAsync(pool_ready.as<int>() + n_rays, 0, (size_t)(cap - n_rays) * sizeof(int), s), "pool flags");
				int ctl_h[4] = {0, n_rays, n_rays, 0};
				CK(cudaMemcpyAsync(ctl, ctl_h, sizeof ctl_h, cudaMemcpyHostToDevice, s), "pool control");
				h2d += sizeof ctl_h;
				ShadeOut so;
				so.qo = q[cur ^ 1];
				so.qo.cap = child_cap(so.qo.cap);
				so.gq = gq.as<GatherReq>();
				so.gq_count = cnt + 2;
				so.gq_cap = (int)std::min<size_t>(gq.bytes / sizeof(GatherReq), (size_t)INT_MAX);
				so.sq = sq.as<ShadowReq>();
				so.sq_count = cnt + 5;
				so.sq_cap = (int)std::min<size_t>(sq.bytes / sizeof(ShadowReq), (size_t)INT_MAX);
				LAUNCH(*this, "render_pool", s, k_render_pool<<<nsm * tune.pool_blocks_per_sm, 128, 0, s>>>(S, q[cur],
						pool_ready.as<int>(), ctl, so,
						acc.as<float4>(), ctr.as<DevCounters>(), g_faults.spin_limit.load() > 0 ? g_faults.spin_limit.load() : POOL_SPIN_LIMIT));
				if(int r = shadow_rays(so.sq_cap, s)) return r;
				LAUNCH(*this, "gather", s, k_gather<<<grid_for(so.gq_cap, GATHER_WARPS), GATHER_WARPS * 32, 0, s>>>(S,
						gq.as<GatherReq>(), cnt + 2, acc.as<float4>(), ctr.as<DevCounters>()));
				CK(cudaMemcpyAsync(pin, q[cur ^ 1].count, sizeof(int), cudaMemcpyDeviceToHost, s), "read queue count");
				CK(cudaMemcpyAsync(pin + 1, ctl + 3, sizeof(int), cudaMemcpyDeviceToHost, s), "read pool error");
				CK(cudaStreamSynchronize(s), "shading tail");
				int h_cnt = pin[0], h_err = pin[1];
				d2h += 2 * sizeof(int);
				prof_collect();
				if(h_err) return fail(SRAY_EDEVICE, "shading pool: a wait for work ran out");
				if(h_cnt > so.qo.cap) return queue_overflow(h_cnt, so.qo.cap);
				n_rays = h_cnt;
				cur ^= 1;
				continue;
			}
			int64_t need64 = (int64_t)n_rays * per_ray_children + rec_extra;
			int need = need64 > INT_MAX / 2 ? INT_MAX / 2 : (int)need64;
			if(need < n_rays) need = n_rays;
			int r = ensure_queue(cur ^ 1, need);
			if(r) return r;
			CK(hits.ensure((size_t)n_rays * 16), "hits");
			if(deferring && gq_upper + n_rays > gq_defer_cap) {
				bool grown = !photon_finished.load() && !S.nrc.mode && grow_deferred(gq_upper + n_rays);
				if(!grown && (r = flush_gathers())) return r;
			}
			q[0].count = cnt + 0;
			q[1].count = cnt + 1;
			CK(cudaMemsetAsync(q[cur ^ 1].count, 0, sizeof(int), s), "reset queue");
			/* side_shadow: this bounce's light samples (and, once the photon
			 * maps exist, its gathers) go to the buffers of its parity, once
			 * the bounce before last has finished with them */
			const int par = depth & 1;
			DevBuf &sqb = sides && par ? sq2 : sq;
			int *sqc = sides ? cnt + 40 + par : cnt + 5;
			DevBuf &gqb = sides && par ? gq2 : gq;
			int *gqc = sides ? cnt + 42 + par : cnt + 2;
			if(sides && side_busy[par]) {
				CK(cudaStreamWaitEvent(s, xs_done[par], 0), "light-sample buffer");
				side_busy[par] = false;
			}
			if(!deferring) {
				CK(gqb.ensure((size_t)n_rays * sizeof(GatherReq)), "gather queue");
				CK(cudaMemsetAsync(gqc, 0, sizeof(int), s), "reset gather queue");
			}
			CK(cudaMemsetAsync(sqc, 0, sizeof(int), s), "reset shadow queue");
			CK(sqb.ensure((size_t)n_rays * shadow_per_ray * sizeof(ShadowReq)), "shadow queue");
			if(depth >= 1 && tune.sort_rays > 0 && n_rays >= tune.sort_rays && (r = sort_pass(cur, n_rays, s))) return r;
			r = trace_rays(q[cur], n_rays, "trace", (prof_flags & 2) != 0, s, depth == 0);
			if(r) return r;
			ShadeOut so;
			so.qo = q[cur ^ 1];
			so.qo.cap = child_cap(so.qo.cap);
			so.gq = deferring ? gq.as<GatherReq>() : gqb.as<GatherReq>();
			so.gq_count = deferring ? cnt + 2 : gqc;
			so.gq_cap = deferring ? (int)gq_defer_cap : n_rays;
			so.sq = sqb.as<ShadowReq>();
			so.sq_count = sqc;
			so.sq_cap = n_rays * shadow_per_ray;
			LAUNCH(*this, "shade", s, k_shade<<<grid_for(n_rays, 128), 128, 0, s>>>(S, q[cur], hits.as<int4>(), so, acc.as<float4>(), depth,
					ctr.as<DevCounters>()));
			if(sides) {
				/* traced beside the next bounce's closest hits and shading */
				CK(cudaEventRecord(xs_fork, s), "light-sample fork");
				CK(cudaStreamWaitEvent(xs, xs_fork, 0), "light-sample fork");
				if(int r = shadow_rays_on(sqb.as<ShadowReq>(), sqc, n_rays * shadow_per_ray, fbs[par], xs)) return r;
				if(!deferring)
					LAUNCH(*this, "gather", xs, k_gather<<<grid_for(n_rays, GATHER_WARPS), GATHER_WARPS * 32, 0, xs>>>(S,
							gqb.as<GatherReq>(), gqc, acc.as<float4>(), ctr.as<DevCounters>()));
				CK(cudaEventRecord(xs_done[par], xs), "light-sample done");
				side_busy[par] = true;
			} else if(int r = shadow_rays(n_rays * shadow_per_ray, s)) {
				return r;
			}
			if(deferring)
				gq_upper += n_rays;
			else if(!sides)
				LAUNCH(*this, "gather", s, k_gather<<<grid_for(n_rays, GATHER_WARPS), GATHER_WARPS * 32, 0, s>>>(S, gq.as<GatherReq>(),
						cnt + 2, acc.as<float4>(), ctr.as<DevCounters>()));
			stats.secondary_rays += depth ? n_rays : 0;
			CK(cudaMemcpyAsync(pin, q[cur ^ 1].count, sizeof(int), cudaMemcpyDeviceToHost, s), "read queue count");
			double tw = host_now_ms();
			CK(cudaStreamSynchronize(s), "bounce");
			host_time("host.bounce_wait", tw);
			int h_cnt = pin[0];
			d2h += sizeof(int);
			prof_collect();
			/* children beyond the queue were dropped (the count kept going):
			 * the frame stops here rather than trace entries never written */
			if(h_cnt > so.qo.cap) return queue_overflow(h_cnt, so.qo.cap);
			n_rays = h_cnt;
			cur ^= 1;
		}
		if(int r = join_shadows()) return r;
		/* the wave's gathers and radiance-cache queries; while the photon
		 * maps are still being traced and more waves follow, the gathers stay
		 * queued (the radiance cache, whose records are gather estimates,
		 * takes them wave by wave) */
		bool more_waves = a0 + wave_pix < n_active;
		if(!(deferring && more_waves && !S.nrc.mode && !photon_finished.load()))
			if(int r = flush_gathers()) return r;
		if(int r = join_side()) return r;
		if(int r = nrc_wave_done(s)) return r;
		}
		if(int r = flush_gathers()) return r;
		if(int r = join_side()) return r;
		if(int r = nrc_batch_done(b, s)) return r;
		CK(cudaMemsetAsync(next_count, 0, sizeof(int), s), "reset next active");
		LAUNCH(*this, "finish", s, k_finish<<<grid_for(n_active, 256), 256, 0, s>>>(act, S.njobs > 0 ? 0 : S.width, S.height, act_count, s0, width, acc.as<float4>(),
				hist.as<float4>(), sums.as<float4>(), maxs, opt.min_samples, opt.max_var, next_list, next_count, fbd,
				spp.as<int>()));
		stats.samples += (int64_t)n_active * width;
		CK(cudaMemcpyAsync(pin + 2, next_count, sizeof(int), cudaMemcpyDeviceToHost, s), "read active count");
		CK(cudaStreamSynchronize(s), "sample pass");
		d2h += sizeof(int);
		prof_collect();
		n_active = pin[2];
	}
	if(photons_pending) {
		/* no sample batch ran: the maps are still the frame's */
		int r = shoot(s, nullptr, nullptr);
		if(r) return r;
	}
	DevCounters hc;
	CK(cudaMemcpyAsync(&hc, ctr.p, sizeof hc, cudaMemcpyDeviceToHost, s), "read counters");
	if(!fb_is_device) CK(cudaMemcpyAsync(fb, fbd, (size_t)npix * 16, cudaMemcpyDeviceToHost, s), "copy framebuffer");
	CK(cudaStreamSynchronize(s), "render");
	d2h += sizeof hc + (fb_is_device ? 0 : (int64_t)npix * 16);
	stats.primary_rays = (int64_t)hc.rays[0];
	stats.secondary_rays += (int64_t)hc.rays[1];
	stats.shadow_rays = (int64_t)hc.rays[2];
	stats.gathers = (int64_t)hc.rays[3];
	stats.kernel_launches = (int)(launch_count - l0);
	stats.h2d_bytes = h2d;
	stats.d2h_bytes = d2h;
	stats.node_visits = (int64_t)hc.nodes;
	stats.prim_tests = (int64_t)hc.prims;
	stats.shadow_node_visits = (int64_t)hc.snodes;
	stats.shadow_prim_tests = (int64_t)hc.sprims;
	stats.gather_tested = (int64_t)hc.g_tested;
	stats.gather_candidates = (int64_t)hc.g_cand;
	stats.gather_selects = (int64_t)hc.g_select;
	stats.gather_spills = (int64_t)hc.g_spill;
	stats.bvh_fallbacks = (int64_t)hc.bvh_fallbacks;
	retrace_hint = stats.bvh_fallbacks;
	if(overlap_photons && !sc.lights.empty()) stats.photons_emitted = (int64_t)opt.caust_photons + opt.gi_photons;
	if(S.nrc.mode) {
		nrc_expect = (int64_t)hc.nrc[0];
		nrc_last_vertices = (int64_t)(hc.nrc[0] + hc.nrc[2]);
		nrc_last_cached = (int64_t)(hc.nrc[1] + hc.nrc[3]);
	}
	if(hc.overflow) return fail(SRAY_EDEVICE, "device queue or traversal stack overflow");
	int r_nrc = 0;
	if(S.nrc.mode && (r_nrc = nrc_device_error(s)) != 0) return fail(r_nrc, nrc_error());
	return 0;
}

/* the child queue's capacity as the emitters see it (an injected cap for
 * the fault tests, else the allocation's) */
int Renderer::child_cap(int cap) const
{
	int f = g_faults.queue_cap.load();
	return f > 0 && f < cap ? f : cap;
}

int Renderer::queue_overflow(int count, int cap)
{
	char msg[160];
	snprintf(msg, sizeof msg, "device ray queue overflow: %d child rays for a queue of %d", count, cap);
	return fail(SRAY_EDEVICE, msg);
}

/* closest hits of the first n (upper bound; the queue's count decides)
 * rays of q into hits: the hierarchy pass, then the octree pass over the
 * rays it listed */
int Renderer::trace_rays_with(const DScene &D, const RayQueue &qq, int n, const char *name, bool count, cudaStream_t s,
		int4 *hit_out, DevBuf &fb, DevCounters *c, bool short_blocks, bool coherent)
{
	CK(fb.ensure(((size_t)n + 1) * sizeof(int)), "fallback list");
	CK(cudaMemsetAsync(fb.p, 0, sizeof(int), s), "reset fallback list");
	/* short_blocks (the photon stream's passes): a block per 128 rays
	 * instead of a capped grid that strides, so that its blocks free their
	 * SMs for the frame's stream as they finish */
	int g = short_blocks ? std::max(1, (n + 127) / 128) : grid_for(n, 128);
	if(!count && coherent && D.nscenes <= 1 && n > tune.warp_rays) {
		LAUNCH(*this, name, s, k_trace_packet<<<g, SRAY_TRACE_THREADS, 0, s>>>(D, qq, hit_out, c, fb.as<int>()));
		LAUNCH(*this, "octree_retrace", s, k_trace<false, false><<<retrace_grid(), 128, 0, s>>>(D, qq, hit_out, c, fb.as<int>()));
		return 0;
	}
	if(!count && n <= tune.warp_rays) {
		/* a pass of few rays: one warp per ray */
		LAUNCH(*this, name, s, k_trace_warp<<<grid_for(n, 4), 128, 0, s>>>(D, qq, hit_out, fb.as<int>()));
		LAUNCH(*this, "octree_retrace", s, k_trace<false, false><<<retrace_grid(), 128, 0, s>>>(D, qq, hit_out, c, fb.as<int>()));
		return 0;
	}
	if(count) {
		LAUNCH(*this, name, s, k_trace<true, true><<<g, 128, 0, s>>>(D, qq, hit_out, c, fb.as<int>()));
		LAUNCH(*this, "octree_retrace", s, k_trace<true, false><<<retrace_grid(), 128, 0, s>>>(D, qq, hit_out, c, fb.as<int>()));
	} else {
		LAUNCH(*this, name, s, k_trace<false, true><<<g, 128, 0, s>>>(D, qq, hit_out, c, fb.as<int>()));
		LAUNCH(*this, "octree_retrace", s, k_trace<false, false><<<retrace_grid(), 128, 0, s>>>(D, qq, hit_out, c, fb.as<int>()));
	}
	return 0;
}

/* the light samples queued in sq (count at cnt[5]): any-hit traversal by
 * the tuning's kernel, then the octree retrace of the undecided ones */
int Renderer::shadow_rays(int cap, cudaStream_t s)
{
	return shadow_rays_on(sq.as<ShadowReq>(), counts.as<int>() + 5, cap, fbl, s);
}

/* the light samples q (count at *count, at most cap) on stream st, with the
 * fallback list fb */
int Renderer::shadow_rays_on(const ShadowReq *q, int *count, int cap, DevBuf &fb, cudaStream_t st)
{
	CK(fb.ensure(((size_t)cap + 1) * sizeof(int)), "fallback list");
	CK(cudaMemsetAsync(fb.p, 0, sizeof(int), st), "reset fallback list");
	int g = grid_for(cap, 128);
	float4 *a = acc.as<float4>();
	DevCounters *c = ctr.as<DevCounters>();
	int *f = fb.as<int>();
	if(prof_flags & 2)   /* counting the traversal work: every pass thread per segment */
		LAUNCH(*this, "shadow", st, k_shadow<true, true, true><<<g, 128, 0, st>>>(S, q, count, a, c, f));
	else if(cap <= tune.warp_segments)
		LAUNCH(*this, "shadow", st, k_shadow_warp<<<grid_for(cap, 4), 128, 0, st>>>(S, q, count, a, c, f));
	else if(tune.shadow_order)
		LAUNCH(*this, "shadow", st, k_shadow<true, false><<<g, 128, 0, st>>>(S, q, count, a, c, f));
	else
		LAUNCH(*this, "shadow", st, k_shadow<true><<<g, 128, 0, st>>>(S, q, count, a, c, f));
	LAUNCH(*this, "octree_retrace", st, k_shadow<false><<<retrace_grid(), 128, 0, st>>>(S, q, count, a, c, f));
	return 0;
}

/* the light-sample stream at the frame's priority: the device's greatest
 * when the frame runs on the priority stream (stream_priority 2), else the
 * least, as the caller's stream */
int Renderer::side_stream()
{
	int want = tune.stream_priority == 2 ? 1 : 0;
	if(xs && xs_priority == want) return 0;
	if(xs) {
		CK(cudaStreamSynchronize(xs), "light-sample stream");
		CK(cudaStreamDestroy(xs), "light-sample stream");
		xs = nullptr;
	}
	int least = 0, greatest = 0;
	CK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
	CK(cudaStreamCreateWithPriority(&xs, cudaStreamNonBlocking, want ? greatest : least), "light-sample stream");
	xs_priority = want;
	if(!xs_fork) {
		CK(cudaEventCreateWithFlags(&xs_fork, cudaEventDisableTiming), "light-sample stream event");
		for(int k = 0; k < 2; k++) CK(cudaEventCreateWithFlags(&xs_done[k], cudaEventDisableTiming), "light-sample stream event");
	}
	return 0;
}

int Renderer::trace_rays(const RayQueue &qq, int n, const char *name, bool count, cudaStream_t s, bool coherent)
{
	return trace_rays_with(S, qq, n, name, count, s, hits.as<int4>(), fbl, ctr.as<DevCounters>(), false, coherent);
}

/* photon passes: the photon buffers and counters */
int launch_trace(Renderer &R, const DScene &D, const RayQueue &q, int n, const char *name, cudaStream_t s)
{
	return R.trace_rays_with(D, q, n, name, false, s, R.phits.as<int4>(), R.pfbl, R.pctr.as<DevCounters>(), true);
}

int Renderer::photon_stream()
{
	int want = tune.stream_priority == 1 ? 1 : 0;
	if(ps && ps_priority == want) return 0;
	if(ps) {
		/* no photon work is in flight between frames */
		CK(cudaStreamSynchronize(ps), "photon stream");
		CK(cudaStreamDestroy(ps), "photon stream");
		ps = nullptr;
	}
	int least = 0, greatest = 0;
	CK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
	CK(cudaStreamCreateWithPriority(&ps, cudaStreamNonBlocking, want ? greatest : least), "photon stream");
	ps_priority = want;
	if(!ps_done) CK(cudaEventCreateWithFlags(&ps_done, cudaEventDisableTiming), "photon event");
	return 0;
}

int Renderer::gather_stream()
{
	if(gs) return 0;
	int least = 0, greatest = 0;
	CK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
	CK(cudaStreamCreateWithPriority(&gs, cudaStreamNonBlocking, least), "gather stream");
	CK(cudaEventCreateWithFlags(&gs_fork, cudaEventDisableTiming), "gather stream event");
	CK(cudaEventCreateWithFlags(&gs_done, cudaEventDisableTiming), "gather stream event");
	return 0;
}

int Renderer::priority_stream()
{
	if(hs) return 0;
	int least = 0, greatest = 0;
	CK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
	CK(cudaStreamCreateWithPriority(&hs, cudaStreamNonBlocking, greatest), "priority stream");
	CK(cudaEventCreateWithFlags(&hs_fork, cudaEventDisableTiming), "priority stream event");
	CK(cudaEventCreateWithFlags(&hs_join, cudaEventDisableTiming), "priority stream event");
	return 0;
}

/* a batch of jobs in one wavefront (sray_gpu_render_batch) */
int Renderer::render_batch(const sray_job *jobs, int n, cudaStream_t s)
{
	if(!loaded) return fail(SRAY_ESTATE, "no scene loaded");
	if(!jobs || n < 1 || n > 4096) return fail(SRAY_EINVAL, "a batch holds 1 to 4096 jobs");
	int nsc = sc.ranges.empty() ? 1 : (int)sc.ranges.size();
	if(nsc > 1 && opt.nrc) return fail(SRAY_EINVAL, "the radiance cache serves one scene: a scene set renders with nrc = 0");
	std::vector<DevJob> hj(n);
	std::vector<long> f0(n), f1(n);
	int64_t total = 0;
	long bt0 = 0, bt1 = 0;
	batch_scene.assign(n, 0);
	batch_caust.assign(n, 0);
	batch_gi.assign(n, 0);
	for(int j = 0; j < n; j++) {
		const sray_job &J = jobs[j];
		if(J.width <= 0 || J.height <= 0 || !J.fb) return fail(SRAY_EINVAL, "bad job");
		if(J.scene < 0 || J.scene >= nsc) return fail(SRAY_EINVAL, "job scene out of range");
		if(J.caust_photons < 0 || J.gi_photons < 0) return fail(SRAY_EINVAL, "negative job photon count");
		const Camera &cam = nsc > 1 ? sc.ranges[J.scene].cam : sc.cam;
		long shutter = cam.shutter;
		batch_scene[j] = J.scene;
		batch_caust[j] = J.caust_photons;
		batch_gi[j] = J.gi_photons;
		f0[j] = J.msec - shutter / 2;
		f1[j] = f0[j] + shutter;
		bt0 = j ? std::min(bt0, f0[j]) : f0[j];
		bt1 = j ? std::max(bt1, f1[j]) : f1[j];
		DevJob &d = hj[j];
		memset(&d, 0, sizeof d);
		d.pix0 = (int)total;
		d.width = J.width;
		d.height = J.height;
		d.t0 = (int)f0[j];
		d.cam_f = (float)(1.0 / tan(0.5 * cam.vfov));
		d.cam_xsz = (float)(cam.aspect * 2.0);   /* the camera's aspect, as for a single frame */
		d.cam_ysz = 2.0f;
		d.scene = J.scene;
		total += (int64_t)J.width * J.height;
		if(total > (1 << 27)) return fail(SRAY_EINVAL, "a batch holds at most 2^27 pixels");
	}
	in_batch = true;
	double tb = host_now_ms();
	int r = build_frame(bt0, bt1, s);
	host_time("host.build", tb);
	in_batch = false;
	if(r) return r;
	for(int j = 0; j < n; j++) hj[j].cam_base = hj[j].scene * nt;   /* its scene's camera in the frame's table */
	/* each job's photon maps, shot over its own interval by the photon
	 * thread while the batch's first bounces run (their gathers wait) */
	if(job_maps.size() < (size_t)n) job_maps.resize(n);   /* kept: their buffers are reused by the next batch */
	batch_t0.assign(f0.begin(), f0.end());
	batch_t1.assign(f1.begin(), f1.end());
	CK(djobs.upload(hj, s), "job table");
	CK(dmaps.ensure(2 * (size_t)n * sizeof(DPhotonMap)), "job photon maps");
	h2d += (int64_t)(hj.size() * sizeof(DevJob));
	CK(fbdev.ensure((size_t)total * 16), "batch framebuffer");
	CK(cudaStreamSynchronize(s), "job table");
	S.njobs = n;
	S.jobs = djobs.as<DevJob>();
	S.maps = nullptr;
	batch_npix = (int)total;
	double tr = host_now_ms();
	r = render_pixels(bt0, fbdev.as<float>(), 1, s, true);
	host_time("host.render", tr);
	S.njobs = 0;
	S.jobs = nullptr;
	S.maps = nullptr;
	batch_npix = 0;
	batch_t0.clear();
	batch_t1.clear();
	photons_ready = false;
	if(r) return r;
	for(int j = 0; j < n; j++)
		CK(cudaMemcpyAsync(jobs[j].fb, fbdev.as<float4>() + hj[j].pix0, (size_t)hj[j].width * hj[j].height * 16,
				cudaMemcpyDeviceToDevice, s), "job framebuffer");
	CK(cudaStreamSynchronize(s), "batch");
	return 0;
}

FaultState g_faults;
static Renderer *g_R = nullptr;
static std::string g_err;
static std::mutex g_mu;

static cudaStream_t as_stream(void *s) { return (cudaStream_t)s; }

}  // namespace sray

using namespace sray;

/* The context belongs to the device that was current at sray_gpu_init:
 * its buffers, streams and tables live there.  A call made while another
 * device is current is refused instead of launching on the wrong one. */
static int check_ctx_device()
{
	int dev = -1;
	cudaError_t e = cudaGetDevice(&dev);
	if(e != cudaSuccess) { g_err = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return SRAY_ECUDA; }
	if(dev != g_R->device) {
		char msg[160];
		snprintf(msg, sizeof msg, "CUDA device %d is current but the renderer was initialised on device %d; make it current first",
				dev, g_R->device);
		g_err = msg;
		return SRAY_ESTATE;
	}
	return 0;
}

#define NEED_CTX() do { \
		if(!g_R) { g_err = "sray_gpu_init has not been called"; return SRAY_ESTATE; } \
		if(int r_dev_ = check_ctx_device()) return r_dev_; \
	} while(0)

/* entry points of a single scene: a scene set renders through batches */
#define NEED_SINGLE() do { \
		if(g_R->sc.ranges.size() > 1) { g_err = "a scene set renders through sray_gpu_render_batch"; return SRAY_ESTATE; } \
	} while(0)

extern "C" {

void sray_default_opts(sray_opts *o)
{
	memset(o, 0, sizeof *o);
	o->width = 640; o->height = 480;
	o->min_samples = 1; o->max_samples = 1;
	o->max_var = 0.005f;
	o->min_energy = 0.0001f;
	o->shadow_samples = 1;
	o->diffuse_samples = 1;
	o->blk_sz = 48;
	o->iter = 7;
	o->fps = 30;
	o->gather_dist = 0.001f;
	o->photon_energy = 300.0f;
	o->scnoct_max_depth = 5; o->scnoct_max_items = 5;
	o->meshoct_max_depth = 7; o->meshoct_max_items = 14;
	o->gather_rcap = 0.5f;
	o->rng_paths = 1;
	o->seed = 0x5EED0001ull;
	o->nrc = 0;
	o->nrc_train_samples = 65536;
	o->nrc_max_rel_err = 0.05f;
	o->nrc_train_steps = 4;
}

static int check_opts(const sray_opts *o)
{
	if(!o) { g_err = "null options"; return SRAY_EINVAL; }
	if(o->width <= 0 || o->height <= 0 || (int64_t)o->width * o->height > (1 << 27)) { g_err = "bad image size"; return SRAY_EINVAL; }
	if(o->max_samples < 1 || o->max_samples > 64 || o->min_samples < 0) { g_err = "bad sample counts (1..64)"; return SRAY_EINVAL; }
	if(o->diffuse_samples < 0 || o->diffuse_samples > MAX_DS) { g_err = "diffuse samples must be 0..128"; return SRAY_EINVAL; }
	if(o->shadow_samples < 1) { g_err = "shadow samples must be >= 1"; return SRAY_EINVAL; }
	if(o->iter < 0 || o->iter > 13) { g_err = "iter must be 0..13"; return SRAY_EINVAL; }
	if(o->caust_photons < 0 || o->gi_photons < 0) { g_err = "negative photon count"; return SRAY_EINVAL; }
	if(o->caust_k < 0 || o->gi_k < 0) { g_err = "negative k"; return SRAY_EINVAL; }
	if(o->nrc < 0 || o->nrc > 2) { g_err = "nrc must be 0, 1 or 2"; return SRAY_EINVAL; }
	if(o->nrc_train_samples < 0 || o->nrc_train_samples > (1 << 22)) { g_err = "nrc_train_samples must be 0..4194304"; return SRAY_EINVAL; }
	if(o->nrc_train_steps < 0 || o->nrc_train_steps > 64) { g_err = "nrc_train_steps must be 0..64"; return SRAY_EINVAL; }
	if(!(o->nrc_max_rel_err >= 0.0f)) { g_err = "nrc_max_rel_err must be >= 0"; return SRAY_EINVAL; }
	if(o->nrc_fallback_samples < 0 || o->nrc_fallback_samples > MAX_DS) { g_err = "nrc_fallback_samples must be 0..128"; return SRAY_EINVAL; }
	return 0;
}

int sray_gpu_init(const sray_opts *opt)
{
	std::lock_guard<std::mutex> lk(g_mu);
	int r = check_opts(opt);
	if(r) return r;
	if(g_R) {
		if(g_R->pin) cudaFreeHost(g_R->pin);
		delete g_R;
		g_R = nullptr;
	}
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if(e != cudaSuccess) { g_err = std::string("no CUDA device: ") + cudaGetErrorString(e); return SRAY_ECUDA; }
	g_R = new Renderer;
	g_R->opt = *opt;
	g_R->device = dev;
	if(cudaDeviceGetAttribute(&g_R->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || g_R->nsm <= 0) g_R->nsm = 152;
	memset(&g_R->stats, 0, sizeof g_R->stats);
	e = cudaMallocHost(&g_R->pin, 16 * sizeof(int));
	if(e != cudaSuccess) {
		g_R->pin = nullptr;
		delete g_R;
		g_R = nullptr;
		g_err = std::string("pinned host words: ") + cudaGetErrorString(e);
		return SRAY_ECUDA;
	}
	return 0;
}

int sray_gpu_set_opts(const sray_opts *opt)
{
	NEED_CTX();
	int r = check_opts(opt);
	if(r) return r;
	bool geom = opt->meshoct_max_depth != g_R->opt.meshoct_max_depth || opt->meshoct_max_items != g_R->opt.meshoct_max_items;
	if(geom && g_R->loaded) { g_err = "mesh octree options change needs a scene reload"; return SRAY_ESTATE; }
	g_R->opt = *opt;
	g_R->photons_ready = false;
	if(g_R->built) g_R->fill_scene_desc();
	return 0;
}

static int load_scene_text(const char *xml, size_t len, const char *sidecar, int *used)
{
	Renderer &R = *g_R;
	R.loaded = false;
	R.built = false;
	R.photons_ready = false;
	if(!xml) { g_err = "null document"; return SRAY_EINVAL; }
	std::string err;
	bool u = false;
	if(!R.sc.load(xml, len, R.opt, err, sidecar, &u)) { g_err = err; return SRAY_ELOAD; }
	if(used) *used = u ? 1 : 0;
	int r = R.upload_scene(0);
	if(r) { g_err = R.err; return r; }
	R.loaded = true;
	return 0;
}

int sray_gpu_upload_scene(const sray_scene_desc *desc)
{
	NEED_CTX();
	Renderer &R = *g_R;
	R.loaded = false;
	R.built = false;
	R.photons_ready = false;
	if(!desc) { g_err = "null scene description"; return SRAY_EINVAL; }
	std::string err;
	if(!R.sc.from_desc(*desc, R.opt, err)) { g_err = err; return SRAY_EINVAL; }
	int r = R.upload_scene(0);
	if(r) { g_err = R.err; return r; }
	R.loaded = true;
	return 0;
}

int sray_gpu_load_scene_mem(const char *xml, size_t len)
{
	NEED_CTX();
	return load_scene_text(xml, len, nullptr, nullptr);
}

static int read_file(const char *path, std::string &buf)
{
	if(!path) { g_err = "null path"; return SRAY_EINVAL; }
	FILE *fp = fopen(path, "rb");
	if(!fp) { g_err = std::string("failed to open file: ") + path; return SRAY_ELOAD; }
	fseek(fp, 0, SEEK_END);
	long sz = ftell(fp);
	fseek(fp, 0, SEEK_SET);
	buf.assign(sz > 0 ? (size_t)sz : 0, '\0');
	size_t rd = sz > 0 ? fread(&buf[0], 1, (size_t)sz, fp) : 0;
	fclose(fp);
	buf.resize(rd);
	return 0;
}

int sray_gpu_load_scene(const char *path)
{
	NEED_CTX();
	std::string buf;
	int r = read_file(path, buf);
	if(r) return r;
	return load_scene_text(buf.data(), buf.size(), nullptr, nullptr);
}

int sray_gpu_load_scene_sidecar(const char *path, const char *sidecar, int *used)
{
	NEED_CTX();
	if(!sidecar) { g_err = "null side-car path"; return SRAY_EINVAL; }
	std::string buf;
	int r = read_file(path, buf);
	if(r) return r;
	return load_scene_text(buf.data(), buf.size(), sidecar, used);
}

int sray_gpu_load_scene_set(const char *const *xml_paths, int n)
{
	NEED_CTX();
	Renderer &R = *g_R;
	if(!xml_paths || n < 1 || n > 4096) { g_err = "a scene set holds 1 to 4096 documents"; return SRAY_EINVAL; }
	R.loaded = false;
	R.built = false;
	R.photons_ready = false;
	HostScene set;
	for(int k = 0; k < n; k++) {
		if(!xml_paths[k]) { g_err = "null document path"; return SRAY_EINVAL; }
		std::string buf, err;
		int r = read_file(xml_paths[k], buf);
		if(r) return r;
		HostScene one;
		if(!one.load(buf.data(), buf.size(), R.opt, err)) { g_err = std::string(xml_paths[k]) + ": " + err; return SRAY_ELOAD; }
		if(k == 0) set = std::move(one);
		else set.append_scene(std::move(one));
	}
	R.sc = std::move(set);
	int r = R.upload_scene(0);
	if(r) { g_err = R.err; return r; }
	R.loaded = true;
	return 0;
}

int sray_gpu_add_data_path(const char *dir)
{
	if(!dir) { g_err = "null directory"; return SRAY_EINVAL; }
	const char *cur = getenv("SRAY_DATA_PATH");
	std::string v = dir;
	if(cur) v += std::string(":") + cur;
	if(setenv("SRAY_DATA_PATH", v.c_str(), 1) != 0) { g_err = "setenv failed"; return SRAY_EINVAL; }
	return 0;
}

int sray_gpu_scene_info(int *n_objects, int *n_lights, int *n_materials, int64_t *n_triangles, int *n_unique_meshes)
{
	NEED_CTX();
	Renderer &R = *g_R;
	if(!R.loaded) { g_err = "no scene loaded"; return SRAY_ESTATE; }
	if(n_objects) *n_objects = (int)R.sc.objs.size();
	if(n_lights) *n_lights = (int)R.sc.lights.size();
	if(n_materials) *n_materials = (int)R.sc.mats.size();
	if(n_triangles) *n_triangles = R.sc.n_tris;
	if(n_unique_meshes) *n_unique_meshes = (int)R.sc.meshes.size();
	return 0;
}

int sray_gpu_build(long t0, long t1)
{
	NEED_CTX();
	NEED_SINGLE();
	int r = g_R->build_frame(t0, t1, 0);
	if(r) g_err = g_R->err;
	return r;
}

int sray_gpu_shoot_photons(long t0, long t1, int *caust_stored, int *gi_stored, void *stream)
{
	NEED_CTX();
	NEED_SINGLE();
	Renderer &R = *g_R;
	if(!R.built || R.t0 != (int)t0 || R.t1 != (int)t1) {
		int r = R.build_frame(t0, t1, as_stream(stream));
		if(r) { g_err = R.err; return r; }
	}
	int r = R.shoot(as_stream(stream), caust_stored, gi_stored);
	if(r) g_err = R.err;
	return r;
}

static void frame_interval(const Renderer &R, long msec, long *t0, long *t1)
{
	long shutter = R.sc.cam.shutter;
	*t0 = msec - shutter / 2;
	*t1 = *t0 + shutter;
}

int sray_gpu_render_pixels(long msec, float *fb, int fb_is_device, void *stream)
{
	NEED_CTX();
	NEED_SINGLE();
	if(!fb) { g_err = "null framebuffer"; return SRAY_EINVAL; }
	g_R->h2d = g_R->d2h = 0;
	int r = g_R->render_pixels(msec, fb, fb_is_device, as_stream(stream));
	if(r) g_err = g_R->err;
	return r;
}

static int render_frame(Renderer &R, long msec, float *fb, int fb_is_device, cudaStream_t s)
{
	long t0, t1;
	frame_interval(R, msec, &t0, &t1);
	long long l0 = R.launch_count;
	R.h2d = R.d2h = 0;
	/* stream_priority 2: the frame runs on an internal stream of the
	 * greatest priority, after the caller's stream's earlier work and
	 * before its later work */
	cudaStream_t rs = s;
	int r = 0;
	if(R.tune.stream_priority == 2) {
		r = R.priority_stream();
		if(!r && (cudaEventRecord(R.hs_fork, s) != cudaSuccess || cudaStreamWaitEvent(R.hs, R.hs_fork, 0) != cudaSuccess))
			r = R.fail(SRAY_ECUDA, "priority stream fork");
		rs = R.hs;
	}
	if(!r) r = R.build_frame(t0, t1, rs);
	if(!r) r = R.render_pixels(msec, fb, fb_is_device, rs, true);
	if(rs != s && (cudaEventRecord(R.hs_join, rs) != cudaSuccess || cudaStreamWaitEvent(s, R.hs_join, 0) != cudaSuccess) && !r)
		r = R.fail(SRAY_ECUDA, "priority stream join");
	if(r) g_err = R.err;
	else R.stats.kernel_launches = (int)(R.launch_count - l0);
	return r;
}

int sray_gpu_render(long msec, float *fb, int fb_is_device, void *stream)
{
	NEED_CTX();
	NEED_SINGLE();
	Renderer &R = *g_R;
	if(!R.loaded) { g_err = "no scene loaded"; return SRAY_ESTATE; }
	if(!fb) { g_err = "null framebuffer"; return SRAY_EINVAL; }
	return render_frame(R, msec, fb, fb_is_device, as_stream(stream));
}

static int check_tuning(const sray_tuning *t)
{
	if(!t) { g_err = "null tuning"; return SRAY_EINVAL; }
	if(t->render_tail < 0 || t->render_tail > (1 << 26)) { g_err = "render_tail must be 0..2^26"; return SRAY_EINVAL; }
	if(t->pool_blocks_per_sm < 1 || t->pool_blocks_per_sm > 16) { g_err = "pool_blocks_per_sm must be 1..16"; return SRAY_EINVAL; }
	if(t->photon_tail < 0 || t->photon_tail > (1 << 26)) { g_err = "photon_tail must be 0..2^26"; return SRAY_EINVAL; }
	if(t->shadow_order != 0 && t->shadow_order != 1) { g_err = "shadow_order must be 0 or 1"; return SRAY_EINVAL; }
	if(t->stream_priority < 0 || t->stream_priority > 2) { g_err = "stream_priority must be 0, 1 or 2"; return SRAY_EINVAL; }
	if(t->warp_rays < 0 || t->warp_rays > (1 << 24)) { g_err = "warp_rays must be 0..2^24"; return SRAY_EINVAL; }
	if(t->warp_segments < 0 || t->warp_segments > (1 << 24)) { g_err = "warp_segments must be 0..2^24"; return SRAY_EINVAL; }
	if(t->side_gather < 0 || t->side_gather > 2) { g_err = "side_gather must be 0, 1 or 2"; return SRAY_EINVAL; }
	if(t->sort_rays < 0) { g_err = "sort_rays must be >= 0"; return SRAY_EINVAL; }
	if(t->side_shadow != 0 && t->side_shadow != 1) { g_err = "side_shadow must be 0 or 1"; return SRAY_EINVAL; }
	if(t->queue_depth != 0 && (t->queue_depth < 1024 || t->queue_depth > (1 << 27))) {
		g_err = "queue_depth must be 0 or 1024..2^27";
		return SRAY_EINVAL;
	}
	return 0;
}

int sray_gpu_get_tuning(sray_tuning *t)
{
	NEED_CTX();
	if(!t) { g_err = "null tuning"; return SRAY_EINVAL; }
	*t = g_R->tune;
	return 0;
}

int sray_gpu_set_tuning(const sray_tuning *t)
{
	NEED_CTX();
	int r = check_tuning(t);
	if(r) return r;
	g_R->tune = *t;
	return 0;
}

/* Coordinate descent over the tunables: each field in turn takes each of
 * its candidate values with the others at the best found so far; a trial is
 * one warm-up frame and `frames` frames timed with CUDA events on the
 * stream.  Trials already measured are not repeated. */
int sray_gpu_autotune(long msec, float *fb, int frames, void *stream, sray_tuning *best, float *best_ms,
		sray_tune_trial *log, int log_cap, int *n_log)
{
	NEED_CTX();
	NEED_SINGLE();
	Renderer &R = *g_R;
	if(!R.loaded) { g_err = "no scene loaded"; return SRAY_ESTATE; }
	if(!fb || frames < 1) { g_err = "bad arguments"; return SRAY_EINVAL; }
	cudaStream_t s = as_stream(stream);
	static const int tails[] = {0, 2048, 8192, 32768, 131072};
	static const int pools[] = {2, 4, 8, 16};
	static const int ptails[] = {16384, 65536, 262144, 1048576};
	static const int binary[] = {0, 1}, prios[] = {0, 1, 2}, wrays[] = {0, 4096, 16384, 65536, 262144};
	static const int depths[] = {0, 1 << 16, 1 << 18, 1 << 20};
	struct Knob { int sray_tuning::*field; const int *vals; int n; };
	const Knob knobs[] = {{&sray_tuning::render_tail, tails, 5}, {&sray_tuning::pool_blocks_per_sm, pools, 4},
		{&sray_tuning::photon_tail, ptails, 4}, {&sray_tuning::shadow_order, binary, 2}, {&sray_tuning::stream_priority, prios, 3},
		{&sray_tuning::warp_rays, wrays, 5}, {&sray_tuning::warp_segments, wrays, 5}, {&sray_tuning::queue_depth, depths, 4},
		{&sray_tuning::side_gather, binary, 2}, {&sray_tuning::side_shadow, binary, 2}};
	std::vector<sray_tune_trial> done;
	cudaEvent_t e0, e1;
	if(cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) { g_err = "autotune events"; return SRAY_ECUDA; }
	auto trial = [&](const sray_tuning &t, float *ms) -> int {
		for(const sray_tune_trial &d : done) {
			if(memcmp(&d.tuning, &t, sizeof t) == 0) {
				*ms = d.ms_per_frame;
				return 0;
			}
		}
		R.tune = t;
		int r = render_frame(R, msec, fb, 1, s);
		if(r) return r;
		/* two groups of `frames` frames, the slower group counting: a
		 * choice whose frames vary (two streams of equal priority taking
		 * turns at random) is judged by its bad runs */
		float worst = 0.0f;
		for(int grp = 0; grp < 2; grp++) {
			cudaEventRecord(e0, s);
			for(int i = 0; i < frames && !r; i++) r = render_frame(R, msec, fb, 1, s);
			cudaEventRecord(e1, s);
			if(r) return r;
			if(cudaEventSynchronize(e1) != cudaSuccess) { g_err = "autotune timing"; return SRAY_ECUDA; }
			float t_ms = 0.0f;
			cudaEventElapsedTime(&t_ms, e0, e1);
			worst = std::max(worst, t_ms);
		}
		sray_tune_trial tr;
		memset(&tr, 0, sizeof tr);
		tr.tuning = t;
		tr.ms_per_frame = worst / (float)frames;
		done.push_back(tr);
		*ms = tr.ms_per_frame;
		return 0;
	};
	sray_tuning cur = R.tune;
	float cur_ms = 0.0f;
	int r = trial(cur, &cur_ms);
	for(const Knob &k : knobs) {
		for(int i = 0; i < k.n && !r; i++) {
			sray_tuning t = cur;
			t.*(k.field) = k.vals[i];
			float ms = 0.0f;
			r = trial(t, &ms);
			if(!r && ms < cur_ms) {
				cur = t;
				cur_ms = ms;
			}
		}
		if(r) break;
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	R.tune = cur;
	if(r) return r;
	if(best) *best = cur;
	if(best_ms) *best_ms = cur_ms;
	if(n_log) *n_log = (int)done.size();
	for(int i = 0; log && i < log_cap && i < (int)done.size(); i++) log[i] = done[i];
	return 0;
}

int sray_gpu_autotune_batch(const sray_job *jobs, int n, int frames, void *stream, sray_tuning *best, float *best_ms,
		sray_tune_trial *log, int log_cap, int *n_log)
{
	NEED_CTX();
	Renderer &R = *g_R;
	if(!R.loaded) { g_err = "no scene loaded"; return SRAY_ESTATE; }
	if(!jobs || n < 1 || frames < 1) { g_err = "bad arguments"; return SRAY_EINVAL; }
	cudaStream_t s = as_stream(stream);
	/* the configuration's sweep (64k, 256k, 1M primary rays per wave), then
	 * deeper waves for batches whose memory allows them */
	static const int depths[] = {1 << 16, 1 << 18, 1 << 20, 1 << 22, 1 << 24};
	const int nd = (int)(sizeof depths / sizeof depths[0]);
	/* thread per ray; warp per ray in the tails; warp per ray everywhere */
	static const int modes[] = {0, 16384, 1 << 24};
	std::vector<sray_tune_trial> done;
	cudaEvent_t e0, e1;
	if(cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) { g_err = "autotune events"; return SRAY_ECUDA; }
	sray_tuning base = R.tune, cur = R.tune;
	float cur_ms = 0.0f;
	int r = 0;
	/* the pairs of depth and mode, then the best pair with the shading
	 * tree's tail in the persistent pool launch (below 32k and 128k rays in
	 * flight) */
	static const int tails[] = {1 << 15, 1 << 17};
	for(int k = 0; k < nd * 3 + 2 && !r; k++) {
		sray_tuning t = base;
		if(k < nd * 3) {
			t.queue_depth = depths[k / 3];
			t.warp_rays = t.warp_segments = modes[k % 3];
			t.render_tail = 0;
		} else {
			t = cur;
			t.render_tail = tails[k - nd * 3];
		}
		R.tune = t;
		r = R.render_batch(jobs, n, s);
		if(r) { g_err = R.err; break; }
		cudaEventRecord(e0, s);
		for(int i = 0; i < frames && !r; i++) r = R.render_batch(jobs, n, s);
		cudaEventRecord(e1, s);
		if(r) { g_err = R.err; break; }
		if(cudaEventSynchronize(e1) != cudaSuccess) { g_err = "autotune timing"; r = SRAY_ECUDA; break; }
		float t_ms = 0.0f;
		cudaEventElapsedTime(&t_ms, e0, e1);
		sray_tune_trial tr;
		memset(&tr, 0, sizeof tr);
		tr.tuning = t;
		tr.ms_per_frame = t_ms / (float)frames;
		done.push_back(tr);
		if(done.size() == 1 || tr.ms_per_frame < cur_ms) {
			cur = t;
			cur_ms = tr.ms_per_frame;
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	R.tune = r ? base : cur;
	if(r) return r;
	if(best) *best = cur;
	if(best_ms) *best_ms = cur_ms;
	if(n_log) *n_log = (int)done.size();
	for(int i = 0; log && i < log_cap && i < (int)done.size(); i++) log[i] = done[i];
	return 0;
}

int sray_gpu_render_batch(const sray_job *jobs, int n, void *stream)
{
	NEED_CTX();
	Renderer &R = *g_R;
	long long l0 = R.launch_count;
	R.h2d = R.d2h = 0;
	int r = R.render_batch(jobs, n, as_stream(stream));
	if(r) g_err = R.err;
	else R.stats.kernel_launches = (int)(R.launch_count - l0);
	return r;
}

int sray_gpu_cast_rays(int n, const float *orig, const float *dir, const int *time, int *obj, int *prim, float *t,
		unsigned char *tie, void *stream)
{
	NEED_CTX();
	NEED_SINGLE();
	Renderer &R = *g_R;
	if(!R.built) { g_err = "acceleration structures not built"; return SRAY_ESTATE; }
	if(n < 0 || (n > 0 && (!orig || !dir || !obj || !prim || !t || !tie))) { g_err = "bad arguments"; return SRAY_EINVAL; }
	if(n == 0) return 0;
	cudaStream_t s = as_stream(stream);
	cudaError_t e = R.ctr.ensure(sizeof(DevCounters));
	if(e == cudaSuccess) e = cudaMemsetAsync(R.ctr.p, 0, sizeof(DevCounters), s);
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	k_cast<<<grid_for(n, 128), 128, 0, s>>>(R.S, n, orig, dir, time, obj, prim, t, tie, R.ctr.as<DevCounters>());
	DevCounters hc;
	e = cudaMemcpyAsync(&hc, R.ctr.p, sizeof hc, cudaMemcpyDeviceToHost, s);
	if(e == cudaSuccess) e = cudaStreamSynchronize(s);
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	if(hc.overflow) { g_err = "traversal stack overflow"; return SRAY_EDEVICE; }
	return 0;
}

int sray_gpu_primary_hits(long msec, int *obj, int *prim, float *t, unsigned char *tie, void *stream)
{
	NEED_CTX();
	NEED_SINGLE();
	Renderer &R = *g_R;
	if(!R.loaded) { g_err = "no scene loaded"; return SRAY_ESTATE; }
	if(!obj || !prim || !t || !tie) { g_err = "bad arguments"; return SRAY_EINVAL; }
	cudaStream_t s = as_stream(stream);
	long t0, t1;
	frame_interval(R, msec, &t0, &t1);
	if(!R.built || R.t0 != (int)t0 || R.t1 != (int)t1) {
		int r = R.build_frame(t0, t1, s);
		if(r) { g_err = R.err; return r; }
	}
	int npix = R.opt.width * R.opt.height;
	if(R.ensure_queue(0, npix)) { g_err = R.err; return SRAY_ECUDA; }
	cudaError_t e = R.hits.ensure((size_t)npix * 16);
	if(e == cudaSuccess) e = R.ctr.ensure(sizeof(DevCounters));
	if(e == cudaSuccess) e = R.counts.ensure(64 * sizeof(int));
	if(e == cudaSuccess) e = cudaMemsetAsync(R.ctr.p, 0, sizeof(DevCounters), s);
	if(e == cudaSuccess) e = R.acc.ensure((size_t)npix * 16);
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	int *cnt = R.counts.as<int>();
	e = cudaMemcpyAsync(cnt + 3, &npix, sizeof(int), cudaMemcpyHostToDevice, s);
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	R.q[0].count = cnt + 0;
	k_camera<<<grid_for(npix, 256), 256, 0, s>>>(R.S, nullptr, 0, npix, 0, 1, R.q[0], R.acc.as<float4>(), R.ctr.as<DevCounters>());
	if(R.trace_rays(R.q[0], npix, "trace", false, s, true)) { g_err = R.err; return SRAY_ECUDA; }
	k_primary_hits<<<grid_for(npix, 256), 256, 0, s>>>(R.S, R.q[0], R.hits.as<int4>(), obj, prim, t, tie);
	DevCounters hc;
	e = cudaMemcpyAsync(&hc, R.ctr.p, sizeof hc, cudaMemcpyDeviceToHost, s);
	if(e == cudaSuccess) e = cudaStreamSynchronize(s);
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	if(hc.overflow) { g_err = "traversal stack overflow"; return SRAY_EDEVICE; }
	return 0;
}

int sray_gpu_photon_gather(int which, int n, const float *pos, const float *norm, float *out, void *stream)
{
	NEED_CTX();
	Renderer &R = *g_R;
	if(!R.photons_ready) { g_err = "photon maps not built"; return SRAY_ESTATE; }
	if((which != 0 && which != 1) || n < 0 || (n > 0 && (!pos || !norm || !out))) { g_err = "bad arguments"; return SRAY_EINVAL; }
	if(n == 0) return 0;
	cudaStream_t s = as_stream(stream);
	cudaError_t e = R.gq.ensure((size_t)n * sizeof(GatherReq));
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	k_pack_gather<<<grid_for(n, 256), 256, 0, s>>>(which, n, pos, norm, R.gq.as<GatherReq>());
	k_gather_points<<<grid_for(n, GATHER_WARPS), GATHER_WARPS * 32, 0, s>>>(R.S, R.gq.as<GatherReq>(), n, out);
	e = cudaStreamSynchronize(s);
	if(e == cudaSuccess) e = cudaGetLastError();
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	return 0;
}

/* Fixed staging for sray_gpu_photon_gather_noalloc.  Host code must not
 * take this symbol as a device address: the device address is looked up
 * once per device with cudaGetSymbolAddress while that device is current. */
static __device__ __align__(256) GatherReq g_noalloc_req[SRAY_NOALLOC_MAX_POINTS];
static GatherReq *g_noalloc_addr[64];
static std::mutex g_noalloc_mu;

/* the staging's address on the renderer's device (which the caller has
 * made current: NEED_CTX refuses calls from another device) */
static int noalloc_requests(int dev, GatherReq **out)
{
	if(dev < 0 || dev >= 64) { g_err = "device index out of range for the fixed gather staging"; return SRAY_EINVAL; }
	std::lock_guard<std::mutex> lk(g_noalloc_mu);
	if(!g_noalloc_addr[dev]) {
		void *p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_req);
		if(e != cudaSuccess || !p) {
			g_err = std::string("cudaGetSymbolAddress of the gather staging: ") + cudaGetErrorString(e);
			return SRAY_ECUDA;
		}
		g_noalloc_addr[dev] = (GatherReq *)p;
	}
	*out = g_noalloc_addr[dev];
	return 0;
}

int sray_gpu_photon_gather_noalloc(int which, int n, const float *pos, const float *norm, float *out, void *stream)
{
	NEED_CTX();
	Renderer &R = *g_R;
	if(!R.photons_ready) { g_err = "photon maps not built"; return SRAY_ESTATE; }
	if((which != 0 && which != 1) || n < 0 || (n > 0 && (!pos || !norm || !out))) { g_err = "bad arguments"; return SRAY_EINVAL; }
	if(n > SRAY_NOALLOC_MAX_POINTS) {
		char msg[160];
		snprintf(msg, sizeof msg, "sray_gpu_photon_gather_noalloc: %d points exceed its fixed capacity of %d; split the call",
				n, SRAY_NOALLOC_MAX_POINTS);
		g_err = msg;
		return SRAY_EINVAL;
	}
	if(n == 0) return 0;
	GatherReq *req = nullptr;
	int r = noalloc_requests(R.device, &req);
	if(r) return r;
	cudaStream_t s = as_stream(stream);
	k_pack_gather<<<grid_for(n, 256), 256, 0, s>>>(which, n, pos, norm, req);
	k_gather_points<<<grid_for(n, GATHER_WARPS), GATHER_WARPS * 32, 0, s>>>(R.S, req, n, out);
	cudaError_t e = cudaStreamSynchronize(s);
	if(e == cudaSuccess) e = cudaGetLastError();
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	return 0;
}

int sray_gpu_get_photons(int which, float *out, int cap, int *n_out)
{
	NEED_CTX();
	Renderer &R = *g_R;
	const PhotonBufs &P = which ? R.gi : R.caust;
	int n = P.map.n;
	if(n_out) *n_out = n;
	if(!out || cap <= 0 || n == 0) return 0;
	int m = n < cap ? n : cap;
	std::vector<DevPhoton> h(m);
	cudaError_t e = cudaMemcpy(h.data(), P.ph.p, (size_t)m * sizeof(DevPhoton), cudaMemcpyDeviceToHost);
	if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	for(int i = 0; i < m; i++) {
		float *f = out + (size_t)i * 16;
		f[0] = h[i].p[0]; f[1] = h[i].p[1]; f[2] = h[i].p[2];
		f[3] = h[i].d[0]; f[4] = h[i].d[1]; f[5] = h[i].d[2];
		f[6] = h[i].n[0]; f[7] = h[i].n[1]; f[8] = h[i].n[2];
		f[9] = h[i].p[3]; f[10] = h[i].d[3]; f[11] = h[i].n[3]; f[12] = 0.0f;
		f[13] = f[14] = f[15] = 0.0f;
	}
	return 0;
}

/* PhotonMap::dump (src/pmap.cc:180-205): "energy %f", then per photon
 * "<pos> <dir> <norm> <col>" with %f components */
int sray_gpu_dump_photons(int which, const char *path)
{
	NEED_CTX();
	Renderer &R = *g_R;
	if(!path || (which != 0 && which != 1)) { g_err = "bad arguments"; return SRAY_EINVAL; }
	const PhotonBufs &P = which ? R.gi : R.caust;
	int n = P.map.n;
	std::vector<DevPhoton> h(n > 0 ? n : 0);
	if(n > 0) {
		cudaError_t e = cudaMemcpy(h.data(), P.ph.p, (size_t)n * sizeof(DevPhoton), cudaMemcpyDeviceToHost);
		if(e != cudaSuccess) { g_err = cudaGetErrorString(e); return SRAY_ECUDA; }
	}
	FILE *fp = fopen(path, "w");
	if(!fp) { g_err = std::string("failed to dump photon map: ") + path; return SRAY_EIO; }
	fprintf(fp, "energy %f\n", R.opt.photon_energy);
	for(const DevPhoton &p : h) {
		fprintf(fp, "<%f %f %f> ", p.p[0], p.p[1], p.p[2]);
		fprintf(fp, "<%f %f %f> ", p.d[0], p.d[1], p.d[2]);
		fprintf(fp, "<%f %f %f> ", p.n[0], p.n[1], p.n[2]);
		fprintf(fp, "<%f %f %f>\n", p.p[3], p.d[3], p.n[3]);
	}
	if(fclose(fp) != 0) { g_err = std::string("failed to write photon map: ") + path; return SRAY_EIO; }
	return 0;
}

/* PhotonMap::restore (src/pmap.cc:207-251): powers scaled by this
 * renderer's photon_energy over the dump's; the map is built on the device
 * over the current frame's scene bounds (sray_gpu_build first) */
int sray_gpu_restore_photons(int which, const char *path, int *n_out)
{
	NEED_CTX();
	Renderer &R = *g_R;
	if(!path || (which != 0 && which != 1)) { g_err = "bad arguments"; return SRAY_EINVAL; }
	if(!R.built) { g_err = "acceleration structures not built"; return SRAY_ESTATE; }
	FILE *fp = fopen(path, "r");
	if(!fp) { g_err = std::string("failed to open photon dump: ") + path; return SRAY_EIO; }
	float prev = 0.0f;
	if(fscanf(fp, "energy %f\n", &prev) < 1 || !(prev > 0.0f)) {
		fclose(fp);
		g_err = std::string("failed to restore photon dump: ") + path;
		return SRAY_ELOAD;
	}
	float scale = R.opt.photon_energy / prev;
	std::vector<DevPhoton> h;
	for(;;) {
		float v[12];
		int res = fscanf(fp, "<%f %f %f> <%f %f %f> <%f %f %f> <%f %f %f>\n", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &v[7],
				&v[8], &v[9], &v[10], &v[11]);
		if(res == EOF) break;
		bool finite = res == 12;
		for(int k = 0; k < 12 && finite; k++) finite = std::isfinite(v[k]);
		if(!finite) {
			fclose(fp);
			g_err = std::string("failed to restore photon dump: ") + path;
			return SRAY_ELOAD;
		}
		DevPhoton p;
		p.p[0] = v[0]; p.p[1] = v[1]; p.p[2] = v[2]; p.p[3] = v[9] * scale;
		p.d[0] = v[3]; p.d[1] = v[4]; p.d[2] = v[5]; p.d[3] = v[10] * scale;
		p.n[0] = v[6]; p.n[1] = v[7]; p.n[2] = v[8]; p.n[3] = v[11] * scale;
		h.push_back(p);
	}
	fclose(fp);
	if(h.size() > (size_t)INT_MAX / 2) { g_err = "photon dump too large"; return SRAY_EINVAL; }
	int r = photon_map_restore(R, which, h, 0);
	if(r) { g_err = R.err; return r; }
	R.photons_ready = true;
	R.fill_scene_desc();
	if(n_out) *n_out = (int)h.size();
	return 0;
}

int sray_gpu_get_stats(sray_stats *st)
{
	NEED_CTX();
	if(!st) { g_err = "null stats"; return SRAY_EINVAL; }
	*st = g_R->stats;
	st->photons_stored = (int64_t)g_R->caust.map.n + g_R->gi.map.n;
	return 0;
}

int sray_gpu_nrc_stats(sray_nrc_stats *st)
{
	NEED_CTX();
	if(!st) { g_err = "null stats"; return SRAY_EINVAL; }
	Renderer &R = *g_R;
	memset(st, 0, sizeof *st);
	st->frames = R.nrc_frames;
	st->vertices = R.nrc_last_vertices;
	st->cached = R.nrc_last_cached;
	st->train_samples = R.nrc_last_train;
	st->val_samples = R.nrc_last_val;
	st->regions = NRC_REGIONS;
	if(R.nrc_regions_ready) {
		float sm[4];
		cudaError_t e = cudaMemcpy(sm, R.nrc_regions.as<NrcRegionStats>()->summary, sizeof sm, cudaMemcpyDeviceToHost);
		if(e != cudaSuccess) { g_err = std::string("radiance cache stats: ") + cudaGetErrorString(e); return SRAY_ECUDA; }
		st->regions_validated = (int)sm[0];
		st->regions_cached = (int)sm[1];
		st->val_rel_err = sm[2];
		float *lp = nrc_loss_ptr();
		if(lp && cudaMemcpy(&st->loss, lp, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) st->loss = -1.0f;
	}
	return 0;
}

int sray_gpu_nrc_reset(uint64_t seed)
{
	NEED_CTX();
	Renderer &R = *g_R;
	int r = sray_nrc_reset(seed);
	if(r) { g_err = std::string("radiance cache: ") + nrc_error(); return r; }
	R.nrc_frames = 0;
	R.nrc_expect = 0;
	R.nrc_last_train = R.nrc_last_val = 0;
	R.nrc_last_vertices = R.nrc_last_cached = 0;
	if(R.nrc_regions_ready) {
		r = R.nrc_reset_regions(0);
		if(r) { g_err = R.err; return r; }
		if(cudaDeviceSynchronize() != cudaSuccess) { g_err = "radiance cache reset"; return SRAY_ECUDA; }
	}
	return 0;
}

int sray_gpu_set_profiling(int flags)
{
	NEED_CTX();
	g_R->prof_flags = flags;
	return 0;
}

int sray_gpu_kernel_times(char *names, size_t names_cap, double *ms, int64_t *launches, int max, int *n_out, int reset)
{
	NEED_CTX();
	Renderer &R = *g_R;
	std::lock_guard<std::mutex> lk(R.prof_mu);
	int n = (int)R.ktimes.size();
	if(n_out) *n_out = n;
	size_t off = 0;
	for(int i = 0; i < n && i < max; i++) {
		if(ms) ms[i] = R.ktimes[i].ms;
		if(launches) launches[i] = R.ktimes[i].launches;
		if(names) {
			const std::string &nm = R.ktimes[i].name;
			if(off + nm.size() + 1 <= names_cap) {
				memcpy(names + off, nm.c_str(), nm.size() + 1);
				off += nm.size() + 1;
			}
		}
	}
	if(reset) for(auto &k : R.ktimes) { k.ms = 0.0; k.launches = 0; }
	return 0;
}

int sray_gpu_set_faults(const sray_faults *f)
{
	if(!f) { g_err = "null fault settings"; return SRAY_EINVAL; }
	if(f->fail_alloc_after < -1 || f->queue_cap < 0 || f->pool_spin_limit < 0 || f->photon_group < 0) {
		g_err = "bad fault settings";
		return SRAY_EINVAL;
	}
	g_faults.alloc_left.store(f->fail_alloc_after);
	g_faults.queue_cap.store(f->queue_cap);
	g_faults.spin_limit.store(f->pool_spin_limit);
	g_faults.photon_group.store(f->photon_group);
	return 0;
}

int sray_gpu_last_error(char *buf, size_t cap)
{
	if(!buf || cap == 0) return SRAY_EINVAL;
	size_t n = g_err.size() < cap - 1 ? g_err.size() : cap - 1;
	memcpy(buf, g_err.data(), n);
	buf[n] = 0;
	return 0;
}

void sray_gpu_shutdown(void)
{
	std::lock_guard<std::mutex> lk(g_mu);
	if(!g_R) return;
	Renderer &R = *g_R;
	if(R.photon_thread.joinable()) R.photon_thread.join();
	for(Renderer::JobMaps &jm : R.job_maps) {
		PhotonBufs *jp[] = {&jm.caust, &jm.gi};
		for(PhotonBufs *p : jp) {
			DevBuf *pbufs[] = {&p->ph, &p->cells, &p->tmp_ph, &p->keys, &p->keys2, &p->vals, &p->vals2, &p->lin, &p->hist, &p->scan};
			for(DevBuf *b : pbufs) b->release();
		}
	}
	R.djobs.release();
	R.dmaps.release();
	DevBuf *bufs[] = {&R.mnodes, &R.mtris, &R.mprim, &R.tri_pos, &R.tri_attr, &R.objs, &R.mats, &R.texs, &R.texels, &R.lights,
		&R.anims, &R.key_t, &R.key_v,
		&R.snodes, &R.sslots,
		&R.xf, &R.light_pos, &R.cam_m, &R.qbuf[0], &R.qbuf[1], &R.hits, &R.gq, &R.sq, &R.acc, &R.hist, &R.sums,
		&R.active[0], &R.active[1], &R.spp, &R.fbdev, &R.ctr, &R.counts, &R.bnodes, &R.btris, &R.bprim, &R.bhome,
		&R.fbl, &R.tnodes, &R.ohome, &R.pool_ready, &R.pqbuf[0], &R.pqbuf[1], &R.phits, &R.pfbl, &R.pcounts, &R.pctr,
		&R.pw_jobs, &R.pw_prefix, &R.pw_scale, &R.pw_bits, &R.pw_cov, &R.pw_pix, &R.pw_out, &R.pw_valid,
		&R.pw_part, &R.pw_tiles, &R.pw_bounds, &R.pw_offs, &R.pw_ph, &R.pw_sorted, &R.pw_grids, &R.pw_morton, &R.pw_cellbase,
		&R.pw_keys, &R.pw_lin, &R.pw_cells, &R.pw_hist, &R.qsbuf, &R.rs_keys, &R.rs_hist, &R.rs_part, &R.sq2, &R.gq2, &R.fbs[0], &R.fbs[1],
		&R.pqsbuf, &R.ps_keys, &R.ps_hist, &R.ps_part,
		&R.nrc_qx, &R.nrc_qw, &R.nrc_rx, &R.nrc_rt, &R.nrc_ry, &R.nrc_regions};
	if(R.ps) cudaStreamSynchronize(R.ps);
	if(R.xs) cudaStreamSynchronize(R.xs);
	for(DevBuf *b : bufs) b->release();
	PhotonBufs *pb[] = {&R.caust, &R.gi};
	for(PhotonBufs *p : pb) {
		DevBuf *pbufs[] = {&p->ph, &p->cells, &p->tmp_ph, &p->keys, &p->keys2, &p->vals, &p->vals2, &p->lin, &p->hist, &p->scan};
		for(DevBuf *b : pbufs) b->release();
	}
	if(R.pin) cudaFreeHost(R.pin);
	R.pin = nullptr;
	if(R.ps_done) cudaEventDestroy(R.ps_done);
	if(R.ps) cudaStreamDestroy(R.ps);
	if(R.gs) {
		cudaStreamSynchronize(R.gs);
		cudaStreamDestroy(R.gs);
		cudaEventDestroy(R.gs_fork);
		cudaEventDestroy(R.gs_done);
	}
	if(R.xs) {
		cudaStreamSynchronize(R.xs);
		cudaStreamDestroy(R.xs);
		cudaEventDestroy(R.xs_fork);
		cudaEventDestroy(R.xs_done[0]);
		cudaEventDestroy(R.xs_done[1]);
	}
	R.gq_side.release();
	if(R.hs) {
		cudaStreamSynchronize(R.hs);
		cudaStreamDestroy(R.hs);
		cudaEventDestroy(R.hs_fork);
		cudaEventDestroy(R.hs_join);
	}
	delete g_R;
	g_R = nullptr;
}

}  /* extern "C" */
