/* dev_common.cuh -- device routines shared by the render and photon kernels:
 * the scene descriptor, float intersection tests written in the reference's
 * operation order, the two-level octree traversal (closest hit and any
 * hit), surface-point reconstruction and light sampling.
 *
 * All files that include this are compiled with -fmad=false (no FMA
 * contraction) and IEEE division/square root, so every float operation
 * below rounds exactly like the CPU oracle's float path.
 */
#ifndef SRAY_DEV_COMMON_CUH_
#define SRAY_DEV_COMMON_CUH_

#include <stdint.h>
#include <float.h>
#include <cuda_runtime.h>
#include "sray_device.h"
#include "sray_rng.h"

namespace sray {

/* photon map on the device: photons in Morton order of their grid cell,
 * a dense table of (first, count) per cell */
struct DPhotonMap {
	const DevPhoton *ph;
	const uint2 *cells;       /* per linear cell: first photon, count */
	int n;
	int dims[3];
	float org[3];
	float cell;
	int k;                    /* 0 = fixed-radius range gather, >0 = k nearest */
	double range;             /* query radius as the kd-tree sees it (float-rounded) */
	float inv_area;           /* range mode: 1 / (pi r^2) of the unrounded radius */
	float range_f;            /* the same radius as a float */
	float r2_hi, r2_lo;       /* range_f^2 exactly, as an unevaluated float sum */
	float screen;             /* float squared distances above this are out of range */
};

/* The radiance cache as the shading kernels see it.  At a final-gather
 * vertex (a Phong hit with the global map on) the network's inputs are the
 * position scaled to the scene box, the normal and the incident direction,
 * each mapped to [0, 1]; the region of a vertex is its cell of an
 * NRC_GRID^3 grid over the box.  A vertex in a region the network serves
 * becomes a query (inputs, weight, accumulator slot) instead of diffuse
 * rays; a vertex the frame's hash selects also becomes a training or
 * validation record whose target (the plain final gather's estimate,
 * without the vertex's weight and kd) accumulates in slot t0 + record. */
#define NRC_GRID 8
#define NRC_VAL_RAYS 8                /* final-gather rays (at least) of a validation record */
#define NRC_REGIONS (NRC_GRID * NRC_GRID * NRC_GRID)
struct DNrc {
	int mode;                         /* 0 off, 1 cache with per-region fallback, 2 cache everywhere */
	float lo[3], sc[3];               /* box corner and 1 / box size */
	const unsigned char *fallback;    /* per region: 1 = plain final gather */
	float *qx;                        /* query inputs, 9 floats each */
	float4 *qw;                       /* query weight rgb, accumulator slot */
	int *qcount;
	int qcap;
	float *tx;                        /* training records [0, tcap), validation records [tcap, tcap + vcap) */
	int *tcount;                      /* [0] training records, [1] validation records */
	int tcap, vcap;
	int t0;                           /* accumulator slot of record 0 */
	uint32_t p_train, p_val;          /* a vertex whose hash is below p_train trains, below p_train + p_val validates */
	uint32_t key;                     /* per-frame key of the selection hash */
	int fb_samples;                   /* final-gather rays in a fallback region (0: diffuse_samples) */
	unsigned long long *counters;     /* [0] final-gather vertices, [1] cached */
};

/* one job of a batch (sray_gpu_render_batch): its pixels are
 * [pix0, pix0 + width * height) of the batch's pixel space */
struct DevJob {
	int pix0, width, height, t0;
	float cam_f, cam_xsz, cam_ysz;
	int scene;                /* its scene in a scene set (0 otherwise) */
	int cam_base;             /* first time slot of its scene's camera in cam_m */
	int pad[3];
};

/* one scene of a scene set: the roots of its scene octree and object
 * hierarchy in the set's tables, its lights and environment */
struct DevSceneRef {
	int sroot, troot;         /* troot < 0: no objects */
	int light0, nlights;
	float env_col[4], env_amb[4];
};

struct DScene {
	const DevNode *snodes;    /* top-level octree (world space) */
	const int *sslots;
	int has_scene;
	int sroot;                /* root node index in snodes */
	const DevNode *mnodes;    /* mesh octrees (object space) */
	const DevTri *mtris;
	const int *mprim;
	const DevBvh4 *bnodes;    /* mesh hierarchies, 4-wide (object space) */
	const DevTri *btris;      /* triangles in hierarchy leaf order */
	const int *bprim;         /* their face indices */
	const int *bhome;         /* their home nodes in the mesh octrees */
	const DevBvh4 *tnodes;    /* object hierarchy, 4-wide (world space), null if none */
	const int *ohome;         /* per object: its home node in the scene octree */
	unsigned long long *bvh_fallbacks;   /* hits the octree did not confirm */
	const DevObj *objs;
	int nobj;
	const float *xf;          /* per object per time, XF_STRIDE floats */
	int tlo, nt;
	const float *tri_pos;     /* 9 floats per unique-mesh triangle */
	const float *tri_attr;    /* 24 floats per unique-mesh triangle */
	const DevMat *mats;
	DevMat defmat;
	const DevTex *texs;       /* textures of the materials' attributes */
	const float4 *texels;     /* their RGBA texels */
	const DevLight *lights;
	int nlights;
	const float *light_pos;   /* 4 floats per light per time */
	const float *cam_m;       /* 12 floats per time */
	float cam_f, cam_xsz, cam_ysz, cam_maxd;
	float env_col[4], env_amb[4];
	float eps, xsmall;
	float min_energy;
	int iter, diffuse_samples, shadow_samples;
	int gi_on, caust_on;
	int width, height;
	int mblur, shutter;
	int t0, t1;
	uint64_t seed;
	float photon_energy;
	float max_cos;
	DPhotonMap caust, gi;
	DNrc nrc;
	/* a batch of jobs (njobs > 0): the jobs and their photon maps, caustic
	 * and global of job j at maps[2j], maps[2j + 1]; a gather request's kind
	 * is then the map index */
	int njobs;
	const DevJob *jobs;
	const DPhotonMap *maps;
	/* the object hierarchy's root (0 for one scene; a batch job's photon
	 * view points it, sroot and the light tables at its scene's) */
	int troot;
	/* a scene set (nscenes > 1): a ray's scene is its job's */
	int nscenes;
	const DevSceneRef *scenes;
};

/* the job of a pixel of the batch's pixel space */
__device__ __forceinline__ int job_of(const DScene &S, int pixel)
{
	int lo = 0, hi = S.njobs - 1;
	while(lo < hi) {
		int mid = (lo + hi + 1) >> 1;
		if(S.jobs[mid].pix0 <= pixel) lo = mid;
		else hi = mid - 1;
	}
	return lo;
}

/* the scene of a batch pixel in a scene set (-1: the view's own scene) */
__device__ __forceinline__ int pixel_scene(const DScene &S, int pixel)
{
	return S.nscenes > 1 && S.njobs > 0 ? S.jobs[job_of(S, pixel)].scene : -1;
}

/* ---------------- float3 helpers (no contraction: built with -fmad=false) */
struct V3 { float x, y, z; };
__device__ __forceinline__ V3 mk(float x, float y, float z) { V3 v; v.x = x; v.y = y; v.z = z; return v; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ float len(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalized(V3 a) { float l = len(a); return mk(a.x / l, a.y / l, a.z / l); }
/* reflection of a vector travelling towards the surface */
__device__ __forceinline__ V3 reflection(V3 v, V3 n) { return v - n * (2.0f * dot(v, n)); }
__device__ __forceinline__ V3 refraction(V3 v, V3 n, float ior)
{
	float cos_inc = dot(v, -n);
	float radical = 1.0f + (ior * ior) * (cos_inc * cos_inc - 1.0f);
	if(radical < 0.0f) return reflection(v, n);
	float beta = ior * cos_inc - sqrtf(radical);
	return v * ior + n * beta;
}

__device__ __forceinline__ V3 mul_pt(const float *m, V3 p)
{
	return mk(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
			m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
			m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
}
__device__ __forceinline__ V3 mul_dir(const float *m, V3 p)
{
	return mk(m[0] * p.x + m[1] * p.y + m[2] * p.z,
			m[4] * p.x + m[5] * p.y + m[6] * p.z,
			m[8] * p.x + m[9] * p.y + m[10] * p.z);
}
__device__ __forceinline__ V3 mul_n(const float *m, V3 p)
{
	return mk(m[0] * p.x + m[1] * p.y + m[2] * p.z,
			m[3] * p.x + m[4] * p.y + m[5] * p.z,
			m[6] * p.x + m[7] * p.y + m[8] * p.z);
}

__device__ __forceinline__ int time_index(const DScene &S, int time)
{
	int ti = time - S.tlo;
	return ti < 0 ? 0 : (ti >= S.nt ? S.nt - 1 : ti);
}

__device__ __forceinline__ const float *obj_xf(const DScene &S, int obj, int ti)
{
	return S.xf + ((size_t)obj * S.nt + ti) * XF_STRIDE;
}

/* ---------------- random draws (float) ---------------- */
__device__ __forceinline__ float frand(sray_rng *s, float range) { return range * sray_rng_uniform_f(s); }
__device__ __forceinline__ V3 sphrand(sray_rng *s, float rad)
{
	float u0 = sray_rng_uniform_f(s);
	float u1 = sray_rng_uniform_f(s);
	float z = 2.0f * u1 - 1.0f;
	float sxy = sqrtf(1.0f - z * z);
	float sn, cs;
	sray_sincos_turns_f(u0, &sn, &cs);
	return mk(rad * cs * sxy, rad * sn * sxy, rad * z);
}

/* ---------------- intersection tests ---------------- */
struct RayT {
	V3 o, d, inv;
};

/* AABox::intersect (src/aabb.cc:81-125); also returns the entry parameter */
__device__ __forceinline__ bool box_hit(const float *mn, const float *mx, const RayT &r, float &tentry)
{
	int xs = r.d.x < 0.0f;
	float tmin = ((xs ? mx[0] : mn[0]) - r.o.x) * r.inv.x;
	float tmax = ((xs ? mn[0] : mx[0]) - r.o.x) * r.inv.x;
	int ys = r.d.y < 0.0f;
	float tymin = ((ys ? mx[1] : mn[1]) - r.o.y) * r.inv.y;
	float tymax = ((ys ? mn[1] : mx[1]) - r.o.y) * r.inv.y;
	if((tmin > tymax) || (tymin > tmax)) return false;
	if(tymin > tmin) tmin = tymin;
	if(tymax < tmax) tmax = tymax;
	int zs = r.d.z < 0.0f;
	float tzmin = ((zs ? mx[2] : mn[2]) - r.o.z) * r.inv.z;
	float tzmax = ((zs ? mn[2] : mx[2]) - r.o.z) * r.inv.z;
	if((tmin > tzmax) || (tzmin > tmax)) return false;
	if(tzmin > tmin) tmin = tzmin;
	if(tzmax < tmax) tmax = tzmax;
	tentry = tmin;
	return (tmin < 1.0f) && (tmax > 0.0f);
}

/* Triangle::intersect (src/mesh.cc:117-165) without the surface point;
 * `limit` lets the caller skip the edge tests of candidates that cannot win */
__device__ __forceinline__ bool tri_hit(const float4 a, const float4 b, const float4 c, const RayT &r, float eps,
		float limit, float &t)
{
	V3 n = mk(a.w, b.w, c.w);
	float ndd = dot(n, r.d);
	if(fabsf(ndd) < eps) return false;
	V3 v0 = mk(a.x, a.y, a.z);
	V3 vo = r.o - v0;
	t = -dot(n, vo) / ndd;
	if(t < eps || t > 1.0f) return false;
	if(t > limit) return false;
	V3 v1 = mk(b.x, b.y, b.z), v2 = mk(c.x, c.y, c.z);
	V3 pos = r.o + r.d * t;
	if(!(dot(cross(v1 - v0, pos - v0), n) >= 0.0f)) return false;
	if(!(dot(cross(v2 - v1, pos - v1), n) >= 0.0f)) return false;
	if(!(dot(cross(v0 - v2, pos - v2), n) >= 0.0f)) return false;
	return true;
}

/* Sphere::intersect (src/sphere.cc:85-131), object space */
/* The reference solves a t^2 + b t + c = 0 with the textbook formula.  In
 * float, with the reference's ray lengths (primary rays 10^4 long) b^2 and
 * 4ac cancel and the hit point drifts off the surface by ~1e-4, so that
 * light samples from it hit the surface again.  These solvers compute the
 * same roots without the cancellation: the discriminant from the ray's
 * closest approach to the axis / centre, r^2 - |o - (o.d / d.d) d|^2, and
 * the near root as c / q (q = -(o.d) -+ sqrt(...)).  The root selection that
 * follows is the reference's. */
__device__ __forceinline__ void stable_roots(float a, float bh, float dh, float c, float &t1, float &t2)
{
	float sq = sqrtf(dh * a);
	float q = -(bh + (bh < 0.0f ? -sq : sq));
	float ta = q / a, tb = q != 0.0f ? c / q : ta;
	t1 = ta > tb ? ta : tb;
	t2 = ta > tb ? tb : ta;
}

__device__ __forceinline__ bool sphere_hit(const RayT &r, float rad, float eps, float &dist)
{
	float a = dot(r.d, r.d);
	float bh = dot(r.o, r.d);
	V3 pp = r.o - r.d * (bh / a);
	float dh = rad * rad - dot(pp, pp);
	if(dh < 0.0f) return false;
	float c = dot(r.o, r.o) - rad * rad;
	float t1, t2;
	stable_roots(a, bh, dh, c, t1, t2);
	if((t1 < eps && t2 < eps) || (t1 > 1.0f && t2 > 1.0f)) return false;
	if(t1 < eps) t1 = t2;
	if(t2 < eps) t2 = t1;
	dist = t1 < t2 ? t1 : t2;
	return true;
}

/* Cylinder::intersect (src/cylinder.cc:125-185), object space */
__device__ __forceinline__ bool cylinder_hit(const RayT &r, float rad, float start, float end, float eps, float &dist)
{
	float a = r.d.x * r.d.x + r.d.z * r.d.z;
	float t1, t2;
	if(a > 0.0f) {
		float bh = r.d.x * r.o.x + r.d.z * r.o.z;
		float px = r.o.x - r.d.x * (bh / a), pz = r.o.z - r.d.z * (bh / a);
		float dh = rad * rad - (px * px + pz * pz);
		if(dh < 0.0f) return false;
		float c = r.o.x * r.o.x + r.o.z * r.o.z - rad * rad;
		stable_roots(a, bh, dh, c, t1, t2);
	} else {
		/* a ray parallel to the axis: the reference's formula */
		float b = 2.0f * r.d.x * r.o.x + 2.0f * r.d.z * r.o.z;
		float c = r.o.x * r.o.x + r.o.z * r.o.z - rad * rad;
		float d = b * b - 4.0f * a * c;
		if(d < 0.0f) return false;
		float sq = sqrtf(d);
		t1 = (-b + sq) / (2.0f * a);
		t2 = (-b - sq) / (2.0f * a);
	}
	if((t1 < eps && t2 < eps) || (t1 > 1.0f && t2 > 1.0f)) return false;
	V3 p1 = r.o + r.d * t1;
	V3 p2 = r.o + r.d * t2;
	bool v0 = true, v1 = true;
	if(t1 < eps || p1.y < start || p1.y >= end) { v0 = false; t1 = t2; }
	if(t2 < eps || p2.y < start || p2.y >= end) { v1 = false; t2 = t1; }
	if(!v0 && !v1) return false;
	dist = t1 < t2 ? t1 : t2;
	return true;
}

__device__ __forceinline__ RayT make_ray(V3 o, V3 d)
{
	RayT r;
	r.o = o;
	r.d = d;
	r.inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
	return r;
}

struct Hit {
	float t;
	int obj, prim, tie;
};

/* candidate update: strict '<' keeps the first hit found among equals, as the
 * reference's octree does; a different primitive at exactly the same t is
 * flagged as a tie */
__device__ __forceinline__ void consider(Hit &h, float t, int obj, int prim)
{
	if(t < h.t) {
		h.t = t;
		h.obj = obj;
		h.prim = prim;
		h.tie = 0;
	} else if(t == h.t && (obj != h.obj || prim != h.prim)) {
		h.tie = 1;
	}
}

/* pruning slack: a node is skipped only when its entry lies clearly behind
 * the best hit, so rounding differences between a hit point and the box that
 * contains it can never hide a candidate the exhaustive search would find */
#define SRAY_PRUNE(te, best) ((te) > (best) * 1.00001f + 1e-30f)

#define SRAY_STACK 128
#define SRAY_MAILBOX 8

struct TraceCounters {
	unsigned long long nodes, prims;
};

/* octant of the ray direction: children are stored in slot order
 * x | y << 1 | z << 2, so visiting slots (k ^ octant) for k = 0..7 goes
 * front to back along the ray */
__device__ __forceinline__ int octant(const RayT &r)
{
	return (r.d.x < 0.0f ? 1 : 0) | (r.d.y < 0.0f ? 2 : 0) | (r.d.z < 0.0f ? 4 : 0);
}

struct TStack {
	int node[SRAY_STACK];
	float te[SRAY_STACK];
};

/* test the children of an inner node and push the hit ones far to near.
 * A child's box is one octant of the node's box split at `mid`, so its slab
 * parameters are three of the nine plane parameters (mn, mid, mx per axis)
 * computed once here; each child's test then makes exactly the comparisons
 * of box_hit on exactly the values box_hit would compute from its box. */
__device__ __forceinline__ void half_planes(float lo, float mid, float hi, float o, float inv, bool neg, float &n0, float &f0,
		float &n1, float &f1)
{
	float ta = (lo - o) * inv, tm = (mid - o) * inv, tb = (hi - o) * inv;
	/* lower half [lo, mid], upper half [mid, hi]; a negative direction
	 * enters through the upper plane */
	n0 = neg ? tm : ta;
	f0 = neg ? ta : tm;
	n1 = neg ? tb : tm;
	f1 = neg ? tm : tb;
}

template <bool COUNT>
__device__ __forceinline__ int push_children(float4 n0, float4 n1, float4 n2, int oct, const RayT &r, float best, TStack &st,
		int sp, int limit, TraceCounters *tc, int *overflow)
{
	int first = __float_as_int(n0.w);
	unsigned mask = __float_as_uint(n2.w);
	float nx0, fx0, nx1, fx1, ny0, fy0, ny1, fy1, nz0, fz0, nz1, fz1;
	half_planes(n0.x, n2.x, n1.x, r.o.x, r.inv.x, r.d.x < 0.0f, nx0, fx0, nx1, fx1);
	half_planes(n0.y, n2.y, n1.y, r.o.y, r.inv.y, r.d.y < 0.0f, ny0, fy0, ny1, fy1);
	half_planes(n0.z, n2.z, n1.z, r.o.z, r.inv.z, r.d.z < 0.0f, nz0, fz0, nz1, fz1);
	#pragma unroll
	for(int k = 7; k >= 0; k--) {
		int c = k ^ oct;
		if(!((mask >> c) & 1u)) continue;
		float tmin = (c & 1) ? nx1 : nx0, tmax = (c & 1) ? fx1 : fx0;
		float tymin = (c & 2) ? ny1 : ny0, tymax = (c & 2) ? fy1 : fy0;
		float tzmin = (c & 4) ? nz1 : nz0, tzmax = (c & 4) ? fz1 : fz0;
		if((tmin > tymax) || (tymin > tmax)) continue;
		if(tymin > tmin) tmin = tymin;
		if(tymax < tmax) tmax = tymax;
		if((tmin > tzmax) || (tzmin > tmax)) continue;
		if(tzmin > tmin) tmin = tzmin;
		if(tzmax < tmax) tmax = tzmax;
		if(!((tmin < 1.0f) && (tmax > 0.0f)) || SRAY_PRUNE(tmin, best)) continue;
		if(sp >= limit) { *overflow = 1; continue; }
		st.node[sp] = first + c;
		st.te[sp] = tmin;
		sp++;
	}
	return sp;
}

/* a node record: n0 = mn + first, n1 = mx + count, n2 = mid + child mask
 * (the third part is read for inner nodes only) */
__device__ __forceinline__ void load_node(const DevNode *nodes, int ni, float4 &n0, float4 &n1)
{
	const float4 *np = reinterpret_cast<const float4 *>(nodes + ni);
	n0 = __ldg(np);
	n1 = __ldg(np + 1);
}

__device__ __forceinline__ float4 load_split(const DevNode *nodes, int ni)
{
	return __ldg(reinterpret_cast<const float4 *>(nodes + ni) + 2);
}

/* Triangle mailbox.  A triangle whose bounds overlap several octree leaves
 * is listed in each of them, and a ray crossing those leaves would test it
 * again with the same result (a repeated test can neither improve the best
 * hit nor flag a tie that the first test did not).  Each thread keeps the
 * last triangle seen per slot of a 16-way direct-mapped table, cleared
 * whenever the ray enters a mesh, and skips repeats.  The table is the
 * thread's own (local memory), not shared memory: the octree-only kernels
 * run between the hierarchy kernels, which use no shared memory, and a
 * kernel that needs shared memory waits for SMs to drain the other
 * stream's blocks before it can start. */
#define SRAY_TRACE_THREADS 128
#define SRAY_TRI_MBOX 16

__device__ __forceinline__ void tri_mailbox_clear(int *mb)
{
	#pragma unroll
	for(int k = 0; k < SRAY_TRI_MBOX; k++) mb[k] = -1;
}

/* true when `prim` was tested since the last clear; records it otherwise */
__device__ __forceinline__ bool tri_mailbox_seen(int *mb, int prim)
{
	int *e = mb + (prim & (SRAY_TRI_MBOX - 1));
	if(*e == prim) return true;
	*e = prim;
	return false;
}

/* closest hit inside one mesh (object space), sharing the best hit so far */
template <bool COUNT>
__device__ __forceinline__ void mesh_closest(const DScene &S, int root, int obj, const RayT &r, Hit &h, TStack &st, int base,
		TraceCounters *tc, int *overflow)
{
	int sp = base;
	float te;
	const DevNode &rn = S.mnodes[root];
	if(!box_hit(rn.mn, rn.mx, r, te)) return;
	int oct = octant(r);
	int mb[SRAY_TRI_MBOX];
	tri_mailbox_clear(mb);
	st.node[sp] = root;
	st.te[sp] = te;
	sp++;
	while(sp > base) {
		sp--;
		int ni = st.node[sp];
		if(SRAY_PRUNE(st.te[sp], h.t)) continue;
		if(COUNT) tc->nodes++;
		float4 n0, n1;
		load_node(S.mnodes, ni, n0, n1);
		int count = __float_as_int(n1.w), first = __float_as_int(n0.w);
		if(count < 0) {
			sp = push_children<COUNT>(n0, n1, load_split(S.mnodes, ni), oct, r, h.t, st, sp, SRAY_STACK, tc, overflow);
		} else {
			const float4 *tp = reinterpret_cast<const float4 *>(S.mtris + first);
			for(int s = 0; s < count; s++) {
				int prim = __ldg(S.mprim + first + s);
				if(tri_mailbox_seen(mb, prim)) continue;
				float4 a = __ldg(tp + 3 * s), b = __ldg(tp + 3 * s + 1), c = __ldg(tp + 3 * s + 2);
				if(COUNT) tc->prims++;
				float t;
				if(tri_hit(a, b, c, r, S.eps, h.t, t)) consider(h, t, obj, prim);
			}
		}
	}
}

/* ---------------- octree traversal (the reference's structure) ---------------- */

template <bool COUNT>
__device__ __forceinline__ void object_closest(const DScene &S, int oi, int ti, V3 wo, V3 wd, Hit &h, TStack &st, int base,
		TraceCounters *tc, int *overflow)
{
	const DevObj ob = S.objs[oi];
	const float *m = obj_xf(S, oi, ti);
	const float *inv = m + 12;
	RayT r = make_ray(mul_pt(inv, wo), mul_dir(inv, wd));
	if(ob.type == 2) {
		if(ob.mesh_root >= 0) mesh_closest<COUNT>(S, ob.mesh_root, oi, r, h, st, base, tc, overflow);
		return;
	}
	if(COUNT) tc->prims++;
	float t;
	bool hit = ob.type == 0 ? sphere_hit(r, ob.rad, S.eps, t) : cylinder_hit(r, ob.rad, ob.start, ob.end, S.eps, t);
	if(hit) consider(h, t, oi, 0);
}

/* Object mailbox.  An object spanning several top-level leaves gives the
 * same closest hit each time it is tested, so it is tested once per ray.
 * Scenes of up to SRAY_OBJ_EXACT objects keep an exact per-ray set (one bit
 * per object, in the thread's local memory as the triangle mailbox); larger
 * scenes remember the last SRAY_MAILBOX objects. */
#define SRAY_OBJ_EXACT 1024

struct ObjMailbox {
	unsigned bits[SRAY_OBJ_EXACT / 32];
	int ring[SRAY_MAILBOX];
	int next;
	bool exact;
};

__device__ __forceinline__ void obj_mailbox_init(const DScene &S, ObjMailbox &m)
{
	m.exact = S.nobj <= SRAY_OBJ_EXACT;
	m.next = 0;
	if(m.exact) {
		int words = (S.nobj + 31) >> 5;
		for(int w = 0; w < words; w++) m.bits[w] = 0u;
	} else {
		#pragma unroll
		for(int k = 0; k < SRAY_MAILBOX; k++) m.ring[k] = -1;
	}
}

__device__ __forceinline__ bool mailbox_seen(ObjMailbox &m, int oi)
{
	if(m.exact) {
		unsigned *w = m.bits + (oi >> 5);
		unsigned bit = 1u << (oi & 31);
		unsigned v = *w;
		if(v & bit) return true;
		*w = v | bit;
		return false;
	}
	bool seen = false;
	#pragma unroll
	for(int k = 0; k < SRAY_MAILBOX; k++) seen |= m.ring[k] == oi;
	if(!seen) {
		m.ring[m.next] = oi;
		m.next = (m.next + 1) & (SRAY_MAILBOX - 1);
	}
	return seen;
}

/* The roots a traversal starts from: those of scene `scene` of a scene set
 * (scene >= 0), else the view's own.  x: the scene octree's root (< 0: no
 * scene), y: the object hierarchy's (< 0: none, the octree decides). */
__device__ __forceinline__ int2 scene_roots(const DScene &S, int scene)
{
	if(scene >= 0) {
		const DevSceneRef &R = S.scenes[scene];
		return make_int2(S.has_scene ? R.sroot : -1, R.troot);
	}
	return make_int2(S.has_scene ? S.sroot : -1, S.tnodes ? S.troot : -1);
}

/* closest hit of a world-space segment (Scene::cast_ray, src/scene.cc:764-794):
 * front to back over the top-level octree with the pruning above; an object
 * straddling several leaves gives the same closest hit every time, so each
 * object is tested once per ray */
template <bool COUNT>
__device__ __forceinline__ void trace_closest_octree_impl(const DScene &S, V3 wo, V3 wd, int time, Hit &h, TraceCounters *tc,
		int *overflow, int scene = -1)
{
	const int sroot_i = scene_roots(S, scene).x;
	h.t = FLT_MAX;
	h.obj = -1;
	h.prim = -1;
	h.tie = 0;
	if(sroot_i < 0) return;
	int ti = time_index(S, time);
	RayT r = make_ray(wo, wd);
	int oct = octant(r);
	TStack st;
	int sp = 0;
	float te;
	ObjMailbox mbox;
	obj_mailbox_init(S, mbox);
	const DevNode &root = S.snodes[sroot_i];
	if(!box_hit(root.mn, root.mx, r, te)) return;
	st.node[sp] = sroot_i;
	st.te[sp] = te;
	sp++;
	while(sp > 0) {
		sp--;
		int ni = st.node[sp];
		if(SRAY_PRUNE(st.te[sp], h.t)) continue;
		if(COUNT) tc->nodes++;
		float4 n0, n1;
		load_node(S.snodes, ni, n0, n1);
		int count = __float_as_int(n1.w), first = __float_as_int(n0.w);
		if(count < 0) {
			sp = push_children<COUNT>(n0, n1, load_split(S.snodes, ni), oct, r, h.t, st, sp, SRAY_STACK / 2, tc, overflow);
		} else {
			for(int s = 0; s < count; s++) {
				int oi = __ldg(S.sslots + first + s);
				if(mailbox_seen(mbox, oi)) continue;
				object_closest<COUNT>(S, oi, ti, wo, wd, h, st, sp, tc, overflow);
			}
		}
	}
}

/* any hit: the reference's shadow test is cast_ray(shadow_ray) != 0
 * (src/shader.cc:266), i.e. whether any candidate intersection exists */
__device__ inline bool mesh_any(const DScene &S, int root, const RayT &r, TStack &st, int base, int *overflow)
{
	int sp = base;
	float te;
	const DevNode &rn = S.mnodes[root];
	if(!box_hit(rn.mn, rn.mx, r, te)) return false;
	int oct = octant(r);
	int mb[SRAY_TRI_MBOX];
	tri_mailbox_clear(mb);
	st.node[sp++] = root;
	while(sp > base) {
		int ni = st.node[--sp];
		float4 n0, n1;
		load_node(S.mnodes, ni, n0, n1);
		int count = __float_as_int(n1.w), first = __float_as_int(n0.w);
		if(count < 0) {
			sp = push_children<false>(n0, n1, load_split(S.mnodes, ni), oct, r, FLT_MAX, st, sp, SRAY_STACK, nullptr, overflow);
		} else {
			const float4 *tp = reinterpret_cast<const float4 *>(S.mtris + first);
			for(int s = 0; s < count; s++) {
				if(tri_mailbox_seen(mb, __ldg(S.mprim + first + s))) continue;
				float4 a = __ldg(tp + 3 * s), b = __ldg(tp + 3 * s + 1), c = __ldg(tp + 3 * s + 2);
				float t;
				if(tri_hit(a, b, c, r, S.eps, FLT_MAX, t)) return true;
			}
		}
	}
	return false;
}

__device__ __forceinline__ bool trace_any_octree_impl(const DScene &S, V3 wo, V3 wd, int time, int *overflow, int scene = -1)
{
	const int sroot_i = scene_roots(S, scene).x;
	if(sroot_i < 0) return false;
	int ti = time_index(S, time);
	RayT r = make_ray(wo, wd);
	int oct = octant(r);
	TStack st;
	int sp = 0;
	ObjMailbox mbox;
	obj_mailbox_init(S, mbox);
	float te;
	const DevNode &root = S.snodes[sroot_i];
	if(!box_hit(root.mn, root.mx, r, te)) return false;
	st.node[sp++] = sroot_i;
	while(sp > 0) {
		int ni = st.node[--sp];
		float4 n0, n1;
		load_node(S.snodes, ni, n0, n1);
		int count = __float_as_int(n1.w), first = __float_as_int(n0.w);
		if(count < 0) {
			sp = push_children<false>(n0, n1, load_split(S.snodes, ni), oct, r, FLT_MAX, st, sp, SRAY_STACK / 2, nullptr, overflow);
		} else {
			for(int s = 0; s < count; s++) {
				int oi = __ldg(S.sslots + first + s);
				if(mailbox_seen(mbox, oi)) continue;
				const DevObj ob = S.objs[oi];
				const float *inv = obj_xf(S, oi, ti) + 12;
				RayT orr = make_ray(mul_pt(inv, wo), mul_dir(inv, wd));
				float t;
				if(ob.type == 2) {
					if(ob.mesh_root >= 0 && mesh_any(S, ob.mesh_root, orr, st, sp, overflow)) return true;
				} else if(ob.type == 0) {
					if(sphere_hit(orr, ob.rad, S.eps, t)) return true;
				} else {
					if(cylinder_hit(orr, ob.rad, ob.start, ob.end, S.eps, t)) return true;
				}
			}
		}
	}
	return false;
}

/* ---------------- two-level hierarchy traversal confirmed by the octrees ----------------
 * The octrees define the result: the closest hit among the objects listed in
 * the top-level leaves the ray reaches, each object's own hit being the
 * closest among the faces listed in the mesh-octree leaves the ray reaches
 * (a leaf is reached when its box test and every ancestor's pass).
 *
 * Two binary hierarchies find the same hit faster: one over the objects,
 * each boxed by the union of the top-level leaves that list it, and one per
 * unique mesh over its faces.  Their boxes are widened per ray, so neither
 * skips an object the octree would test or a face the triangle test accepts;
 * the hit found is therefore the closest over a superset of the octrees'
 * candidates.  If it is unique at its distance and both octrees reach it
 * (the hit point's leaf lists the face, resp. the object, and that leaf's
 * box test passes), the octrees return it too.  Otherwise -- a second hit at
 * the same distance, or a hit an octree would not reach, both confined to
 * rounding-level coincidences and to objects moving outside their frame
 * bounds -- the ray is marked and traced again by the octrees alone. */

/* A ray prepared for the widened box test: the inverse direction clamped to
 * finite values, and per axis the widening in units of t.
 *
 * The widening must cover, for a face the triangle test accepts at t, the
 * distance by which the segment's exact point at t can lie outside the
 * face's box, plus the rounding of the slab parameters.  The computed hit
 * point o + d t is within 2^-23 (|o| + |p|) of the exact one, and the edge
 * tests accept it at most a few units in the last place of those
 * coordinates outside the face.  A slab parameter (x - o) / d_a is rounded
 * by at most 3 * 2^-24 of |x - o|.  Every point and plane involved lies in
 * the hierarchy's bounds, so all of this is below 2^-20.5 (|o| + R), where
 * R is the largest coordinate of those bounds.  The widening is 2^-17 of that
 * (a factor of 11 over it).  It does not grow with the segment's length, which
 * is RAY_MAGNITUDE times the unit direction (src/opt.h:21), while the scene is
 * a few hundred units across. */
struct RayC {
	V3 inv;
	V3 cn, cf;            /* slab constants of the entry / exit planes: -(o inv) -/+ slack */
	unsigned neg;         /* bit a: the direction's axis a is negative (the entry plane
	                         is the box's upper bound) */
};

/* a 4-wide node's six bound vectors (lo x, y, z, hi x, y, z) as entry planes
 * (n) and exit planes (f) of the ray */
struct NodePlanes {
	float4 nx, ny, nz, fx, fy, fz;
};

__device__ __forceinline__ NodePlanes node_planes(const float4 *np, const RayC &c)
{
	int sx = (c.neg & 1u) ? 3 : 0, sy = (c.neg & 2u) ? 3 : 0, sz = (c.neg & 4u) ? 3 : 0;
	NodePlanes p;
	p.nx = __ldg(np + sx);
	p.ny = __ldg(np + 1 + sy);
	p.nz = __ldg(np + 2 + sz);
	p.fx = __ldg(np + 3 - sx);
	p.fy = __ldg(np + 4 - sy);
	p.fz = __ldg(np + 5 - sz);
	return p;
}

__device__ __forceinline__ RayC make_rayc(const RayT &r, float bound)
{
	RayC c;
	c.inv = mk(fminf(fmaxf(r.inv.x, -1e20f), 1e20f), fminf(fmaxf(r.inv.y, -1e20f), 1e20f), fminf(fmaxf(r.inv.z, -1e20f), 1e20f));
	float om = fmaxf(fmaxf(fabsf(r.o.x), fabsf(r.o.y)), fabsf(r.o.z));
	float delta = (om + bound) * 7.6293945e-6f;   /* 2^-17 */
	V3 sl = mk(delta * fabsf(c.inv.x), delta * fabsf(c.inv.y), delta * fabsf(c.inv.z));
	V3 oi = mk(r.o.x * c.inv.x, r.o.y * c.inv.y, r.o.z * c.inv.z);
	c.cn = mk(-oi.x - sl.x, -oi.y - sl.y, -oi.z - sl.z);
	c.cf = mk(sl.x - oi.x, sl.y - oi.y, sl.z - oi.z);
	c.neg = (c.inv.x < 0.0f ? 1u : 0u) | (c.inv.y < 0.0f ? 2u : 0u) | (c.inv.z < 0.0f ? 4u : 0u);
	return c;
}

/* the largest coordinate of a box */
__device__ __forceinline__ float box_bound(const float *mn, const float *mx)
{
	return fmaxf(fmaxf(fmaxf(fabsf(mn[0]), fabsf(mn[1])), fmaxf(fabsf(mn[2]), fabsf(mx[0]))), fmaxf(fabsf(mx[1]), fabsf(mx[2])));
}

/* The widened box test with the entry planes (nx, ny, nz) and exit planes
 * (fx, fy, fz) picked by the direction's signs: each slab parameter is one
 * FMA, x inv + c, with the widening in c.  Against (x - o) inv - slack this
 * moves each parameter by a few units in the last place of o inv (and by
 * the cancellation when x is near o, also of order ulp(o inv)); the slack is
 * 2^-17 (|o| + R) |inv| >= 2^-17 |o inv|, over a hundred times that, so the
 * test stays a superset of the octrees' candidates.  A box with its bounds
 * swapped (an object no leaf lists) gives an empty interval. */
__device__ __forceinline__ bool wide_box(const RayC &c, float nx, float ny, float nz, float fx, float fy, float fz, float limit,
		float &tn)
{
	float tnear = fmaxf(fmaxf(fmaf(nx, c.inv.x, c.cn.x), fmaf(ny, c.inv.y, c.cn.y)), fmaf(nz, c.inv.z, c.cn.z));
	float tfar = fminf(fminf(fmaf(fx, c.inv.x, c.cf.x), fmaf(fy, c.inv.y, c.cf.y)), fmaf(fz, c.inv.z, c.cf.z));
	tn = tnear;
	return tnear <= tfar && tfar >= 0.0f && tnear <= limit;
}

/* Would an octree (nodes, and the item ids its leaves list) test item `id`
 * for this ray, with best hit t?  The leaves listing the item all lie below
 * its home node; the hit point (computed as the intersection tests compute
 * it) picks the leaf.  The octree reaches that leaf if the leaf's own box
 * test passes: slab parameters are monotone in the planes, so each
 * ancestor's intervals contain the leaf's and its test (and the pruning test,
 * its entry parameter being no larger) passes too. */
__device__ inline bool octree_reaches(const DevNode *nodes, const int *ids, int home, const RayT &r, int id, float t, bool prune)
{
	V3 P = r.o + r.d * t;
	int ni = home;
	for(int level = 0; level < 64; level++) {
		const float4 *np = reinterpret_cast<const float4 *>(nodes + ni);
		float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
		int count = __float_as_int(n1.w), first = __float_as_int(n0.w);
		if(count >= 0) {
			float mn[3] = {n0.x, n0.y, n0.z}, mx[3] = {n1.x, n1.y, n1.z};
			float te;
			if(!box_hit(mn, mx, r, te)) return false;
			if(prune && SRAY_PRUNE(te, t)) return false;
			for(int s = 0; s < count; s++) if(__ldg(ids + first + s) == id) return true;
			return false;
		}
		int c = (P.x >= n2.x ? 1 : 0) | (P.y >= n2.y ? 2 : 0) | (P.z >= n2.z ? 4 : 0);
		if(!((__float_as_uint(n2.w) >> c) & 1u)) return false;
		ni = first + c;
	}
	return false;
}

/* the object-space ray of object o at time index ti */
__device__ __forceinline__ RayT object_ray(const DScene &S, int o, int ti, V3 wo, V3 wd)
{
	const float *inv = obj_xf(S, o, ti) + 12;
	return make_ray(mul_pt(inv, wo), mul_dir(inv, wd));
}

/* ANY = false: closest hit into h, returns false when the octrees must
 * decide.  ANY = true: returns 1 when a hit the octrees reach exists, 0 when
 * no hit exists, 2 when the octrees must decide.  SORT: a node's hit
 * children are visited nearest first (always for closest hits); an any-hit
 * query may visit them in the node's order instead. */
template <bool COUNT, bool ANY, bool SORT = true>
__device__ __forceinline__ int trace_two_level(const DScene &S, V3 wo, V3 wd, int time, Hit &h, TraceCounters *tc, int *overflow,
		int scene = -1)
{
	h.t = FLT_MAX;
	h.obj = -1;
	h.prim = -1;
	h.tie = 0;
	const int2 roots = scene_roots(S, scene);
	if(roots.x < 0) return ANY ? 0 : 1;
	if(roots.y < 0) return ANY ? 2 : 0;
	int ti = time_index(S, time);
	RayT wr = make_ray(wo, wd);
	const DevNode &sroot = S.snodes[roots.x];
	RayC wc = make_rayc(wr, box_bound(sroot.mn, sroot.mx));
	RayT r = wr;
	RayC rc = wc;
	TStack st;
	float best = ANY ? 1.0f : FLT_MAX;
	int bobj = -1, bprim = -1, bslot = -1;
	bool eq = false;
	int sp = 0, inst_base = 0, iobj = -1;
	bool inst = false;
	int cur = roots.y;   /* the object hierarchy's root */
	for(;;) {
		if(cur == BVH_NONE) {
			bool found = false;
			while(sp > 0) {
				int k = sp - 1;
				if(inst && k < inst_base) {   /* the instance's entries are done */
					inst = false;
					iobj = -1;
					r = wr;
					rc = wc;
				}
				sp = k;
				if(ANY || st.te[k] <= best) {
					cur = st.node[k];
					found = true;
					break;
				}
			}
			if(!found) break;
		}
		if(!inst && cur < 0) {
			/* enter object ~cur */
			int o = ~cur;
			cur = BVH_NONE;
			const DevObj ob = S.objs[o];
			RayT orr = object_ray(S, o, ti, wo, wd);
			if(ob.type != 2) {
				if(COUNT) tc->prims++;
				float t;
				bool hit = ob.type == 0 ? sphere_hit(orr, ob.rad, S.eps, t) : cylinder_hit(orr, ob.rad, ob.start, ob.end, S.eps, t);
				if(hit && t <= best) {
					if(ANY) {
						bobj = o;
						bprim = 0;
						best = t;
						break;
					}
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
			if(ob.bvh_root < 0) return ANY ? 2 : 0;
			/* the mesh octree's entry test: a mesh it would not enter gives
			 * no candidates (nor one beating the best, when pruned) */
			float te;
			const DevNode &rn = S.mnodes[ob.mesh_root];
			if(!box_hit(rn.mn, rn.mx, orr, te) || (!ANY && SRAY_PRUNE(te, best))) continue;
			r = orr;
			rc = make_rayc(orr, box_bound(rn.mn, rn.mx));
			inst = true;
			inst_base = sp;
			iobj = o;
			cur = ob.bvh_root;
			continue;
		}
		if(inst && cur < 0) {
			/* a leaf of the mesh hierarchy: its faces */
			unsigned v = ~(unsigned)cur;
			cur = BVH_NONE;
			int start = (int)(v >> 4), cnt = (int)(v & 15u);
			const float4 *tp = reinterpret_cast<const float4 *>(S.btris + start);
			bool done = false;
			for(int k = 0; k < cnt; k++) {
				float4 a = __ldg(tp + 3 * k), b = __ldg(tp + 3 * k + 1), c = __ldg(tp + 3 * k + 2);
				if(COUNT) tc->prims++;
				float t;
				if(!tri_hit(a, b, c, r, S.eps, best, t)) continue;
				int prim = __ldg(S.bprim + start + k);
				if(ANY) {
					bobj = iobj;
					bprim = prim;
					bslot = start + k;
					best = t;
					done = true;
					break;
				}
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
			if(ANY && done) break;
			continue;
		}
		/* a node of the object hierarchy (world space) or of a mesh's: up to
		 * four children in one 128-byte line; the hit ones (nodes, leaves, or
		 * objects) are visited nearest first, each leaf and object in an
		 * iteration of its own so that the lanes of a warp stay together */
		const float4 *np = reinterpret_cast<const float4 *>((inst ? S.bnodes : S.tnodes) + cur);
		const NodePlanes pl = node_planes(np, rc);
		const float4 &nx = pl.nx, &ny = pl.ny, &nz = pl.nz, &fx = pl.fx, &fy = pl.fy, &fz = pl.fz;
		int4 ch = __ldg(reinterpret_cast<const int4 *>(np) + 6);
		if(COUNT) tc->nodes++;
		float lim = fminf(best, 1.0f);
		int ref[4] = {ch.x, ch.y, ch.z, ch.w};
		float key[4];
		float tn;
		key[0] = (ref[0] != BVH_NONE && wide_box(rc, nx.x, ny.x, nz.x, fx.x, fy.x, fz.x, lim, tn)) ? tn : INFINITY;
		key[1] = (ref[1] != BVH_NONE && wide_box(rc, nx.y, ny.y, nz.y, fx.y, fy.y, fz.y, lim, tn)) ? tn : INFINITY;
		key[2] = (ref[2] != BVH_NONE && wide_box(rc, nx.z, ny.z, nz.z, fx.z, fy.z, fz.z, lim, tn)) ? tn : INFINITY;
		key[3] = (ref[3] != BVH_NONE && wide_box(rc, nx.w, ny.w, nz.w, fx.w, fy.w, fz.w, lim, tn)) ? tn : INFINITY;
		if(ANY && !SORT) {
			/* the hit children in node order: the first is next, the rest
			 * are stacked so that they pop in order */
			int nxt = BVH_NONE;
			#pragma unroll
			for(int k = 3; k >= 0; k--) {
				if(key[k] == INFINITY) continue;
				if(nxt != BVH_NONE) {
					if(sp >= SRAY_STACK) { *overflow = 1; return 0; }
					st.node[sp++] = nxt;
				}
				nxt = ref[k];
			}
			cur = nxt;
			continue;
		}
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
			if(sp >= SRAY_STACK) { *overflow = 1; return ANY ? 0 : 1; }
			st.node[sp] = ref[k];
			if(!ANY) st.te[sp] = key[k];   /* any hit visits every entry */
			sp++;
		}
		cur = ref[0];
	}
	if(bobj < 0) return ANY ? 0 : 1;
	if(!ANY && eq) return 0;
	/* confirm against the octrees */
	if(bslot >= 0 && !octree_reaches(S.mnodes, S.mprim, __ldg(S.bhome + bslot), object_ray(S, bobj, ti, wo, wd), bprim, best, !ANY))
		return ANY ? 2 : 0;
	if(!octree_reaches(S.snodes, S.sslots, __ldg(S.ohome + bobj), wr, bobj, best, !ANY)) return ANY ? 2 : 0;
	if(ANY) return 1;
	h.t = best;
	h.obj = bobj;
	h.prim = bprim;
	h.tie = 0;
	return 1;
}

/* the octrees alone, kept out of line so that the hierarchy traversal's
 * registers are not shaped by them */
template <bool COUNT>
static __device__ __noinline__ void trace_closest_octree(const DScene &S, V3 wo, V3 wd, int time, Hit &h, TraceCounters *tc, int *overflow)
{
	trace_closest_octree_impl<COUNT>(S, wo, wd, time, h, tc, overflow);
}

static __device__ __noinline__ bool trace_any_octree(const DScene &S, V3 wo, V3 wd, int time, int *overflow)
{
	return trace_any_octree_impl(S, wo, wd, time, overflow);
}

/* closest hit, the octrees deciding when the hierarchies cannot */
template <bool COUNT>
__device__ inline void trace_closest(const DScene &S, V3 wo, V3 wd, int time, Hit &h, TraceCounters *tc, int *overflow)
{
	if(!trace_two_level<COUNT, false>(S, wo, wd, time, h, tc, overflow)) {
		atomicAdd(S.bvh_fallbacks, 1ull);
		trace_closest_octree<COUNT>(S, wo, wd, time, h, tc, overflow);
	}
}

__device__ inline bool trace_any(const DScene &S, V3 wo, V3 wd, int time, int *overflow)
{
	Hit h;
	int res = trace_two_level<false, true>(S, wo, wd, time, h, nullptr, overflow);
	if(res != 2) return res == 1;
	atomicAdd(S.bvh_fallbacks, 1ull);
	return trace_any_octree(S, wo, wd, time, overflow);
}

/* ---------------- surface point ---------------- */
struct Surf {
	V3 pos, normal;
	V3 gn;            /* geometric normal, unit, world space */
	V3 tangent;       /* filled when asked for (a normal-mapped material) */
	float tex[2];
};

/* The origin of a light sample's shadow ray.  The reference starts it at the
 * surface point and ignores hits closer than ERROR_MARGIN (in units of the
 * segment); in double the surface's own hit is ~1e-15 away, in float the
 * point is off the surface by a few ulps and a segment leaving at a shallow
 * angle can hit its own surface beyond the margin (dark speckles near the
 * shadow terminator).  The ray therefore starts 2^-18 (|p|max + 1) off the
 * surface along the geometric normal, on the side it leaves to. */
#define SHADOW_OFFSET 3.814697265625e-06f   /* 2^-18 */
__device__ __forceinline__ V3 shadow_origin(const Surf &sp, V3 dir)
{
	float side = dot(dir, sp.gn);
	if(side == 0.0f) return sp.pos;
	float ax = fabsf(sp.pos.x), ay = fabsf(sp.pos.y), az = fabsf(sp.pos.z);
	float m = ax > ay ? ax : ay;
	m = m > az ? m : az;
	float off = (m + 1.0f) * SHADOW_OFFSET;
	if(side < 0.0f) off = -off;
	return sp.pos + sp.gn * off;
}

/* The patch inversion's discriminant: ~0 where the hit lies on the patch's
 * fold, and float rounding can make it negative, where the reference's
 * sqrt (in double, never negative there) would give a NaN normal.  Clamped
 * to 0. */
__device__ __forceinline__ float root_disc(float d) { return sqrtf(d > 0.0f ? d : 0.0f); }

/* interp_face (src/mesh.cc:321-445): bilinear-patch inversion after Haines */
__device__ inline void interp_face(const float *P, const float *A, V3 ispos, V3 normal, float xsmall, V3 *onorm, float *otex, bool want_tex,
		V3 *otang = nullptr)
{
	V3 p00 = mk(P[0], P[1], P[2]), p10 = mk(P[3], P[4], P[5]), p01 = mk(P[6], P[7], P[8]), p11 = p01;
	V3 pa = (p00 - p10) + (p11 - p01);
	V3 pb = p10 - p00;
	V3 pc = p01 - p00;
	V3 pd = p00;
	V3 na = cross(pa, normal), nb = cross(pb, normal), nc = cross(pc, normal);
	float du0 = dot(nc, pd);
	float du1 = dot(na, pd) + dot(nc, pb);
	float du2 = dot(na, pb);
	float dv0 = dot(nb, pd);
	float dv1 = dot(na, pd) + dot(nb, pc);
	float dv2 = dot(na, pc);
	float rx, ry;
	if(fabsf(du2) <= xsmall) {
		float divisor = du1 - dot(na, ispos);
		rx = fabsf(divisor) > xsmall ? ((dot(nc, ispos) - du0) / divisor) : 0.0f;
	} else {
		V3 qux = na / (2.0f * du2);
		V3 quy = -nc / du2;
		float dux = -du1 / (2.0f * du2);
		float duy = du0 / du2;
		float ka = dux + dot(qux, ispos);
		float kb = duy + dot(quy, ispos);
		float sq = root_disc(ka * ka - kb);
		float u0 = ka - sq;
		float u1 = ka + sq;
		rx = (u0 < 0.0f || u0 > 1.0f) ? u1 : u0;
	}
	if(fabsf(dv2) <= xsmall) {
		float divisor = dv1 - dot(na, ispos);
		ry = fabsf(divisor) > xsmall ? ((dot(nb, ispos) - dv0) / divisor) : 0.0f;
	} else {
		V3 qvx = na / (2.0f * dv2);
		V3 qvy = -nb / dv2;
		float dvx = -dv1 / (2.0f * dv2);
		float dvy = dv0 / dv2;
		float ka = dvx + dot(qvx, ispos);
		float kb = dvy + dot(qvy, ispos);
		float sq = root_disc(ka * ka - kb);
		float v0 = ka - sq;
		float v1 = ka + sq;
		ry = (v0 < 0.0f || v0 > 1.0f) ? v1 : v0;
	}
#define DLERP(a, b, t) ((a) + ((b) - (a)) * (t))
	float nn[3];
	for(int k = 0; k < 3; k++) {
		float n0 = DLERP(A[0 * 3 + k], A[2 * 3 + k], ry);
		float n1 = DLERP(A[1 * 3 + k], A[2 * 3 + k], ry);
		nn[k] = DLERP(n0, n1, rx);
	}
	*onorm = mk(nn[0], nn[1], nn[2]);
	if(want_tex) {
		for(int k = 0; k < 2; k++) {
			float s0 = DLERP(A[18 + 0 * 2 + k], A[18 + 2 * 2 + k], ry);
			float s1 = DLERP(A[18 + 1 * 2 + k], A[18 + 2 * 2 + k], ry);
			otex[k] = DLERP(s0, s1, rx);
		}
	}
	if(otang) {
		float g[3];
		for(int k = 0; k < 3; k++) {
			float g0 = DLERP(A[9 + 0 * 3 + k], A[9 + 2 * 3 + k], ry);
			float g1 = DLERP(A[9 + 1 * 3 + k], A[9 + 2 * 3 + k], ry);
			g[k] = DLERP(g0, g1, rx);
		}
		*otang = mk(g[0], g[1], g[2]);
	}
#undef DLERP
}

__device__ __forceinline__ void sph_tex(V3 p, float *tex, bool cyl)
{
	double th = atan2((double)p.z, (double)p.x) + 3.14159265358979323846;
	double r = sqrt((double)p.x * p.x + (double)p.y * p.y + (double)p.z * p.z);
	double ph = acos((double)p.y / r);
	tex[0] = (float)(th / (2.0 * 3.14159265358979323846));
	tex[1] = cyl ? p.y : (float)(ph / 3.14159265358979323846);
}

/* world-space surface point of a hit, as the intersectors fill SurfPoint
 * (object-space position and normal, then forward / inverse-transpose).
 * Texture coordinates with want_tex, the tangent with want_tan: the
 * quadrics' (0,1,0) x normal, unnormalised (src/sphere.cc:120,
 * src/cylinder.cc:173), a mesh's interpolated vertex tangents, normalised
 * (src/mesh.cc:162, 302-305). */
__device__ inline void surface_point(const DScene &S, const Hit &h, V3 wo, V3 wd, int time, Surf &sp, bool want_tex,
		bool want_tan = false)
{
	int ti = time_index(S, time);
	const DevObj ob = S.objs[h.obj];
	const float *m = obj_xf(S, h.obj, ti);
	const float *inv = m + 12, *it = m + 24;
	V3 o = mul_pt(inv, wo), d = mul_dir(inv, wd);
	V3 pos = o + d * h.t;
	V3 nrm;
	sp.tex[0] = sp.tex[1] = 0.0f;
	if(ob.type == 0) {
		nrm = pos / ob.rad;
		if(want_tex) sph_tex(pos, sp.tex, false);
		if(want_tan) sp.tangent = mul_n(it, cross(mk(0.0f, 1.0f, 0.0f), nrm));
		sp.pos = mul_pt(m, pos);
		sp.normal = mul_n(it, nrm);
		sp.gn = normalized(sp.normal);
	} else if(ob.type == 1) {
		nrm = mk(1.0f * pos.x, 0.0f * pos.y, 1.0f * pos.z) / ob.rad;
		if(want_tex) sph_tex(pos, sp.tex, true);
		if(want_tan) sp.tangent = mul_n(it, cross(mk(0.0f, 1.0f, 0.0f), nrm));
		sp.pos = mul_pt(m, pos);
		sp.normal = mul_n(it, nrm);
		sp.gn = normalized(sp.normal);
	} else {
		const float *P = S.tri_pos + (size_t)(ob.tri_base + h.prim) * 9;
		const float *A = S.tri_attr + (size_t)(ob.tri_base + h.prim) * 24;
		V3 v0 = mk(P[0], P[1], P[2]), v1 = mk(P[3], P[4], P[5]), v2 = mk(P[6], P[7], P[8]);
		V3 fn = cross(v1 - v0, v2 - v0);
		V3 in, tg;
		interp_face(P, A, pos, fn, S.xsmall, &in, sp.tex, want_tex, want_tan ? &tg : nullptr);
		nrm = dot(in, in) < S.xsmall ? fn : in;
		if(want_tan) sp.tangent = normalized(mul_n(it, tg));
		sp.pos = mul_pt(m, pos);
		sp.normal = normalized(mul_n(it, nrm));
		sp.gn = normalized(mul_n(it, fn));
	}
}

/* ---------------- textures ---------------- */
/* Texture::lookup (src/texture.cc:60-83), the texture's transform being the
 * identity: texel (int)(tc * size) averaged with its four edge neighbours,
 * each wrapped by the repeat mode of Texture::get_texel
 * (src/texture.cc:85-101). */
__device__ __forceinline__ float4 tex_lookup(const DScene &S, int ti, const float *tc)
{
	const DevTex t = S.texs[ti];
	int tx = (int)(tc[0] * (float)t.xsz);
	int ty = (int)(tc[1] * (float)t.ysz);
	const int ox[5] = {0, 1, -1, 0, 0}, oy[5] = {0, 0, 0, 1, -1};
	float4 sum = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
	#pragma unroll
	for(int i = 0; i < 5; i++) {
		int x = (tx + ox[i]) % t.xsz, y = (ty + oy[i]) % t.ysz;
		if(x < 0) x += t.xsz;
		if(y < 0) y += t.ysz;
		float4 c = __ldg(S.texels + t.off + (long long)y * t.xsz + x);
		if(i == 0) sum = c;
		else { sum.x = sum.x + c.x; sum.y = sum.y + c.y; sum.z = sum.z + c.z; sum.w = sum.w + c.w; }
	}
	return make_float4(sum.x / 5.0f, sum.y / 5.0f, sum.z / 5.0f, sum.w / 5.0f);
}

/* a material's attributes at a surface point (MatAttrib::get_color /
 * get_value, src/material.inl:18-29): the colour, times the texel where the
 * attribute has a texture; a scalar is the colour's x, as float */
struct MatVals {
	float kd[3], ks[3];
	float shin, refl, refr, ior;
};
__device__ __forceinline__ void mat_values(const DScene &S, const DevMat &m, const float *tc, MatVals &v)
{
	#pragma unroll
	for(int k = 0; k < 3; k++) { v.kd[k] = m.kd[k]; v.ks[k] = m.ks[k]; }
	v.shin = m.shin;
	v.refl = m.refl;
	v.refr = m.refr;
	v.ior = m.ior;
	if(!m.textured) return;
	if(m.tex[TA_DIFFUSE] >= 0) {
		float4 c = tex_lookup(S, m.tex[TA_DIFFUSE], tc);
		v.kd[0] = c.x * m.kd[0]; v.kd[1] = c.y * m.kd[1]; v.kd[2] = c.z * m.kd[2];
	}
	if(m.tex[TA_SPECULAR] >= 0) {
		float4 c = tex_lookup(S, m.tex[TA_SPECULAR], tc);
		v.ks[0] = c.x * m.ks[0]; v.ks[1] = c.y * m.ks[1]; v.ks[2] = c.z * m.ks[2];
	}
	if(m.tex[TA_SHININESS] >= 0) v.shin = tex_lookup(S, m.tex[TA_SHININESS], tc).x * m.scol[TA_SHININESS];
	if(m.tex[TA_REFLECT] >= 0) v.refl = tex_lookup(S, m.tex[TA_REFLECT], tc).x * m.scol[TA_REFLECT];
	if(m.tex[TA_REFRACT] >= 0) v.refr = tex_lookup(S, m.tex[TA_REFRACT], tc).x * m.scol[TA_REFRACT];
	if(m.tex[TA_IOR] >= 0) v.ior = tex_lookup(S, m.tex[TA_IOR], tc).x * m.scol[TA_IOR];
}

/* get_bump_normal (src/shader.cc:296-318): the unflipped surface normal,
 * tilted by the normal map's texel in the frame (tangent, normal x tangent,
 * normal) where the "normal" attribute has a texture */
__device__ __forceinline__ V3 bump_normal(const DScene &S, const DevMat &m, const Surf &sp)
{
	V3 normal = sp.normal;
	if(m.tex[TA_NORMAL] < 0) return normal;
	float4 c = tex_lookup(S, m.tex[TA_NORMAL], sp.tex);
	V3 n = mk(c.x * 2.0f - 1.0f, c.y * 2.0f - 1.0f, c.z * 2.0f - 1.0f);
	n.x = n.x * m.scol[TA_NORMAL];
	n.y = n.y * m.scol[TA_NORMAL];
	n = normalized(n);
	V3 bitan = cross(normal, sp.tangent);
	return mk(sp.tangent.x * n.x + bitan.x * n.y + normal.x * n.z, sp.tangent.y * n.x + bitan.y * n.y + normal.y * n.z,
			sp.tangent.z * n.x + bitan.z * n.y + normal.z * n.z);
}

/* ---------------- lights ---------------- */
/* Light::get_point / SphLight::get_point / BoxLight::get_point (src/light.cc:107, 272, 346) */
__device__ __forceinline__ V3 light_point(const DScene &S, int li, int time, sray_rng *s)
{
	const DevLight &L = S.lights[li];
	const float *p = S.light_pos + ((size_t)li * S.nt + time_index(S, time)) * 4;
	V3 pos = mk(p[0], p[1], p[2]);
	if(L.type == 1) return pos + sphrand(s, L.radius);
	if(L.type == 2) {
		V3 v;
		v.x = frand(s, L.dim[0]) - 0.5f * L.dim[0];
		v.y = frand(s, L.dim[1]) - 0.5f * L.dim[1];
		v.z = frand(s, L.dim[2]) - 0.5f * L.dim[2];
		return mul_pt(L.box_m, v);
	}
	return pos;
}

__device__ __forceinline__ const DevMat &mat_of(const DScene &S, int obj)
{
	int m = S.objs[obj].mat;
	return m >= 0 ? S.mats[m] : S.defmat;
}

__device__ __forceinline__ float fresnel(float r, float cosa)
{
	float inv = 1.0f - cosa;
	float inv_sq = inv * inv;
	return r + (1.0f - r) * inv_sq * inv_sq * inv;
}

/* ray IOR stack (depth 4): enter / leave / calc_ior */
struct IorStack {
	float ior;
	float stk[4];
	int sp;
	__device__ void enter(float n) { ior = n; if(sp < 4) stk[sp++] = n; }
	__device__ void leave()
	{
		if(sp == 0) return;
		sp--;
		ior = sp ? stk[sp - 1] : 1.0f;
	}
	__device__ float calc_ior(bool entering, float mat_ior) const
	{
		if(entering) return ior / mat_ior;
		IorStack t = *this;
		t.leave();
		return ior / t.ior;
	}
};

}  // namespace sray

#endif
