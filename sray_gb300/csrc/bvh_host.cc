/* bvh_host.cc -- binned surface-area-heuristic hierarchy over a mesh's
 * triangles (host side).
 *
 * The reference finds triangle candidates with a per-mesh octree
 * (src/octree.inl, built in Mesh::build_octree, src/mesh.cc); the octree stays
 * the definition of which hit a ray gets.  Its leaves follow the mesh's
 * bounding box, so a thin, wide mesh (a terrain) gets leaves that are thin
 * slabs, lists each triangle in many of them and spreads over far more
 * memory than the L2 cache holds.  This hierarchy has one entry per triangle
 * and tight boxes; the GPU traversal uses it to find the closest candidate
 * and then confirms that candidate against the octree.
 *
 * Boxes are the exact float bounds of the float vertices the triangle test
 * reads; the traversal widens them by a per-ray margin, so the hierarchy
 * never loses a triangle that the test would accept.
 */
#include <math.h>
#include <float.h>
#include <string.h>
#include <algorithm>
#include <numeric>
#include "scene_host.h"

namespace sray {

namespace {

struct Bounds {
	float mn[3], mx[3];
	void clear()
	{
		for(int a = 0; a < 3; a++) { mn[a] = FLT_MAX; mx[a] = -FLT_MAX; }
	}
	void grow(const Bounds &b)
	{
		for(int a = 0; a < 3; a++) {
			mn[a] = std::min(mn[a], b.mn[a]);
			mx[a] = std::max(mx[a], b.mx[a]);
		}
	}
	double area() const
	{
		double e[3];
		for(int a = 0; a < 3; a++) e[a] = mx[a] > mn[a] ? (double)mx[a] - (double)mn[a] : 0.0;
		return e[0] * e[1] + e[1] * e[2] + e[2] * e[0];
	}
};

enum { NBINS = 16, LEAF_MIN = 4, LEAF_MAX = 8, MEDIAN_DEPTH = 36 };

struct Builder {
	const std::vector<Bounds> *tb;
	const std::vector<float> *cen;   /* 3 per face */
	std::vector<int> *order;
	std::vector<DevBvhNode> *nodes;
	int max_depth = 0;
	int leaf_min = LEAF_MIN, leaf_max = LEAF_MAX;

	Bounds range_bounds(int b, int e) const
	{
		Bounds r;
		r.clear();
		for(int i = b; i < e; i++) r.grow((*tb)[(*order)[i]]);
		return r;
	}

	static int leaf_ref(int b, int e) { return ~((b << 4) | (e - b)); }

	/* reference to a subtree over order[b, e) */
	int build(int b, int e, int depth)
	{
		max_depth = std::max(max_depth, depth);
		int n = e - b;
		if(n <= leaf_min) return leaf_ref(b, e);
		Bounds cb;
		cb.clear();
		for(int i = b; i < e; i++) {
			const float *c = &(*cen)[(size_t)(*order)[i] * 3];
			for(int a = 0; a < 3; a++) {
				cb.mn[a] = std::min(cb.mn[a], c[a]);
				cb.mx[a] = std::max(cb.mx[a], c[a]);
			}
		}
		int axis = -1, split = -1;
		double best = DBL_MAX;
		if(depth < MEDIAN_DEPTH) {
			Bounds pb = range_bounds(b, e);
			double parea = pb.area();
			for(int a = 0; a < 3; a++) {
				double ext = (double)cb.mx[a] - (double)cb.mn[a];
				if(!(ext > 0.0)) continue;
				Bounds bin[NBINS];
				int cnt[NBINS] = {0};
				for(int k = 0; k < NBINS; k++) bin[k].clear();
				double sc = NBINS / ext;
				for(int i = b; i < e; i++) {
					int f = (*order)[i];
					int k = (int)(((double)(*cen)[(size_t)f * 3 + a] - (double)cb.mn[a]) * sc);
					k = k < 0 ? 0 : (k >= NBINS ? NBINS - 1 : k);
					cnt[k]++;
					bin[k].grow((*tb)[f]);
				}
				double ra[NBINS];
				int rn[NBINS];
				Bounds acc;
				acc.clear();
				int accn = 0;
				for(int k = NBINS - 1; k > 0; k--) {
					acc.grow(bin[k]);
					accn += cnt[k];
					ra[k] = acc.area();
					rn[k] = accn;
				}
				acc.clear();
				accn = 0;
				for(int k = 0; k < NBINS - 1; k++) {
					acc.grow(bin[k]);
					accn += cnt[k];
					if(accn == 0 || rn[k + 1] == 0) continue;
					double cost = 1.0 + (acc.area() * accn + ra[k + 1] * rn[k + 1]) / (parea > 0.0 ? parea : 1.0);
					if(cost < best) {
						best = cost;
						axis = a;
						split = k;
					}
				}
			}
			if(n <= leaf_max && (axis < 0 || best >= (double)n)) return leaf_ref(b, e);
		}
		int mid;
		if(axis >= 0) {
			double ext = (double)cb.mx[axis] - (double)cb.mn[axis];
			double sc = NBINS / ext;
			int *beg = order->data() + b, *end = order->data() + e;
			int *m = std::partition(beg, end, [&](int f) {
				int k = (int)(((double)(*cen)[(size_t)f * 3 + axis] - (double)cb.mn[axis]) * sc);
				k = k < 0 ? 0 : (k >= NBINS ? NBINS - 1 : k);
				return k <= split;
			});
			mid = (int)(m - order->data());
		} else {
			mid = b;
		}
		if(mid <= b || mid >= e) {
			/* no useful split (coincident centroids or the depth cap): halve
			 * the range along the widest centroid axis */
			int a = 0;
			for(int k = 1; k < 3; k++) if(cb.mx[k] - cb.mn[k] > cb.mx[a] - cb.mn[a]) a = k;
			mid = b + n / 2;
			std::nth_element(order->begin() + b, order->begin() + mid, order->begin() + e,
					[&](int x, int y) { return (*cen)[(size_t)x * 3 + a] < (*cen)[(size_t)y * 3 + a]; });
		}
		int id = (int)nodes->size();
		nodes->push_back(DevBvhNode());
		int l = build(b, mid, depth + 1);
		int r = build(mid, e, depth + 1);
		Bounds lb = range_bounds(b, mid), rbx = range_bounds(mid, e);
		DevBvhNode &nd = (*nodes)[id];
		memset(&nd, 0, sizeof nd);
		for(int a = 0; a < 3; a++) {
			nd.lmn[a] = lb.mn[a];
			nd.lmx[a] = lb.mx[a];
			nd.rmn[a] = rbx.mn[a];
			nd.rmx[a] = rbx.mx[a];
		}
		nd.left = l;
		nd.right = r;
		return id;
	}
};

}  // namespace

void MeshBvh::build_items(const float *mn, const float *mx, size_t n, int leaf_max)
{
	nodes.clear();
	order.clear();
	depth = 0;
	/* leaf references hold a 27-bit start: larger item sets use the octree alone */
	if(n == 0 || n >= ((size_t)1 << 27)) return;
	std::vector<Bounds> tb(n);
	std::vector<float> cen(n * 3);
	for(size_t i = 0; i < n; i++) {
		for(int a = 0; a < 3; a++) {
			tb[i].mn[a] = mn[i * 3 + a];
			tb[i].mx[a] = mx[i * 3 + a];
			cen[i * 3 + a] = (float)(((double)mn[i * 3 + a] + (double)mx[i * 3 + a]) * 0.5);
		}
	}
	order.resize(n);
	std::iota(order.begin(), order.end(), 0);
	Builder B;
	B.tb = &tb;
	B.cen = &cen;
	B.order = &order;
	B.nodes = &nodes;
	B.leaf_min = leaf_max < LEAF_MIN ? leaf_max : LEAF_MIN;
	B.leaf_max = leaf_max;
	nodes.reserve(n / 2 + 1);
	int ref = B.build(0, (int)n, 1);
	if(ref < 0) {
		/* at most leaf_min items: a root node with one leaf */
		DevBvhNode nd;
		memset(&nd, 0, sizeof nd);
		Bounds bb;
		bb.clear();
		for(size_t i = 0; i < n; i++) bb.grow(tb[i]);
		for(int a = 0; a < 3; a++) {
			nd.lmn[a] = bb.mn[a];
			nd.lmx[a] = bb.mx[a];
			nd.rmn[a] = FLT_MAX;
			nd.rmx[a] = -FLT_MAX;
		}
		nd.left = ref;
		nd.right = BVH_NONE;
		nodes.push_back(nd);
	}
	/* otherwise build() created the root first: it is node 0 */
	depth = B.max_depth;
}

namespace {
struct Entry {
	int ref;
	float mn[3], mx[3];
	double area() const
	{
		if(ref == BVH_NONE) return -1.0;
		double e[3];
		for(int a = 0; a < 3; a++) e[a] = mx[a] > mn[a] ? (double)mx[a] - (double)mn[a] : 0.0;
		return e[0] * e[1] + e[1] * e[2] + e[2] * e[0];
	}
};

void children_of(const DevBvhNode &n, Entry *e)
{
	e[0].ref = n.left;
	e[1].ref = n.right;
	for(int a = 0; a < 3; a++) {
		e[0].mn[a] = n.lmn[a];
		e[0].mx[a] = n.lmx[a];
		e[1].mn[a] = n.rmn[a];
		e[1].mx[a] = n.rmx[a];
	}
}

int collapse_node(const std::vector<DevBvhNode> &b2, int n2, std::vector<DevBvh4> &out)
{
	Entry c[4];
	int nc = 2;
	children_of(b2[n2], c);
	while(nc < 4) {
		int best = -1;
		double ba = -1.0;
		for(int k = 0; k < nc; k++) {
			if(c[k].ref < 0 || c[k].ref == BVH_NONE) continue;
			double a = c[k].area();
			if(a > ba) { ba = a; best = k; }
		}
		if(best < 0) break;
		Entry two[2];
		children_of(b2[c[best].ref], two);
		c[best] = two[0];
		c[nc++] = two[1];
	}
	int id = (int)out.size();
	out.push_back(DevBvh4());
	int refs[4];
	for(int k = 0; k < 4; k++) {
		if(k >= nc || c[k].ref == BVH_NONE) refs[k] = BVH_NONE;
		else if(c[k].ref >= 0) refs[k] = collapse_node(b2, c[k].ref, out);
		else refs[k] = c[k].ref;
	}
	DevBvh4 &d = out[id];
	memset(&d, 0, sizeof d);
	for(int k = 0; k < 4; k++) {
		bool ok = k < nc && refs[k] != BVH_NONE;
		d.lox[k] = ok ? c[k].mn[0] : FLT_MAX;
		d.loy[k] = ok ? c[k].mn[1] : FLT_MAX;
		d.loz[k] = ok ? c[k].mn[2] : FLT_MAX;
		d.hix[k] = ok ? c[k].mx[0] : -FLT_MAX;
		d.hiy[k] = ok ? c[k].mx[1] : -FLT_MAX;
		d.hiz[k] = ok ? c[k].mx[2] : -FLT_MAX;
		d.child[k] = refs[k];
	}
	return id;
}
}  // namespace

void MeshBvh::collapse4(std::vector<DevBvh4> &out) const
{
	out.clear();
	if(nodes.empty()) return;
	out.reserve(nodes.size() / 2 + 1);
	collapse_node(nodes, 0, out);
}

void MeshBvh::build(const std::vector<float> &pos)
{
	size_t nf = pos.size() / 9;
	std::vector<float> mn(nf * 3), mx(nf * 3);
	for(size_t i = 0; i < nf; i++) {
		for(int a = 0; a < 3; a++) {
			float lo = pos[i * 9 + a], hi = lo;
			for(int v = 1; v < 3; v++) {
				float c = pos[i * 9 + v * 3 + a];
				lo = std::min(lo, c);
				hi = std::max(hi, c);
			}
			mn[i * 3 + a] = lo;
			mx[i * 3 + a] = hi;
		}
	}
	build_items(mn.data(), mx.data(), nf, LEAF_MAX);
}

}  // namespace sray
