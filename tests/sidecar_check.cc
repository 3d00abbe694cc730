/* Host-side check of the mesh side-car (no GPU): a document loaded through
 * a side-car it wrote has the same meshes, octrees, hierarchies and objects
 * as the document parsed in full; a changed document ignores a stale
 * side-car.  Built and run by tests/test_sidecar.py. */
#include <stdio.h>
#include <string.h>
#include <string>
#include <vector>
#include "scene_host.h"

using namespace sray;

static std::string slurp(const char *path)
{
	FILE *f = fopen(path, "rb");
	if(!f) return std::string();
	std::string s;
	char buf[1 << 16];
	size_t n;
	while((n = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
	fclose(f);
	return s;
}

static bool same(const HostScene &a, const HostScene &b)
{
	if(a.n_tris != b.n_tris || a.meshes.size() != b.meshes.size() || a.objs.size() != b.objs.size()) return false;
	for(size_t i = 0; i < a.objs.size(); i++) {
		if(a.objs[i].type != b.objs[i].type || a.objs[i].mesh != b.objs[i].mesh || a.objs[i].mat != b.objs[i].mat ||
				a.objs[i].name != b.objs[i].name) return false;
	}
	for(size_t u = 0; u < a.meshes.size(); u++) {
		const Mesh &x = a.meshes[u], &y = b.meshes[u];
		if(x.posd != y.posd || x.pos != y.pos || x.attr != y.attr || x.hash != y.hash) return false;
		if(x.oct.nodes.size() != y.oct.nodes.size()) return false;
		for(size_t n = 0; n < x.oct.nodes.size(); n++) {
			const BuildOctree::Node &p = x.oct.nodes[n], &q = y.oct.nodes[n];
			if(memcmp(&p.box, &q.box, sizeof p.box) || p.child != q.child || p.items != q.items) return false;
		}
		if(x.bvh.nodes.size() != y.bvh.nodes.size() || x.bvh.order != y.bvh.order || x.bvh.depth != y.bvh.depth) return false;
		if(!x.bvh.nodes.empty() && memcmp(x.bvh.nodes.data(), y.bvh.nodes.data(), x.bvh.nodes.size() * sizeof(x.bvh.nodes[0])))
			return false;
	}
	return true;
}

int main(int argc, char **argv)
{
	if(argc < 3) return 2;
	std::string doc = slurp(argv[1]);
	const char *car = argv[2];
	if(doc.empty()) { printf("cannot read %s\n", argv[1]); return 2; }
	sray_opts o;
	memset(&o, 0, sizeof o);
	o.width = 64; o.height = 64;
	o.meshoct_max_depth = 8; o.meshoct_max_items = 8; o.scnoct_max_depth = 8; o.scnoct_max_items = 8;
	std::string err;
	bool used = true;
	HostScene full, first, cached;
	if(!full.load(doc.data(), doc.size(), o, err)) { printf("load: %s\n", err.c_str()); return 1; }
	remove(car);
	if(!first.load(doc.data(), doc.size(), o, err, car, &used) || used) { printf("first side-car load: %s used %d\n", err.c_str(), used); return 1; }
	if(!cached.load(doc.data(), doc.size(), o, err, car, &used) || !used) { printf("second side-car load: %s used %d\n", err.c_str(), used); return 1; }
	if(!same(full, first) || !same(full, cached)) { printf("side-car scene differs from the document\n"); return 1; }
	/* a changed document (one vertex moved) must not take the stale side-car */
	std::string doc2 = doc;
	size_t at = doc2.find("<vertex");
	if(at == std::string::npos) { printf("no vertex element\n"); return 1; }
	size_t val = doc2.find("val=\"", at);
	doc2[val + 5] = doc2[val + 5] == '1' ? '2' : '1';
	HostScene full2, cached2;
	if(!full2.load(doc2.data(), doc2.size(), o, err)) { printf("load 2: %s\n", err.c_str()); return 1; }
	if(!cached2.load(doc2.data(), doc2.size(), o, err, car, &used) || used) { printf("stale side-car used\n"); return 1; }
	if(!same(full2, cached2) || same(full, full2)) { printf("changed document loaded wrongly\n"); return 1; }
	/* other octree options: the side-car (now of doc2) is not used */
	o.meshoct_max_depth = 6;
	HostScene other;
	if(!other.load(doc2.data(), doc2.size(), o, err, car, &used) || used) { printf("side-car used with other octree options\n"); return 1; }
	printf("side-car ok: %lld triangles, %zu unique meshes, %zu objects\n", (long long)full.n_tris, full.meshes.size(), full.objs.size());
	return 0;
}
