/* The reference-side adapter (sray_gb300/adapter/render_gpu.cc) on the
 * reference's own in-memory scene, without a GPU: load a document with the
 * reference's Scene::load (src/scene.cc:93-183), flatten it with
 * sray_tables_from_scene, and check that the GPU library's host scene
 * built from those tables equals the one its XML loader builds from the
 * document (desc_matches_xml, tests/desc_check.cc).  Built and run by
 * tests/test_scene_desc.py where the reference's sources are present.
 * usage: adapter_check scene.xml t_lo t_hi [reference options...] */
#include <stdio.h>
#include <stdlib.h>
#include <string>
#include <vector>
#include "render_gpu.h"
#include "opt.h"
#include "camera.h"

extern "C" int desc_matches_xml(const sray_scene_desc *d, const char *xml, size_t len, const sray_opts *opt, int lo, int hi,
		int check_textures, char *msg, size_t cap);

int main(int argc, char **argv)
{
	if(argc < 4) {
		fprintf(stderr, "usage: %s scene.xml t_lo t_hi [options]\n", argv[0]);
		return 2;
	}
	const char *path = argv[1];
	int lo = atoi(argv[2]), hi = atoi(argv[3]);
	std::vector<char *> av;
	av.push_back(argv[0]);
	for(int i = 4; i < argc; i++) av.push_back(argv[i]);
	av.push_back((char *)path);
	av.push_back(0);
	if(parse_opt((int)av.size() - 1, av.data()) == -1) return 2;
	opt.verb = -1;
	Scene *scn = new Scene;
	if(!scn->load(path)) return 2;
	if(!scn->get_camera()) scn->set_camera(new Camera);
	SceneTables T;
	std::string err;
	if(!sray_tables_from_scene(scn, lo, hi, &T, &err)) {
		printf("tables: %s\n", err.c_str());
		return 1;
	}
	FILE *f = fopen(path, "rb");
	if(!f) return 2;
	std::string xml;
	char buf[1 << 16];
	size_t n;
	while((n = fread(buf, 1, sizeof buf, f)) > 0) xml.append(buf, n);
	fclose(f);
	sray_opts o;
	sray_default_opts(&o);
	o.width = opt.width;
	o.height = opt.height;
	o.shutter = opt.shutter;
	o.meshoct_max_depth = opt.meshoct_max_depth;
	o.meshoct_max_items = opt.meshoct_max_items;
	char msg[512];
	int ok = desc_matches_xml(&T.desc, xml.data(), xml.size(), &o, lo, hi, 0, msg, sizeof msg);
	printf("%s: %d materials, %d objects, %d lights, window %d..%d ms: %s\n", path, T.desc.n_materials, T.desc.n_objects,
			T.desc.n_lights, lo, hi, msg);
	return ok ? 0 : 1;
}
