/* Host-side checks of the scene loader (no GPU), built and run by
 * tests/test_host_scene.py:
 *   textures  load_texture reads binary PPM (P6) as RGBA floats (v / 255,
 *             alpha 1) from the FIRST directory of SRAY_DATA_PATH only and
 *             rejects other formats; a material attribute's "map" gets the
 *             texture, a map that fails to load leaves it untextured, a
 *             later attribute of the same name replaces colour and texture
 *   keyframes XForm::matrix at the key times equals the node matrix of the
 *             keys; linear keys repeated past the last key are periodic;
 *             step keys hold between keys; clamped tracks hold the end keys
 *   documents malformed or inconsistent scene documents (empty, truncated,
 *             unbalanced tags, unknown types, dangling references, face
 *             indices out of range) are refused with a message
 * Usage: host_check <scratch dir> <animated scene xml> */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>
#include <vector>
#include "scene_host.h"

using namespace sray;

static int failures = 0;

static sray_opts host_opts()
{
	sray_opts o;
	memset(&o, 0, sizeof o);
	o.meshoct_max_depth = 8; o.meshoct_max_items = 8; o.scnoct_max_depth = 8; o.scnoct_max_items = 8;
	return o;
}
#define CHECK(c) do { if(!(c)) { printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); failures++; } } while(0)

static void write_file(const std::string &path, const std::string &data)
{
	FILE *f = fopen(path.c_str(), "wb");
	if(!f) { printf("cannot write %s\n", path.c_str()); exit(2); }
	fwrite(data.data(), 1, data.size(), f);
	fclose(f);
}

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

static void check_textures(const std::string &dir)
{
	std::string a = dir + "/a", b = dir + "/b";
	std::string cmd = "mkdir -p " + a + " " + b;
	if(system(cmd.c_str()) != 0) { printf("mkdir failed\n"); exit(2); }
	/* 2x1 image: (255, 0, 51) (102, 204, 255), with a header comment */
	std::string ppm = "P6\n# made by host_check\n2 1\n255\n";
	const unsigned char px[6] = {255, 0, 51, 102, 204, 255};
	ppm.append((const char *)px, 6);
	write_file(b + "/t.ppm", ppm);
	write_file(b + "/ascii.ppm", "P3\n1 1\n255\n1 2 3\n");
	std::string wide = "P6\n1 1\n65535\n";
	wide.append(6, '\0');
	write_file(b + "/wide.ppm", wide);
	write_file(b + "/short.ppm", "P6\n4 4\n255\nabc");

	Texture t;
	setenv("SRAY_DATA_PATH", (a + ":" + b).c_str(), 1);
	CHECK(!load_texture("t.ppm", t));          /* only the first directory is searched */
	setenv("SRAY_DATA_PATH", (b + ":" + a).c_str(), 1);
	CHECK(load_texture("t.ppm", t));
	CHECK(t.xsz == 2 && t.ysz == 1 && t.pix.size() == 8);
	if(t.pix.size() == 8) {
		const float want[8] = {1.0f, 0.0f, 51 / 255.0f, 1.0f, 102 / 255.0f, 204 / 255.0f, 1.0f, 1.0f};
		for(int i = 0; i < 8; i++) CHECK(t.pix[i] == want[i]);
	}
	CHECK(!load_texture("ascii.ppm", t));
	CHECK(!load_texture("wide.ppm", t));
	CHECK(!load_texture("short.ppm", t));
	CHECK(!load_texture("missing.ppm", t));
	unsetenv("SRAY_DATA_PATH");
	CHECK(!load_texture("t.ppm", t));

	/* materials: textured attributes, a failing map, a replaced attribute */
	setenv("SRAY_DATA_PATH", b.c_str(), 1);
	const char *xml =
		"<scene>\n"
		"<material name=\"m\" shader=\"phong\">\n"
		"<mattr name=\"diffuse\" value=\"0.5 0.6 0.7\" map=\"t.ppm\"/>\n"
		"<mattr name=\"specular\" value=\"0.3\" map=\"nothere.ppm\"/>\n"
		"<mattr name=\"ior\" value=\"1.4\" map=\"t.ppm\"/>\n"
		"<mattr name=\"ior\" value=\"1.6\"/>\n"
		"<mattr name=\"normal\" value=\"2.0\" map=\"t.ppm\"/>\n"
		"</material>\n"
		"<material name=\"n\" shader=\"phong\"><mattr name=\"normal\" value=\"1\"/></material>\n"
		"<object type=\"sphere\" name=\"s\"><matref name=\"m\"/><sphere rad=\"1.0\"/></object>\n"
		"</scene>\n";
	sray_opts opt = host_opts();
	HostScene sc;
	std::string err;
	bool ok = sc.load(xml, strlen(xml), opt, err);
	CHECK(ok);
	if(ok) {
		CHECK(sc.mats.size() == 2);
		CHECK(sc.texs.size() == 3);               /* one copy per map that loaded */
		const Material &m = sc.mats[0];
		/* XML numbers are read as float (src/xmltree.c:75-93) */
		CHECK(m.tex[TA_DIFFUSE] >= 0 && m.kd[0] == 0.5 && m.kd[2] == (double)0.7f);
		CHECK(m.tex[TA_SPECULAR] == -1 && m.ks[0] == (double)0.3f);
		CHECK(m.tex[TA_IOR] == -1 && m.ior == (double)1.6f);
		CHECK(m.have_normal && m.tex[TA_NORMAL] >= 0 && m.nrm_scale == 2.0);
		CHECK(sc.mats[1].have_normal && sc.mats[1].tex[TA_NORMAL] == -1 && sc.mats[1].nrm_scale == 1.0);
	} else {
		printf("load: %s\n", err.c_str());
	}
	unsetenv("SRAY_DATA_PATH");
}

static double mdiff(const double a[4][4], const double b[4][4])
{
	double d = 0.0;
	for(int i = 0; i < 4; i++) for(int j = 0; j < 4; j++) d = fmax(d, fabs(a[i][j] - b[i][j]));
	return d;
}

static void check_keyframes(const char *scene)
{
	std::string text = slurp(scene);
	sray_opts opt = host_opts();
	HostScene sc;
	std::string err;
	if(!sc.load(text.data(), text.size(), opt, err)) { printf("load: %s\n", err.c_str()); failures++; return; }
	int checked = 0;
	for(const Object &o : sc.objs) {
		const XForm &x = o.xf;
		/* at each position key time (with the other tracks' values there), the node matrix of the keys */
		for(size_t k = 0; k < x.pos.time.size(); k++) {
			int t = x.pos.time[k];
			double m[4][4], want[4][4];
			x.matrix(t, m);
			double p[3] = {x.pos.val[k].x, x.pos.val[k].y, x.pos.val[k].z}, q[4], s[3];
			KeyView kr = {x.rot.time.data(), (const double *)x.rot.val.data(), (const double *)&x.rot.def, (int)x.rot.time.size(), 4,
				x.rot.interp, x.rot.extrap};
			KeyView ks = {x.scale.time.data(), (const double *)x.scale.val.data(), (const double *)&x.scale.def, (int)x.scale.time.size(), 3,
				x.scale.interp, x.scale.extrap};
			key_eval(kr, t, q);
			key_eval(ks, t, s);
			double pv[3] = {x.pivot.x, x.pivot.y, x.pivot.z};
			node_matrix(p, q, s, pv, want);
			CHECK(mdiff(m, want) == 0.0);
			checked++;
		}
		size_t n = x.pos.time.size();
		if(n >= 2) {
			int first = x.pos.time[0], last = x.pos.time[n - 1];
			double a[4][4], b[4][4];
			if(x.pos.extrap == EXTRAP_REPEAT) {
				for(int t = last + 1; t < last + 600; t += 37) {
					x.matrix(t, a);
					x.matrix(t - (last - first), b);
					CHECK(mdiff(a, b) < 1e-12);
					checked++;
				}
			} else {
				x.matrix(last + 500, a);
				x.matrix(last, b);
				CHECK(mdiff(a, b) == 0.0);
				x.matrix(first - 500, a);
				x.matrix(first, b);
				CHECK(mdiff(a, b) == 0.0);
				checked++;
			}
			if(x.pos.interp == INTERP_STEP) {
				int t0 = x.pos.time[0], t1 = x.pos.time[1];
				/* the nearest key decides the interval: before the midpoint the first key holds */
				x.matrix(t0, a);
				x.matrix(t0 + (t1 - t0) / 2 - 1, b);
				CHECK(mdiff(a, b) == 0.0);
				checked++;
			}
		}
	}
	printf("keyframe checks: %d\n", checked);
	CHECK(checked > 10);
}

/* malformed documents: every one is refused with a message, none crashes
 * (the reference's loader prints and returns false, src/scene.cc:79-90) */
static void check_bad_documents(const char *good_path)
{
	std::string good = slurp(good_path);
	CHECK(good.size() > 200);
	struct Case { const char *what; std::string text; const char *needle; };
	std::vector<Case> cases = {
		{"empty", "", "no root element"},
		{"not xml", "this is not a scene", "no root element"},
		{"truncated", good.substr(0, good.size() / 2), "end of document"},
		{"unclosed", "<scene><material name=\"m\"></scene>", "mismatched closing tag"},
		{"bad attribute", "<scene><material name=m/></scene>", "unquoted attribute value"},
		{"unknown object", "<scene><object name=\"o\" type=\"torus\"/></scene>", "unknown type"},
		{"missing material", "<scene><object name=\"o\" type=\"sphere\"><matref name=\"nope\"/><sphere rad=\"1.0\"/></object></scene>",
			"does not exist"},
		{"face index", "<scene><object name=\"m\" type=\"mesh\"><mesh><vertex id=\"0\" val=\"0 0 0\"/>"
			"<vertex id=\"1\" val=\"1 0 0\"/><vertex id=\"2\" val=\"0 1 0\"/>"
			"<face><vref vertex=\"0\"/><vref vertex=\"1\"/><vref vertex=\"7\"/></face></mesh></object></scene>",
			"out of range"},
		{"light type", "<scene><light type=\"spot\"/></scene>", "unknown type"},
	};
	for(const Case &c : cases) {
		HostScene sc;
		std::string err;
		bool ok = sc.load(c.text.data(), c.text.size(), host_opts(), err);
		printf("bad document (%s): %s\n", c.what, ok ? "LOADED" : err.c_str());
		CHECK(!ok);
		CHECK(err.find(c.needle) != std::string::npos);
	}
	HostScene sc;
	std::string err;
	CHECK(sc.load(good.data(), good.size(), host_opts(), err));
}

int main(int argc, char **argv)
{
	if(argc < 3) {
		printf("usage: %s scratch_dir animated_scene.xml\n", argv[0]);
		return 2;
	}
	check_textures(argv[1]);
	check_keyframes(argv[2]);
	check_bad_documents(argv[2]);
	if(failures) {
		printf("%d failures\n", failures);
		return 1;
	}
	printf("host checks ok\n");
	return 0;
}
