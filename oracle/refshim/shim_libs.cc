/* shim_libs.cc -- TEST INFRASTRUCTURE: implementations behind the stand-in
 * headers (vmath random streams, kdtree, imago2) for the compiled reference. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <utility>
#include <vector>
#include "vmath/vmath.h"
#include "kdtree.h"
#include "imago2.h"

scalar_t Ray::env_ior = 1.0;

static thread_local sray_rng *g_cur = nullptr;
static thread_local sray_rng g_fallback;
static thread_local bool g_fallback_init = false;

sray_rng *shim_rng_current(void)
{
	if(g_cur) return g_cur;
	if(!g_fallback_init) {
		sray_rng_init(&g_fallback, 0x5EED0001ull, SRAY_DOM_USER, 0, 0);
		g_fallback_init = true;
	}
	return &g_fallback;
}

void shim_rng_select(sray_rng *s) { g_cur = s; }

extern "C" int shim_rand(void) { return sray_rng_int(shim_rng_current()); }

/* ---- kdtree ---- */
struct kdpoint { float pos[3]; void *data; };
/* The index (points sorted by the cell of the query radius) is built by the
 * first query and reused while the radius stays the same.  Queries come from
 * the reference's tpool workers at once (the real library's queries only
 * read the tree), so the build runs under a lock and the others wait for it;
 * a query with another radius rebuilds, which the reference never does
 * while others query (each map has one gather radius per frame). */
struct kdtree {
	std::vector<kdpoint> pts;
	void (*destr)(void *) = nullptr;
	std::atomic<bool> built{false};
	double cell = 0.0;
	std::mutex mu;
	std::vector<std::pair<unsigned long long, int> > keys;
};
struct kdres {
	std::vector<std::pair<void *, const float *> > items;
	size_t cur = 0;
};

static unsigned long long pack_key(long long x, long long y, long long z)
{
	return ((unsigned long long)(x & 0x1fffff) << 42) | ((unsigned long long)(y & 0x1fffff) << 21) | (unsigned long long)(z & 0x1fffff);
}

static void build_index(struct kdtree *t, double cell)
{
	t->built.store(false, std::memory_order_release);
	t->cell = cell;
	t->keys.resize(t->pts.size());
	for(size_t i = 0; i < t->pts.size(); i++) {
		long long c[3];
		for(int k = 0; k < 3; k++) c[k] = (long long)floor((double)t->pts[i].pos[k] / t->cell);
		t->keys[i] = std::make_pair(pack_key(c[0], c[1], c[2]), (int)i);
	}
	std::sort(t->keys.begin(), t->keys.end());
	t->built.store(true, std::memory_order_release);
}

extern "C" {

struct kdtree *kd_create(int k) { return k == 3 ? new kdtree : nullptr; }
void kd_clear(struct kdtree *t)
{
	if(t->destr) for(auto &p : t->pts) t->destr(p.data);
	t->pts.clear();
	t->keys.clear();
	t->built.store(false);
}
void kd_free(struct kdtree *t) { if(t) { kd_clear(t); delete t; } }
void kd_data_destructor(struct kdtree *t, void (*d)(void *)) { t->destr = d; }
int kd_insert3f(struct kdtree *t, float x, float y, float z, void *data)
{
	kdpoint p;
	p.pos[0] = x; p.pos[1] = y; p.pos[2] = z;
	p.data = data;
	t->pts.push_back(p);
	t->built.store(false);
	return 0;
}

struct kdres *kd_nearest_range3f(struct kdtree *t, float x, float y, float z, float range)
{
	kdres *r = new kdres;
	double q[3] = {x, y, z}, rg = range, r2 = rg * rg;
	double want = rg > 0.0 ? rg : 1.0;
	if(!t->built.load(std::memory_order_acquire) || t->cell != want) {
		std::lock_guard<std::mutex> lk(t->mu);
		if(!t->built.load(std::memory_order_acquire) || t->cell != want) build_index(t, want);
	}
	long long lo[3], hi[3];

	for(int k = 0; k < 3; k++) { lo[k] = (long long)floor((q[k] - rg) / t->cell); hi[k] = (long long)floor((q[k] + rg) / t->cell); }
	for(long long a = lo[0]; a <= hi[0]; a++)
	for(long long b = lo[1]; b <= hi[1]; b++)
	for(long long c = lo[2]; c <= hi[2]; c++) {
		unsigned long long key = pack_key(a, b, c);
		auto it = std::lower_bound(t->keys.begin(), t->keys.end(), std::make_pair(key, -1));
		for(; it != t->keys.end() && it->first == key; ++it) {
			const kdpoint &p = t->pts[it->second];
			double d2 = 0.0;
			for(int k = 0; k < 3; k++) { double d = (double)p.pos[k] - q[k]; d2 += d * d; }
			if(d2 <= r2) r->items.push_back(std::make_pair(p.data, p.pos));
		}
	}
	return r;
}

void kd_res_free(struct kdres *s) { delete s; }
int kd_res_size(struct kdres *s) { return (int)s->items.size(); }
int kd_res_end(struct kdres *s) { return s->cur >= s->items.size(); }
int kd_res_next(struct kdres *s) { s->cur++; return s->cur < s->items.size(); }
void *kd_res_item(struct kdres *s, double *pos)
{
	if(s->cur >= s->items.size()) return nullptr;
	if(pos) for(int k = 0; k < 3; k++) pos[k] = s->items[s->cur].second[k];
	return s->items[s->cur].first;
}

/* ---- imago2 ----
 * Loading reads binary PPM (P6, maxval <= 255) into RGBA floats (v / 255,
 * alpha 1), rows top first, the subset of libimago's formats the texture
 * tests use; other files fail to load. */
static int ppm_token(FILE *fp)
{
	int c, v = 0, any = 0;
	while((c = fgetc(fp)) != EOF) {
		if(c == '#') { while((c = fgetc(fp)) != EOF && c != '\n') {} continue; }
		if(c >= '0' && c <= '9') { v = v * 10 + (c - '0'); any = 1; }
		else if(any) break;
	}
	return any ? v : -1;
}

void *img_load_pixels(const char *fname, int *xsz, int *ysz, int fmt)
{
	if(fmt != IMG_FMT_RGBAF) return nullptr;
	FILE *fp = fopen(fname, "rb");
	if(!fp) return nullptr;
	char magic[2];
	if(fread(magic, 1, 2, fp) != 2 || magic[0] != 'P' || magic[1] != '6') { fclose(fp); return nullptr; }
	int w = ppm_token(fp), h = ppm_token(fp), maxv = ppm_token(fp);
	if(w <= 0 || h <= 0 || maxv <= 0 || maxv > 255) { fclose(fp); return nullptr; }
	size_t n = (size_t)w * h;
	unsigned char *rgb = (unsigned char *)malloc(n * 3);
	float *out = (float *)malloc(n * 4 * sizeof(float));
	if(!rgb || !out || fread(rgb, 1, n * 3, fp) != n * 3) { free(rgb); free(out); fclose(fp); return nullptr; }
	fclose(fp);
	for(size_t i = 0; i < n; i++) {
		for(int k = 0; k < 3; k++) out[i * 4 + k] = rgb[i * 3 + k] / 255.0f;
		out[i * 4 + 3] = 1.0f;
	}
	free(rgb);
	*xsz = w;
	*ysz = h;
	return out;
}
void img_free_pixels(void *p) { free(p); }
int img_save_pixels(const char *fname, void *pix, int xsz, int ysz, int fmt)
{
	if(fmt != IMG_FMT_RGBAF) return -1;
	FILE *fp = fopen(fname, "wb");
	if(!fp) return -1;
	fprintf(fp, "PF\n%d %d\n-1.0\n", xsz, ysz);
	const float *f = (const float *)pix;
	for(int y = ysz - 1; y >= 0; y--)
		for(int x = 0; x < xsz; x++) fwrite(f + ((size_t)y * xsz + x) * 4, sizeof(float), 3, fp);
	fclose(fp);
	return 0;
}

}  /* extern "C" */
