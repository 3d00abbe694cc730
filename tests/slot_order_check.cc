/* Host check of slot_pixel (sray_gb300/csrc/slot_order.h), built and run by
 * tests/test_slot_order.py: for frames of many sizes the first batch's slot
 * -> pixel map is a bijection on the frame's pixels, every 32 slots of a
 * full band cover an 8 x 4 patch (frames at least 8 pixels wide), an
 * active list is followed as given, and tw = 0 maps slot a to pixel a. */
#include <stdio.h>
#include <vector>
#include "slot_order.h"

using namespace sray;

static int failures = 0;

static void check(bool ok, const char *what, int w, int h)
{
	if(!ok) {
		failures++;
		fprintf(stderr, "FAIL %s (%d x %d)\n", what, w, h);
	}
}

int main()
{
	const int sizes[][2] = {{1, 1}, {1, 7}, {7, 1}, {8, 4}, {9, 5}, {31, 17}, {64, 64}, {192, 108}, {1920, 1080}, {1921, 1083},
			{4096, 2160}, {3, 2}};
	for(const auto &sz : sizes) {
		const int w = sz[0], h = sz[1], n = w * h;
		std::vector<int> seen(n, 0);
		bool in_range = true;
		for(int a = 0; a < n; a++) {
			int p = slot_pixel(nullptr, a, w, h);
			if(p < 0 || p >= n) { in_range = false; continue; }
			seen[p]++;
		}
		bool bij = in_range;
		for(int p = 0; p < n; p++) bij = bij && seen[p] == 1;
		check(bij, "bijection", w, h);
		if(w >= 8) {
			bool patches = true;
			for(int band = 0; band < h / 4; band++)
				for(int a0 = band * 4 * w; a0 + 32 <= (band + 1) * 4 * w; a0 += 32) {
					int x0 = w, x1 = -1, y0 = h, y1 = -1;
					for(int a = a0; a < a0 + 32; a++) {
						int p = slot_pixel(nullptr, a, w, h), x = p % w, y = p / w;
						x0 = x < x0 ? x : x0; x1 = x > x1 ? x : x1;
						y0 = y < y0 ? y : y0; y1 = y > y1 ? y : y1;
					}
					patches = patches && x1 - x0 == 7 && y1 - y0 == 3;
				}
			check(patches, "8 x 4 patches", w, h);
		}
	}
	const int list[] = {5, 3, 9, 0};
	bool listed = true;
	for(int a = 0; a < 4; a++) listed = listed && slot_pixel(list, a, 16, 16) == list[a];
	check(listed, "active list", 16, 16);
	bool ident = true;
	for(int a = 0; a < 1000; a++) ident = ident && slot_pixel(nullptr, a, 0, 7) == a;
	check(ident, "identity without a frame size", 0, 7);
	if(failures) return 1;
	printf("slot order: all checks passed\n");
	return 0;
}
