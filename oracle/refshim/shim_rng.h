/* shim_rng.h -- TEST INFRASTRUCTURE: force-included into every reference
 * source file when the reference is compiled as the oracle's pin.  It routes
 * the C library's rand() to the Philox stream selected by the harness.  The
 * standard headers that mention rand() are included first so the macro only
 * affects the reference's own code (unistd.h too: src/render.cc calls write()
 * without including it). */
#ifndef SHIM_RNG_H_
#define SHIM_RNG_H_
#include <stdlib.h>
#include <unistd.h>
#ifdef __cplusplus
#include <cstdlib>
#include <algorithm>
#include <vector>
#include <list>
#include <string>
#include <queue>
#include <set>
#include <map>
extern "C" {
#endif
int shim_rand(void);
#ifdef __cplusplus
}
#endif
#define rand() shim_rand()
#endif
