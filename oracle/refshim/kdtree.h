/* kdtree.h -- TEST INFRASTRUCTURE: a stand-in for the kdtree library
 * (code.google.com/p/kdtree, by the reference's author; not shipped with the
 * reference).  Only the calls of src/pmap.cc are provided, with the
 * library's semantics: positions inserted by kd_insert3f and the query of
 * kd_nearest_range3f are rounded to float, a point is in range when its
 * squared distance (in double) is <= range^2.  Points are kept in a list and
 * bucketed in a uniform grid built on the first query. */
#ifndef SHIM_KDTREE_H_
#define SHIM_KDTREE_H_

#ifdef __cplusplus
extern "C" {
#endif

struct kdtree;
struct kdres;

struct kdtree *kd_create(int k);
void kd_free(struct kdtree *tree);
void kd_clear(struct kdtree *tree);
void kd_data_destructor(struct kdtree *tree, void (*destr)(void *));
int kd_insert3f(struct kdtree *tree, float x, float y, float z, void *data);
struct kdres *kd_nearest_range3f(struct kdtree *tree, float x, float y, float z, float range);
void kd_res_free(struct kdres *set);
int kd_res_size(struct kdres *set);
int kd_res_end(struct kdres *set);
int kd_res_next(struct kdres *set);
void *kd_res_item(struct kdres *set, double *pos);

#ifdef __cplusplus
}
#endif

#endif
