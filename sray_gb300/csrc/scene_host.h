/* scene_host.h -- host side of the GB300 renderer: the S-ray scene database
 * (XML loader, transforms, materials, objects, lights, camera), the octree
 * builds and their flattening into the device layouts.
 *
 * Everything here runs once per scene load (meshes) or once per frame
 * (top-level octree, per-time matrices, projection maps) in double
 * precision, exactly as the reference computes it, and is rounded to float
 * only when written into the device tables.
 */
#ifndef SRAY_SCENE_HOST_H_
#define SRAY_SCENE_HOST_H_

#include <stdint.h>
#include <string>
#include <vector>
#include "sray_gpu.h"
#include "sray_device.h"
#include "anim_eval.h"

namespace sray {


struct Vec3 {
	double x, y, z;
	Vec3() : x(0), y(0), z(0) {}
	Vec3(double a, double b, double c) : x(a), y(b), z(c) {}
	double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct Quat { double s, x, y, z; };

template <class T> struct Track {
	T def;
	std::vector<int> time;
	std::vector<T> val;
	int interp = INTERP_LINEAR, extrap = EXTRAP_CLAMP;
};

struct XForm {
	Track<Vec3> pos, scale;
	Track<Quat> rot;
	Vec3 pivot;
	XForm();
	Vec3 position(int t) const;
	Vec3 scaling(int t) const;
	void matrix(int t, double m[4][4]) const;
};

struct Material {
	std::string name;
	int phong = 0;
	double kd[4] = {1, 1, 1, 0}, ks[4] = {0, 0, 0, 0};
	double shin = 1.0, refl = 0.0, refr = 0.0, ior = 1.5;
	bool have_normal = false;         /* a "normal" attribute is present */
	double nrm_scale = 1.0;           /* its colour's x */
	int tex[TA_COUNT] = {-1, -1, -1, -1, -1, -1, -1};   /* texture per attribute, -1 = none */
};

/* a texture image: RGBA floats, rows top first */
struct Texture {
	int xsz = 0, ysz = 0;
	std::vector<float> pix;
};

/* Texture::load (src/texture.cc:28-36): the file found by find_file
 * (src/datapath.c:57-77) in the first directory of SRAY_DATA_PATH (the
 * reference's list parser stops after the first entry), read as RGBA
 * floats.  Binary PPM (P6, maxval <= 255) is the format read. */
bool load_texture(const char *name, Texture &t);

enum { OBJ_SPHERE = 0, OBJ_CYLINDER = 1, OBJ_MESH = 2 };
enum { LT_POINT = 0, LT_SPHERE = 1, LT_BOX = 2 };

struct Box { double mn[3], mx[3]; };

/* an octree in build form: children of a node are 8 consecutive entries */
struct BuildOctree {
	struct Node { Box box; std::vector<int> items; int child = -1; };
	std::vector<Node> nodes;
	void build(const std::vector<Box> &item_boxes, int max_depth, int max_items);
};

/* A binary bounding-volume hierarchy over a mesh's triangles, built by the
 * surface-area heuristic over 16 bins per axis.  It only speeds up finding
 * candidates; which hit counts is still decided by the mesh octree (the
 * traversal confirms every hit against it). */
struct MeshBvh {
	std::vector<DevBvhNode> nodes;   /* child references relative to this hierarchy */
	std::vector<int> order;          /* items in leaf order */
	int depth = 0;
	void build(const std::vector<float> &pos);   /* over faces: 9 floats each */
	/* over boxes (3 floats min, 3 max per item), at most leaf_max per leaf */
	void build_items(const float *mn, const float *mx, size_t n, int leaf_max);
	/* the same hierarchy with up to four children per node: each node takes
	 * over the children of its largest inner children (by surface area) */
	void collapse4(std::vector<DevBvh4> &out) const;
};

/* one unique triangle mesh (identical meshes of several objects share it) */
struct Mesh {
	std::vector<float> pos;    /* 9 floats per face: the three vertices (object space) */
	std::vector<double> posd;  /* same, as parsed */
	std::vector<float> attr;   /* 24 floats per face: normals 9, tangents 9, texcoords 6 */
	uint64_t hash = 0;
	BuildOctree oct;
	MeshBvh bvh;
	int node_base = 0;         /* first node in the device mesh-node array */
	int bvh_base = -1;         /* root in the device hierarchy-node array */
	int tri_base = 0;          /* first face in the device attribute table */
};

struct Object {
	int type = OBJ_SPHERE;
	std::string name;
	int mat = -1;
	XForm xf;
	double rad = 1.0, start = -1.0, end = 1.0;
	int mesh = -1;
	bool is_static = false;    /* every transform track has at most one key */
	Box static_box;
	Box bounds(const std::vector<Mesh> &meshes, int t) const;
};

struct ProjMap {
	int udiv = 64, vdiv = 32;
	std::vector<char> cells;
	std::vector<double> cell_area;
	double total_area = 0.0, coverage = 0.0;
	ProjMap();
	void corner_dir(int uc, int vc, int corner, double out[3]) const;
	void cell_from_dir(const double d[3], int *uc, int *vc) const;
	void set_cell(int uc, int vc, bool v);
	void set_all(bool v);
	void clear();
	double get_coverage() const;
};

struct Light {
	int type = LT_POINT;
	double col[4] = {1, 1, 1, 1};
	XForm xf;
	float radius = 1.0f;
	Vec3 dim = Vec3(1, 1, 1);
	ProjMap pm, spm;
};

struct Camera {
	int target = 0;
	XForm xf, txf;
	double vfov = 0.78539816339744830962, aspect = 1.0, max_dist = SRAY_RAY_MAGNITUDE;
	int shutter = 0;
	void matrix(int t, double m[4][4]) const;
};

/* one scene of a scene set: its objects and lights (index ranges into the
 * set's tables), camera and environment */
struct SceneRange {
	int obj0 = 0, nobj = 0, light0 = 0, nlight = 0;
	Camera cam;
	double env_ior = 1.0, env_col[4] = {0, 0, 0, 0}, env_amb[4] = {0, 0, 0, 0};
};

struct HostScene {
	std::vector<Material> mats;
	Material defmat;
	std::vector<Texture> texs;
	std::vector<Object> objs;
	std::vector<Light> lights;
	std::vector<Mesh> meshes;
	Camera cam;
	double env_ior = 1.0, env_col[4] = {0, 0, 0, 0}, env_amb[4] = {0, 0, 0, 0};
	int64_t n_tris = 0;

	/* a scene set (several documents loaded together for batches whose jobs
	 * render different scenes): one range per scene; empty for one scene */
	std::vector<SceneRange> ranges;
	/* append `other` as the set's next scene (materials, textures, meshes,
	 * objects and lights re-indexed) */
	void append_scene(HostScene &&other);

	/* per-frame state */
	BuildOctree oct;
	double gather_dist = 0.0;
	int bt0 = 0, bt1 = 0;
	std::vector<Box> box_t0, box_t1;   /* object bounds at the frame's t0 / t1 */
	std::vector<Box> oct_boxes;        /* the boxes the scene octree was built from */
	Box object_bounds(size_t i, int t) const;

	/* Load an S-ray XML document.  With a side-car path: when the file
	 * there holds the meshes of this exact document (and their octrees and
	 * hierarchies for the same mesh octree options), they are read from it
	 * and the XML's <mesh> elements are skipped; otherwise the document is
	 * loaded in full and the side-car is written.  *used tells which. */
	bool load(const char *text, size_t len, const sray_opts &opt, std::string &err, const char *sidecar = nullptr,
			bool *used = nullptr);
	/* Load a scene given as tables (sray_gpu_upload_scene). */
	bool from_desc(const sray_scene_desc &d, const sray_opts &opt, std::string &err);
	void finish_load(const sray_opts &opt, bool build_meshes);
	void build_tree(int t0, int t1, const sray_opts &opt);
	/* build_tree's object bounds cache, root box and gather radius without
	 * the octree (a scene set's scenes have octrees of their own): oct keeps
	 * its root node only */
	void bound_objects(int t0, int t1, const sray_opts &opt);
	/* the root box and gather radius build_tree(t0, t1) would give the
	 * objects obj0 .. obj0 + nobj, without building */
	Box box_at(int t0, int t1, int obj0 = 0, int nobj = -1) const;
	double gather_dist_at(int t0, int t1, const sray_opts &opt, int obj0 = 0, int nobj = -1) const;
	/* the projection maps of lights [light0, light0 + nlight) over objects
	 * [obj0, obj0 + nobj) (all by default); a light's stream is keyed by its
	 * index within that range */
	void build_projmaps(int t0, int t1, uint64_t seed, int light0 = 0, int nlight = -1, int obj0 = 0, int nobj = -1);
	void build_light_projmaps(size_t li, int t0, int t1, uint64_t seed, int key, int obj0, int nobj);
	/* the same maps of light li into pm / spm (the light's own are untouched) */
	void light_projmaps(size_t li, int t0, int t1, uint64_t seed, int key, int obj0, int nobj, ProjMap &pm, ProjMap &spm) const;
};

/* general 4x4 inverse by the adjugate */
void mat_inverse(double out[4][4], const double m[4][4]);

/* Flatten an octree breadth first into device nodes; leaf items are
 * appended to `slots` (their indices into the item array). */
void flatten_octree(const BuildOctree &oct, std::vector<DevNode> &nodes, std::vector<int> &slots,
		std::vector<int> *index_of = nullptr);

/* For every face of a mesh: the deepest node of its octree whose box holds
 * the face's bounds (the node below which all the leaves listing the face
 * lie), as an index into the flattened nodes (index_of from flatten_octree). */
void octree_homes(const BuildOctree &oct, const std::vector<double> &posd, const std::vector<int> &index_of,
		std::vector<int> &home);
/* the same for items given by their boxes */
void octree_homes_boxes(const BuildOctree &oct, const std::vector<Box> &boxes, const std::vector<int> &index_of,
		std::vector<int> &home);

}  // namespace sray

#endif
