/* sray_device.h -- device-resident scene layout shared by the host builder
 * and the CUDA kernels (plain structs, no CUDA types).
 *
 * HBM layout (all arrays 16-byte aligned):
 *   mesh_nodes   DevNode[ ]  octree nodes of every unique mesh, breadth first,
 *                            the 8 children of a node consecutive (32 B each)
 *   mesh_tris    DevTri[ ]   one 48 B record per leaf slot: the triangle's three
 *                            object-space vertices and its unnormalised normal
 *                            cross(v1-v0, v2-v0), duplicated into every leaf
 *                            the triangle overlaps, so a leaf is one
 *                            contiguous, 16 B-vector-loadable run
 *   mesh_prim    int[ ]      triangle index of each slot (read on a hit only)
 *   tri_pos/attr float[ ]    per unique-mesh triangle: vertices (9 floats) and
 *                            normals/tangents/texcoords (24 floats), read once
 *                            per shaded hit for the attribute interpolation
 *   scene_nodes/scene_slots  top-level octree over objects (rebuilt per frame)
 *   objs         DevObj[ ]   type, material, mesh root, xform table index
 *   xf           float[ ]    per object per integer time: forward 3x4,
 *                            inverse 3x4, inverse-transpose 3x3 (36 floats)
 */
#ifndef SRAY_DEVICE_H_
#define SRAY_DEVICE_H_

#include <stdint.h>

namespace sray {

/* an octree node; the children of an inner node are the octants of its box
 * split at `mid`, so their boxes are not stored */
struct alignas(16) DevNode {
	float mn[3];
	int first;      /* inner: index of child slot 0; leaf: first slot */
	float mx[3];
	int count;      /* inner: -1; leaf: number of slots */
	float mid[3];   /* inner: split point (the reference's box centre) */
	unsigned mask;  /* inner: bit k set when child slot k holds items */
};

/* a node of a mesh's bounding-volume hierarchy: the boxes of its two
 * children and their references.  A reference >= 0 is a node index, BVH_NONE
 * an absent child, and any other negative value r a leaf holding the
 * (~r) & 15 triangles that start at (~r) >> 4 in the hierarchy's triangle
 * order. */
#define BVH_NONE 0x7fffffff

struct alignas(16) DevBvhNode {
	float lmn[3], lmx[3];
	float rmn[3], rmx[3];
	int left, right;
	int pad[2];
};

/* a node of the 4-wide hierarchies the GPU traverses, one 128-byte line:
 * the boxes of up to four children (planes in structure-of-arrays order)
 * and their references, encoded as in DevBvhNode */
struct alignas(128) DevBvh4 {
	float lox[4], loy[4], loz[4];
	float hix[4], hiy[4], hiz[4];
	int child[4];
	int pad[4];
};

struct alignas(16) DevTri {
	float a[4];     /* v0.xyz, n.x */
	float b[4];     /* v1.xyz, n.y */
	float c[4];     /* v2.xyz, n.z */
};

struct alignas(16) DevObj {
	int type;       /* 0 sphere, 1 cylinder, 2 mesh */
	int mat;        /* material index, -1 = default material */
	int mesh_root;  /* mesh: root node in mesh_nodes, -1 if the mesh is empty */
	int tri_base;   /* mesh: first triangle of its unique mesh in tri_pos/tri_attr */
	float rad, start, end;
	int bvh_root;   /* mesh: root node in the mesh hierarchies, -1 if none */
};

/* attributes that can carry a texture, in DevMat::tex order */
enum { TA_DIFFUSE, TA_SPECULAR, TA_SHININESS, TA_REFLECT, TA_REFRACT, TA_IOR, TA_NORMAL, TA_COUNT };

struct alignas(16) DevMat {
	float kd[4], ks[4];
	float shin, refl, refr, ior;
	int phong;
	int textured;      /* some attribute has a texture */
	int have_normal;   /* the material has a "normal" attribute (src/shader.cc:136-139) */
	int pad;
	int tex[8];        /* texture of each attribute (TA_*), -1 = none */
	float scol[8];     /* the attribute colour's x: factor of a textured scalar, bump scale */
};

/* a texture: RGBA float texels, rows top first, at `off` (in texels) in the
 * scene's texel table */
struct alignas(16) DevTex {
	long long off;
	int xsz, ysz;
};

struct alignas(16) DevLight {
	int type;       /* 0 point, 1 sphere, 2 box */
	float radius;
	float pad0[2];
	float col[4];
	float dim[4];
	float box_m[12];   /* transform at time 0 (BoxLight::get_point) */
};

enum { XF_STRIDE = 36 };

/* the keyframe tracks of an object (or a light: position only) on the
 * device: per track (position, rotation, scale) its first key time in the
 * key-time table, its first value in the key-value table (3 doubles per
 * position / scale key, 4 per rotation key), its key count, interpolation
 * and extrapolation; the pivot; the defaults of empty tracks */
struct alignas(16) DevAnim {
	int toff[3], voff[3], n[3], interp[3], extrap[3];
	int pad;
	double pivot[3];
	double def[10];   /* position 0-2, rotation 3-6, scale 7-9 */
};

/* photon record: 48 B */
struct alignas(16) DevPhoton {
	float p[4];     /* pos.xyz, power.r */
	float d[4];     /* dir.xyz, power.g */
	float n[4];     /* norm.xyz, power.b */
};

}  // namespace sray

#endif
