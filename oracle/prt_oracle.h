/*
 * prt_oracle.h - CPU oracle for portableRT's nearest-hit path (TEST INFRASTRUCTURE).
 *
 * Plain-C restatement of the reference CPU backend (include/portableRT/core.hpp,
 * include/portableRT/bvh.hpp, include/portableRT/intersect_cpu.hpp).  It exists only
 * to check the CUDA path: tests/, __graft_entry__.smoke() and the CPU-baseline leg
 * of bench.py load it; the product library never does.
 *
 * Parity pin: tests/test_oracle_pin.py checks every output of this file against
 * golden vectors written by the reference's own CPU backend (compiled from its
 * sources by oracle/Makefile into oracle/_ref/ref_oracle).
 */
#ifndef PRT_ORACLE_H
#define PRT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Byte-for-byte the layout of portableRT::FullHitReg (HitReg with all five tags):
 * u@0 v@4 t@8 primitive_id@12 valid@16 px@20 py@24 pz@28, size 32. */
typedef struct {
	float u, v, t;
	uint32_t primitive_id;
	uint8_t valid;
	uint8_t pad_[3];
	float px, py, pz;
} orc_hit;

/* One node of the reference BVH2 (bvh.hpp:20-26), flattened. */
typedef struct {
	uint32_t is_leaf;
	uint32_t tri;   /* 0xFFFFFFFF = no triangle */
	uint32_t left;  /* 0xFFFFFFFF = none */
	uint32_t right; /* 0xFFFFFFFF = none */
	float lo[3];
	float hi[3];
} orc_node;

typedef struct orc_bvh orc_bvh;

/* Extra per-ray information the reference does not produce, used by the parity
 * rules: how many accepted triangles share the best t, the smallest t strictly
 * above it, and the FP64 Moller-Trumbore t of the winning triangle. */
typedef struct {
	float best_t;
	uint32_t n_best;      /* accepted triangles whose t == best_t */
	uint32_t pid_min;     /* smallest primitive id among them */
	uint32_t pid_max;     /* largest primitive id among them */
	float second_t;       /* smallest accepted t > best_t (inf if none) */
	uint32_t n_accepted;  /* triangles accepted (MT true and every box passed) */
	uint32_t n_nodes;     /* nodes popped */
	uint32_t pad_;
	double t64;           /* FP64 t of the reference's winning triangle (nan on miss) */
} orc_stats;

int orc_intersect_tri(const float *tri9, const float *ray6, float *t, float *u, float *v);
int orc_ray_box(const float *ray6, const float *bmin, const float *bmax);
double orc_intersect_tri_f64(const float *tri9, const float *ray6, int *hit);

orc_bvh *orc_bvh_build(const float *tris9, size_t n_tris);
void orc_bvh_free(orc_bvh *bvh);
size_t orc_bvh_node_count(const orc_bvh *bvh);
void orc_bvh_nodes(const orc_bvh *bvh, orc_node *out);

/* nthreads <= 0: one thread per online CPU (the reference uses
 * std::thread::hardware_concurrency()). */
void orc_nearest_hits(const orc_bvh *bvh, const float *rays6, size_t n_rays, orc_hit *out,
                      int nthreads);
void orc_hit_stats(const orc_bvh *bvh, const float *rays6, size_t n_rays, orc_stats *out,
                   int nthreads);

/* Pinhole sensor camera of portableRT's examples; the same fields as prt_b200_camera.
 * form 0: bunny/main.cpp:101-124 (sensor plane at z = sensor_z, direction normalised
 *         by its own length); form 1: validation/main.cpp:170-198 (the same, normalised
 *         by the length of the sensor position); form 2: sponza/main.cpp:193-218 (sensor
 *         rotated about y by an angle with cosine cos_a and sine sin_a, at sensor_dist).
 * Ray i is pixel x = i % width of row y = height - 1 - i / width. */
typedef struct {
	uint32_t width, height, form, pad_;
	float pos[3];
	float sensor_size, sensor_dist, sensor_z, cos_a, sin_a;
} orc_camera;

void orc_camera_rays(const orc_camera *cam, float *rays6);

/* Lambert shade of sponza/main.cpp:11-32 and its pixel loop (:228-243): RGBA8 per ray,
 * grey = 255 * clamp(N . -d) for a hit (t != inf), black otherwise; alpha 255. */
void orc_lambert(const float *tris9, const float *rays6, const orc_hit *hits, size_t n,
                 uint8_t *rgba);

/* Leaf-only semantics by exhaustive search: a triangle counts when the reference slab
 * test passes on its own box and Moller-Trumbore accepts it; best = smallest t, ties
 * broken by the smaller primitive id.  No tree involved. */
void orc_brute_force(const float *tris9, size_t n_tris, const float *rays6, size_t n_rays,
                     orc_hit *out, int nthreads);

/* As orc_brute_force but ignoring triangles whose own-box test passes only through the
 * NaN of a zero x direction on the box's lower x face.  The reference's answer for a ray
 * lies between the two: it admits such a triangle only when all its SAH ancestors pass,
 * so a ray whose two brute-force answers differ is "tree-dependent". */
void orc_brute_force_robust(const float *tris9, size_t n_tris, const float *rays6,
                            size_t n_rays, orc_hit *out, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
