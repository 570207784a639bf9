/*
 * prt_oracle.c - CPU oracle for portableRT's nearest-hit path (TEST INFRASTRUCTURE).
 *
 * A plain-C restatement of the reference CPU backend, used only to check the CUDA
 * path and to time a CPU baseline.  Nothing in the product library links it.
 *
 *   intersect_tri          <- include/portableRT/core.hpp:27-65   (Moller-Trumbore)
 *   ray_box                <- include/portableRT/bvh.hpp:195-222  (slab test)
 *   make/extend/harea      <- include/portableRT/bvh.hpp:13-56
 *   sah_split              <- include/portableRT/bvh.hpp:58-129   (14 bins x 3 axes)
 *   build_rec / bvh_build  <- include/portableRT/bvh.hpp:131-193
 *   nearest_tri            <- include/portableRT/bvh.hpp:224-265  (DFS, stack of 1024)
 *   orc_nearest_hits       <- include/portableRT/intersect_cpu.hpp:12-43 (static split)
 *
 * Float rules that make the results bit-identical to the reference on x86-64 and
 * aarch64: build with -O2 -ffp-contract=off and no -march (no FMA contraction), keep
 * every expression in the reference's evaluation order, and use the std::min /
 * std::max select semantics (min(a,b) = b<a ? b : a) wherever the reference does,
 * because they decide what a NaN does.
 *
 * Parity pin: tests/test_oracle_pin.py compares these functions with golden vectors
 * written by the reference itself (oracle/_ref/ref_oracle, built from its sources).
 */
#include "prt_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define ORC_NONE 0xFFFFFFFFu

/* std::min / std::max as the reference calls them (select on operator<). */
static inline float rmin(float a, float b) { return (b < a) ? b : a; }
static inline float rmax(float a, float b) { return (a < b) ? b : a; }

typedef struct {
	float lo[3], hi[3];
} box3;

/* core.hpp:27-65.  Every product and sum is a separate float operation in the
 * reference's order; the compiler flags above keep it that way. */
int orc_intersect_tri(const float *tri, const float *ray, float *t, float *u, float *v) {
	const float *o = ray, *d = ray + 3;
	float e1x = tri[3] - tri[0], e1y = tri[4] - tri[1], e1z = tri[5] - tri[2];
	float e2x = tri[6] - tri[0], e2y = tri[7] - tri[1], e2z = tri[8] - tri[2];

	float px = d[1] * e2z - d[2] * e2y;
	float py = d[2] * e2x - d[0] * e2z;
	float pz = d[0] * e2y - d[1] * e2x;

	float det = e1x * px + e1y * py + e1z * pz;
	if (det == 0.0f)
		return 0;
	float inv = 1.0f / det;

	float tx = o[0] - tri[0], ty = o[1] - tri[1], tz = o[2] - tri[2];
	float uu = (tx * px + ty * py + tz * pz) * inv;
	*u = uu;
	if (uu < 0.0f || uu > 1.0f)
		return 0;

	float qx = ty * e1z - tz * e1y;
	float qy = tz * e1x - tx * e1z;
	float qz = tx * e1y - ty * e1x;

	float vv = (d[0] * qx + d[1] * qy + d[2] * qz) * inv;
	*v = vv;
	if (vv < 0.0f || uu + vv > 1.0f)
		return 0;

	*t = (e2x * qx + e2y * qy + e2z * qz) * inv;
	return 1;
}

/* The same formula evaluated in double from the FP32 inputs; used to score t error. */
double orc_intersect_tri_f64(const float *tri, const float *ray, int *hit) {
	double o[3] = {ray[0], ray[1], ray[2]}, d[3] = {ray[3], ray[4], ray[5]};
	double v0[3] = {tri[0], tri[1], tri[2]};
	double e1[3] = {(double)tri[3] - v0[0], (double)tri[4] - v0[1], (double)tri[5] - v0[2]};
	double e2[3] = {(double)tri[6] - v0[0], (double)tri[7] - v0[1], (double)tri[8] - v0[2]};
	double p[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2],
	               d[0] * e2[1] - d[1] * e2[0]};
	double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
	*hit = 0;
	if (det == 0.0)
		return NAN;
	double inv = 1.0 / det;
	double tv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
	double u = (tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2]) * inv;
	double q[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2],
	               tv[0] * e1[1] - tv[1] * e1[0]};
	double v = (d[0] * q[0] + d[1] * q[1] + d[2] * q[2]) * inv;
	*hit = !(u < 0.0 || u > 1.0 || v < 0.0 || u + v > 1.0);
	return (e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2]) * inv;
}

/* bvh.hpp:195-222.  The reciprocal is recomputed per call exactly like the
 * reference; IEEE division makes the value identical to a cached one. */
int orc_ray_box(const float *ray, const float *bmin, const float *bmax) {
	float fx = 1.0f / ray[3], fy = 1.0f / ray[4], fz = 1.0f / ray[5];
	float t1 = (bmin[0] - ray[0]) * fx;
	float t2 = (bmax[0] - ray[0]) * fx;
	float t3 = (bmin[1] - ray[1]) * fy;
	float t4 = (bmax[1] - ray[1]) * fy;
	float t5 = (bmin[2] - ray[2]) * fz;
	float t6 = (bmax[2] - ray[2]) * fz;
	float tmin = rmax(rmax(rmin(t1, t2), rmin(t3, t4)), rmin(t5, t6));
	float tmax = rmin(rmin(rmax(t1, t2), rmax(t3, t4)), rmax(t5, t6));
	if (tmax < 0)
		return 0;
	if (tmin > tmax)
		return 0;
	return 1;
}

/* bvh.hpp:13-56 */
static box3 box_empty(void) {
	box3 b;
	for (int k = 0; k < 3; ++k) {
		b.lo[k] = FLT_MAX;
		b.hi[k] = -FLT_MAX;
	}
	return b;
}

static box3 box_of_tri(const float *t) {
	box3 b;
	for (int k = 0; k < 3; ++k) {
		b.lo[k] = rmin(t[k], rmin(t[k + 3], t[k + 6]));
		b.hi[k] = rmax(t[k], rmax(t[k + 3], t[k + 6]));
	}
	return b;
}

/* extend_aabb(a, b): a is the running box, b the one being added. */
static box3 box_grow(box3 a, box3 b) {
	box3 r;
	for (int k = 0; k < 3; ++k) {
		r.lo[k] = rmin(a.lo[k], b.lo[k]);
		r.hi[k] = rmax(a.hi[k], b.hi[k]);
	}
	return r;
}

static float box_half_area(box3 b) {
	float dx = b.hi[0] - b.lo[0];
	float dy = b.hi[1] - b.lo[1];
	float dz = b.hi[2] - b.lo[2];
	return dx * dy + dx * dz + dy * dz;
}

struct orc_bvh {
	orc_node *nodes;
	size_t count, cap;
	float *tris;
	size_t n_tris;
};

static uint32_t node_new(orc_bvh *b) {
	if (b->count == b->cap) {
		b->cap = b->cap ? 2 * b->cap : 64;
		b->nodes = (orc_node *)realloc(b->nodes, b->cap * sizeof(orc_node));
		if (!b->nodes)
			abort();
	}
	orc_node *n = &b->nodes[b->count];
	box3 e = box_empty();
	n->is_leaf = 0;
	n->tri = ORC_NONE;
	n->left = ORC_NONE;
	n->right = ORC_NONE;
	memcpy(n->lo, e.lo, sizeof e.lo);
	memcpy(n->hi, e.hi, sizeof e.hi);
	return (uint32_t)b->count++;
}

static inline const float *tri_at(const orc_bvh *b, uint32_t i) { return b->tris + 9 * (size_t)i; }

/* bvh.hpp:58-129.  Fourteen candidate planes per axis, evaluated bin-major then
 * axis-major; the first strictly cheaper candidate wins.  Both output lists keep
 * the input order.  One side empty -> split by position at n/2. */
static void sah_split(const orc_bvh *b, const uint32_t *in, size_t n, uint32_t *left,
                      size_t *nl, uint32_t *right, size_t *nr) {
	const int n_bins = 14;
	float min_cost = FLT_MAX;
	int best_axis = 0, best_bin = n_bins / 2;

	box3 nb = box_empty();
	for (size_t i = 0; i < n; ++i)
		nb = box_grow(nb, box_of_tri(tri_at(b, in[i])));

	for (int bin = 0; bin < n_bins; ++bin) {
		for (int axis = 0; axis < 3; ++axis) {
			float plane = nb.lo[axis] + (nb.hi[axis] - nb.lo[axis]) * (float)bin / (float)n_bins;
			box3 lb = box_empty(), rb = box_empty();
			int lc = 0, rc = 0;
			for (size_t i = 0; i < n; ++i) {
				const float *t = tri_at(b, in[i]);
				float c = (t[axis] + t[axis + 3] + t[axis + 6]) / 3.0f;
				if (c < plane) {
					lb = box_grow(lb, box_of_tri(t));
					++lc;
				} else {
					rb = box_grow(rb, box_of_tri(t));
					++rc;
				}
			}
			float cost = box_half_area(lb) * (float)lc + box_half_area(rb) * (float)rc;
			if (cost < min_cost) {
				min_cost = cost;
				best_axis = axis;
				best_bin = bin;
			}
		}
	}

	float plane = nb.lo[best_axis] +
	              (nb.hi[best_axis] - nb.lo[best_axis]) * (float)best_bin / (float)n_bins;
	*nl = *nr = 0;
	for (size_t i = 0; i < n; ++i) {
		const float *t = tri_at(b, in[i]);
		float c = (t[best_axis] + t[best_axis + 3] + t[best_axis + 6]) / 3.0f;
		if (c < plane)
			left[(*nl)++] = in[i];
		else
			right[(*nr)++] = in[i];
	}
	if (*nl == 0 || *nr == 0) {
		*nl = *nr = 0;
		for (size_t i = 0; i < n; ++i) {
			if (i < n / 2)
				left[(*nl)++] = in[i];
			else
				right[(*nr)++] = in[i];
		}
	}
}

/* bvh.hpp:131-156.  Preorder numbering: a node is appended before its subtrees,
 * the left subtree is built completely before the right one. */
static uint32_t build_rec(orc_bvh *b, const uint32_t *in, size_t n) {
	uint32_t me = node_new(b);
	if (n == 0) {
		b->nodes[me].is_leaf = 1;
	} else if (n == 1) {
		box3 tb = box_of_tri(tri_at(b, in[0]));
		b->nodes[me].is_leaf = 1;
		b->nodes[me].tri = in[0];
		memcpy(b->nodes[me].lo, tb.lo, sizeof tb.lo);
		memcpy(b->nodes[me].hi, tb.hi, sizeof tb.hi);
	} else {
		box3 bb = box_empty();
		for (size_t i = 0; i < n; ++i)
			bb = box_grow(bb, box_of_tri(tri_at(b, in[i])));
		memcpy(b->nodes[me].lo, bb.lo, sizeof bb.lo);
		memcpy(b->nodes[me].hi, bb.hi, sizeof bb.hi);
		uint32_t *l = (uint32_t *)malloc(n * sizeof(uint32_t));
		uint32_t *r = (uint32_t *)malloc(n * sizeof(uint32_t));
		if (!l || !r)
			abort();
		size_t nl, nr;
		sah_split(b, in, n, l, &nl, r, &nr);
		uint32_t li = build_rec(b, l, nl);
		b->nodes[me].left = li;
		free(l);
		uint32_t ri = build_rec(b, r, nr);
		b->nodes[me].right = ri;
		free(r);
	}
	return me;
}

/* bvh.hpp:158-193, including the three-node special case for one triangle. */
orc_bvh *orc_bvh_build(const float *tris, size_t n) {
	orc_bvh *b = (orc_bvh *)calloc(1, sizeof(orc_bvh));
	if (!b)
		abort();
	b->n_tris = n;
	b->tris = (float *)malloc((n ? n : 1) * 9 * sizeof(float));
	if (!b->tris)
		abort();
	if (n)
		memcpy(b->tris, tris, n * 9 * sizeof(float));
	if (n == 1) {
		box3 tb = box_of_tri(b->tris);
		uint32_t root = node_new(b);
		uint32_t leaf = node_new(b);
		uint32_t empty = node_new(b);
		b->nodes[root].left = leaf;
		b->nodes[root].right = empty;
		memcpy(b->nodes[root].lo, tb.lo, sizeof tb.lo);
		memcpy(b->nodes[root].hi, tb.hi, sizeof tb.hi);
		b->nodes[leaf].is_leaf = 1;
		b->nodes[leaf].tri = 0;
		memcpy(b->nodes[leaf].lo, tb.lo, sizeof tb.lo);
		memcpy(b->nodes[leaf].hi, tb.hi, sizeof tb.hi);
		b->nodes[empty].is_leaf = 1;
	} else {
		uint32_t *idx = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
		if (!idx)
			abort();
		for (size_t i = 0; i < n; ++i)
			idx[i] = (uint32_t)i;
		build_rec(b, idx, n);
		free(idx);
	}
	return b;
}

void orc_bvh_free(orc_bvh *b) {
	if (!b)
		return;
	free(b->nodes);
	free(b->tris);
	free(b);
}

size_t orc_bvh_node_count(const orc_bvh *b) { return b->count; }

void orc_bvh_nodes(const orc_bvh *b, orc_node *out) {
	memcpy(out, b->nodes, b->count * sizeof(orc_node));
}

/* bvh.hpp:224-265.  Depth-first with an explicit stack; every popped node (leaves
 * included) is box-tested; children are pushed left then right, so the right child
 * is visited first; a hit replaces the record only when t < t_near. */
#define ORC_STACK 1024

typedef struct {
	float t_near, u, v;
	uint32_t pid;
	orc_stats *st; /* optional bookkeeping */
} trav_state;

static void nearest_tri(const orc_bvh *b, const float *ray, trav_state *s) {
	uint32_t stack[ORC_STACK];
	uint32_t sp = 0;
	stack[sp++] = 0;
	s->t_near = INFINITY;
	s->u = 0.0f;
	s->v = 0.0f;
	s->pid = 0;
	if (b->count == 0)
		return;
	while (sp > 0) {
		const orc_node *node = &b->nodes[stack[--sp]];
		if (s->st)
			s->st->n_nodes++;
		if (!orc_ray_box(ray, node->lo, node->hi))
			continue;
		if (node->is_leaf) {
			if (node->tri == ORC_NONE)
				continue;
			float t, u, v;
			if (orc_intersect_tri(tri_at(b, node->tri), ray, &t, &u, &v)) {
				if (s->st) {
					orc_stats *st = s->st;
					st->n_accepted++;
					if (t < st->best_t) {
						st->second_t = st->best_t;
						st->best_t = t;
						st->n_best = 1;
						st->pid_min = st->pid_max = node->tri;
					} else if (t == st->best_t && t < INFINITY) {
						st->n_best++;
						if (node->tri < st->pid_min)
							st->pid_min = node->tri;
						if (node->tri > st->pid_max)
							st->pid_max = node->tri;
					} else if (t < st->second_t) {
						st->second_t = t;
					}
				}
				if (t < s->t_near) {
					s->t_near = t;
					s->u = u;
					s->v = v;
					s->pid = node->tri;
				}
			}
		} else {
			if (sp + 2 > ORC_STACK)
				abort(); /* the reference does not check; it would corrupt memory */
			stack[sp++] = node->left;
			stack[sp++] = node->right;
		}
	}
}

static void fill_hit(const float *ray, const trav_state *s, orc_hit *h) {
	memset(h, 0, sizeof *h);
	h->u = s->u;
	h->v = s->v;
	h->primitive_id = s->pid;
	h->t = s->t_near;
	h->valid = s->t_near < INFINITY;
	h->px = ray[0] + s->t_near * ray[3];
	h->py = ray[1] + s->t_near * ray[4];
	h->pz = ray[2] + s->t_near * ray[5];
}

/* ---- threading: the reference's static split (intersect_cpu.hpp:20-43) ---- */

typedef struct {
	const orc_bvh *bvh;
	const float *tris;
	size_t n_tris;
	const float *rays;
	size_t begin, end;
	orc_hit *out;
	orc_stats *stats;
	int mode; /* 0 hits, 1 stats, 2 brute force, 3 brute force without NaN admissions */
} job;

/* 1 when the slab test on this box passes only because (min_x - o_x) * (1 / d_x) is
 * NaN: a zero-x-direction ray starting on the box's lower x face.  In the reference
 * that NaN makes the whole test pass (bvh.hpp:208-209 nest it first), so such a
 * triangle is admitted at its own leaf and the answer then depends on its ancestors. */
static int nan_admitted(const float *ray, const box3 *b) {
	float fx = 1.0f / ray[3];
	float t1 = (b->lo[0] - ray[0]) * fx;
	return t1 != t1;
}

static void brute_one(const float *tris, size_t n_tris, const float *ray, orc_hit *h,
                      int skip_nan) {
	trav_state s = {INFINITY, 0.0f, 0.0f, 0, NULL};
	for (size_t i = 0; i < n_tris; ++i) {
		const float *t9 = tris + 9 * i;
		box3 tb = box_of_tri(t9);
		if (!orc_ray_box(ray, tb.lo, tb.hi))
			continue;
		if (skip_nan && nan_admitted(ray, &tb))
			continue;
		float t, u, v;
		if (!orc_intersect_tri(t9, ray, &t, &u, &v))
			continue;
		if (t < s.t_near || (t == s.t_near && s.t_near < INFINITY && (uint32_t)i < s.pid)) {
			s.t_near = t;
			s.u = u;
			s.v = v;
			s.pid = (uint32_t)i;
		}
	}
	fill_hit(ray, &s, h);
}

static void run_range(job *j) {
	for (size_t r = j->begin; r < j->end; ++r) {
		const float *ray = j->rays + 6 * r;
		if (j->mode == 0) {
			trav_state s = {0};
			nearest_tri(j->bvh, ray, &s);
			fill_hit(ray, &s, &j->out[r]);
		} else if (j->mode == 1) {
			orc_stats *st = &j->stats[r];
			memset(st, 0, sizeof *st);
			st->best_t = INFINITY;
			st->second_t = INFINITY;
			st->pid_min = st->pid_max = ORC_NONE;
			trav_state s = {0};
			s.st = st;
			nearest_tri(j->bvh, ray, &s);
			if (s.t_near < INFINITY) {
				int hit;
				st->t64 = orc_intersect_tri_f64(tri_at(j->bvh, s.pid), ray, &hit);
			} else {
				st->t64 = NAN;
			}
		} else {
			brute_one(j->tris, j->n_tris, ray, &j->out[r], j->mode == 3);
		}
	}
}

static void *thread_main(void *arg) {
	run_range((job *)arg);
	return NULL;
}

static void run_parallel(job proto, size_t n_rays, int nthreads) {
	if (nthreads <= 0) {
		long c = sysconf(_SC_NPROCESSORS_ONLN);
		nthreads = c > 0 ? (int)c : 1;
	}
	size_t per = n_rays / (size_t)nthreads;
	pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
	job *jobs = (job *)malloc(sizeof(job) * (size_t)nthreads);
	if (!th || !jobs)
		abort();
	for (int i = 0; i < nthreads; ++i) {
		jobs[i] = proto;
		jobs[i].begin = (size_t)i * per;
		jobs[i].end = (size_t)(i + 1) * per;
		if (pthread_create(&th[i], NULL, thread_main, &jobs[i]) != 0)
			abort();
	}
	for (int i = 0; i < nthreads; ++i)
		pthread_join(th[i], NULL);
	job rest = proto;
	rest.begin = (size_t)nthreads * per;
	rest.end = n_rays;
	run_range(&rest);
	free(th);
	free(jobs);
}

void orc_nearest_hits(const orc_bvh *bvh, const float *rays, size_t n, orc_hit *out,
                      int nthreads) {
	job p = {bvh, NULL, 0, rays, 0, 0, out, NULL, 0};
	run_parallel(p, n, nthreads);
}

void orc_hit_stats(const orc_bvh *bvh, const float *rays, size_t n, orc_stats *out,
                   int nthreads) {
	job p = {bvh, NULL, 0, rays, 0, 0, NULL, out, 1};
	run_parallel(p, n, nthreads);
}

void orc_brute_force(const float *tris, size_t n_tris, const float *rays, size_t n,
                     orc_hit *out, int nthreads) {
	job p = {NULL, tris, n_tris, rays, 0, 0, out, NULL, 2};
	run_parallel(p, n, nthreads);
}

void orc_brute_force_robust(const float *tris, size_t n_tris, const float *rays, size_t n,
                            orc_hit *out, int nthreads) {
	job p = {NULL, tris, n_tris, rays, 0, 0, out, NULL, 3};
	run_parallel(p, n, nthreads);
}


/* ---------------------------------------------------------------- camera and shading */

/* The sensor coordinate: sensor_size * (float(k) / extent - 0.5), evaluated as the
 * reference writes it (the float quotient widened to double by the 0.5 literal, the
 * product rounded to float on assignment): bunny/main.cpp:103-104. */
static float sensor_coord(float size, uint32_t k, uint32_t extent) {
	return (float)((double)size * ((double)((float)k / (float)extent) - 0.5));
}

void orc_camera_rays(const orc_camera *c, float *rays) {
	const uint64_t n = (uint64_t)c->width * c->height;
	for (uint64_t i = 0; i < n; ++i) {
		const uint32_t x = (uint32_t)(i % c->width);
		const uint32_t y = c->height - 1u - (uint32_t)(i / c->width);
		const float sx = sensor_coord(c->sensor_size, x, c->width);
		const float sy = sensor_coord(c->sensor_size, y, c->height);
		float sp[3];
		if (c->form == 2) { /* sponza/main.cpp:199-207 */
			const float dx = c->cos_a * sx + c->sin_a * c->sensor_dist;
			const float dz = -c->sin_a * sx + c->cos_a * c->sensor_dist;
			sp[0] = c->pos[0] + dx;
			sp[1] = c->pos[1] + sy;
			sp[2] = c->pos[2] + dz;
		} else { /* bunny/main.cpp:106-107 */
			sp[0] = sx;
			sp[1] = sy;
			sp[2] = c->sensor_z;
		}
		float d[3] = {sp[0] - c->pos[0], sp[1] - c->pos[1], sp[2] - c->pos[2]};
		/* bunny/main.cpp:113-115 (|direction|); validation/main.cpp:187-188 (|sensor|) */
		const float *l = c->form == 1 ? sp : d;
		const float len = sqrtf(l[0] * l[0] + l[1] * l[1] + l[2] * l[2]);
		float *r = rays + 6 * i;
		r[0] = c->pos[0];
		r[1] = c->pos[1];
		r[2] = c->pos[2];
		r[3] = d[0] / len;
		r[4] = d[1] / len;
		r[5] = d[2] / len;
	}
}

/* sponza/main.cpp:11-32 */
static float lambert_shade(const float *tri, const float *ray) {
	const float e1[3] = {tri[3] - tri[0], tri[4] - tri[1], tri[5] - tri[2]};
	const float e2[3] = {tri[6] - tri[0], tri[7] - tri[1], tri[8] - tri[2]};
	float N[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
	              e1[0] * e2[1] - e1[1] * e2[0]};
	const float lenN = sqrtf(N[0] * N[0] + N[1] * N[1] + N[2] * N[2]);
	if ((double)fabsf(lenN) > 0.001) {
		N[0] /= lenN;
		N[1] /= lenN;
		N[2] /= lenN;
	}
	const float dotNV = N[0] * -ray[3] + N[1] * -ray[4] + N[2] * -ray[5];
	const float m = (1.0f < dotNV) ? 1.0f : dotNV; /* std::min(dotNV, 1.0f) */
	return (0.0f < m) ? m : 0.0f;                  /* std::max(0.0f, m) */
}

/* sponza/main.cpp:228-243 */
void orc_lambert(const float *tris, const float *rays, const orc_hit *hits, size_t n,
                 uint8_t *rgba) {
	for (size_t i = 0; i < n; ++i) {
		uint8_t g = 0;
		if (hits[i].t != INFINITY) {
			const float color = 255 * lambert_shade(tris + 9 * (size_t)hits[i].primitive_id,
			                                        rays + 6 * i);
			g = (uint8_t)color;
		}
		rgba[4 * i + 0] = g;
		rgba[4 * i + 1] = g;
		rgba[4 * i + 2] = g;
		rgba[4 * i + 3] = 255;
	}
}
