/*
 * oracle.c — CPU oracle for the sparse-voxel-octree hot path.  TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Compile with -ffp-contract=off: the march and the ray/bounce generation must round every float
 * operation separately, exactly as the CUDA kernels do (they use explicitly rounded intrinsics).
 *
 * Reference files cited below are paths inside AdamYuan/SparseVoxelOctree.
 */
#include "oracle.h"
#include "svo_trig.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ====================================================================== threads */

static int g_threads = 0;

void oracle_set_threads(int n) { g_threads = n; }

int oracle_get_threads(void) {
	if (g_threads > 0)
		return g_threads;
	long n = sysconf(_SC_NPROCESSORS_ONLN);
	return n > 0 ? (int)n : 1;
}

typedef void (*range_fn)(void *ctx, uint64_t begin, uint64_t end);

typedef struct {
	range_fn fn;
	void *ctx;
	uint64_t n, chunk;
	uint64_t next; /* atomic */
} pfor_job;

static void *pfor_worker(void *arg) {
	pfor_job *job = (pfor_job *)arg;
	for (;;) {
		uint64_t b = __atomic_fetch_add(&job->next, job->chunk, __ATOMIC_RELAXED);
		if (b >= job->n)
			break;
		uint64_t e = b + job->chunk < job->n ? b + job->chunk : job->n;
		job->fn(job->ctx, b, e);
	}
	return NULL;
}

/* Dynamic-chunked parallel loop over [0, n). */
static void parallel_for(uint64_t n, uint64_t min_chunk, range_fn fn, void *ctx) {
	if (n == 0)
		return;
	int nt = oracle_get_threads();
	uint64_t chunk = n / ((uint64_t)nt * 16u);
	if (chunk < min_chunk)
		chunk = min_chunk;
	if (nt <= 1 || n <= chunk) {
		fn(ctx, 0, n);
		return;
	}
	pfor_job job = {fn, ctx, n, chunk, 0};
	pthread_t th[256];
	if (nt > 256)
		nt = 256;
	for (int i = 0; i < nt - 1; ++i)
		pthread_create(&th[i], NULL, pfor_worker, &job);
	pfor_worker(&job);
	for (int i = 0; i < nt - 1; ++i)
		pthread_join(th[i], NULL);
}

/* ====================================================================== voxelize
 *
 * The reference rasterises each triangle with Vulkan conservative rasterisation (src/Voxelizer.cpp:92-127)
 * or, without the extension, dilates it by half a pixel in a geometry shader
 * (shader/voxelizer_conservative.geom:46-58) and clips to the triangle's pixel AABB in the fragment
 * shader (shader/voxelizer.frag:17-25).  The fixed-function raster has no source, so the rule is
 * restated here exactly, in integers:
 *
 *  1. every coordinate is snapped to 1/256 voxel: X = round_to_nearest_even(clamp(p,0,1) * R * 256);
 *  2. the dominant axis of the (integer) normal picks the projection (shader/voxelizer.geom:27-36):
 *     x if |n.x| > |n.y| and |n.x| > |n.z|, else y if |n.y| > |n.z|, else z;
 *     projected (a, b, depth) = (y,z,x) / (z,x,y) / (x,y,z);
 *  3. pixel (i, j) is covered when, for each of the three edges, the edge function's maximum over
 *     the closed pixel square is >= 0 (the half-pixel dilation of the conservative geometry shader),
 *     and i, j lie inside [floor(min)/256, floor(max)/256] of the projected vertices (gAABB,
 *     shader/voxelizer.geom:39-40; discard test shader/voxelizer.frag:21-22);
 *  4. depth = floor(plane depth at the pixel centre), clamped to [0, R-1] and then to the triangle's
 *     [floor(min depth), floor(max depth)] (shader/voxelizer.frag:18-23, gDepthRange geom:41-42);
 *  5. voxel = un-swizzled (i, j, depth) (shader/voxelizer.frag:24); packing as shader/voxelizer.frag:40-42;
 *     colour = per-channel floor((c0 + c1 + c2) / 3) of the vertex colours;
 *  6. triangles whose integer normal is zero produce nothing.
 *
 * Canonical fragment order: triangles in input order; inside a triangle, spans along the longer AABB
 * side (rows when the AABB is at least as wide as tall, columns otherwise), spans in increasing order,
 * pixels inside a span in increasing order.  The oracle visits every pixel of the AABB and tests it
 * directly; the CUDA kernel computes span intervals arithmetically.
 */

typedef struct {
	int axis, degenerate, cols;
	int64_t a[3], b[3], c[3]; /* projected vertices, counter-clockwise in (a, b) */
	int64_t na, nb, nc;       /* plane normal in projected order, nc > 0 */
	int64_t ea[3], eb[3];     /* edge k: E_k(x,y) = ea*(x - a[k]) + eb*(y - b[k]) >= 0 inside */
	int32_t i0, i1, j0, j1, z0, z1;
	uint32_t rgb;
} vox_setup;

static int64_t snap(float p, float scale) {
	float q = p > 0.0f ? p : 0.0f; /* also maps NaN to 0 */
	q = q < 1.0f ? q : 1.0f;
	return (int64_t)nearbyintf(q * scale);
}

static int64_t floor_div(int64_t a, int64_t b) { /* b > 0 */
	int64_t q = a / b;
	return (a % b != 0 && a < 0) ? q - 1 : q;
}

static int32_t clampi(int64_t v, int64_t lo, int64_t hi) { return (int32_t)(v < lo ? lo : (v > hi ? hi : v)); }

static uint32_t tri_color(const svo_triangle *t) {
	uint32_t out = 0;
	for (int ch = 0; ch < 3; ++ch) {
		uint32_t s = 0;
		for (int k = 0; k < 3; ++k)
			s += (t->rgb[k] >> (8 * ch)) & 0xffu;
		out |= (s / 3u) << (8 * ch);
	}
	return out;
}

static void vox_triangle_setup(const svo_triangle *t, uint32_t level, vox_setup *s) {
	const int64_t R = (int64_t)1 << level;
	const float scale = (float)(R * 256);
	int64_t V[3][3];
	for (int k = 0; k < 3; ++k)
		for (int c = 0; c < 3; ++c)
			V[k][c] = snap(t->v[3 * k + c], scale);
	int64_t e1[3], e2[3], n[3];
	for (int c = 0; c < 3; ++c) {
		e1[c] = V[1][c] - V[0][c];
		e2[c] = V[2][c] - V[0][c];
	}
	n[0] = e1[1] * e2[2] - e1[2] * e2[1];
	n[1] = e1[2] * e2[0] - e1[0] * e2[2];
	n[2] = e1[0] * e2[1] - e1[1] * e2[0];
	memset(s, 0, sizeof(*s));
	s->rgb = tri_color(t);
	if (n[0] == 0 && n[1] == 0 && n[2] == 0) {
		s->degenerate = 1;
		return;
	}
	int64_t ax = llabs(n[0]), ay = llabs(n[1]), az = llabs(n[2]);
	int axis = (ax > ay && ax > az) ? 0 : (ay > az ? 1 : 2);
	s->axis = axis;
	/* (a, b, depth) component indices for each axis: yzx, zxy, xyz (shader/voxelizer.geom:15-19) */
	static const int perm[3][3] = {{1, 2, 0}, {2, 0, 1}, {0, 1, 2}};
	const int *p = perm[axis];
	int order[3] = {0, 1, 2};
	int64_t na = n[p[0]], nb = n[p[1]], nc = n[p[2]];
	if (nc < 0) { /* make the projected triangle counter-clockwise */
		order[1] = 2;
		order[2] = 1;
		na = -na;
		nb = -nb;
		nc = -nc;
	}
	for (int k = 0; k < 3; ++k) {
		s->a[k] = V[order[k]][p[0]];
		s->b[k] = V[order[k]][p[1]];
		s->c[k] = V[order[k]][p[2]];
	}
	s->na = na;
	s->nb = nb;
	s->nc = nc;
	for (int k = 0; k < 3; ++k) {
		int q = (k + 1) % 3;
		s->ea[k] = -(s->b[q] - s->b[k]);
		s->eb[k] = s->a[q] - s->a[k];
	}
	int64_t amin = s->a[0], amax = s->a[0], bmin = s->b[0], bmax = s->b[0], cmin = s->c[0], cmax = s->c[0];
	for (int k = 1; k < 3; ++k) {
		amin = s->a[k] < amin ? s->a[k] : amin;
		amax = s->a[k] > amax ? s->a[k] : amax;
		bmin = s->b[k] < bmin ? s->b[k] : bmin;
		bmax = s->b[k] > bmax ? s->b[k] : bmax;
		cmin = s->c[k] < cmin ? s->c[k] : cmin;
		cmax = s->c[k] > cmax ? s->c[k] : cmax;
	}
	s->i0 = clampi(amin >> 8, 0, R - 1);
	s->i1 = clampi(amax >> 8, 0, R - 1);
	s->j0 = clampi(bmin >> 8, 0, R - 1);
	s->j1 = clampi(bmax >> 8, 0, R - 1);
	s->z0 = clampi(cmin >> 8, 0, R - 1);
	s->z1 = clampi(cmax >> 8, 0, R - 1);
	s->cols = (s->j1 - s->j0) > (s->i1 - s->i0);
}

static int vox_covered(const vox_setup *s, int64_t i, int64_t j) {
	for (int k = 0; k < 3; ++k) {
		int64_t x = 256 * i + (s->ea[k] > 0 ? 256 : 0);
		int64_t y = 256 * j + (s->eb[k] > 0 ? 256 : 0);
		if (s->ea[k] * (x - s->a[k]) + s->eb[k] * (y - s->b[k]) < 0)
			return 0;
	}
	return 1;
}

static uint64_t vox_fragment(const vox_setup *s, int64_t i, int64_t j, uint32_t level) {
	const int64_t R = (int64_t)1 << level;
	int64_t x = 256 * i + 128, y = 256 * j + 128;
	int64_t num = s->c[0] * s->nc - s->na * (x - s->a[0]) - s->nb * (y - s->b[0]);
	int64_t z = floor_div(num, 256 * s->nc);
	z = z < 0 ? 0 : (z > R - 1 ? R - 1 : z);
	z = z < s->z0 ? s->z0 : (z > s->z1 ? s->z1 : z);
	uint32_t vx, vy, vz;
	if (s->axis == 0) { /* u.zxy */
		vx = (uint32_t)z;
		vy = (uint32_t)i;
		vz = (uint32_t)j;
	} else if (s->axis == 1) { /* u.yzx */
		vx = (uint32_t)j;
		vy = (uint32_t)z;
		vz = (uint32_t)i;
	} else {
		vx = (uint32_t)i;
		vy = (uint32_t)j;
		vz = (uint32_t)z;
	}
	uint32_t fx = vx | (vy << 12) | ((vz & 0xffu) << 24);
	uint32_t fy = ((vz >> 8) << 28) | (s->rgb & 0xffffffu);
	return (uint64_t)fx | ((uint64_t)fy << 32);
}

/* Visits covered pixels in canonical order; emit may be NULL (count only). */
static uint64_t vox_walk(const vox_setup *s, uint32_t level, uint64_t *emit) {
	if (s->degenerate)
		return 0;
	uint64_t n = 0;
	if (!s->cols) {
		for (int64_t j = s->j0; j <= s->j1; ++j)
			for (int64_t i = s->i0; i <= s->i1; ++i)
				if (vox_covered(s, i, j)) {
					if (emit)
						emit[n] = vox_fragment(s, i, j, level);
					++n;
				}
	} else {
		for (int64_t i = s->i0; i <= s->i1; ++i)
			for (int64_t j = s->j0; j <= s->j1; ++j)
				if (vox_covered(s, i, j)) {
					if (emit)
						emit[n] = vox_fragment(s, i, j, level);
					++n;
				}
	}
	return n;
}

void oracle_triangle_info(const svo_triangle *tri, uint32_t level, oracle_tri_info *info) {
	vox_setup s;
	vox_triangle_setup(tri, level, &s);
	info->axis = s.axis;
	info->i0 = s.i0;
	info->i1 = s.i1;
	info->j0 = s.j0;
	info->j1 = s.j1;
	info->z0 = s.z0;
	info->z1 = s.z1;
	info->cols = s.cols;
	info->degenerate = s.degenerate;
	info->rgb = s.rgb;
}

typedef struct {
	const svo_triangle *tris;
	uint32_t level;
	uint32_t *counts;
	const uint64_t *offsets;
	uint64_t *frags;
	uint64_t total; /* atomic */
} vox_ctx;

static void vox_count_range(void *p, uint64_t b, uint64_t e) {
	vox_ctx *c = (vox_ctx *)p;
	uint64_t sum = 0;
	for (uint64_t t = b; t < e; ++t) {
		vox_setup s;
		vox_triangle_setup(&c->tris[t], c->level, &s);
		uint64_t n = vox_walk(&s, c->level, NULL);
		if (c->counts)
			c->counts[t] = (uint32_t)n;
		sum += n;
	}
	__atomic_fetch_add(&c->total, sum, __ATOMIC_RELAXED);
}

static void vox_emit_range(void *p, uint64_t b, uint64_t e) {
	vox_ctx *c = (vox_ctx *)p;
	for (uint64_t t = b; t < e; ++t) {
		vox_setup s;
		vox_triangle_setup(&c->tris[t], c->level, &s);
		vox_walk(&s, c->level, c->frags + c->offsets[t]);
	}
}

uint64_t oracle_voxelize_count(const svo_triangle *tris, uint32_t n, uint32_t level, uint32_t *counts) {
	vox_ctx c = {tris, level, counts, NULL, NULL, 0};
	parallel_for(n, 64, vox_count_range, &c);
	return c.total;
}

void oracle_voxelize_emit(const svo_triangle *tris, uint32_t n, uint32_t level, const uint64_t *offsets,
                          uint64_t *frags) {
	vox_ctx c = {tris, level, NULL, offsets, frags, 0};
	parallel_for(n, 64, vox_emit_range, &c);
}

/* ====================================================================== build
 *
 * The level loop of src/OctreeBuilder.cpp:142-210 with build info {begin = 0, num = 8}
 * (src/OctreeBuilder.cpp:25-30):
 *   init   zero words [begin, begin+num)                         shader/octree_init_node.comp:7-11
 *   tag    every fragment walks from the root (TraverseOctree)   shader/octree_tag_node.comp:18-31
 *          and marks 0x80000000, or merges its colour at a leaf   shader/octree_tag_node.comp:33-60
 *   alloc  every marked word in [begin, begin+num) gets a block  shader/octree_alloc_node.comp:9-23
 *   modify begin += num; num = counter*8 - begin + 8             shader/octree_modify_arg.comp:9-13
 * Blocks are handed out in word order (one invocation at a time), which is the breadth-first canonical
 * order the engine's prefix-sum allocation produces.
 */

typedef struct {
	const uint64_t *frags;
	uint32_t level;
	uint32_t *pool;
	uint64_t leaf_begin;
	uint64_t *sums; /* det mode: per leaf word r, g, b, n */
} tag_ctx;

/* TraverseOctree: descend until the node pointer is 0 or the unit level is reached. */
static uint64_t traverse(const uint32_t *pool, uint32_t level, uint64_t frag, int *is_leaf) {
	uint32_t fx = (uint32_t)frag, fy = (uint32_t)(frag >> 32);
	uint32_t pos[3] = {fx & 0xfffu, (fx >> 12) & 0xfffu, (fx >> 24) | ((fy >> 28) << 8)};
	uint32_t dim = 1u << level;
	uint32_t idx = 0, cur = 0;
	do {
		dim >>= 1;
		uint32_t cx = pos[0] >= dim, cy = pos[1] >= dim, cz = pos[2] >= dim;
		idx = cur | cx | (cy << 1) | (cz << 2);
		cur = __atomic_load_n(&pool[idx], __ATOMIC_RELAXED) & 0x3fffffffu;
		pos[0] -= cx * dim;
		pos[1] -= cy * dim;
		pos[2] -= cz * dim;
	} while (cur != 0 && dim > 1);
	*is_leaf = dim == 1;
	return idx;
}

static void tag_range(void *p, uint64_t b, uint64_t e) {
	tag_ctx *c = (tag_ctx *)p;
	for (uint64_t f = b; f < e; ++f) {
		int leaf;
		uint64_t idx = traverse(c->pool, c->level, c->frags[f], &leaf);
		if (leaf) {
			uint32_t rgb = (uint32_t)(c->frags[f] >> 32) & 0xffffffu;
			uint64_t *s = c->sums + 4 * (idx - c->leaf_begin);
			__atomic_fetch_add(&s[0], rgb & 0xffu, __ATOMIC_RELAXED);
			__atomic_fetch_add(&s[1], (rgb >> 8) & 0xffu, __ATOMIC_RELAXED);
			__atomic_fetch_add(&s[2], (rgb >> 16) & 0xffu, __ATOMIC_RELAXED);
			__atomic_fetch_add(&s[3], 1, __ATOMIC_RELAXED);
		} else {
			__atomic_store_n(&c->pool[idx], 0x80000000u, __ATOMIC_RELAXED);
		}
	}
}

/* The reference's leaf merge (shader/octree_tag_node.comp:47-57) applied sequentially: the CAS loop
 * succeeds on its first retry, so each fragment folds into the running mean in list order. */
static void tag_leaf_ref(uint32_t *word, uint32_t rgb) {
	uint32_t prev = *word;
	uint32_t nr = rgb & 0xffu, ng = (rgb >> 8) & 0xffu, nb = (rgb >> 16) & 0xffu;
	if (prev == 0) {
		*word = 0xC1000000u | (rgb & 0xffffffu);
		return;
	}
	uint32_t pr = prev & 0xffu, pg = (prev >> 8) & 0xffu, pb = (prev >> 16) & 0xffu, pc = (prev >> 24) & 0x3fu;
	uint32_t cnt = pc + 1u;
	uint32_t r = (pr * pc + nr) / cnt, g = (pg * pc + ng) / cnt, bl = (pb * pc + nb) / cnt;
	uint32_t w = cnt < 0x3fu ? cnt : 0x3fu;
	*word = (w << 24) | (r & 0xffu) | ((g & 0xffu) << 8) | ((bl & 0xffu) << 16) | 0xC0000000u;
}

typedef struct {
	uint32_t *pool;
	uint64_t begin;
	const uint64_t *sums;
} fin_ctx;

static void finalize_range(void *p, uint64_t b, uint64_t e) {
	fin_ctx *c = (fin_ctx *)p;
	for (uint64_t w = b; w < e; ++w) {
		const uint64_t *s = c->sums + 4 * w;
		if (s[3] == 0)
			continue;
		uint64_t n = s[3];
		uint32_t r = (uint32_t)(s[0] / n), g = (uint32_t)(s[1] / n), bl = (uint32_t)(s[2] / n);
		uint32_t cnt = n < 63 ? (uint32_t)n : 63u;
		c->pool[c->begin + w] = 0xC0000000u | (cnt << 24) | (bl << 16) | (g << 8) | r;
	}
}

uint64_t oracle_build(const uint64_t *frags, uint64_t count, uint32_t level, int color_mode, uint32_t *pool,
                      uint64_t capacity, uint32_t *level_nodes, int *status) {
	*status = SVO_OK;
	if (level < SVO_LEVEL_MIN || level > SVO_LEVEL_MAX) {
		*status = SVO_ERR_INVALID;
		return 0;
	}
	uint64_t begin = 0, num = 8, counter = 0;
	for (uint32_t i = 1; i <= level; ++i) {
		if (begin + num > capacity) {
			*status = SVO_ERR_CAPACITY;
			return 0;
		}
		memset(pool + begin, 0, num * sizeof(uint32_t)); /* init */
		if (i < level) {
			tag_ctx c = {frags, level, pool, 0, NULL};
			parallel_for(count, 4096, tag_range, &c);
		} else if (color_mode == ORACLE_COLOR_REF) {
			for (uint64_t f = 0; f < count; ++f) {
				int leaf;
				uint64_t idx = traverse(pool, level, frags[f], &leaf);
				tag_leaf_ref(&pool[idx], (uint32_t)(frags[f] >> 32) & 0xffffffu);
			}
		} else {
			uint64_t *sums = (uint64_t *)calloc(num * 4 + 4, sizeof(uint64_t));
			tag_ctx c = {frags, level, pool, begin, sums};
			parallel_for(count, 4096, tag_range, &c);
			fin_ctx fc = {pool, begin, sums};
			parallel_for(num, 4096, finalize_range, &fc);
			free(sums);
		}
		uint64_t nodes = 0;
		for (uint64_t w = begin; w < begin + num; ++w)
			nodes += (pool[w] & 0x80000000u) != 0;
		if (level_nodes)
			level_nodes[i - 1] = (uint32_t)nodes;
		if (i < level) { /* alloc + modify_arg */
			for (uint64_t w = begin; w < begin + num; ++w)
				if (pool[w] & 0x80000000u) {
					pool[w] = (uint32_t)(((counter + 1) << 3) | 0x80000000u);
					++counter;
				}
			begin += num;
			num = counter * 8 - begin + 8;
			if ((counter + 1) * 8 > SVO_MAX_POOL_WORDS) {
				*status = SVO_ERR_CAPACITY;
				return 0;
			}
		}
	}
	return (counter + 1) * 8;
}

int oracle_canonicalize(const uint32_t *pool, uint64_t range, uint32_t *out) {
	if (range < 8 || range % 8)
		return -1;
	uint64_t nblocks = range / 8;
	uint64_t *queue = (uint64_t *)malloc(nblocks * sizeof(uint64_t));
	uint8_t *seen = (uint8_t *)calloc(nblocks, 1);
	uint64_t head = 0, tail = 0;
	queue[tail++] = 0;
	seen[0] = 1;
	int rc = 0;
	while (head < tail) {
		uint64_t blk = queue[head], nb = head;
		++head;
		for (int k = 0; k < 8; ++k) {
			uint32_t w = pool[blk * 8 + k];
			if ((w & 0xC0000000u) == 0x80000000u) {
				uint64_t child = (w & 0x3fffffffu);
				if (child % 8 || child / 8 >= nblocks || seen[child / 8]) {
					rc = -1;
					goto done;
				}
				seen[child / 8] = 1;
				out[nb * 8 + k] = (uint32_t)(0x80000000u | (tail * 8));
				queue[tail++] = child / 8;
			} else {
				out[nb * 8 + k] = w;
			}
		}
	}
	if (tail != nblocks)
		rc = -1;
done:
	free(queue);
	free(seen);
	return rc;
}

/* ====================================================================== march
 *
 * Octree_RayMarchLeaf with the iteration counter (shader/octree.glsl:179-340), the variant the
 * tracer calls (shader/octree_tracer.frag:37).  The octree occupies [1,2]^3; coordinates are mirrored
 * so the ray direction is negative on every axis; cube positions are exact dyadic floats whose bits
 * drive the pop (highest differing bit).  Every float operation is rounded separately.
 *
 * This section (march_one, march_traverse and the path-tracer vertex built on them) restates the ray
 * cast of Laine and Karras, "Efficient Sparse Voxel Octrees" (NVIDIA Research, 2010), as the reference
 * carries it in shader/octree.glsl:15-42,179-629.  That code is distributed under the following notice,
 * which applies to this restatement:
 *
 *   Copyright (c) 2009-2011, NVIDIA Corporation
 *   All rights reserved.
 *
 *   Redistribution and use in source and binary forms, with or without
 *   modification, are permitted provided that the following conditions are met:
 *       * Redistributions of source code must retain the above copyright
 *         notice, this list of conditions and the following disclaimer.
 *       * Redistributions in binary form must reproduce the above copyright
 *         notice, this list of conditions and the following disclaimer in the
 *         documentation and/or other materials provided with the distribution.
 *       * Neither the name of NVIDIA Corporation nor the
 *         names of its contributors may be used to endorse or promote products
 *         derived from this software without specific prior written permission.
 *
 *   THIS SOFTWARE IS PROVIDED BY THE COPYRIGHT HOLDERS AND CONTRIBUTORS "AS IS"
 *   AND ANY EXPRESS OR IMPLIED WARRANTIES, INCLUDING, BUT NOT LIMITED TO, THE
 *   IMPLIED WARRANTIES OF MERCHANTABILITY AND FITNESS FOR A PARTICULAR PURPOSE
 *   ARE DISCLAIMED. IN NO EVENT SHALL <COPYRIGHT HOLDER> BE LIABLE FOR ANY
 *   DIRECT, INDIRECT, INCIDENTAL, SPECIAL, EXEMPLARY, OR CONSEQUENTIAL DAMAGES
 *   (INCLUDING, BUT NOT LIMITED TO, PROCUREMENT OF SUBSTITUTE GOODS OR SERVICES;
 *   LOSS OF USE, DATA, OR PROFITS; OR BUSINESS INTERRUPTION) HOWEVER CAUSED AND
 *   ON ANY THEORY OF LIABILITY, WHETHER IN CONTRACT, STRICT LIABILITY, OR TORT
 *   (INCLUDING NEGLIGENCE OR OTHERWISE) ARISING IN ANY WAY OUT OF THE USE OF
 *   THIS SOFTWARE, EVEN IF ADVISED OF THE POSSIBILITY OF SUCH DAMAGE.
 */

#define MARCH_EPS 3.552713678800501e-15f

static inline float fmax_glsl(float x, float y) { return x < y ? y : x; }
static inline float fmin_glsl(float x, float y) { return y < x ? y : x; }
static inline uint32_t f2u(float f) {
	uint32_t u;
	memcpy(&u, &f, 4);
	return u;
}
static inline float u2f(uint32_t u) {
	float f;
	memcpy(&f, &u, 4);
	return f;
}
static inline float eps_clamp(float v) { return fabsf(v) > MARCH_EPS ? v : (v >= 0.0f ? MARCH_EPS : -MARCH_EPS); }

static void march_one(const uint32_t *pool, uint64_t range, uint32_t level, const svo_ray *ray, svo_hit *hit,
                      uint32_t *fetches) {
	const float o[3] = {ray->o[0], ray->o[1], ray->o[2]};
	float d[3] = {ray->d[0], ray->d[1], ray->d[2]};
	uint32_t nfetch = 0;
	if (d[0] == 0.0f && d[1] == 0.0f && d[2] == 0.0f) { /* ABI convention: no ray */
		memset(hit, 0, sizeof(*hit));
		hit->pos[0] = o[0];
		hit->pos[1] = o[1];
		hit->pos[2] = o[2];
		hit->voxel[0] = hit->voxel[1] = hit->voxel[2] = 0xffffu;
		if (fetches)
			*fetches = 0;
		return;
	}
	uint32_t stack[SVO_STACK_SIZE] = {0};
	uint32_t iter = 0;
	for (int k = 0; k < 3; ++k)
		d[k] = eps_clamp(d[k]);

	float coef[3], bias[3];
	for (int k = 0; k < 3; ++k) {
		coef[k] = 1.0f / -fabsf(d[k]);
		bias[k] = coef[k] * o[k];
	}
	uint32_t oct_mask = 0;
	for (int k = 0; k < 3; ++k)
		if (d[k] > 0.0f) {
			oct_mask ^= 1u << k;
			bias[k] = 3.0f * coef[k] - bias[k];
		}
	float t_min = fmax_glsl(fmax_glsl(2.0f * coef[0] - bias[0], 2.0f * coef[1] - bias[1]), 2.0f * coef[2] - bias[2]);
	float t_max = fmin_glsl(fmin_glsl(coef[0] - bias[0], coef[1] - bias[1]), coef[2] - bias[2]);
	t_min = fmax_glsl(t_min, 0.0f);
	float h = t_max;

	uint32_t parent = 0, cur = 0, idx = 0;
	float pos[3] = {1.0f, 1.0f, 1.0f};
	for (int k = 0; k < 3; ++k)
		if (1.5f * coef[k] - bias[k] > t_min) {
			idx ^= 1u << k;
			pos[k] = 1.5f;
		}
	uint32_t scale = SVO_STACK_SIZE - 1;
	float scale_exp2 = 0.5f;

	/* Malformed pools stop the ray as an aborted miss (the engine's guard; the shader has none):
	 * a pointer outside the pool, an interior word below the octree level, or the iteration bound. */
	int aborted = 0;
	const uint32_t min_scale = SVO_STACK_SIZE - level;
	while (scale < SVO_STACK_SIZE) {
		++iter;
		if (cur == 0u) {
			uint64_t w = (uint64_t)parent + (idx ^ oct_mask);
			if (w >= range) {
				aborted = 1;
				scale = 0xffffffffu;
				break;
			}
			cur = pool[w];
			++nfetch;
		}
		float tc[3];
		for (int k = 0; k < 3; ++k)
			tc[k] = pos[k] * coef[k] - bias[k];
		float tc_max = fmin_glsl(fmin_glsl(tc[0], tc[1]), tc[2]);

		if ((cur & 0x80000000u) != 0 && t_min <= t_max) {
			float half = scale_exp2 * 0.5f;
			float t_center[3];
			for (int k = 0; k < 3; ++k)
				t_center[k] = half * coef[k] + tc[k];
			if ((cur & 0x40000000u) != 0)
				break; /* leaf */
			if (scale <= min_scale) { /* interior word at the leaf level */
				aborted = 1;
				scale = 0xffffffffu;
				break;
			}
			if (tc_max < h) /* push */
				stack[scale] = parent;
			h = tc_max;
			parent = cur & 0x3fffffffu;
			idx = 0;
			--scale;
			scale_exp2 = half;
			for (int k = 0; k < 3; ++k)
				if (t_center[k] > t_min) {
					idx ^= 1u << k;
					pos[k] += scale_exp2;
				}
			cur = 0;
			continue;
		}
		/* advance.  The iteration bound is tested here, not in every iteration: pushes in a row are
		 * limited by the tree depth, so every endless sequence has advances (also with NaN arithmetic,
		 * where nothing is fetched); never reached on a valid octree. */
		if (iter >= SVO_MARCH_MAX_ITER) {
			aborted = 1;
			break;
		}
		uint32_t step_mask = 0;
		for (int k = 0; k < 3; ++k)
			if (tc[k] <= tc_max) {
				step_mask ^= 1u << k;
				pos[k] -= scale_exp2;
			}
		t_min = tc_max;
		idx ^= step_mask;
		if ((idx & step_mask) != 0) { /* pop */
			uint32_t diff = 0;
			for (int k = 0; k < 3; ++k)
				if (step_mask & (1u << k))
					diff |= f2u(pos[k]) ^ f2u(pos[k] + scale_exp2);
			scale = diff ? 31u - (uint32_t)__builtin_clz(diff) : 0xffffffffu; /* findMSB */
			if (scale >= SVO_STACK_SIZE)
				break;
			scale_exp2 = u2f((scale - SVO_STACK_SIZE + 127u) << 23u);
			parent = stack[scale];
			uint32_t sh[3];
			for (int k = 0; k < 3; ++k) {
				sh[k] = f2u(pos[k]) >> scale;
				pos[k] = u2f(sh[k] << scale);
			}
			idx = (sh[0] & 1u) | ((sh[1] & 1u) << 1) | ((sh[2] & 1u) << 2);
			h = 0.0f;
			cur = 0;
		}
	}

	/* normal from the exit corner (shader/octree.glsl:307-317) */
	float tc[3];
	for (int k = 0; k < 3; ++k)
		tc[k] = coef[k] * (pos[k] + scale_exp2) - bias[k];
	int nax = (tc[0] > tc[1] && tc[0] > tc[2]) ? 0 : (tc[1] > tc[2] ? 1 : 2);
	float norm[3] = {0.0f, 0.0f, 0.0f};
	norm[nax] = -1.0f;
	if ((oct_mask & (1u << nax)) == 0u)
		norm[nax] = 1.0f;
	/* undo mirroring (shader/octree.glsl:319-325) */
	for (int k = 0; k < 3; ++k)
		if (oct_mask & (1u << k))
			pos[k] = 3.0f - scale_exp2 - pos[k];
	/* o_pos (shader/octree.glsl:327-334) */
	for (int k = 0; k < 3; ++k) {
		float v = o[k] + t_min * d[k];
		float lo = pos[k], hi = pos[k] + scale_exp2;
		v = fmin_glsl(fmax_glsl(v, lo), hi);
		if (k == nax)
			v = norm[k] > 0.0f ? pos[k] + scale_exp2 + MARCH_EPS * 2.0f : pos[k] - MARCH_EPS;
		hit->pos[k] = v;
	}
	int is_hit = !aborted && scale < SVO_STACK_SIZE && t_min <= t_max;
	hit->t = t_min;
	hit->iter = iter;
	hit->flags = (uint16_t)((is_hit ? SVO_HIT_FLAG_HIT : 0u) | ((uint32_t)nax << 1) |
	                        (norm[nax] < 0.0f ? SVO_HIT_NORMAL_NEG : 0u) | (aborted ? SVO_HIT_FLAG_ABORTED : 0u));
	if (is_hit) {
		hit->node = cur;
		float res = (float)(1u << level);
		for (int k = 0; k < 3; ++k)
			hit->voxel[k] = (uint16_t)(uint32_t)((pos[k] - 1.0f) * res);
	} else {
		hit->node = 0;
		hit->voxel[0] = hit->voxel[1] = hit->voxel[2] = 0xffffu;
	}
	if (fetches)
		*fetches = nfetch;
}

typedef struct {
	const uint32_t *pool;
	uint64_t range;
	uint32_t level;
	const svo_ray *rays;
	svo_hit *hits;
	uint32_t *fetches;
} march_ctx;

static void march_range(void *p, uint64_t b, uint64_t e) {
	march_ctx *c = (march_ctx *)p;
	for (uint64_t r = b; r < e; ++r)
		march_one(c->pool, c->range, c->level, &c->rays[r], &c->hits[r], c->fetches ? &c->fetches[r] : NULL);
}

void oracle_raycast(const uint32_t *pool, uint64_t range, uint32_t level, const svo_ray *rays, uint64_t n,
                    svo_hit *hits, uint32_t *fetches) {
	march_ctx c = {pool, range, level, rays, hits, fetches};
	parallel_for(n, 256, march_range, &c);
}

/* ====================================================================== rays */

/* Camera_GenRay(coord) = normalize(look - side*(2c.x-1) - up*(2c.y-1)) (shader/camera.glsl:11-14);
 * normalize is v / sqrt(x*x + y*y + z*z), each operation rounded. */
void oracle_camera_rays(const svo_camera *cam, uint32_t width, uint32_t height, svo_ray *rays) {
	for (uint32_t y = 0; y < height; ++y)
		for (uint32_t x = 0; x < width; ++x) {
			float cx = (float)x / (float)width, cy = (float)y / (float)height;
			cx = cx * 2.0f - 1.0f;
			cy = cy * 2.0f - 1.0f;
			float v[3];
			for (int k = 0; k < 3; ++k)
				v[k] = (cam->look[k] - cam->side[k] * cx) - cam->up[k] * cy;
			float len = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
			svo_ray *r = &rays[(uint64_t)y * width + x];
			for (int k = 0; k < 3; ++k) {
				r->o[k] = cam->pos[k];
				r->d[k] = v[k] / len;
			}
		}
}

/* ====================================================================== occlusion and beam */

/* The traversal of Octree_RayMarchOcclude (shader/octree.glsl:504-629; coarse = 0) and of
 * Octree_RayMarchCoarse (shader/octree.glsl:47-177; coarse = 1).  They differ from the leaf march only in
 * the direction clamp (occlude keeps |d| >= EPS, coarse keeps |d| > EPS, :505-507 and :48-50) and, for
 * coarse, a stop at the first non-empty node at least as large as the cone footprint
 * orig_sz + t * dir_sz (:96-97).  Returns 1 on a hit with *t_out = t_min and *size_out = the node size.
 * The engine's guards end a ray on a malformed pool as a miss. */
static int march_traverse(const uint32_t *pool, uint64_t range, uint32_t level, const float *o, const float *din,
                          int coarse, float orig_sz, float dir_sz, float *t_out, float *size_out) {
	float d[3];
	for (int k = 0; k < 3; ++k)
		d[k] = (coarse ? fabsf(din[k]) > MARCH_EPS : fabsf(din[k]) >= MARCH_EPS) ? din[k]
		                                                                     : (din[k] >= 0.0f ? MARCH_EPS : -MARCH_EPS);
	uint32_t stack[SVO_STACK_SIZE] = {0};
	float coef[3], bias[3];
	for (int k = 0; k < 3; ++k) {
		coef[k] = 1.0f / -fabsf(d[k]);
		bias[k] = coef[k] * o[k];
	}
	uint32_t oct_mask = 0;
	for (int k = 0; k < 3; ++k)
		if (d[k] > 0.0f) {
			oct_mask ^= 1u << k;
			bias[k] = 3.0f * coef[k] - bias[k];
		}
	float t_min = fmax_glsl(fmax_glsl(2.0f * coef[0] - bias[0], 2.0f * coef[1] - bias[1]), 2.0f * coef[2] - bias[2]);
	float t_max = fmin_glsl(fmin_glsl(coef[0] - bias[0], coef[1] - bias[1]), coef[2] - bias[2]);
	t_min = fmax_glsl(t_min, 0.0f);
	float h = t_max;
	uint32_t parent = 0, cur = 0, idx = 0;
	float pos[3] = {1.0f, 1.0f, 1.0f};
	for (int k = 0; k < 3; ++k)
		if (1.5f * coef[k] - bias[k] > t_min) {
			idx ^= 1u << k;
			pos[k] = 1.5f;
		}
	uint32_t scale = SVO_STACK_SIZE - 1, iter = 0;
	float scale_exp2 = 0.5f;
	int aborted = 0;
	const uint32_t min_scale = SVO_STACK_SIZE - level;
	while (scale < SVO_STACK_SIZE) {
		if (++iter > SVO_MARCH_MAX_ITER) {
			aborted = 1;
			break;
		}
		if (cur == 0u) {
			uint64_t w = (uint64_t)parent + (idx ^ oct_mask);
			if (w >= range) {
				aborted = 1;
				break;
			}
			cur = pool[w];
		}
		float tc[3];
		for (int k = 0; k < 3; ++k)
			tc[k] = pos[k] * coef[k] - bias[k];
		float tc_max = fmin_glsl(fmin_glsl(tc[0], tc[1]), tc[2]);
		if ((cur & 0x80000000u) != 0 && t_min <= t_max) {
			if (coarse && orig_sz + tc_max * dir_sz >= scale_exp2)
				break;
			float half = scale_exp2 * 0.5f;
			float t_center[3];
			for (int k = 0; k < 3; ++k)
				t_center[k] = half * coef[k] + tc[k];
			if ((cur & 0x40000000u) != 0)
				break;
			if (scale <= min_scale) {
				aborted = 1;
				break;
			}
			if (tc_max < h)
				stack[scale] = parent;
			h = tc_max;
			parent = cur & 0x3fffffffu;
			idx = 0;
			--scale;
			scale_exp2 = half;
			for (int k = 0; k < 3; ++k)
				if (t_center[k] > t_min) {
					idx ^= 1u << k;
					pos[k] += scale_exp2;
				}
			cur = 0;
			continue;
		}
		uint32_t step_mask = 0;
		for (int k = 0; k < 3; ++k)
			if (tc[k] <= tc_max) {
				step_mask ^= 1u << k;
				pos[k] -= scale_exp2;
			}
		t_min = tc_max;
		idx ^= step_mask;
		if ((idx & step_mask) != 0) {
			uint32_t diff = 0;
			for (int k = 0; k < 3; ++k)
				if (step_mask & (1u << k))
					diff |= f2u(pos[k]) ^ f2u(pos[k] + scale_exp2);
			scale = diff ? 31u - (uint32_t)__builtin_clz(diff) : 0xffffffffu;
			if (scale >= SVO_STACK_SIZE)
				break;
			scale_exp2 = u2f((scale - SVO_STACK_SIZE + 127u) << 23u);
			parent = stack[scale];
			uint32_t sh[3];
			for (int k = 0; k < 3; ++k) {
				sh[k] = f2u(pos[k]) >> scale;
				pos[k] = u2f(sh[k] << scale);
			}
			idx = (sh[0] & 1u) | ((sh[1] & 1u) << 1) | ((sh[2] & 1u) << 2);
			h = 0.0f;
			cur = 0;
		}
	}
	*t_out = t_min;
	*size_out = scale_exp2;
	return !aborted && scale < SVO_STACK_SIZE && t_min <= t_max;
}

typedef struct {
	const uint32_t *pool;
	uint64_t range;
	uint32_t level;
	const svo_ray *rays;
	uint32_t *out;
} occlude_ctx;

static void occlude_range(void *p, uint64_t b, uint64_t e) {
	occlude_ctx *c = (occlude_ctx *)p;
	for (uint64_t r = b; r < e; ++r) {
		const svo_ray *ray = &c->rays[r];
		float t, sz;
		const int none = ray->d[0] == 0.0f && ray->d[1] == 0.0f && ray->d[2] == 0.0f; /* ABI: no ray */
		c->out[r] =
		    none ? 0u : (uint32_t)march_traverse(c->pool, c->range, c->level, ray->o, ray->d, 0, 0.0f, 0.0f, &t, &sz);
	}
}

void oracle_occlude(const uint32_t *pool, uint64_t range, uint32_t level, const svo_ray *rays, uint64_t n,
                    uint32_t *occluded) {
	occlude_ctx c = {pool, range, level, rays, occluded};
	parallel_for(n, 256, occlude_range, &c);
}

/* Camera_GenRay of a normalised image coordinate (shader/camera.glsl:11-14). */
static void gen_ray(const svo_camera *cam, float cx, float cy, float d[3]) {
	cx = cx * 2.0f - 1.0f;
	cy = cy * 2.0f - 1.0f;
	float v[3];
	for (int k = 0; k < 3; ++k)
		v[k] = (cam->look[k] - cam->side[k] * cx) - cam->up[k] * cy;
	float len = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
	for (int k = 0; k < 3; ++k)
		d[k] = v[k] / len;
}

/* RayTangent of shader/octree_tracer_beam.frag:17-20: tan of the angle between two unit vectors. */
static float ray_tangent(const float x[3], const float y[3]) {
	float c = (x[0] * y[0] + x[1] * y[1]) + x[2] * y[2];
	return sqrtf(1.0f - c * c) / fabsf(c);
}

typedef struct {
	const uint32_t *pool;
	uint64_t range;
	uint32_t level;
	const svo_camera *cam;
	uint32_t width, height, beam_size, bw;
	float *beam;
} beam_ctx;

static void beam_range(void *p, uint64_t b, uint64_t e) {
	beam_ctx *c = (beam_ctx *)p;
	const float W = (float)c->width, H = (float)c->height, bs = (float)c->beam_size;
	const float orig_sz = ldexpf(1.0f, 1 - (int)c->level); /* exp2f(1 - level), src/OctreeTracer.cpp:205 */
	static const float bias[4][2] = {{0.5f, 0.5f}, {-0.5f, 0.5f}, {0.5f, -0.5f}, {-0.5f, -0.5f}};
	for (uint64_t i = b; i < e; ++i) {
		const uint32_t bx = (uint32_t)(i % c->bw), by = (uint32_t)(i / c->bw);
		float d[3], tg[4];
		gen_ray(c->cam, (float)bx / W * bs, (float)by / H * bs, d);
		for (int k = 0; k < 4; ++k) {
			float dk[3];
			gen_ray(c->cam, ((float)bx + bias[k][0]) / W * bs, ((float)by + bias[k][1]) / H * bs, dk);
			tg[k] = ray_tangent(d, dk);
		}
		const float dir_sz = 2.0f * fmax_glsl(fmax_glsl(tg[0], tg[1]), fmax_glsl(tg[2], tg[3]));
		float t, sz;
		const float o[3] = {c->cam->pos[0], c->cam->pos[1], c->cam->pos[2]};
		c->beam[i] = march_traverse(c->pool, c->range, c->level, o, d, 1, orig_sz, dir_sz, &t, &sz)
		                 ? fmax_glsl(0.0f, t - sz)
		                 : 1e10f;
	}
}

/* The beam pre-pass (shader/octree_tracer_beam.frag:22-30, src/OctreeTracer.cpp:183-211): one start
 * distance per corner of each beam_size x beam_size pixel tile, (W + bs - 1)/bs + 1 by (H + bs - 1)/bs + 1
 * texels (src/OctreeTracer.cpp:6), row-major. */
void oracle_beam(const uint32_t *pool, uint64_t range, uint32_t level, const svo_camera *cam, uint32_t width,
                 uint32_t height, uint32_t beam_size, float *beam) {
	const uint32_t bw = (width + beam_size - 1) / beam_size + 1, bh = (height + beam_size - 1) / beam_size + 1;
	beam_ctx c = {pool, range, level, cam, width, height, beam_size, bw, beam};
	parallel_for((uint64_t)bw * bh, 64, beam_range, &c);
}

/* Primary rays advanced by the beam (shader/octree_tracer.frag:27-33): o += d * min of the 4 texels
 * around the pixel's tile. */
void oracle_camera_rays_beam(const svo_camera *cam, uint32_t width, uint32_t height, const float *beam,
                             uint32_t beam_size, svo_ray *rays) {
	const uint32_t bw = (width + beam_size - 1) / beam_size + 1;
	oracle_camera_rays(cam, width, height, rays);
	for (uint32_t y = 0; y < height; ++y)
		for (uint32_t x = 0; x < width; ++x) {
			const uint32_t bx = x / beam_size, by = y / beam_size;
			const float *t0 = beam + (uint64_t)by * bw + bx, *t1 = t0 + bw;
			const float m = fmin_glsl(fmin_glsl(t0[0], t0[1]), fmin_glsl(t1[0], t1[1]));
			svo_ray *r = &rays[(uint64_t)y * width + x];
			for (int k = 0; k < 3; ++k)
				r->o[k] = r->o[k] + r->d[k] * m;
		}
}

/* Counter hash for the bounce sample: splitmix64 finaliser of seed + golden * (index + 1). */
static uint64_t mix64(uint64_t z) {
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

/* sin / cos / atan / acos: the engine's restatements (svo_trig.h). */

/* Diffuse_Sample (shader/diffuse.glsl:7-14) with AlignDirection (shader/util.glsl:5-9) for an
 * axis-aligned normal; sin/cos from sincos_2pi. */
void oracle_diffuse_sample(const float nrm_in[3], float u1, float u2, float out[3]) {
	float rr = sqrtf(u1), sn, cs;
	sincos_2pi(u2, &sn, &cs);
	float dl[3] = {rr * cs, rr * sn, sqrtf(1.0f - u1)};
	float nrm[3] = {nrm_in[0], nrm_in[1], nrm_in[2]};
	float ref[3] = {0.0f, 0.0f, 0.0f};
	if (fabsf(nrm[0]) > 0.01f)
		ref[1] = 1.0f;
	else
		ref[0] = 1.0f;
	float u[3] = {ref[1] * nrm[2] - ref[2] * nrm[1], ref[2] * nrm[0] - ref[0] * nrm[2],
	              ref[0] * nrm[1] - ref[1] * nrm[0]};
	float ul = sqrtf((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]);
	for (int k = 0; k < 3; ++k)
		u[k] = u[k] / ul;
	float v[3] = {nrm[1] * u[2] - nrm[2] * u[1], nrm[2] * u[0] - nrm[0] * u[2], nrm[0] * u[1] - nrm[1] * u[0]};
	for (int k = 0; k < 3; ++k)
		out[k] = (dl[0] * u[k] + dl[1] * v[k]) + dl[2] * nrm[k];
}

void oracle_bounce_rays(const svo_hit *hits, uint64_t n, uint64_t seed, svo_ray *rays) {
	for (uint64_t i = 0; i < n; ++i) {
		const svo_hit *h = &hits[i];
		svo_ray *r = &rays[i];
		for (int k = 0; k < 3; ++k) {
			r->o[k] = h->pos[k];
			r->d[k] = 0.0f;
		}
		if (!(h->flags & SVO_HIT_FLAG_HIT))
			continue;
		uint64_t z = mix64(seed + 0x9E3779B97F4A7C15ull * (i + 1));
		float u1 = (float)(uint32_t)(z >> 40) * (1.0f / 16777216.0f);
		float u2 = (float)(uint32_t)((z >> 16) & 0xffffffu) * (1.0f / 16777216.0f);
		int ax = SVO_HIT_NORMAL_AXIS(h->flags);
		float nrm[3] = {0.0f, 0.0f, 0.0f};
		nrm[ax] = (h->flags & SVO_HIT_NORMAL_NEG) ? -1.0f : 1.0f;
		oracle_diffuse_sample(nrm, u1, u2, r->d);
	}
}

/* ====================================================================== path tracer */

#define PT_PI 3.14159265358979323846f

typedef struct pt_env {
	const float *texels; /* 4 floats per texel: radiance rgb, pdf weight */
	const uint32_t *alias;
	uint32_t w, h;
} pt_env;

/* texture() with a linear filter and repeat addressing: the 4 texels around (u W - 1/2, v H - 1/2). */
static void env_texture(const pt_env *e, float u, float v, float out[4]) {
	float x = u * (float)e->w - 0.5f, y = v * (float)e->h - 0.5f;
	float fx = floorf(x), fy = floorf(y);
	float a = x - fx, b = y - fy;
	int64_t W = e->w, H = e->h;
	int64_t i0 = (((int64_t)fx % W) + W) % W, j0 = (((int64_t)fy % H) + H) % H;
	int64_t i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
	const float *t00 = e->texels + 4 * (j0 * W + i0), *t10 = e->texels + 4 * (j0 * W + i1);
	const float *t01 = e->texels + 4 * (j1 * W + i0), *t11 = e->texels + 4 * (j1 * W + i1);
	float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
	for (int k = 0; k < 4; ++k)
		out[k] = ((w00 * t00[k] + w10 * t10[k]) + w01 * t01[k]) + w11 * t11[k];
}

static const float kTwoPiPi = 2.0f * PT_PI * PT_PI;

/* EnvMap_Dir2Coord + texture (shader/environment_map.glsl:16-25). */
static void env_lookup(const pt_env *e, const float d[3], float rot, float out[4]) {
	float u = (svo_atan2(d[0], d[2]) + rot) / PT_PI * 0.5f;
	float v = svo_acos(d[1]) / PT_PI;
	env_texture(e, u, v, out);
}

/* EnvMap_Sample (shader/environment_map.glsl:31-48) with the engine's sin/cos rule. */
static void env_sample(const pt_env *e, float s0, float s1, float rot, float d[3], float light[3], float *pdf) {
	uint32_t sz = e->w * e->h;
	uint32_t idx = (uint32_t)(s0 * (float)sz);
	if (idx > sz - 1u)
		idx = sz - 1u;
	uint32_t prob = (uint32_t)(s1 * 4294967296.0f);
	uint32_t pix = idx;
	if (prob > e->alias[2 * idx])
		pix = e->alias[2 * idx + 1];
	uint32_t py = pix / e->w, px = pix - py * e->w;
	float u = ((float)px + 0.5f) / (float)e->w, v = ((float)py + 0.5f) / (float)e->h;
	float phi = 2.0f * PT_PI * u - rot, theta = PT_PI * v;
	float st, ct, sp, cp;
	svo_sincos(theta, &st, &ct);
	svo_sincos(phi, &sp, &cp);
	const float *tx = e->texels + 4 * (size_t)pix;
	light[0] = tx[0], light[1] = tx[1], light[2] = tx[2];
	*pdf = tx[3] / (kTwoPiPi * st);
	d[0] = st * sp, d[1] = ct, d[2] = st * cp;
}

static float mis_power(float a, float b) {
	float t = a * a;
	return t / (b * b + t);
}

static float sobol_f(uint32_t v) { return (float)v * 2.3283064365386963e-10f; }

static float unorm8_load(uint32_t w, int k) { return (float)((w >> (8 * k)) & 0xffu) / 255.0f; }
static uint32_t unorm8_store(float v) { return (uint32_t)floorf(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f + 0.5f); }
static float snorm8_load(uint32_t w, int k) { return fmaxf((float)(int32_t)(int8_t)((w >> (8 * k)) & 0xffu) / 127.0f, -1.0f); }
static uint32_t snorm8_store(float v) {
	return (uint32_t)(int32_t)floorf(fminf(fmaxf(v, -1.0f), 1.0f) * 127.0f + 0.5f) & 0xffu;
}

typedef struct pt_ctx {
	const uint32_t *pool;
	uint64_t range;
	uint32_t level;
	const svo_camera *cam;
	uint32_t width, height, bounce, light_type;
	const float *const_color;
	float rot, mult;
	pt_env env;
	const uint32_t *sobol;
	const uint8_t *noise;
	float *color;
	uint32_t *albedo, *normal;
} pt_ctx;

/* AlignDirection (shader/util.glsl:5-9). */
static void align_direction(const float dl[3], const float nrm[3], float out[3]) {
	float ref[3] = {0.0f, 0.0f, 0.0f};
	if (fabsf(nrm[0]) > 0.01f)
		ref[1] = 1.0f;
	else
		ref[0] = 1.0f;
	float u[3] = {ref[1] * nrm[2] - ref[2] * nrm[1], ref[2] * nrm[0] - ref[0] * nrm[2],
	              ref[0] * nrm[1] - ref[1] * nrm[0]};
	float ul = sqrtf((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]);
	for (int k = 0; k < 3; ++k)
		u[k] = u[k] / ul;
	float v[3] = {nrm[1] * u[2] - nrm[2] * u[1], nrm[2] * u[0] - nrm[0] * u[2], nrm[0] * u[1] - nrm[1] * u[0]};
	for (int k = 0; k < 3; ++k)
		out[k] = (dl[0] * u[k] + dl[1] * v[k]) + dl[2] * nrm[k];
}

/* Diffuse_Sample (shader/diffuse.glsl:7-14) as the path tracer calls it: phi = 2 * PI * samp.y, cos and
 * sin of phi, pdf = d.z / PI. */
static void pt_diffuse_sample(const float nrm[3], float s0, float s1, float out[3], float *pdf) {
	float r = sqrtf(s0), phi = 2.0f * PT_PI * s1;
	float sn, cs;
	svo_sincos(phi, &sn, &cs);
	float dl[3] = {r * cs, r * sn, sqrtf(1.0f - s0)};
	*pdf = dl[2] / PT_PI;
	align_direction(dl, nrm, out);
}

/* The 5-argument Octree_RayMarchLeaf (shader/octree.glsl:342-502) as the path tracer reads it: the
 * |d| >= EPS clamp (applied first; the leaf march's > EPS clamp then keeps d), hit, o_pos,
 * o_color = rgb * (1/255), o_normal. */
static int pt_leaf(const pt_ctx *c, const float o[3], const float din[3], float pos[3], float alb[3], float nrm[3]) {
	float d[3];
	for (int k = 0; k < 3; ++k)
		d[k] = fabsf(din[k]) >= MARCH_EPS ? din[k] : (din[k] >= 0.0f ? MARCH_EPS : -MARCH_EPS);
	svo_ray r = {{o[0], o[1], o[2]}, {d[0], d[1], d[2]}};
	svo_hit h;
	march_one(c->pool, c->range, c->level, &r, &h, NULL);
	for (int k = 0; k < 3; ++k) {
		pos[k] = h.pos[k];
		alb[k] = (float)((h.node >> (8 * k)) & 0xffu) * 0.00392156862745098f;
		nrm[k] = 0.0f;
	}
	nrm[SVO_HIT_NORMAL_AXIS(h.flags)] = (h.flags & SVO_HIT_NORMAL_NEG) ? -1.0f : 1.0f;
	return (h.flags & SVO_HIT_FLAG_HIT) != 0;
}

/* One sample of one pixel: ConstColorPathTrace / EnvMapPathTrace and main()
 * (shader/path_tracer.comp:32-135). */
static void pt_pixel(const pt_ctx *c, uint32_t x, uint32_t y) {
	uint32_t spp = c->sobol[2 * (c->bounce + 1)];
	uint32_t ni = (((y & 255u) << 8) | (x & 255u)) * 2u;
	float nz[2] = {(float)c->noise[ni] / 255.0f, (float)c->noise[ni + 1] / 255.0f};
	float o[3] = {c->cam->pos[0], c->cam->pos[1], c->cam->pos[2]}, d[3];
	gen_ray(c->cam, ((float)x + sobol_f(c->sobol[0])) / (float)c->width,
	        ((float)y + sobol_f(c->sobol[1])) / (float)c->height, d);
	float acc[3] = {1.0f, 1.0f, 1.0f}, rad[3] = {0.0f, 0.0f, 0.0f};
	float dalb[3] = {0.0f, 0.0f, 0.0f}, dnrm[3] = {0.0f, 0.0f, 0.0f};
	float pos[3], alb[3], nrm[3];
	if (pt_leaf(c, o, d, pos, alb, nrm)) {
		for (int k = 0; k < 3; ++k) {
			acc[k] *= alb[k];
			dalb[k] = alb[k];
			dnrm[k] = nrm[k];
		}
		for (uint32_t cur = 1; cur < c->bounce; ++cur) {
			float samp[2] = {sobol_f(c->sobol[2 * cur]) + nz[0], sobol_f(c->sobol[2 * cur + 1]) + nz[1]};
			samp[0] = samp[0] - floorf(samp[0]);
			samp[1] = samp[1] - floorf(samp[1]);
			for (int k = 0; k < 3; ++k)
				o[k] = pos[k];
			if (c->light_type == 1) {
				float ld[3], light[3], light_pdf;
				env_sample(&c->env, samp[0], samp[1], c->rot, ld, light, &light_pdf);
				float ndd = (nrm[0] * ld[0] + nrm[1] * ld[1]) + nrm[2] * ld[2];
				if (ndd > 0.0f && !isnan(light_pdf) && light_pdf > 0.0f) {
					float t, sz;
					if (!march_traverse(c->pool, c->range, c->level, o, ld, 0, 0.0f, 0.0f, &t, &sz)) {
						float bsdf_pdf = ndd / PT_PI;
						float w = mis_power(light_pdf, bsdf_pdf);
						for (int k = 0; k < 3; ++k)
							rad[k] += acc[k] * light[k] * c->mult * w * ndd * (1.0f / PT_PI) / light_pdf;
					}
				}
			}
			float bsdf_pdf;
			pt_diffuse_sample(nrm, samp[0], samp[1], d, &bsdf_pdf);
			if (pt_leaf(c, o, d, pos, alb, nrm)) {
				for (int k = 0; k < 3; ++k)
					acc[k] *= alb[k];
			} else {
				if (c->light_type == 1) {
					float env[4];
					env_lookup(&c->env, d, c->rot, env);
					float light_pdf = env[3] / (kTwoPiPi * sqrtf(1.0f - d[1] * d[1]));
					if (!isnan(light_pdf) && light_pdf > 0.0f) {
						float w = mis_power(bsdf_pdf, light_pdf);
						for (int k = 0; k < 3; ++k)
							rad[k] += acc[k] * env[k] * c->mult * w;
					}
				} else {
					for (int k = 0; k < 3; ++k)
						rad[k] = acc[k] * c->const_color[k];
				}
				break;
			}
		}
	} else if (c->light_type == 1) {
		float env[4];
		env_lookup(&c->env, d, c->rot, env);
		rad[0] = env[0], rad[1] = env[1], rad[2] = env[2];
	} else {
		for (int k = 0; k < 3; ++k)
			rad[k] = c->const_color[k];
	}
	size_t p = (size_t)y * c->width + x;
	float fs = (float)spp, fn = (float)(spp + 1u);
	float *col = c->color + 4 * p;
	for (int k = 0; k < 3; ++k)
		col[k] = (col[k] * fs + rad[k]) / fn;
	col[3] = 1.0f;
	uint32_t wa = c->albedo[p], wn = c->normal[p];
	uint32_t oa = 255u << 24, on = 127u << 24;
	for (int k = 0; k < 3; ++k) {
		oa |= unorm8_store((unorm8_load(wa, k) * fs + dalb[k]) / fn) << (8 * k);
		on |= snorm8_store((snorm8_load(wn, k) * fs + dnrm[k]) / fn) << (8 * k);
	}
	c->albedo[p] = oa;
	c->normal[p] = on;
}

static void pt_range(void *p, uint64_t b, uint64_t e) {
	const pt_ctx *c = (const pt_ctx *)p;
	for (uint64_t i = b; i < e; ++i)
		pt_pixel(c, (uint32_t)(i % c->width), (uint32_t)(i / c->width));
}

void oracle_pt_render(const uint32_t *pool, uint64_t range, uint32_t level, const svo_camera *cam, uint32_t width,
                      uint32_t height, uint32_t bounce, uint32_t light_type, const float *const_color, float rot,
                      float mult, const float *env_texels, const uint32_t *env_alias, uint32_t env_w, uint32_t env_h,
                      const uint32_t *sobol, const uint8_t *noise, float *color, uint32_t *albedo, uint32_t *normal) {
	pt_ctx c = {pool, range, level, cam, width, height, bounce, light_type, const_color, rot, mult,
	            {env_texels, env_alias, env_w, env_h}, sobol, noise, color, albedo, normal};
	parallel_for((uint64_t)width * height, 64, pt_range, &c);
}

/* Sobol::CmdNext (shader/sobol.comp:70-86). */
void oracle_sobol_next(uint32_t *sobol, const uint32_t *matrices, uint32_t dim) {
	uint32_t i = sobol[dim];
	if (i == 0xffffffffu) {
		sobol[dim] = 0;
		return;
	}
	uint32_t c = (uint32_t)__builtin_ctz(~i);
	sobol[dim] = i + 1u;
	for (uint32_t j = 0; j < dim; ++j)
		sobol[j] ^= matrices[j * 32 + c];
}

/* EnvironmentMap::weigh_hdr_image + generate_alias_table (src/EnvironmentMap.cpp:83-160) on a copy:
 * rgba[4i+3] becomes the weight (float), alias gets (prob, alias) per texel.  Returns 0 when the image
 * has no positive luminance. */
int oracle_envmap_build(float *rgba, uint32_t w, uint32_t h, uint32_t *alias) {
	size_t n = (size_t)w * h;
	double *wt = (double *)malloc(n * sizeof(double));
	uint32_t *sm = (uint32_t *)malloc(n * sizeof(uint32_t)), *lg = (uint32_t *)malloc(n * sizeof(uint32_t));
	double sum = 0.0;
	for (uint32_t j = 0; j < h; ++j) {
		double st = sin(3.14159265358979323846 * ((double)j + 0.5) / (double)h);
		for (uint32_t i = 0; i < w; ++i) {
			const float *c = rgba + 4 * ((size_t)j * w + i);
			float lum = 0.2126f * c[0] + 0.7152f * c[1] + 0.0722f * c[2];
			wt[(size_t)j * w + i] = (double)lum * st;
			sum += wt[(size_t)j * w + i];
		}
	}
	int ok = sum > 0.0 && isfinite(sum);
	if (ok) {
		double mul = (double)n / sum;
		for (size_t i = 0; i < n; ++i) {
			wt[i] *= mul;
			rgba[4 * i + 3] = (float)wt[i];
		}
		size_t ns = 0, nl = 0;
		for (size_t i = 0; i < n; ++i) {
			if (wt[i] < 1.0)
				sm[ns++] = (uint32_t)i;
			else
				lg[nl++] = (uint32_t)i;
		}
		while (ns && nl) {
			uint32_t s = sm[--ns], l = lg[nl - 1];
			double p = wt[s] * 4294967296.0;
			alias[2 * s] = (uint32_t)(p < 0.0 ? 0.0 : (p > 4294967295.0 ? 4294967295.0 : p));
			alias[2 * s + 1] = l;
			wt[l] -= 1.0 - wt[s];
			if (wt[l] < 1.0) {
				--nl;
				sm[ns++] = l;
			}
		}
		while (nl) {
			uint32_t l = lg[--nl];
			alias[2 * l] = alias[2 * l + 1] = 0xffffffffu;
		}
		while (ns) {
			uint32_t s = sm[--ns];
			alias[2 * s] = alias[2 * s + 1] = 0xffffffffu;
		}
	}
	free(wt);
	free(sm);
	free(lg);
	return ok;
}

/* The engine's transcendental restatements, for accuracy tests: sin x, cos x, atan2(y, x), acos x. */
void oracle_trig(float x, float y, float *out) {
	svo_sincos(x, &out[0], &out[1]);
	out[2] = svo_atan2(y, x);
	out[3] = svo_acos(x);
}

/* ====================================================================== textured voxelization */

static double srgb_decode_d(double c) { return c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4); }
static double srgb_encode_d(double x) { return x <= 0.0031308 ? 12.92 * x : 1.055 * pow(x, 1.0 / 2.4) - 0.055; }
static uint8_t to_byte_d(double x) { return (uint8_t)floor(fmin(fmax(x, 0.0), 1.0) * 255.0 + 0.5); }

/* The texture's mip chain (CmdGenerateMipmap2D as the engine states it): level l+1 texel (i, j) is the
 * bilinear, clamp-to-edge, linear-space sample of level l at ((i + 1/2) w / w' - 1/2, (j + 1/2) h / h' - 1/2),
 * re-encoded to sRGB bytes (alpha linear), rounding to nearest.  out: every level's RGBA8 bytes, level
 * 0 first; returns the number of levels.  out must hold the chain (< 4/3 w h 4 + 4 * levels bytes). */
uint32_t oracle_texture_mips(const uint8_t *rgba, uint32_t w, uint32_t h, uint8_t *out) {
	double lin[256];
	for (int c = 0; c < 256; ++c)
		lin[c] = srgb_decode_d(c / 255.0);
	memcpy(out, rgba, (size_t)w * h * 4);
	uint8_t *src = out;
	uint32_t levels = 1;
	while (w > 1 || h > 1) {
		uint32_t w2 = w > 1 ? w / 2 : 1, h2 = h > 1 ? h / 2 : 1;
		uint8_t *dst = src + (size_t)w * h * 4;
		for (uint32_t j = 0; j < h2; ++j)
			for (uint32_t i = 0; i < w2; ++i) {
				double x = ((double)i + 0.5) * (double)w / (double)w2 - 0.5;
				double y = ((double)j + 0.5) * (double)h / (double)h2 - 0.5;
				double fx = floor(x), fy = floor(y), a = x - fx, b = y - fy;
				int64_t i0 = (int64_t)fx, j0 = (int64_t)fy;
				size_t xs[2], ys[2];
				for (int q = 0; q < 2; ++q) {
					int64_t xi = i0 + q, yj = j0 + q;
					xs[q] = (size_t)(xi < 0 ? 0 : (xi >= (int64_t)w ? w - 1 : xi));
					ys[q] = (size_t)(yj < 0 ? 0 : (yj >= (int64_t)h ? h - 1 : yj));
				}
				double wt[4] = {(1 - a) * (1 - b), a * (1 - b), (1 - a) * b, a * b};
				for (int ch = 0; ch < 4; ++ch) {
					double acc = 0.0;
					for (int q = 0; q < 4; ++q) {
						uint8_t v = src[(ys[q >> 1] * w + xs[q & 1]) * 4 + ch];
						acc += wt[q] * (ch < 3 ? lin[v] : v / 255.0);
					}
					dst[((size_t)j * w2 + i) * 4 + ch] = to_byte_d(ch < 3 ? srgb_encode_d(acc) : acc);
				}
			}
		src = dst;
		w = w2;
		h = h2;
		++levels;
	}
	return levels;
}

typedef struct tex_view {
	const float *texels; /* linear rgba floats of every level of every texture */
	const uint64_t *level_off; /* [texture * 16 + level]: first texel of the level */
	const uint32_t *dims;      /* [texture * 3]: width, height, levels */
	uint32_t count;
} tex_view;

static float log2_svo(float x) {
	if (!(x > 0.0f))
		return -1e30f;
	uint32_t bits = f2u(x);
	int e = (int)((bits >> 23) & 255u) - 127;
	float m = u2f((bits & 0x7fffffu) | 0x3f800000u);
	if (m > 1.41421356237309505f) {
		m = m * 0.5f;
		e += 1;
	}
	float s = (m - 1.0f) / (m + 1.0f), s2 = s * s;
	float p = 1.0f / 11.0f;
	p = p * s2 + 1.0f / 9.0f;
	p = p * s2 + 1.0f / 7.0f;
	p = p * s2 + 1.0f / 5.0f;
	p = p * s2 + 1.0f / 3.0f;
	p = p * s2 + 1.0f;
	return (float)e + (2.0f * (s * p)) * 1.44269504088896341f;
}

static void tex_bilinear(const tex_view *tv, uint32_t t, uint32_t l, float u, float v, float out[4]) {
	int64_t W = tv->dims[3 * t] >> l, H = tv->dims[3 * t + 1] >> l;
	if (W < 1) W = 1;
	if (H < 1) H = 1;
	float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
	float fx = floorf(x), fy = floorf(y);
	float a = x - fx, b = y - fy;
	int64_t ix = (int64_t)fminf(fmaxf(fx, -4e18f), 4e18f), jy = (int64_t)fminf(fmaxf(fy, -4e18f), 4e18f);
	int64_t i0 = ((ix % W) + W) % W, j0 = ((jy % H) + H) % H;
	int64_t i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
	const float *L = tv->texels + 4 * tv->level_off[16 * t + l];
	const float *t00 = L + 4 * (j0 * W + i0), *t10 = L + 4 * (j0 * W + i1);
	const float *t01 = L + 4 * (j1 * W + i0), *t11 = L + 4 * (j1 * W + i1);
	float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
	for (int k = 0; k < 4; ++k)
		out[k] = ((w00 * t00[k] + w10 * t10[k]) + w01 * t01[k]) + w11 * t11[k];
}

static uint32_t unorm8_tex(float v) { return (uint32_t)floorf(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f + 0.5f); }

/* shader/voxelizer.frag:27-36 for one candidate fragment of triangle tri: returns 0 when discarded. */
static int tex_fragment(uint64_t *frag, const svo_triangle *tri, const svo_triangle_uv *uv, uint32_t level,
                        const tex_view *tv) {
	if (uv->texture == 0xffffffffu || uv->texture >= tv->count)
		return 1;
	float scale = (float)(256 << level);
	int64_t X[3], Y[3], Z[3];
	for (int k = 0; k < 3; ++k) {
		X[k] = snap(tri->v[3 * k], scale);
		Y[k] = snap(tri->v[3 * k + 1], scale);
		Z[k] = snap(tri->v[3 * k + 2], scale);
	}
	int64_t e1x = X[1] - X[0], e1y = Y[1] - Y[0], e1z = Z[1] - Z[0];
	int64_t e2x = X[2] - X[0], e2y = Y[2] - Y[0], e2z = Z[2] - Z[0];
	int64_t nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
	int64_t ax = nx < 0 ? -nx : nx, ay = ny < 0 ? -ny : ny, az = nz < 0 ? -nz : nz;
	int axis = (ax > ay && ax > az) ? 0 : (ay > az ? 1 : 2);
	int64_t A[3], B[3];
	for (int k = 0; k < 3; ++k) {
		A[k] = axis == 0 ? Y[k] : (axis == 1 ? Z[k] : X[k]);
		B[k] = axis == 0 ? Z[k] : (axis == 1 ? X[k] : Y[k]);
	}
	uint32_t fx = (uint32_t)*frag, fy = (uint32_t)(*frag >> 32);
	int64_t vx = fx & 0xfffu, vy = (fx >> 12) & 0xfffu, vz = (fx >> 24) | ((fy >> 28) << 8);
	int64_t pi = axis == 0 ? vy : (axis == 1 ? vz : vx), pj = axis == 0 ? vz : (axis == 1 ? vx : vy);
	int64_t px = 256 * pi + 128, py = 256 * pj + 128;
	int64_t a0 = A[1] - A[0], a1 = B[1] - B[0], b0 = A[2] - A[0], b1 = B[2] - B[0];
	int64_t area = a0 * b1 - a1 * b0;
	if (area == 0)
		return 1;
	int64_t q0 = px - A[0], q1 = py - B[0];
	float fa = (float)area;
	float l1 = (float)(q0 * b1 - q1 * b0) / fa, l2 = (float)(a0 * q1 - a1 * q0) / fa;
	float du1 = uv->uv[2] - uv->uv[0], dv1 = uv->uv[3] - uv->uv[1];
	float du2 = uv->uv[4] - uv->uv[0], dv2 = uv->uv[5] - uv->uv[1];
	float u = (uv->uv[0] + l1 * du1) + l2 * du2, v = (uv->uv[1] + l1 * dv1) + l2 * dv2;
	float g1i = (float)(256 * b1) / fa, g1j = (float)(-256 * b0) / fa;
	float g2i = (float)(-256 * a1) / fa, g2j = (float)(256 * a0) / fa;
	uint32_t t = uv->texture, levels = tv->dims[3 * t + 2];
	float W = (float)tv->dims[3 * t], H = (float)tv->dims[3 * t + 1];
	float dux = (g1i * du1 + g2i * du2) * W, dvx = (g1i * dv1 + g2i * dv2) * H;
	float duy = (g1j * du1 + g2j * du2) * W, dvy = (g1j * dv1 + g2j * dv2) * H;
	float rho = fmaxf(sqrtf(dux * dux + dvx * dvx), sqrtf(duy * duy + dvy * dvy));
	float lod = log2_svo(rho), c[4];
	if (!(lod > 0.0f)) {
		tex_bilinear(tv, t, 0, u, v, c);
	} else {
		float d = fminf(lod, (float)(levels - 1));
		uint32_t lo = (uint32_t)floorf(d), hi = lo + 1 < levels ? lo + 1 : levels - 1;
		float f = d - (float)lo, c0[4], c1[4];
		tex_bilinear(tv, t, lo, u, v, c0);
		tex_bilinear(tv, t, hi, u, v, c1);
		for (int k = 0; k < 4; ++k)
			c[k] = (1.0f - f) * c0[k] + f * c1[k];
	}
	if (c[3] < 0.5f)
		return 0;
	uint32_t rgb = unorm8_tex(c[0]) | (unorm8_tex(c[1]) << 8) | (unorm8_tex(c[2]) << 16);
	*frag = (*frag & 0xF0000000FFFFFFFFull) | ((uint64_t)rgb << 32);
	return 1;
}

/* Voxelization with texture-sampled colour: the canonical fragments of every triangle, each textured
 * one's coloured or dropped.  textures: `count` RGBA8 images (sizes in widths / heights).  Returns the
 * fragment count written to out (out holds at least oracle_voxelize_count's total). */
uint64_t oracle_voxelize_textured(const svo_triangle *tris, const svo_triangle_uv *uvs, uint32_t n, uint32_t level,
                                  const uint8_t *const *textures, const uint32_t *widths, const uint32_t *heights,
                                  uint32_t count, uint64_t *out) {
	/* linear texels of every level */
	uint64_t total_texels = 0;
	uint64_t *level_off = (uint64_t *)calloc((size_t)count * 16 + 1, sizeof(uint64_t));
	uint32_t *dims = (uint32_t *)calloc((size_t)count * 3 + 1, sizeof(uint32_t));
	uint8_t **chains = (uint8_t **)calloc((size_t)count + 1, sizeof(uint8_t *));
	for (uint32_t t = 0; t < count; ++t) {
		size_t bytes = (size_t)widths[t] * heights[t] * 4 * 2 + 64 * 4;
		chains[t] = (uint8_t *)malloc(bytes);
		uint32_t levels = oracle_texture_mips(textures[t], widths[t], heights[t], chains[t]);
		dims[3 * t] = widths[t], dims[3 * t + 1] = heights[t], dims[3 * t + 2] = levels;
		for (uint32_t l = 0; l < levels; ++l) {
			uint64_t w = widths[t] >> l, h = heights[t] >> l;
			level_off[16 * t + l] = total_texels;
			total_texels += (w ? w : 1) * (h ? h : 1);
		}
	}
	float lin[256];
	for (int c = 0; c < 256; ++c)
		lin[c] = (float)srgb_decode_d(c / 255.0);
	float *texels = (float *)malloc((size_t)(total_texels + 1) * 16);
	for (uint32_t t = 0; t < count; ++t) {
		const uint8_t *p = chains[t];
		for (uint32_t l = 0; l < dims[3 * t + 2]; ++l) {
			uint64_t w = widths[t] >> l, h = heights[t] >> l, m = (w ? w : 1) * (h ? h : 1);
			float *dst = texels + 4 * level_off[16 * t + l];
			for (uint64_t i = 0; i < m; ++i, p += 4) {
				dst[4 * i] = lin[p[0]], dst[4 * i + 1] = lin[p[1]], dst[4 * i + 2] = lin[p[2]];
				dst[4 * i + 3] = (float)(p[3] / 255.0);
			}
		}
	}
	tex_view tv = {texels, level_off, dims, count};
	uint32_t *counts = (uint32_t *)malloc(((size_t)n + 1) * sizeof(uint32_t));
	uint64_t total = oracle_voxelize_count(tris, n, level, counts);
	uint64_t *offsets = (uint64_t *)malloc(((size_t)n + 1) * sizeof(uint64_t));
	offsets[0] = 0;
	for (uint32_t t = 0; t < n; ++t)
		offsets[t + 1] = offsets[t] + counts[t];
	uint64_t *cand = (uint64_t *)malloc((size_t)(total + 1) * sizeof(uint64_t));
	oracle_voxelize_emit(tris, n, level, offsets, cand);
	uint64_t kept = 0;
	for (uint32_t t = 0; t < n; ++t)
		for (uint64_t f = offsets[t]; f < offsets[t + 1]; ++f) {
			uint64_t fr = cand[f];
			if (tex_fragment(&fr, &tris[t], &uvs[t], level, &tv))
				out[kept++] = fr;
		}
	for (uint32_t t = 0; t < count; ++t)
		free(chains[t]);
	free(chains);
	free(level_off);
	free(dims);
	free(texels);
	free(counts);
	free(offsets);
	free(cand);
	return kept;
}
