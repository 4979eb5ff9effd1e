// march.cu — stack-based leaf ray march over the octree (replaces Octree_RayMarchLeaf,
// shader/octree.glsl:179-340, as called per pixel by shader/octree_tracer.frag:23-37 and per bounce by
// shader/path_tracer.comp:35-47).
//
// This translation unit is compiled with -fmad=false and IEEE division/square root: every float
// operation is rounded separately, so results are bit-identical to the oracle's scalar restatement.
//
// GB300 design:
//   * persistent grid; each warp claims 32 rays at a time from a global ticket (one ray per lane), so
//     rays of very different lengths do not leave the tail of the launch idle (measured: 4 rays per lane
//     per ticket took 1.7x longer on the 2^10 room scene);
//   * camera rays are claimed as 8x4-pixel tiles, so a warp's lanes march neighbouring rays that share
//     traversal paths and node words;
//   * the traversal stack (one parent word per level, at most 12) lives in shared memory, laid out
//     [level][thread] so a warp's accesses hit 32 distinct banks; it never touches local memory;
//   * node words are read through the read-only path (ld.global.nc), so hot upper levels stay in L1/L2;
//   * camera rays are generated in the kernel (no ray buffer), hits are written as two 16 B stores
//     (row-major by pixel, whatever the claim order).
//
// The traversal (ray_init / ray_step / ray_finish below, and the occlusion, coarse and path-tracer
// marches built on it) restates the sparse-voxel-octree ray cast of Laine and Karras, "Efficient Sparse
// Voxel Octrees" (NVIDIA Research, 2010), as the reference carries it in shader/octree.glsl:15-42,
// 179-629.  That code is distributed under the following notice, which applies to this restatement:
//
//   Copyright (c) 2009-2011, NVIDIA Corporation
//   All rights reserved.
//
//   Redistribution and use in source and binary forms, with or without
//   modification, are permitted provided that the following conditions are met:
//       * Redistributions of source code must retain the above copyright
//         notice, this list of conditions and the following disclaimer.
//       * Redistributions in binary form must reproduce the above copyright
//         notice, this list of conditions and the following disclaimer in the
//         documentation and/or other materials provided with the distribution.
//       * Neither the name of NVIDIA Corporation nor the
//         names of its contributors may be used to endorse or promote products
//         derived from this software without specific prior written permission.
//
//   THIS SOFTWARE IS PROVIDED BY THE COPYRIGHT HOLDERS AND CONTRIBUTORS "AS IS"
//   AND ANY EXPRESS OR IMPLIED WARRANTIES, INCLUDING, BUT NOT LIMITED TO, THE
//   IMPLIED WARRANTIES OF MERCHANTABILITY AND FITNESS FOR A PARTICULAR PURPOSE
//   ARE DISCLAIMED. IN NO EVENT SHALL <COPYRIGHT HOLDER> BE LIABLE FOR ANY
//   DIRECT, INDIRECT, INCIDENTAL, SPECIAL, EXEMPLARY, OR CONSEQUENTIAL DAMAGES
//   (INCLUDING, BUT NOT LIMITED TO, PROCUREMENT OF SUBSTITUTE GOODS OR SERVICES;
//   LOSS OF USE, DATA, OR PROFITS; OR BUSINESS INTERRUPTION) HOWEVER CAUSED AND
//   ON ANY THEORY OF LIABILITY, WHETHER IN CONTRACT, STRICT LIABILITY, OR TORT
//   (INCLUDING NEGLIGENCE OR OTHERWISE) ARISING IN ANY WAY OUT OF THE USE OF
//   THIS SOFTWARE, EVEN IF ADVISED OF THE POSSIBILITY OF SUCH DAMAGE.
#include "common.cuh"
#include "svo_internal.h"

namespace svo {

constexpr int kMarchTPB = 128;
constexpr float kEps = 3.552713678800501e-15f; // EPS of shader/octree.glsl:44 (2^-48)
constexpr uint32_t kBeamSize = SVO_BEAM_SIZE;   // pixels per beam tile edge (kBeamSize, src/Config.hpp:22)

SVO_DEV float max_glsl(float x, float y) { return x < y ? y : x; }
SVO_DEV float min_glsl(float x, float y) { return y < x ? y : x; }
SVO_DEV float eps_clamp(float v) { return fabsf(v) > kEps ? v : (v >= 0.0f ? kEps : -kEps); }

struct MarchOut {
	float t;
	float pos[3];
	uint32_t node, iter;
	uint32_t voxel_lo, voxel_hi; // packed uint16 voxel[3] and flags, as in svo_hit
};

// State of one ray's leaf march (Octree_RayMarchLeaf, shader/octree.glsl:179-340), so a lane can run a
// ray as init + steps + finish and take a new ray as soon as its current one ends.  `stack` points at
// the lane's stack: a column of a shared [level][thread] array (STRIDE = threads per block) or a private
// array in local memory (STRIDE = 1).
struct RayState {
	float o[3], d[3], coef[3], bias[3], pos[3];
	float t_min, t_max, h, scale_exp2;
	uint32_t parent, cur, idx, scale, oct_mask, iter, nfetch, min_scale;
	bool aborted, none;
};

template <int STRIDE>
SVO_DEV void ray_init(RayState &s, const float o[3], const float dir[3], uint32_t level, uint32_t *stack) {
	s.nfetch = 0;
	s.iter = 0;
	s.aborted = false;
	s.none = dir[0] == 0.0f && dir[1] == 0.0f && dir[2] == 0.0f; // no ray (miss of a previous bounce)
#pragma unroll
	for (int k = 0; k < 3; ++k) s.o[k] = o[k];
	if (s.none) {
		s.scale = 0xffffffffu; // ends at once
		return;
	}
	for (uint32_t k = 0; k < level; ++k) stack[k * STRIDE] = 0u;
#pragma unroll
	for (int k = 0; k < 3; ++k) s.d[k] = eps_clamp(dir[k]);
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		s.coef[k] = 1.0f / -fabsf(s.d[k]);
		s.bias[k] = s.coef[k] * o[k];
	}
	s.oct_mask = 0;
#pragma unroll
	for (int k = 0; k < 3; ++k)
		if (s.d[k] > 0.0f) {
			s.oct_mask ^= 1u << k;
			s.bias[k] = 3.0f * s.coef[k] - s.bias[k];
		}
	s.t_min = max_glsl(max_glsl(2.0f * s.coef[0] - s.bias[0], 2.0f * s.coef[1] - s.bias[1]), 2.0f * s.coef[2] - s.bias[2]);
	s.t_max = min_glsl(min_glsl(s.coef[0] - s.bias[0], s.coef[1] - s.bias[1]), s.coef[2] - s.bias[2]);
	s.t_min = max_glsl(s.t_min, 0.0f);
	s.h = s.t_max;
	s.parent = 0, s.cur = 0, s.idx = 0;
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		s.pos[k] = 1.0f;
		if (1.5f * s.coef[k] - s.bias[k] > s.t_min) {
			s.idx ^= 1u << k;
			s.pos[k] = 1.5f;
		}
	}
	s.scale = SVO_STACK_SIZE - 1;
	s.scale_exp2 = 0.5f;
	s.min_scale = SVO_STACK_SIZE - level; // deepest scale a valid tree reaches
}

// One iteration of the march loop; returns true when the ray has ended (the loop of the shader breaks or
// its condition fails).  A malformed pool (pointer outside the range, interior word below the octree
// level, iteration bound) ends the ray as an aborted miss and sets kStatusMalformed.  CHECK_END = false
// skips the loop condition for callers that never step an ended ray (every path that ends the ray
// returns true at once, so only a ray without direction enters the loop ended).  COUNT = false leaves
// the node-fetch counter alone (callers that do not report it).
//
// The iteration bound is tested where an iteration advances, not in every iteration: consecutive pushes
// are limited by the tree depth (a push below the octree level aborts), so every iteration sequence
// that does not end contains advances, and a ray is stopped within SVO_STACK_SIZE iterations of the
// bound, also when its arithmetic is NaN and nothing is fetched.  (Testing the bound in every iteration
// cost 10% of the march on the room frame.)  The oracle tests it at the same place.
template <int STRIDE, bool CHECK_END = true, bool COUNT = true>
SVO_DEV bool ray_step(RayState &s, const uint32_t *__restrict__ pool, uint32_t range, uint32_t *stack,
                      uint32_t *status) {
	if (CHECK_END && s.scale >= SVO_STACK_SIZE) return true;
	++s.iter;
	if (s.cur == 0u) {
		const uint32_t w = s.parent + (s.idx ^ s.oct_mask);
		if (w >= range) {
			atomicOr(status, kStatusMalformed);
			s.aborted = true;
			s.scale = 0xffffffffu;
			return true;
		}
		s.cur = __ldg(pool + w);
		if (COUNT) ++s.nfetch;
	}
	float tc[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) tc[k] = s.pos[k] * s.coef[k] - s.bias[k];
	// GLSL min (y < x ? y : x) as one min instruction.  For a finite origin and direction, pos * coef is
	// finite and nonzero (pos in [1, 2], coef = -1 / max(|d|, EPS)), so tc = pos * coef - bias is never
	// NaN (bias may overflow to an infinity, never both terms) and never -0 (a - b gives -0 only for
	// a = -0); fminf then returns the same value as the GLSL form.
	const float tc_max = fminf(fminf(tc[0], tc[1]), tc[2]);

	if ((s.cur & 0x80000000u) != 0u && s.t_min <= s.t_max) {
		const float half = s.scale_exp2 * 0.5f;
		float t_center[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) t_center[k] = half * s.coef[k] + tc[k];
		if ((s.cur & 0x40000000u) != 0u) return true; // leaf
		if (s.scale <= s.min_scale) {                  // interior node below the leaf level: malformed pool
			atomicOr(status, kStatusMalformed);
			s.aborted = true;
			s.scale = 0xffffffffu;
			return true;
		}
		if (tc_max < s.h) stack[(SVO_STACK_SIZE - 1 - s.scale) * STRIDE] = s.parent; // push
		s.h = tc_max;
		s.parent = s.cur & 0x3fffffffu;
		s.idx = 0;
		--s.scale;
		s.scale_exp2 = half;
#pragma unroll
		for (int k = 0; k < 3; ++k)
			if (t_center[k] > s.t_min) {
				s.idx ^= 1u << k;
				s.pos[k] += s.scale_exp2;
			}
		s.cur = 0;
		return false;
	}
	// advance
	if (s.iter >= SVO_MARCH_MAX_ITER) { // the iteration bound (see above); never reached on a valid octree
		s.aborted = true;
		return true;
	}
	uint32_t step_mask = 0;
#pragma unroll
	for (int k = 0; k < 3; ++k)
		if (tc[k] <= tc_max) {
			step_mask ^= 1u << k;
			s.pos[k] -= s.scale_exp2;
		}
	s.t_min = tc_max;
	s.idx ^= step_mask;
	if ((s.idx & step_mask) != 0u) { // pop
		uint32_t diff = 0;
#pragma unroll
		for (int k = 0; k < 3; ++k)
			if (step_mask & (1u << k)) diff |= __float_as_uint(s.pos[k]) ^ __float_as_uint(s.pos[k] + s.scale_exp2);
		s.scale = diff ? 31u - (uint32_t)__clz(diff) : 0xffffffffu; // findMSB
		if (s.scale >= SVO_STACK_SIZE) return true;
		s.scale_exp2 = __uint_as_float((s.scale - SVO_STACK_SIZE + 127u) << 23u);
		s.parent = stack[(SVO_STACK_SIZE - 1 - s.scale) * STRIDE];
		uint32_t sh[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			sh[k] = __float_as_uint(s.pos[k]) >> s.scale;
			s.pos[k] = __uint_as_float(sh[k] << s.scale);
		}
		s.idx = (sh[0] & 1u) | ((sh[1] & 1u) << 1) | ((sh[2] & 1u) << 2);
		s.h = 0.0f;
		s.cur = 0;
	}
	return false;
}

// The outputs of an ended ray (shader/octree.glsl:307-340): normal from the exit corner, un-mirrored
// cube position, o_pos clamped into the cube and nudged by EPS, hit flag.
SVO_DEV void ray_finish(RayState &s, uint32_t level, MarchOut &out) {
	if (s.none) {
		out.t = 0.0f;
		out.pos[0] = s.o[0], out.pos[1] = s.o[1], out.pos[2] = s.o[2];
		out.node = 0, out.iter = 0;
		out.voxel_lo = 0xffffffffu;
		out.voxel_hi = 0x0000ffffu;
		return;
	}
	float tc[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) tc[k] = s.coef[k] * (s.pos[k] + s.scale_exp2) - s.bias[k];
	const uint32_t nax = (tc[0] > tc[1] && tc[0] > tc[2]) ? 0u : (tc[1] > tc[2] ? 1u : 2u);
	const bool neg = (s.oct_mask >> nax) & 1u; // normal is -axis exactly when that axis was mirrored
#pragma unroll
	for (int k = 0; k < 3; ++k)
		if (s.oct_mask & (1u << k)) s.pos[k] = 3.0f - s.scale_exp2 - s.pos[k];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		float v = s.o[k] + s.t_min * s.d[k];
		v = min_glsl(max_glsl(v, s.pos[k]), s.pos[k] + s.scale_exp2);
		if ((uint32_t)k == nax) v = neg ? s.pos[k] - kEps : s.pos[k] + s.scale_exp2 + kEps * 2.0f;
		out.pos[k] = v;
	}
	const bool hit = !s.aborted && s.scale < SVO_STACK_SIZE && s.t_min <= s.t_max;
	out.t = s.t_min;
	out.iter = s.iter;
	const uint32_t flags = (hit ? SVO_HIT_FLAG_HIT : 0u) | (nax << 1) | (neg ? SVO_HIT_NORMAL_NEG : 0u) |
	                       (s.aborted ? SVO_HIT_FLAG_ABORTED : 0u);
	if (hit) {
		const float res = (float)(1u << level);
		const uint32_t vx = (uint32_t)((s.pos[0] - 1.0f) * res), vy = (uint32_t)((s.pos[1] - 1.0f) * res);
		const uint32_t vz = (uint32_t)((s.pos[2] - 1.0f) * res);
		out.node = s.cur;
		out.voxel_lo = vx | (vy << 16);
		out.voxel_hi = vz | (flags << 16);
	} else {
		out.node = 0;
		out.voxel_lo = 0xffffffffu;
		out.voxel_hi = 0xffffu | (flags << 16);
	}
}

// One whole ray (nfetch: node words read, when COUNT).
template <int STRIDE, bool COUNT = true>
SVO_DEV void march_ray(const uint32_t *__restrict__ pool, uint32_t range, uint32_t level, const float o[3],
                       const float dir[3], uint32_t *stack, MarchOut &out, uint32_t &nfetch, uint32_t *status) {
	RayState s;
	ray_init<STRIDE>(s, o, dir, level, stack);
	if (!s.none)
		while (!ray_step<STRIDE, false, COUNT>(s, pool, range, stack, status)) {
		}
	ray_finish(s, level, out);
	nfetch = s.nfetch;
}

SVO_DEV void store_hit(svo_hit *hits, uint32_t r, const MarchOut &m) {
	uint4 *dst = reinterpret_cast<uint4 *>(hits + r);
	dst[0] = make_uint4(__float_as_uint(m.t), __float_as_uint(m.pos[0]), __float_as_uint(m.pos[1]),
	                    __float_as_uint(m.pos[2]));
	dst[1] = make_uint4(m.node, m.iter, m.voxel_lo, m.voxel_hi);
}

// Camera_GenRay(ivec2(pixel) / size) (shader/camera.glsl:11-14, shader/octree_tracer.frag:24).
// Camera_GenRay of a normalised image coordinate (shader/camera.glsl:11-14).
SVO_DEV void gen_dir(const svo_camera &cam, float cx, float cy, float d[3]) {
	cx = cx * 2.0f - 1.0f;
	cy = cy * 2.0f - 1.0f;
	float v[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) v[k] = (cam.look[k] - cam.side[k] * cx) - cam.up[k] * cy;
	const float len = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
#pragma unroll
	for (int k = 0; k < 3; ++k) d[k] = v[k] / len;
}

SVO_DEV void camera_ray(const svo_camera &cam, uint32_t width, uint32_t height, uint32_t r, float o[3], float d[3]) {
	const uint32_t y = r / width, x = r - y * width;
	gen_dir(cam, (float)x / (float)width, (float)y / (float)height, d);
#pragma unroll
	for (int k = 0; k < 3; ++k) o[k] = cam.pos[k];
}

// shader/octree_tracer.frag:27-33: a primary ray starts at o + d * (the least of the 4 beam texels at
// the corners of its pixel's tile).
SVO_DEV void beam_advance(const float *__restrict__ beam, uint32_t width, uint32_t r, float o[3], const float d[3]) {
	const uint32_t y = r / width, x = r - y * width;
	const uint32_t bw = (width + kBeamSize - 1) / kBeamSize + 1;
	const float *t0 = beam + (size_t)(y / kBeamSize) * bw + x / kBeamSize, *t1 = t0 + bw;
	const float m = min_glsl(min_glsl(__ldg(t0), __ldg(t0 + 1)), min_glsl(__ldg(t1), __ldg(t1 + 1)));
#pragma unroll
	for (int k = 0; k < 3; ++k) o[k] = o[k] + d[k] * m;
}

// One past the last image row a camera launch traces (the launch covers rows [row0, that)).
SVO_DEV uint32_t camera_row_end(const MarchArgs &a) {
	return a.rows ? min(a.height, a.row0 + a.rows) : a.height;
}

// Variants (chosen per launch from the launch-parameter table): TPB threads per block, RPL rays per lane
// per ticket, SHARED: stack in shared memory ([level][thread], 32 distinct banks per warp) or in a
// private local-memory array.  COUNT: the launch reports node fetches (a.fetches); a separate
// instantiation, so the usual launch carries no counter and no second copy of the loop.
template <bool CAMERA, int TPB, int RPL, bool SHARED, bool COUNT>
__global__ void __launch_bounds__(TPB) march_kernel(MarchArgs a) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	constexpr int kStride = SHARED ? TPB : 1;
	__shared__ uint32_t s_stack[SHARED ? SVO_LEVEL_MAX * TPB : 1];
	uint32_t l_stack[SHARED ? 1 : SVO_LEVEL_MAX];
	uint32_t *stack = SHARED ? s_stack + threadIdx.x : l_stack;
	const uint32_t lane = lane_id();
	// work slots: ray indices, or for camera rays 32 slots per 8x4 tile of the (padded) image
	const uint32_t tiles_x = CAMERA ? (a.width + 7u) / 8u : 0u;
	const uint32_t y_end = camera_row_end(a);
	const uint64_t slots = CAMERA ? (uint64_t)tiles_x * ((y_end - a.row0 + 3u) / 4u) * 32u : (uint64_t)a.n;
	unsigned long long fetched = 0;
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(a.ticket, (unsigned long long)(32u * RPL));
		base = __shfl_sync(kFullMask, base, 0);
		if (base >= slots) break;
#pragma unroll 1
		for (uint32_t k = 0; k < (uint32_t)RPL; ++k) {
			const uint64_t slot = base + k * 32u + lane;
			if (slot >= slots) break;
			float o[3], d[3];
			uint32_t r;
			if constexpr (CAMERA) {
				const uint32_t tile = (uint32_t)(slot >> 5), in = (uint32_t)(slot & 31u);
				const uint32_t x = (tile % tiles_x) * 8u + (in & 7u), y = a.row0 + (tile / tiles_x) * 4u + (in >> 3);
				if (x >= a.width || y >= y_end) continue; // padding slot of a partial edge tile
				r = y * a.width + x;
				camera_ray(a.cam, a.width, a.height, r, o, d);
				if (a.beam) beam_advance(a.beam, a.width, r, o, d);
			} else {
				r = (uint32_t)slot;
				const float2 *src = reinterpret_cast<const float2 *>(a.rays + r);
				const float2 p0 = src[0], p1 = src[1], p2 = src[2];
				o[0] = p0.x, o[1] = p0.y, o[2] = p1.x, d[0] = p1.y, d[1] = p2.x, d[2] = p2.y;
			}
			MarchOut m;
			uint32_t nf = 0;
			march_ray<kStride, COUNT>(a.pool, a.range, a.level, o, d, stack, m, nf, a.status);
			store_hit(a.hits, r, m);
			fetched += nf;
		}
	}
	if (COUNT && a.fetches) {
		fetched = warp_sum(fetched);
		if (lane == 0) atomicAdd(a.fetches, fetched);
	}
}

// Persistent refill: a lane takes a new ray as soon as its ray ends, instead of the warp waiting for its
// slowest ray.  Idle lanes claim consecutive work slots together (one atomic per claim) once at least
// kRefillMin of them are idle, or all of them are.  Per ray the arithmetic is the single-ray march's.
constexpr uint32_t kRefillMin = 8;

template <bool CAMERA, int TPB, bool SHARED, bool COUNT>
__global__ void __launch_bounds__(TPB) march_refill_kernel(MarchArgs a) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	constexpr int kStride = SHARED ? TPB : 1;
	__shared__ uint32_t s_stack[SHARED ? SVO_LEVEL_MAX * TPB : 1];
	uint32_t l_stack[SHARED ? 1 : SVO_LEVEL_MAX];
	uint32_t *stack = SHARED ? s_stack + threadIdx.x : l_stack;
	const uint32_t lane = lane_id(), lt_mask = (1u << lane) - 1u;
	const uint32_t tiles_x = CAMERA ? (a.width + 7u) / 8u : 0u;
	const uint32_t y_end = camera_row_end(a);
	const uint64_t slots = CAMERA ? (uint64_t)tiles_x * ((y_end - a.row0 + 3u) / 4u) * 32u : (uint64_t)a.n;
	RayState s;
	bool active = false, exhausted = false;
	uint32_t r = 0;
	unsigned long long fetched = 0;
	for (;;) {
		const uint32_t idle = __ballot_sync(kFullMask, !active);
		const uint32_t nidle = __popc(idle);
		if (!exhausted && (nidle >= kRefillMin || idle == kFullMask)) {
			const uint32_t leader = __ffs(idle) - 1;
			unsigned long long base = 0;
			if (lane == leader) base = atomicAdd(a.ticket, (unsigned long long)nidle);
			base = __shfl_sync(kFullMask, base, leader);
			if (base + nidle >= slots) exhausted = true; // warp-uniform
			const uint64_t slot = base + __popc(idle & lt_mask);
			if (!active && slot < slots) {
				float o[3], d[3];
				bool live = true;
				if constexpr (CAMERA) {
					const uint32_t tile = (uint32_t)(slot >> 5), in = (uint32_t)(slot & 31u);
					const uint32_t x = (tile % tiles_x) * 8u + (in & 7u), y = a.row0 + (tile / tiles_x) * 4u + (in >> 3);
					live = x < a.width && y < y_end; // padding slots of partial edge tiles
					if (live) {
						r = y * a.width + x;
						camera_ray(a.cam, a.width, a.height, r, o, d);
						if (a.beam) beam_advance(a.beam, a.width, r, o, d);
					}
				} else {
					r = (uint32_t)slot;
					const float2 *src = reinterpret_cast<const float2 *>(a.rays + r);
					const float2 p0 = src[0], p1 = src[1], p2 = src[2];
					o[0] = p0.x, o[1] = p0.y, o[2] = p1.x, d[0] = p1.y, d[1] = p2.x, d[2] = p2.y;
				}
				if (live) {
					ray_init<kStride>(s, o, d, a.level, stack);
					active = true;
				}
			}
		}
		if (!__any_sync(kFullMask, active)) {
			if (exhausted) break;
			continue;
		}
		if (active && ray_step<kStride, true, COUNT>(s, a.pool, a.range, stack, a.status)) {
			MarchOut m;
			ray_finish(s, a.level, m);
			store_hit(a.hits, r, m);
			fetched += s.nfetch;
			active = false;
		}
	}
	if (a.fetches) {
		fetched = warp_sum(fetched);
		if (lane == 0) atomicAdd(a.fetches, fetched);
	}
}

// ------------------------------------------------------------------------------------ occlusion and beam
// The traversal of Octree_RayMarchOcclude (shader/octree.glsl:504-629; COARSE = false) and of
// Octree_RayMarchCoarse (shader/octree.glsl:47-177; COARSE = true): the leaf march without its outputs,
// with the occlusion march's direction clamp (|d| >= EPS is kept) or, for the coarse march, the leaf
// march's clamp and a stop at the first non-empty node at least as large as the cone footprint
// orig_sz + t * dir_sz.  Returns true on a hit, with t = t_min and size = the node's size.  A malformed
// pool ends the ray as a miss and sets kStatusMalformed.
template <bool COARSE, int STRIDE>
SVO_DEV bool march_traverse(const uint32_t *__restrict__ pool, uint32_t range, uint32_t level, const float o[3],
                            const float dir[3], float orig_sz, float dir_sz, uint32_t *stack, float &t_out,
                            float &size_out, uint32_t *status) {
	float d[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
		d[k] = (COARSE ? fabsf(dir[k]) > kEps : fabsf(dir[k]) >= kEps) ? dir[k] : (dir[k] >= 0.0f ? kEps : -kEps);
	for (uint32_t k = 0; k < level; ++k) stack[k * STRIDE] = 0u;
	float coef[3], bias[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		coef[k] = 1.0f / -fabsf(d[k]);
		bias[k] = coef[k] * o[k];
	}
	uint32_t oct_mask = 0;
#pragma unroll
	for (int k = 0; k < 3; ++k)
		if (d[k] > 0.0f) {
			oct_mask ^= 1u << k;
			bias[k] = 3.0f * coef[k] - bias[k];
		}
	float t_min = max_glsl(max_glsl(2.0f * coef[0] - bias[0], 2.0f * coef[1] - bias[1]), 2.0f * coef[2] - bias[2]);
	const float t_max = min_glsl(min_glsl(coef[0] - bias[0], coef[1] - bias[1]), coef[2] - bias[2]);
	t_min = max_glsl(t_min, 0.0f);
	float h = t_max;
	uint32_t parent = 0, cur = 0, idx = 0;
	float pos[3] = {1.0f, 1.0f, 1.0f};
#pragma unroll
	for (int k = 0; k < 3; ++k)
		if (1.5f * coef[k] - bias[k] > t_min) {
			idx ^= 1u << k;
			pos[k] = 1.5f;
		}
	uint32_t scale = SVO_STACK_SIZE - 1, iter = 0;
	float scale_exp2 = 0.5f;
	bool aborted = false;
	const uint32_t min_scale = SVO_STACK_SIZE - level;
	while (scale < SVO_STACK_SIZE) {
		if (++iter > SVO_MARCH_MAX_ITER) {
			aborted = true;
			break;
		}
		if (cur == 0u) {
			const uint32_t w = parent + (idx ^ oct_mask);
			if (w >= range) {
				atomicOr(status, kStatusMalformed);
				aborted = true;
				break;
			}
			cur = __ldg(pool + w);
		}
		float tc[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) tc[k] = pos[k] * coef[k] - bias[k];
		const float tc_max = fminf(fminf(tc[0], tc[1]), tc[2]); // the GLSL min for finite rays (ray_step)
		if ((cur & 0x80000000u) != 0u && t_min <= t_max) {
			if (COARSE && orig_sz + tc_max * dir_sz >= scale_exp2) break;
			const float half = scale_exp2 * 0.5f;
			float t_center[3];
#pragma unroll
			for (int k = 0; k < 3; ++k) t_center[k] = half * coef[k] + tc[k];
			if ((cur & 0x40000000u) != 0u) break; // leaf
			if (scale <= min_scale) {
				atomicOr(status, kStatusMalformed);
				aborted = true;
				break;
			}
			if (tc_max < h) stack[(SVO_STACK_SIZE - 1 - scale) * STRIDE] = parent;
			h = tc_max;
			parent = cur & 0x3fffffffu;
			idx = 0;
			--scale;
			scale_exp2 = half;
#pragma unroll
			for (int k = 0; k < 3; ++k)
				if (t_center[k] > t_min) {
					idx ^= 1u << k;
					pos[k] += scale_exp2;
				}
			cur = 0;
			continue;
		}
		uint32_t step_mask = 0;
#pragma unroll
		for (int k = 0; k < 3; ++k)
			if (tc[k] <= tc_max) {
				step_mask ^= 1u << k;
				pos[k] -= scale_exp2;
			}
		t_min = tc_max;
		idx ^= step_mask;
		if ((idx & step_mask) != 0u) {
			uint32_t diff = 0;
#pragma unroll
			for (int k = 0; k < 3; ++k)
				if (step_mask & (1u << k)) diff |= __float_as_uint(pos[k]) ^ __float_as_uint(pos[k] + scale_exp2);
			scale = diff ? 31u - (uint32_t)__clz(diff) : 0xffffffffu;
			if (scale >= SVO_STACK_SIZE) break;
			scale_exp2 = __uint_as_float((scale - SVO_STACK_SIZE + 127u) << 23u);
			parent = stack[(SVO_STACK_SIZE - 1 - scale) * STRIDE];
			uint32_t sh[3];
#pragma unroll
			for (int k = 0; k < 3; ++k) {
				sh[k] = __float_as_uint(pos[k]) >> scale;
				pos[k] = __uint_as_float(sh[k] << scale);
			}
			idx = (sh[0] & 1u) | ((sh[1] & 1u) << 1) | ((sh[2] & 1u) << 2);
			h = 0.0f;
			cur = 0;
		}
	}
	t_out = t_min;
	size_out = scale_exp2;
	return !aborted && scale < SVO_STACK_SIZE && t_min <= t_max;
}

// RayTangent of shader/octree_tracer_beam.frag:17-20.
SVO_DEV float ray_tangent(const float x[3], const float y[3]) {
	const float c = (x[0] * y[0] + x[1] * y[1]) + x[2] * y[2];
	return sqrtf(1.0f - c * c) / fabsf(c);
}

// The beam pre-pass (shader/octree_tracer_beam.frag:22-30 as src/OctreeTracer.cpp:183-211 draws it): one
// texel per corner of each kBeamSize x kBeamSize pixel tile.  The ray through the corner and the 4 rays
// half a texel away give the cone's tangent; the coarse march stops at the first node the cone does
// not resolve, and the texel is max(0, t - node size), or 1e10 when the cone misses.
SVO_DEV float beam_texel(const MarchArgs &a, uint32_t i, uint32_t bw, float orig_sz, uint32_t *stack) {
	const float W = (float)a.width, H = (float)a.height, bs = (float)kBeamSize;
	const uint32_t by = i / bw, bx = i - by * bw;
	const float fx = (float)bx, fy = (float)by;
	float d[3], dk[3];
	gen_dir(a.cam, fx / W * bs, fy / H * bs, d);
	gen_dir(a.cam, (fx + 0.5f) / W * bs, (fy + 0.5f) / H * bs, dk);
	const float t0 = ray_tangent(d, dk);
	gen_dir(a.cam, (fx + -0.5f) / W * bs, (fy + 0.5f) / H * bs, dk);
	const float t1 = ray_tangent(d, dk);
	gen_dir(a.cam, (fx + 0.5f) / W * bs, (fy + -0.5f) / H * bs, dk);
	const float t2 = ray_tangent(d, dk);
	gen_dir(a.cam, (fx + -0.5f) / W * bs, (fy + -0.5f) / H * bs, dk);
	const float t3 = ray_tangent(d, dk);
	const float dir_sz = 2.0f * max_glsl(max_glsl(t0, t1), max_glsl(t2, t3));
	const float o[3] = {a.cam.pos[0], a.cam.pos[1], a.cam.pos[2]};
	float t, sz;
	const bool hit = march_traverse<true, kMarchTPB>(a.pool, a.range, a.level, o, d, orig_sz, dir_sz, stack, t, sz,
	                                                 a.status);
	return hit ? max_glsl(0.0f, t - sz) : 1e10f;
}

__global__ void __launch_bounds__(kMarchTPB) beam_kernel(MarchArgs a, float *__restrict__ beam, float orig_sz) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_stack[SVO_LEVEL_MAX * kMarchTPB];
	uint32_t *stack = s_stack + threadIdx.x;
	const uint32_t bw = (a.width + kBeamSize - 1) / kBeamSize + 1, bh = (a.height + kBeamSize - 1) / kBeamSize + 1;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < bw * bh; i += gridDim.x * blockDim.x)
		beam[i] = beam_texel(a, i, bw, orig_sz, stack);
}

// Beam pre-pass and beam-advanced primary march in one persistent launch.  Work slots come from one
// ticket: first the texels (32 per claim), then the 8x4-pixel tiles of the image (32 rays per claim).
// A tile's 4 beam texels (an 8x4 tile lies inside one 8x8 beam tile) were all claimed before the
// tile, by warps that are running and wait on nothing, so the tile's warp polls them (acquire loads,
// bounded) and marches as soon as they are published; the slow coarse marches of a few texels overlap
// the other tiles' marches instead of ending a separate launch.  Texels start as the all-ones pattern,
// which no texel value has.  Every value is the separate kernels' value bit for bit.
constexpr uint32_t kBeamUnset = 0xffffffffu;

template <bool COUNT>
__global__ void __launch_bounds__(kMarchTPB) march_beam_fused_kernel(MarchArgs a, float *__restrict__ beam,
                                                                     float orig_sz) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_stack[SVO_LEVEL_MAX * kMarchTPB];
	uint32_t *stack = s_stack + threadIdx.x;
	const uint32_t lane = lane_id();
	const uint32_t bw = (a.width + kBeamSize - 1) / kBeamSize + 1, bh = (a.height + kBeamSize - 1) / kBeamSize + 1;
	const uint64_t texels = (uint64_t)bw * bh, texel_slots = (texels + 31u) / 32u * 32u;
	const uint32_t tiles_x = (a.width + 7u) / 8u;
	const uint64_t slots = texel_slots + (uint64_t)tiles_x * ((a.height + 3u) / 4u) * 32u;
	unsigned long long fetched = 0;
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(a.ticket, 32ull);
		base = __shfl_sync(kFullMask, base, 0);
		if (base >= slots) break;
		if (base < texel_slots) {
			const uint64_t i = base + lane;
			if (i < texels && i != c_wait_fault.withheld) { // (a test may withhold one texel)
				const float v = beam_texel(a, (uint32_t)i, bw, orig_sz, stack);
				asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(beam + i), "r"(__float_as_uint(v)) : "memory");
			}
			continue;
		}
		const uint64_t slot = base - texel_slots + lane;
		const uint32_t tile = (uint32_t)(slot >> 5), in = (uint32_t)(slot & 31u);
		const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
		const uint32_t x = tx * 8u + (in & 7u), y = ty * 4u + (in >> 3);
		// lanes 0..3 fetch texels (bx, by), (bx + 1, by), (bx, by + 1), (bx + 1, by + 1) of the beam tile
		float tv = 0.0f;
		bool gave_up = false;
		if (lane < 4) {
			const uint32_t bx = tx * 8u / kBeamSize, by = ty * 4u / kBeamSize;
			const float *p = beam + (size_t)(by + (lane >> 1)) * bw + bx + (lane & 1u);
			const uint32_t limit = c_wait_fault.limit;
			uint32_t w, spins = 0;
			for (;;) {
				asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(w) : "l"(p) : "memory");
				if (w != kBeamUnset) break;
				if (++spins > limit) { // a texel that never came: report, march from the camera
					atomicOr(a.status, kStatusTimeout);
					w = 0u;
					gave_up = true;
					break;
				}
				__nanosleep(64);
			}
			tv = __uint_as_float(w);
		}
		// a tile whose wait gave up marches from the camera (start distance 0) and flags its rays
		const uint32_t waited_out = __any_sync(kFullMask, gave_up) ? (SVO_HIT_FLAG_BEAM_WAIT << 16) : 0u;
		const float t00 = __shfl_sync(kFullMask, tv, 0), t01 = __shfl_sync(kFullMask, tv, 1);
		const float t10 = __shfl_sync(kFullMask, tv, 2), t11 = __shfl_sync(kFullMask, tv, 3);
		const float m = min_glsl(min_glsl(t00, t01), min_glsl(t10, t11));
		if (x < a.width && y < a.height) {
			const uint32_t r = y * a.width + x;
			float o[3], d[3];
			camera_ray(a.cam, a.width, a.height, r, o, d);
#pragma unroll
			for (int k = 0; k < 3; ++k) o[k] = o[k] + d[k] * m;
			MarchOut mo;
			uint32_t nf = 0;
			march_ray<kMarchTPB, COUNT>(a.pool, a.range, a.level, o, d, stack, mo, nf, a.status);
			mo.voxel_hi |= waited_out;
			store_hit(a.hits, r, mo);
			fetched += nf;
		}
	}
	if (a.fetches) {
		fetched = warp_sum(fetched);
		if (lane == 0) atomicAdd(a.fetches, fetched);
	}
}

__global__ void __launch_bounds__(kMarchTPB) occlude_kernel(MarchArgs a, uint32_t *__restrict__ occluded) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_stack[SVO_LEVEL_MAX * kMarchTPB];
	uint32_t *stack = s_stack + threadIdx.x;
	const uint32_t lane = lane_id();
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(a.ticket, 32ull);
		base = __shfl_sync(kFullMask, base, 0);
		if (base >= a.n) break;
		const uint64_t r = base + lane;
		if (r < a.n) {
			const float2 *src = reinterpret_cast<const float2 *>(a.rays + r);
			const float2 p0 = src[0], p1 = src[1], p2 = src[2];
			const float o[3] = {p0.x, p0.y, p1.x}, d[3] = {p1.y, p2.x, p2.y};
			bool hit = false;
			if (d[0] != 0.0f || d[1] != 0.0f || d[2] != 0.0f) { // a null ray (a missed bounce) hits nothing
				float t, sz;
				hit = march_traverse<false, kMarchTPB>(a.pool, a.range, a.level, o, d, 0.0f, 0.0f, stack, t, sz, a.status);
			}
			occluded[r] = hit ? 1u : 0u;
		}
	}
}

// ------------------------------------------------------------------------------------ bounce rays
SVO_DEV uint64_t mix64(uint64_t z) {
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

// sin and cos of 2*pi*u (u in [0,1)): quadrant split + Taylor polynomials of degree 13/12 on [0, pi/2),
// each operation rounded separately (this file is built with -fmad=false).
SVO_DEV void sincos_2pi(float u, float &s_out, float &c_out) {
	const float q4 = u * 4.0f;
	const int q = (int)q4;
	const float r = q4 - (float)q;
	const float a = r * 1.57079632679489662f;
	const float a2 = a * a;
	float s = 1.0f / 6227020800.0f;
	s = s * a2 + -1.0f / 39916800.0f;
	s = s * a2 + 1.0f / 362880.0f;
	s = s * a2 + -1.0f / 5040.0f;
	s = s * a2 + 1.0f / 120.0f;
	s = s * a2 + -1.0f / 6.0f;
	s = s * a2 + 1.0f;
	s = s * a;
	float c = 1.0f / 479001600.0f;
	c = c * a2 + -1.0f / 3628800.0f;
	c = c * a2 + 1.0f / 40320.0f;
	c = c * a2 + -1.0f / 720.0f;
	c = c * a2 + 1.0f / 24.0f;
	c = c * a2 + -0.5f;
	c = c * a2 + 1.0f;
	switch (q & 3) {
	case 0: s_out = s, c_out = c; break;
	case 1: s_out = c, c_out = -s; break;
	case 2: s_out = -s, c_out = -c; break;
	default: s_out = -c, c_out = s; break;
	}
}

constexpr float kPi = 3.14159265358979323846f; // PI of shader/util.glsl:4 as a float

// AlignDirection (shader/util.glsl:5-9): dl expressed in the frame (u, v, n) about the unit normal n.
SVO_DEV void align_direction(const float dl[3], const float nrm[3], float d[3]) {
	float ref[3] = {0.0f, 0.0f, 0.0f};
	if (fabsf(nrm[0]) > 0.01f)
		ref[1] = 1.0f;
	else
		ref[0] = 1.0f;
	float u[3] = {ref[1] * nrm[2] - ref[2] * nrm[1], ref[2] * nrm[0] - ref[0] * nrm[2], ref[0] * nrm[1] - ref[1] * nrm[0]};
	const float ul = sqrtf((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]);
#pragma unroll
	for (int k = 0; k < 3; ++k) u[k] = u[k] / ul;
	const float v[3] = {nrm[1] * u[2] - nrm[2] * u[1], nrm[2] * u[0] - nrm[0] * u[2], nrm[0] * u[1] - nrm[1] * u[0]};
#pragma unroll
	for (int k = 0; k < 3; ++k) d[k] = (dl[0] * u[k] + dl[1] * v[k]) + dl[2] * nrm[k];
}

// Diffuse_Sample (shader/diffuse.glsl:7-14): cosine-weighted direction about the unit normal and its pdf.
SVO_DEV void diffuse_sample(const float nrm[3], float u1, float u2, float d[3], float &pdf) {
	const float rr = sqrtf(u1);
	float sn, cs;
	sincos_2pi(u2, sn, cs);
	const float dl[3] = {rr * cs, rr * sn, sqrtf(1.0f - u1)};
	pdf = dl[2] / kPi;
	align_direction(dl, nrm, d);
}

// o = hit pos, d = Diffuse_Sample about the hit normal; misses give d = 0.  (u1, u2) come from a
// counter hash of (seed, i).
SVO_DEV svo_ray bounce_one(const svo_hit &h, uint64_t i, uint64_t seed) {
	float d[3] = {0.0f, 0.0f, 0.0f};
	if (h.flags & SVO_HIT_FLAG_HIT) {
		const uint64_t z = mix64(seed + 0x9E3779B97F4A7C15ull * (i + 1));
		const float u1 = (float)(uint32_t)(z >> 40) * (1.0f / 16777216.0f);
		const float u2 = (float)(uint32_t)((z >> 16) & 0xffffffu) * (1.0f / 16777216.0f);
		const uint32_t ax = SVO_HIT_NORMAL_AXIS(h.flags);
		float nrm[3] = {0.0f, 0.0f, 0.0f};
		nrm[ax] = (h.flags & SVO_HIT_NORMAL_NEG) ? -1.0f : 1.0f;
		float pdf;
		diffuse_sample(nrm, u1, u2, d, pdf);
	}
	svo_ray r;
	r.o[0] = h.pos[0], r.o[1] = h.pos[1], r.o[2] = h.pos[2];
	r.d[0] = d[0], r.d[1] = d[1], r.d[2] = d[2];
	return r;
}

__global__ void bounce_kernel(const svo_hit *__restrict__ hits, uint32_t n, uint64_t seed, svo_ray *__restrict__ rays) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		rays[i] = bounce_one(hits[i], i, seed);
}

// ------------------------------------------------------------------------------------ path tracer
// shader/path_tracer.comp:32-135 per pixel, fused on the device: the camera ray, every bounce's leaf
// march, the environment light's shadow march, MIS weights and the accumulation into the target images,
// one lane per pixel for the whole path.  Transcendentals are this file's own restatements (rounded
// operation by operation like the march), so the oracle reproduces every value bit for bit; the
// reference's GPU evaluates sin/cos/atan/acos with its own approximations.

// atan(z) for 0 <= z <= 1: two half-angle reductions z' = z / (1 + sqrt(1 + z^2)) (atan z = 2 atan z'),
// which leave |z''| <= tan(pi/16), then the Taylor series of atan to the z^15 term.
SVO_DEV float atan_unit(float z) {
	z = z / (1.0f + sqrtf(1.0f + z * z));
	z = z / (1.0f + sqrtf(1.0f + z * z));
	const float z2 = z * z;
	float p = -1.0f / 15.0f;
	p = p * z2 + 1.0f / 13.0f;
	p = p * z2 + -1.0f / 11.0f;
	p = p * z2 + 1.0f / 9.0f;
	p = p * z2 + -1.0f / 7.0f;
	p = p * z2 + 1.0f / 5.0f;
	p = p * z2 + -1.0f / 3.0f;
	p = p * z2 + 1.0f;
	return 4.0f * (z * p);
}

// sin and cos of x radians: sincos_2pi of frac(x / (2 pi)).
SVO_DEV void sincos_rad(float x, float &s, float &c) {
	float u = x * 0.159154943091895336f;
	u = u - floorf(u);
	sincos_2pi(u, s, c);
}

// GLSL atan(y, x) in [-pi, pi] (0 for x = y = 0, which GLSL leaves undefined).
SVO_DEV float atan2_svo(float y, float x) {
	const float ax = fabsf(x), ay = fabsf(y);
	if (ax == 0.0f && ay == 0.0f) return 0.0f;
	float a = ay <= ax ? atan_unit(ay / ax) : 1.57079632679489662f - atan_unit(ax / ay);
	if (x < 0.0f) a = kPi - a;
	return y < 0.0f ? -a : a;
}

// GLSL acos(x) in [0, pi] as atan(sqrt((1 - x)(1 + x)), x); x is clamped to [-1, 1].
SVO_DEV float acos_svo(float x) {
	x = fminf(fmaxf(x, -1.0f), 1.0f);
	return atan2_svo(sqrtf((1.0f - x) * (1.0f + x)), x);
}

// texture(uEnvironmentMap, uv) with VK_FILTER_LINEAR and VK_SAMPLER_ADDRESS_MODE_REPEAT
// (src/EnvironmentMap.cpp:10): the 4 texels around (u W - 1/2, v H - 1/2), integer coordinates wrapped,
// weights (1-a)(1-b), a(1-b), (1-a)b, ab summed in that order.
SVO_DEV float4 env_texture(const EnvMapView &e, float u, float v) {
	const float x = u * (float)e.width - 0.5f, y = v * (float)e.height - 0.5f;
	const float fx = floorf(x), fy = floorf(y);
	const float a = x - fx, b = y - fy;
	const int64_t W = e.width, H = e.height;
	const int64_t i0 = (((int64_t)fx % W) + W) % W, j0 = (((int64_t)fy % H) + H) % H;
	const int64_t i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
	const float4 t00 = __ldg(e.texels + j0 * W + i0), t10 = __ldg(e.texels + j0 * W + i1);
	const float4 t01 = __ldg(e.texels + j1 * W + i0), t11 = __ldg(e.texels + j1 * W + i1);
	const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
	float4 r;
	r.x = ((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x;
	r.y = ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y;
	r.z = ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z;
	r.w = ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w;
	return r;
}

constexpr float kTwoPiPi = 2.0f * kPi * kPi; // 2 * PI * PI of shader/environment_map.glsl:24,45

// EnvMap_Dir2Coord + texture (shader/environment_map.glsl:16-25): the filtered texel in direction d; its w
// over 2 pi^2 sqrt(1 - d.y^2) is EnvMap_PDF.
SVO_DEV float4 env_lookup(const EnvMapView &e, const float d[3], float rot) {
	const float u = (atan2_svo(d[0], d[2]) + rot) / kPi * 0.5f;
	const float v = acos_svo(d[1]) / kPi;
	return env_texture(e, u, v);
}

// EnvMap_Sample (shader/environment_map.glsl:31-48): alias-table pick of a texel, its centre's direction
// (phi = 2 PI u - rot, theta = PI v as the shader forms them), radiance and pdf.
SVO_DEV void env_sample(const EnvMapView &e, float s0, float s1, float rot, float d[3], float light[3], float &pdf) {
	const uint32_t sz = e.width * e.height;
	const uint32_t idx = min((uint32_t)(s0 * (float)sz), sz - 1u);
	const uint32_t prob = (uint32_t)(s1 * 4294967296.0f);
	uint32_t pix = idx;
	const uint2 al = __ldg(e.alias + idx);
	if (prob > al.x) pix = al.y;
	const uint32_t py = pix / e.width, px = pix - py * e.width;
	const float u = ((float)px + 0.5f) / (float)e.width, v = ((float)py + 0.5f) / (float)e.height;
	const float phi = 2.0f * kPi * u - rot, theta = kPi * v;
	float st, ct, sp, cp;
	sincos_rad(theta, st, ct);
	sincos_rad(phi, sp, cp);
	const float4 tx = __ldg(e.texels + pix);
	light[0] = tx.x, light[1] = tx.y, light[2] = tx.z;
	pdf = tx.w / (kTwoPiPi * st);
	d[0] = st * sp, d[1] = ct, d[2] = st * cp;
}

// MIS_PowerHeuristic (shader/mis.glsl:4-7).
SVO_DEV float mis_power(float a, float b) {
	const float t = a * a;
	return t / (b * b + t);
}

// Sobol_GetVec2 component (shader/sobol.glsl:10): the 32-bit value over 2^32.
SVO_DEV float sobol_f(uint32_t v) { return (float)v * 2.3283064365386963e-10f; }

// The 5-argument Octree_RayMarchLeaf the path tracer calls (shader/octree.glsl:342-502): its direction
// clamp keeps |d| >= EPS (applied here; the march's own > EPS clamp then leaves d unchanged) and its
// outputs are hit, o_pos, o_color = rgb * (1/255) (:499) and o_normal.
template <int STRIDE>
SVO_DEV bool pt_leaf(const PtArgs &a, const float o[3], const float dir[3], uint32_t *stack, float pos[3],
                     float albedo[3], float nrm[3]) {
	float d[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) d[k] = fabsf(dir[k]) >= kEps ? dir[k] : (dir[k] >= 0.0f ? kEps : -kEps);
	MarchOut m;
	uint32_t nf;
	march_ray<STRIDE, false>(a.pool, a.range, a.level, o, d, stack, m, nf, a.status);
	const uint32_t flags = m.voxel_hi >> 16;
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		pos[k] = m.pos[k];
		albedo[k] = (float)((m.node >> (8 * k)) & 0xffu) * 0.00392156862745098f;
		nrm[k] = 0.0f;
	}
	nrm[(flags >> 1) & 3u] = (flags & SVO_HIT_NORMAL_NEG) ? -1.0f : 1.0f;
	return (flags & SVO_HIT_FLAG_HIT) != 0u;
}

// Accumulation targets: rgba8 unorm / snorm words as imageStore writes them (round to nearest, ties
// up, after clamping) and imageLoad reads them back.
SVO_DEV float unorm8_load(uint32_t w, int k) { return (float)((w >> (8 * k)) & 0xffu) / 255.0f; }
SVO_DEV uint32_t unorm8_store(float v) { return (uint32_t)floorf(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f + 0.5f); }
SVO_DEV float snorm8_load(uint32_t w, int k) {
	return fmaxf((float)(int32_t)(int8_t)((w >> (8 * k)) & 0xffu) / 127.0f, -1.0f);
}
SVO_DEV uint32_t snorm8_store(float v) {
	return (uint32_t)(int32_t)floorf(fminf(fmaxf(v, -1.0f), 1.0f) * 127.0f + 0.5f) & 0xffu;
}

// Wavefront form of ConstColorPathTrace / EnvMapPathTrace (shader/path_tracer.comp:32-109): one launch
// per path vertex over the paths still alive, so a warp's lanes all march one ray (and, with the
// environment light, one shadow ray) instead of waiting for the warp's longest path.  Each path's
// arithmetic is the shader's loop body in its order, so the images are those of the per-pixel loop.
// Path state lives in HBM between launches; the surviving paths of a vertex are appended to a queue
// (warp-aggregated cursor), counts and tickets are device words, so a sample needs no host round trip.
SVO_DEV uint32_t nrm_code(const float n[3]) {
	const uint32_t ax = n[0] != 0.0f ? 0u : (n[1] != 0.0f ? 1u : 2u);
	return ax | ((n[ax] < 0.0f ? 1u : 0u) << 2);
}
SVO_DEV void nrm_decode(uint32_t c, float n[3]) {
	n[0] = n[1] = n[2] = 0.0f;
	if (c != kPathNoNormal) n[c & 3u] = (c & 4u) ? -1.0f : 1.0f;
}

// Appends the lanes with `alive` set to queue `q` (count `*cnt`), in lane order within the warp.
SVO_DEV void queue_append(bool alive, uint32_t p, uint32_t *q, uint32_t *cnt) {
	const uint32_t lane = lane_id(), m = __ballot_sync(kFullMask, alive);
	if (!m) return;
	uint32_t base = 0;
	if (lane == (uint32_t)(__ffs(m) - 1)) base = atomicAdd(cnt, (uint32_t)__popc(m));
	base = __shfl_sync(kFullMask, base, __ffs(m) - 1);
	if (alive) q[base + __popc(m & ((1u << lane) - 1u))] = p;
}

// Vertex 0: the camera ray of every pixel (main(), shader/path_tracer.comp:115-119) and its first hit.
template <uint32_t LIGHT>
__global__ void __launch_bounds__(kMarchTPB) pt_primary_kernel(PtArgs a) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_stack[SVO_LEVEL_MAX * kMarchTPB];
	uint32_t *stack = s_stack + threadIdx.x;
	const uint32_t lane = lane_id();
	const uint32_t tiles_x = (a.width + 7u) / 8u;
	const uint64_t slots = (uint64_t)tiles_x * ((a.height + 3u) / 4u) * 32u;
	const float s0x = sobol_f(__ldg(a.sobol)), s0y = sobol_f(__ldg(a.sobol + 1));
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(a.tickets, 32ull);
		base = __shfl_sync(kFullMask, base, 0);
		if (base >= slots) break;
		const uint64_t slot = base + lane;
		const uint32_t tile = (uint32_t)(slot >> 5), in = (uint32_t)(slot & 31u);
		const uint32_t x = (tile % tiles_x) * 8u + (in & 7u), y = (tile / tiles_x) * 4u + (in >> 3);
		const bool live = x < a.width && y < a.height;
		bool alive = false;
		const uint32_t p = y * a.width + x;
		if (live) {
			float o[3] = {a.cam.pos[0], a.cam.pos[1], a.cam.pos[2]}, d[3];
			gen_dir(a.cam, ((float)x + s0x) / (float)a.width, ((float)y + s0y) / (float)a.height, d);
			float pos[3], alb[3], nrm[3];
			PathState &S = a.paths[p];
			if (pt_leaf<kMarchTPB>(a, o, d, stack, pos, alb, nrm)) {
#pragma unroll
				for (int k = 0; k < 3; ++k) S.acc[k] = 1.0f * alb[k], S.rad[k] = 0.0f, S.pos[k] = pos[k], S.dalb[k] = alb[k];
				S.nrm = S.first_nrm = nrm_code(nrm);
				alive = a.bounce > 1;
			} else {
				float rad[3];
				if (LIGHT == 1) {
					const float4 env = env_lookup(a.env, d, a.env_rotation);
					rad[0] = env.x, rad[1] = env.y, rad[2] = env.z;
				} else {
					rad[0] = a.const_color[0], rad[1] = a.const_color[1], rad[2] = a.const_color[2];
				}
#pragma unroll
				for (int k = 0; k < 3; ++k) S.rad[k] = rad[k], S.dalb[k] = 0.0f;
				S.first_nrm = kPathNoNormal;
			}
		}
		queue_append(alive, p, a.queue[1], a.counts + 1);
	}
}

// Path vertex `cur` with lanes refilled: a lane takes the next queued path as soon as its work on the
// current one ends (idle lanes claim together once kRefillMin of them are idle, or all are), so a warp
// does not wait for its longest incoherent ray.  A lane's path vertex is up to two marches: the shadow
// ray of the environment light's sample (Octree_RayMarchOcclude is the 5-argument leaf march without
// its outputs, shader/octree.glsl:504-629, so the same stepper serves it), then the bounce ray.  Per
// path the arithmetic is the loop body of ConstColorPathTrace / EnvMapPathTrace
// (shader/path_tracer.comp:41-58, 70-105): light sample with its shadow march, diffuse bounce, leaf march.
template <uint32_t LIGHT>
__global__ void __launch_bounds__(kMarchTPB) pt_bounce_refill_kernel(PtArgs a, uint32_t cur) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_stack[SVO_LEVEL_MAX * kMarchTPB];
	uint32_t *stack = s_stack + threadIdx.x;
	const uint32_t lane = lane_id(), lt_mask = (1u << lane) - 1u;
	const uint32_t n = a.counts[cur];
	const uint32_t *qin = a.queue[cur & 1u];
	uint32_t *qout = a.queue[(cur + 1u) & 1u];
	const float sx = sobol_f(__ldg(a.sobol + 2 * cur)), sy = sobol_f(__ldg(a.sobol + 2 * cur + 1));
	RayState s;
	bool active = false, exhausted = false, shadow = false;
	uint32_t p = 0;
	float acc[3] = {0.0f, 0.0f, 0.0f}, rad[3] = {0.0f, 0.0f, 0.0f}, o[3] = {0.0f, 0.0f, 0.0f}, db[3] = {0.0f, 0.0f, 0.0f};
	float light[3] = {0.0f, 0.0f, 0.0f}, light_pdf = 0.0f, ndd = 0.0f, bsdf_pdf = 0.0f;
	for (;;) {
		const uint32_t idle = __ballot_sync(kFullMask, !active);
		const uint32_t nidle = __popc(idle);
		if (!exhausted && (nidle >= kRefillMin || idle == kFullMask)) {
			const uint32_t leader = __ffs(idle) - 1;
			unsigned long long base = 0;
			if (lane == leader) base = atomicAdd(a.tickets + cur, (unsigned long long)nidle);
			base = __shfl_sync(kFullMask, base, leader);
			if (base + nidle >= n) exhausted = true; // warp-uniform
			const uint64_t slot = base + __popc(idle & lt_mask);
			if (!active && slot < n) {
				p = qin[slot];
				const uint32_t y = p / a.width, x = p - y * a.width;
				const PathState &S = a.paths[p];
				const uint32_t ni = (((y & 255u) << 8) | (x & 255u)) * 2u;
				float samp[2] = {sx + (float)__ldg(a.noise + ni) / 255.0f, sy + (float)__ldg(a.noise + ni + 1) / 255.0f};
				samp[0] = samp[0] - floorf(samp[0]);
				samp[1] = samp[1] - floorf(samp[1]);
				float nrm[3];
#pragma unroll
				for (int k = 0; k < 3; ++k) o[k] = S.pos[k], acc[k] = S.acc[k], rad[k] = S.rad[k];
				nrm_decode(S.nrm, nrm);
				shadow = false;
				float sd[3];
				if (LIGHT == 1) { // multiple importance sampling, light sample
					env_sample(a.env, samp[0], samp[1], a.env_rotation, sd, light, light_pdf);
					ndd = (nrm[0] * sd[0] + nrm[1] * sd[1]) + nrm[2] * sd[2];
					shadow = ndd > 0.0f && !isnan(light_pdf) && light_pdf > 0.0f;
				}
				{ // Diffuse_Sample (shader/diffuse.glsl:7-14) with phi = 2 * PI * samp.y
					const float r = sqrtf(samp[0]), phi = 2.0f * kPi * samp[1];
					float sn, cs;
					sincos_rad(phi, sn, cs);
					const float dl[3] = {r * cs, r * sn, sqrtf(1.0f - samp[0])};
					bsdf_pdf = dl[2] / kPi;
					align_direction(dl, nrm, db);
				}
				const float *d = shadow ? sd : db;
				float dc[3];
#pragma unroll
				for (int k = 0; k < 3; ++k) dc[k] = fabsf(d[k]) >= kEps ? d[k] : (d[k] >= 0.0f ? kEps : -kEps);
				ray_init<kMarchTPB>(s, o, dc, a.level, stack);
				active = true;
			}
		}
		if (!__any_sync(kFullMask, active)) {
			if (exhausted) break;
			continue;
		}
		bool alive = false;
		if (active && ray_step<kMarchTPB, true, false>(s, a.pool, a.range, stack, a.status)) {
			MarchOut m;
			ray_finish(s, a.level, m);
			const uint32_t flags = m.voxel_hi >> 16;
			if (shadow) { // the light sample's contribution unless occluded, then the bounce ray
				if (!(flags & SVO_HIT_FLAG_HIT)) {
					const float bp = ndd / kPi;
					const float w = mis_power(light_pdf, bp);
#pragma unroll
					for (int k = 0; k < 3; ++k)
						rad[k] += acc[k] * light[k] * a.env_multiplier * w * ndd * (1.0f / kPi) / light_pdf;
				}
				shadow = false;
				float dc[3];
#pragma unroll
				for (int k = 0; k < 3; ++k) dc[k] = fabsf(db[k]) >= kEps ? db[k] : (db[k] >= 0.0f ? kEps : -kEps);
				ray_init<kMarchTPB>(s, o, dc, a.level, stack);
			} else {
				PathState &S = a.paths[p];
				if (flags & SVO_HIT_FLAG_HIT) {
					float nrm[3] = {0.0f, 0.0f, 0.0f};
					nrm[(flags >> 1) & 3u] = (flags & SVO_HIT_NORMAL_NEG) ? -1.0f : 1.0f;
#pragma unroll
					for (int k = 0; k < 3; ++k) {
						S.acc[k] = acc[k] * ((float)((m.node >> (8 * k)) & 0xffu) * 0.00392156862745098f);
						S.pos[k] = m.pos[k];
					}
					S.nrm = nrm_code(nrm);
					alive = cur + 1u < a.bounce;
				} else if (LIGHT == 1) { // multiple importance sampling, bsdf sample
					const float4 env = env_lookup(a.env, db, a.env_rotation);
					const float lp = env.w / (kTwoPiPi * sqrtf(1.0f - db[1] * db[1]));
					if (!isnan(lp) && lp > 0.0f) {
						const float w = mis_power(bsdf_pdf, lp);
						const float e3[3] = {env.x, env.y, env.z};
#pragma unroll
						for (int k = 0; k < 3; ++k) rad[k] += acc[k] * e3[k] * a.env_multiplier * w;
					}
				} else {
#pragma unroll
					for (int k = 0; k < 3; ++k) rad[k] = acc[k] * a.const_color[k];
				}
#pragma unroll
				for (int k = 0; k < 3; ++k) S.rad[k] = rad[k];
				active = false;
			}
		}
		queue_append(alive, p, qout, a.counts + cur + 1);
	}
}

// main()'s running means (shader/path_tracer.comp:121-134) of every pixel's sample.
__global__ void pt_accumulate_kernel(PtArgs a) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	const uint32_t spp = __ldg(a.sobol + 2u * (a.bounce + 1u)); // Sobol_Current((uBounce + 1) << 1)
	const float fs = (float)spp, fn = (float)(spp + 1u);
	const size_t npx = (size_t)a.width * a.height;
	for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += (size_t)gridDim.x * blockDim.x) {
		const PathState &S = a.paths[p];
		float dnrm[3];
		nrm_decode(S.first_nrm, dnrm);
		const float4 c = a.color[p];
		a.color[p] = make_float4((c.x * fs + S.rad[0]) / fn, (c.y * fs + S.rad[1]) / fn, (c.z * fs + S.rad[2]) / fn, 1.0f);
		const uint32_t wa = a.albedo[p], wn = a.normal[p];
		uint32_t oa = 255u << 24, on = 127u << 24;
#pragma unroll
		for (int k = 0; k < 3; ++k) {
			oa |= unorm8_store((unorm8_load(wa, k) * fs + S.dalb[k]) / fn) << (8 * k);
			on |= snorm8_store((snorm8_load(wn, k) * fs + dnrm[k]) / fn) << (8 * k);
		}
		a.albedo[p] = oa;
		a.normal[p] = on;
	}
}

// Sobol::CmdNext (shader/sobol.comp:70-86): c = index of the lowest zero bit of the sample index, which
// then increments; every dimension's value takes the XOR of its direction number c.
__global__ void sobol_next_kernel(uint32_t *sobol, const uint32_t *__restrict__ matrices, uint32_t dim) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t c;
	if (threadIdx.x == 0) {
		const uint32_t i = sobol[dim];
		c = (uint32_t)__ffs(~i) - 1u; // 0xffffffff when every bit is set: no step
		sobol[dim] = i + 1u;
	}
	__syncthreads();
	if (threadIdx.x < dim && c < 32u) sobol[threadIdx.x] ^= matrices[threadIdx.x * 32u + c];
}

// ------------------------------------------------------------------------------------ shared launches
// Many requests in one launch (the serving loop): work slots are numbered job after job, every job's
// slot count a multiple of 32, so the 32 slots of a warp ticket belong to one job.  Per ray the work is
// exactly the single-request kernel's, so a request's hits do not depend on what it shares a launch with.
SVO_DEV uint32_t job_of(const MarchJob *__restrict__ jobs, uint32_t njobs, uint64_t slot) {
	uint32_t lo = 0, hi = njobs; // jobs[lo].slot_begin <= slot < jobs[hi].slot_begin
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (jobs[mid].slot_begin <= slot)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

template <bool COUNT>
__global__ void __launch_bounds__(kMarchTPB) march_jobs_kernel(const MarchJob *__restrict__ jobs, uint32_t njobs,
                                                                uint64_t total, unsigned long long *ticket,
                                                                uint32_t *status, unsigned long long *fetches) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_stack[SVO_LEVEL_MAX * kMarchTPB];
	uint32_t *stack = s_stack + threadIdx.x;
	const uint32_t lane = lane_id();
	unsigned long long fetched = 0;
	for (;;) {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(ticket, 32ull);
		base = __shfl_sync(kFullMask, base, 0);
		if (base >= total) break;
		const MarchJob &J = jobs[job_of(jobs, njobs, base)]; // warp-uniform (jobs are whole tickets)
		const uint64_t local = base + lane - J.slot_begin;
		float o[3], d[3];
		uint32_t r = 0;
		bool live;
		if (J.rays == nullptr) {
			const uint32_t tiles_x = (J.width + 7u) / 8u;
			const uint32_t tile = (uint32_t)(local >> 5), in = (uint32_t)(local & 31u);
			const uint32_t x = (tile % tiles_x) * 8u + (in & 7u), y = (tile / tiles_x) * 4u + (in >> 3);
			r = y * J.width + x;
			live = x < J.width && r < J.n;
			if (live) camera_ray(J.cam, J.width, J.height, r, o, d);
		} else {
			r = (uint32_t)local;
			live = local < J.n;
			if (live) {
				const float2 *src = reinterpret_cast<const float2 *>(J.rays + r);
				const float2 p0 = src[0], p1 = src[1], p2 = src[2];
				o[0] = p0.x, o[1] = p0.y, o[2] = p1.x, d[0] = p1.y, d[1] = p2.x, d[2] = p2.y;
			}
		}
		if (live) {
			MarchOut m;
			uint32_t nf = 0;
			march_ray<kMarchTPB, COUNT>(J.pool, J.range, J.level, o, d, stack, m, nf, status + J.req);
			store_hit(J.hits, r, m);
			fetched += nf;
		}
	}
	if (COUNT && fetches) {
		fetched = warp_sum(fetched);
		if (lane == 0 && fetched) atomicAdd(fetches, fetched);
	}
}

__global__ void bounce_jobs_kernel(const BounceJob *__restrict__ jobs, uint32_t njobs, uint64_t total) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
		uint32_t lo = 0, hi = njobs;
		while (hi - lo > 1) {
			const uint32_t mid = (lo + hi) >> 1;
			if (jobs[mid].begin <= i)
				lo = mid;
			else
				hi = mid;
		}
		const BounceJob &J = jobs[lo];
		const uint64_t local = i - J.begin;
		J.rays[local] = bounce_one(J.hits[local], local, J.seed);
	}
}

// ---------------------------------------------------------------------------------------------------
template <bool CAMERA, int TPB, int RPL, bool SHARED, bool COUNT = false>
static void launch_variant(const MarchArgs &a, cudaStream_t stream) {
	const int sms = device_sm_count();
	const uint64_t warps_needed = ((uint64_t)a.n + 32 * RPL - 1) / (32 * RPL);
	const uint64_t blocks_needed = (warps_needed + TPB / 32 - 1) / (TPB / 32);
	const uint64_t cap = (uint64_t)sms * (2048 / TPB); // persistent: a full SM's worth of threads
	const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, cap));
	SVO_LAUNCH(CAMERA ? "march_camera" : "march_rays", stream,
	           ::svo::launch_k(march_kernel<CAMERA, TPB, RPL, SHARED, COUNT>, blocks, TPB, 0, stream, a););
}

template <bool CAMERA, int TPB, bool SHARED> static void launch_refill(const MarchArgs &a, cudaStream_t stream) {
	const int sms = device_sm_count();
	const uint64_t blocks_needed = ((uint64_t)a.n + TPB - 1) / TPB;
	const uint64_t cap = (uint64_t)sms * (2048 / TPB);
	const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, cap));
	SVO_LAUNCH(CAMERA ? "march_camera" : "march_rays", stream,
	           ::svo::launch_k(march_refill_kernel<CAMERA, TPB, SHARED, false>, blocks, TPB, 0, stream, a););
}

template <bool CAMERA, int TPB>
static void launch_rpl(const MarchArgs &a, int rpl, bool shared, cudaStream_t stream) {
	if (rpl == 0) {
		if (shared) launch_refill<CAMERA, TPB, true>(a, stream);
		else launch_refill<CAMERA, TPB, false>(a, stream);
	} else if (rpl == 2) {
		if (shared) launch_variant<CAMERA, TPB, 2, true>(a, stream);
		else launch_variant<CAMERA, TPB, 2, false>(a, stream);
	} else {
		if (shared) launch_variant<CAMERA, TPB, 1, true>(a, stream);
		else launch_variant<CAMERA, TPB, 1, false>(a, stream);
	}
}

template <bool CAMERA> static void launch_tuned(const MarchArgs &a, cudaStream_t stream) {
	if (a.fetches) { // a launch that counts node fetches: the default variant with the counter
		launch_variant<CAMERA, 128, 1, true, true>(a, stream);
		return;
	}
	const int tpb = tune_value(kTuneMarchBlock, a.level, a.n);
	// camera rays and ray buffers (bounce rays, usually incoherent) have their own rays-per-lane choice
	const int rpl = tune_value(CAMERA ? kTuneMarchRays : kTuneMarchBufferRays, a.level, a.n);
	const bool shared = tune_value(kTuneMarchShared, a.level, a.n) != 0;
	if (tpb == 64) launch_rpl<CAMERA, 64>(a, rpl, shared, stream);
	else if (tpb == 256) launch_rpl<CAMERA, 256>(a, rpl, shared, stream);
	else launch_rpl<CAMERA, 128>(a, rpl, shared, stream);
}

cudaError_t march_launch(const MarchArgs &a, bool camera, cudaStream_t stream) {
	cudaError_t e = cudaMemsetAsync(a.ticket, 0, sizeof(unsigned long long), stream);
	if (e != cudaSuccess || a.n == 0) return e;
	if (camera)
		launch_tuned<true>(a, stream);
	else
		launch_tuned<false>(a, stream);
	return cudaGetLastError();
}

cudaError_t bounce_launch(const svo_hit *hits, uint32_t n, uint64_t seed, svo_ray *rays, cudaStream_t stream) {
	if (n == 0) return cudaSuccess;
	const int sms = device_sm_count();
	const uint32_t blocks = (uint32_t)std::min<uint64_t>(((uint64_t)n + 255) / 256, (uint64_t)sms * 8);
	SVO_LAUNCH("bounce_kernel", stream, ::svo::launch_k(bounce_kernel, blocks, 256, 0, stream, hits, n, seed, rays););
	return cudaGetLastError();
}

} // namespace svo

namespace svo {

uint64_t march_job_slots(const MarchJob &j) {
	if (j.n == 0) return 0;
	if (j.rays) return (j.n + 31ull) / 32ull * 32ull;
	const uint64_t rows = (j.n + (uint64_t)j.width - 1) / j.width; // rows holding the first n pixels
	return (uint64_t)((j.width + 7u) / 8u) * ((rows + 3) / 4) * 32ull;
}

cudaError_t march_jobs_launch(const MarchJob *jobs, uint32_t njobs, uint64_t total, unsigned long long *ticket,
                              uint32_t *status, unsigned long long *fetches, cudaStream_t stream) {
	cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned long long), stream);
	if (e != cudaSuccess || total == 0 || njobs == 0) return e;
	const int sms = device_sm_count();
	const uint64_t blocks_needed = (total / 32 + kMarchTPB / 32 - 1) / (kMarchTPB / 32);
	const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, (uint64_t)sms * 16));
	if (fetches)
		SVO_LAUNCH("march_jobs", stream,
		           ::svo::launch_k(march_jobs_kernel<true>, blocks, kMarchTPB, 0, stream, jobs, njobs, total, ticket, status, fetches););
	else
		SVO_LAUNCH("march_jobs", stream,
		           ::svo::launch_k(march_jobs_kernel<false>, blocks, kMarchTPB, 0, stream, jobs, njobs, total, ticket, status, nullptr););
	return cudaGetLastError();
}

cudaError_t bounce_jobs_launch(const BounceJob *jobs, uint32_t njobs, uint64_t total, cudaStream_t stream) {
	if (total == 0 || njobs == 0) return cudaSuccess;
	const int sms = device_sm_count();
	const uint32_t blocks = (uint32_t)std::min<uint64_t>((total + 255) / 256, (uint64_t)sms * 8);
	SVO_LAUNCH("bounce_jobs", stream, ::svo::launch_k(bounce_jobs_kernel, blocks, 256, 0, stream, jobs, njobs, total););
	return cudaGetLastError();
}

} // namespace svo

namespace svo {

cudaError_t beam_launch(const MarchArgs &a, float *beam, cudaStream_t stream) {
	const uint64_t texels = (uint64_t)((a.width + kBeamSize - 1) / kBeamSize + 1) * ((a.height + kBeamSize - 1) / kBeamSize + 1);
	const int sms = device_sm_count();
	const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((texels + kMarchTPB - 1) / kMarchTPB,
	                                                                            (uint64_t)sms * 16));
	const float orig_sz = ldexpf(1.0f, 1 - (int)a.level); // exp2f(1 - level), src/OctreeTracer.cpp:205
	SVO_LAUNCH("beam_prepass", stream, ::svo::launch_k(beam_kernel, blocks, kMarchTPB, 0, stream, a, beam, orig_sz););
	return cudaGetLastError();
}

cudaError_t march_set_wait_fault(uint32_t limit, uint32_t withheld) { return set_wait_fault_here(limit, withheld); }

cudaError_t march_beam_fused_launch(const MarchArgs &a, float *beam, cudaStream_t stream) {
	const uint64_t texels = (uint64_t)((a.width + kBeamSize - 1) / kBeamSize + 1) * ((a.height + kBeamSize - 1) / kBeamSize + 1);
	cudaError_t e = cudaMemsetAsync(a.ticket, 0, sizeof(unsigned long long), stream);
	if (e == cudaSuccess) e = cudaMemsetAsync(beam, 0xff, texels * sizeof(float), stream); // kBeamUnset
	if (e != cudaSuccess || a.width == 0 || a.height == 0) return e;
	const int sms = device_sm_count();
	const uint64_t slots = (texels + 31) / 32 * 32 + (uint64_t)((a.width + 7u) / 8u) * ((a.height + 3u) / 4u) * 32u;
	const uint64_t blocks_needed = (slots / 32 + kMarchTPB / 32 - 1) / (kMarchTPB / 32);
	const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, (uint64_t)sms * 16));
	const float orig_sz = ldexpf(1.0f, 1 - (int)a.level);
	if (a.fetches)
		SVO_LAUNCH("march_beam", stream, ::svo::launch_k(march_beam_fused_kernel<true>, blocks, kMarchTPB, 0, stream, a, beam, orig_sz););
	else
		SVO_LAUNCH("march_beam", stream, ::svo::launch_k(march_beam_fused_kernel<false>, blocks, kMarchTPB, 0, stream, a, beam, orig_sz););
	return cudaGetLastError();
}

cudaError_t occlude_launch(const MarchArgs &a, uint32_t *occluded, cudaStream_t stream) {
	cudaError_t e = cudaMemsetAsync(a.ticket, 0, sizeof(unsigned long long), stream);
	if (e != cudaSuccess || a.n == 0) return e;
	const int sms = device_sm_count();
	const uint64_t blocks_needed = ((uint64_t)a.n / 32 + kMarchTPB / 32) / (kMarchTPB / 32);
	const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, (uint64_t)sms * 16));
	SVO_LAUNCH("occlude", stream, ::svo::launch_k(occlude_kernel, blocks, kMarchTPB, 0, stream, a, occluded););
	return cudaGetLastError();
}

cudaError_t pt_render_launch(const PtArgs &a, cudaStream_t stream) {
	// tickets and queue counts of every vertex start at zero
	cudaError_t e = cudaMemsetAsync(a.tickets, 0, kPtScratchBytes, stream);
	if (e != cudaSuccess || a.width == 0 || a.height == 0) return e;
	const int sms = device_sm_count();
	const uint64_t slots = (uint64_t)((a.width + 7u) / 8u) * ((a.height + 3u) / 4u) * 32u;
	const uint64_t blocks_needed = (slots / 32 + kMarchTPB / 32 - 1) / (kMarchTPB / 32);
	const uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(blocks_needed, (uint64_t)sms * 16));
	if (a.light_type == 1) {
		SVO_LAUNCH("pt_primary", stream, ::svo::launch_k(pt_primary_kernel<1>, blocks, kMarchTPB, 0, stream, a););
		for (uint32_t cur = 1; cur < a.bounce; ++cur)
			SVO_LAUNCH("pt_bounce", stream, ::svo::launch_k(pt_bounce_refill_kernel<1>, blocks, kMarchTPB, 0, stream, a, cur););
	} else {
		SVO_LAUNCH("pt_primary", stream, ::svo::launch_k(pt_primary_kernel<0>, blocks, kMarchTPB, 0, stream, a););
		for (uint32_t cur = 1; cur < a.bounce; ++cur)
			SVO_LAUNCH("pt_bounce", stream, ::svo::launch_k(pt_bounce_refill_kernel<0>, blocks, kMarchTPB, 0, stream, a, cur););
	}
	const uint64_t npx = (uint64_t)a.width * a.height;
	const uint32_t ablocks = (uint32_t)std::min<uint64_t>((npx + 255) / 256, (uint64_t)sms * 8);
	SVO_LAUNCH("pt_accumulate", stream, ::svo::launch_k(pt_accumulate_kernel, ablocks, 256, 0, stream, a););
	return cudaGetLastError();
}

cudaError_t sobol_next_launch(uint32_t *sobol, const uint32_t *matrices, uint32_t dim, cudaStream_t stream) {
	SVO_LAUNCH("sobol_next", stream, ::svo::launch_k(sobol_next_kernel, 1, 64, 0, stream, sobol, matrices, dim););
	return cudaGetLastError();
}

} // namespace svo
