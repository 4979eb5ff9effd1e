// build.cu — fragments -> octree node pool (replaces OctreeBuilder::CmdBuild, src/OctreeBuilder.cpp:142-210,
// and the shaders shader/octree_{init,tag,alloc}_node.comp, shader/octree_modify_arg.comp).
//
// Same level-by-level structure and node-word format as the reference:
//   depth i = 1..L:  tag   every fragment marks its depth-i node 0x80000000, or at depth L merges its
//                          colour into the leaf (shader/octree_tag_node.comp:33-60);
//                    alloc every marked word of depth i gets a child block: word = ((b+1)<<3)|0x80000000
//                          (shader/octree_alloc_node.comp:21), and the block's 8 words are zeroed (the
//                          next level's init, shader/octree_init_node.comp:7-11);
//                    the level range advances as shader/octree_modify_arg.comp:9-13 does.
// GB300 design:
//   * each fragment's depth-(i-1) node index is cached (4 B per fragment), so tag reads one parent word
//     instead of re-walking i levels from the root (O(F*L) node reads instead of O(F*L^2));
//   * fragments are swept 4 per thread with 16-byte loads; an interior tag is stored only when the word
//     is not marked yet, so upper levels (millions of fragments on 8 words) cost loads, not stores;
//   * block numbers come from a single-pass decoupled look-back prefix sum over the level's words, so
//     child blocks are in breadth-first word order (canonical, reproducible) instead of atomic order;
//   * leaf colour is the channel-wise integer mean: per leaf two 64-bit accumulators (r | g<<32 and
//     b | n<<32) are added atomically and a finalize pass writes floor(sum/n) and min(n,63);
//   * level sizes stay on the device (BuildState); every kernel has a fixed grid, so the whole build is
//     stream-ordered with no host round trip until the final 1 KB readback (and can be graph-captured).
#include "common.cuh"
#include "svo_internal.h"

namespace svo {

constexpr int kTagTPB = 256;
constexpr int kAllocTPB = 256;
constexpr int kAllocIPT = 8;
constexpr int kAllocTile = kAllocTPB * kAllocIPT;

SVO_DEV uint32_t octant(uint64_t frag, uint32_t shift) {
	const uint32_t fx = (uint32_t)frag, fy = (uint32_t)(frag >> 32);
	const uint32_t x = fx & 0xfffu, y = (fx >> 12) & 0xfffu, z = (fx >> 24) | ((fy >> 28) << 8);
	return ((x >> shift) & 1u) | (((y >> shift) & 1u) << 1) | (((z >> shift) & 1u) << 2);
}

__global__ void build_init(BuildState *state, uint32_t *pool, unsigned long long *sums, uint32_t level) {
	const uint32_t t = threadIdx.x;
	uint32_t *s = reinterpret_cast<uint32_t *>(state);
	for (uint32_t k = t; k < sizeof(BuildState) / 4; k += blockDim.x) s[k] = 0u;
	if (t < 8) pool[t] = 0u;
	if (level == 1 && t < 16) sums[t] = 0ull;
	__syncthreads();
	if (t == 0) {
		state->lv[1].begin = 0;
		state->lv[1].num = 8;
		state->lv[1].blocks_before = 0;
	}
}

template <bool LEAF>
SVO_DEV void tag_one(uint64_t frag, uint32_t &node, uint32_t shift, uint32_t depth, uint32_t *__restrict__ pool,
                     unsigned long long *__restrict__ sums, uint32_t leaf_begin, uint32_t leaf_num) {
	const uint32_t oct = octant(frag, shift);
	const uint32_t idx = depth == 1 ? oct : (pool[node] & 0x3fffffffu) + oct;
	if (LEAF) {
		const uint32_t slot = idx - leaf_begin;
		if (slot < leaf_num) {
			const uint32_t rgb = (uint32_t)(frag >> 32);
			atomicAdd(&sums[2 * (size_t)slot], (unsigned long long)(rgb & 0xffu) | ((unsigned long long)((rgb >> 8) & 0xffu) << 32));
			atomicAdd(&sums[2 * (size_t)slot + 1], (unsigned long long)((rgb >> 16) & 0xffu) | (1ull << 32));
		}
	} else {
		if ((pool[idx] & 0x80000000u) == 0u) pool[idx] = 0x80000000u;
		node = idx;
	}
}

template <bool LEAF>
__global__ void __launch_bounds__(kTagTPB) build_tag(const uint64_t *__restrict__ frags, uint32_t n, uint32_t level,
                                                     uint32_t depth, uint32_t *__restrict__ pool,
                                                     uint32_t *__restrict__ cache, unsigned long long *__restrict__ sums,
                                                     const BuildState *__restrict__ state, int vec_ok) {
	if (state->status & kStatusCapacity) return;
	const uint32_t shift = level - depth;
	const uint32_t leaf_begin = LEAF ? state->lv[depth].begin : 0u, leaf_num = LEAF ? state->lv[depth].num : 0u;
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t nq = (n + 3u) / 4u;
	for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
		const uint64_t f0 = q * 4;
		if (vec_ok && f0 + 4 <= n) {
			const ulonglong2 a = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0));
			const ulonglong2 b = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0 + 2));
			uint4 c = make_uint4(0, 0, 0, 0);
			if (depth > 1) c = __ldcs(reinterpret_cast<const uint4 *>(cache + f0));
			tag_one<LEAF>(a.x, c.x, shift, depth, pool, sums, leaf_begin, leaf_num);
			tag_one<LEAF>(a.y, c.y, shift, depth, pool, sums, leaf_begin, leaf_num);
			tag_one<LEAF>(b.x, c.z, shift, depth, pool, sums, leaf_begin, leaf_num);
			tag_one<LEAF>(b.y, c.w, shift, depth, pool, sums, leaf_begin, leaf_num);
			if (!LEAF) __stcs(reinterpret_cast<uint4 *>(cache + f0), c);
		} else {
			for (uint64_t f = f0; f < f0 + 4 && f < n; ++f) {
				uint32_t c = depth > 1 ? cache[f] : 0u;
				tag_one<LEAF>(frags[f], c, shift, depth, pool, sums, leaf_begin, leaf_num);
				if (!LEAF) cache[f] = c;
			}
		}
	}
}

// Prefix-sum allocation of child blocks for the marked words of depth `depth` (persistent grid, tiles
// claimed in order by a ticket so the look-back always waits on a running or finished tile).
__global__ void __launch_bounds__(kAllocTPB) build_alloc(uint32_t *__restrict__ pool, uint64_t capacity,
                                                         uint32_t depth, uint32_t level,
                                                         unsigned long long *__restrict__ sums, BuildState *state,
                                                         unsigned long long *descs) {
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kAllocTPB / 32 + 1];
	__shared__ uint32_t s_prefix;
	__shared__ uint32_t s_abort;
	// other blocks of this launch may set the capacity flag: decide once per block
	if (threadIdx.x == 0) s_abort = atomicOr(&state->status, 0u) & kStatusCapacity;
	__syncthreads();
	if (s_abort) return;
	const LevelInfo li = state->lv[depth];
	const uint32_t ntiles = (li.num + kAllocTile - 1) / kAllocTile;
	const bool next_is_leaf = depth + 1 == level;
	const uint32_t next_begin = li.begin + li.num;
	if (ntiles == 0) {
		if (blockIdx.x == 0 && threadIdx.x == 0) {
			state->lv[depth].nodes = 0;
			state->lv[depth + 1] = LevelInfo{next_begin, 0u, li.blocks_before, 0u};
		}
		return;
	}
	for (;;) {
		if (threadIdx.x == 0) s_tile = atomicAdd(&state->tiles[depth], 1u);
		__syncthreads();
		const uint32_t tile = s_tile;
		__syncthreads();
		if (tile >= ntiles) break;
		const uint32_t w0 = tile * kAllocTile + threadIdx.x * kAllocIPT; // offset inside the level
		uint32_t w[kAllocIPT];
		if (w0 + kAllocIPT <= li.num) {
			const uint4 *src = reinterpret_cast<const uint4 *>(pool + li.begin + w0);
			const uint4 x = src[0], y = src[1];
			w[0] = x.x, w[1] = x.y, w[2] = x.z, w[3] = x.w, w[4] = y.x, w[5] = y.y, w[6] = y.z, w[7] = y.w;
		} else {
#pragma unroll
			for (int k = 0; k < kAllocIPT; ++k) w[k] = w0 + k < li.num ? pool[li.begin + w0 + k] : 0u;
		}
		uint32_t cnt = 0;
#pragma unroll
		for (int k = 0; k < kAllocIPT; ++k) cnt += (w[k] >> 31);
		uint32_t total;
		const uint32_t rank0 = block_exclusive_sum<uint32_t, kAllocTPB>(cnt, s_warp, total);
		if (threadIdx.x == 0) s_prefix = (uint32_t)tile_lookback(descs, tile, depth, total, &state->status);
		__syncthreads();
		const uint32_t prefix = s_prefix;
		uint32_t rank = rank0;
#pragma unroll
		for (int k = 0; k < kAllocIPT; ++k) {
			if (!(w[k] >> 31)) continue;
			const uint64_t b = (uint64_t)li.blocks_before + prefix + rank++; // 0-based child block number
			const uint64_t ptr = (b + 1) * 8;
			if (ptr + 8 > capacity || ptr + 8 > SVO_MAX_POOL_WORDS) {
				atomicOr(&state->status, kStatusCapacity);
				w[k] = 0x80000000u; // leave unallocated; the build reports SVO_ERR_CAPACITY
				continue;
			}
			w[k] = (uint32_t)ptr | 0x80000000u;
			uint4 *child = reinterpret_cast<uint4 *>(pool + ptr);
			child[0] = make_uint4(0, 0, 0, 0);
			child[1] = make_uint4(0, 0, 0, 0);
			if (next_is_leaf) {
				ulonglong2 *acc = reinterpret_cast<ulonglong2 *>(sums + 2 * (ptr - next_begin));
#pragma unroll
				for (int j = 0; j < 8; ++j) acc[j] = make_ulonglong2(0ull, 0ull);
			}
		}
		if (w0 + kAllocIPT <= li.num) {
			uint4 *dst = reinterpret_cast<uint4 *>(pool + li.begin + w0);
			dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
			dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
		} else {
#pragma unroll
			for (int k = 0; k < kAllocIPT; ++k)
				if (w0 + k < li.num) pool[li.begin + w0 + k] = w[k];
		}
		if (tile == ntiles - 1 && threadIdx.x == 0) {
			const uint32_t nodes = prefix + total;
			state->lv[depth].nodes = nodes;
			state->lv[depth + 1] = LevelInfo{next_begin, nodes * 8u, li.blocks_before + nodes, 0u};
		}
	}
}

__global__ void __launch_bounds__(256) build_finalize(uint32_t *__restrict__ pool,
                                                      const unsigned long long *__restrict__ sums, BuildState *state,
                                                      uint32_t level) {
	__shared__ uint32_t s_warp[256 / 32];
	__shared__ uint32_t s_abort;
	if (threadIdx.x == 0) s_abort = state->status & kStatusCapacity;
	__syncthreads();
	if (s_abort) return;
	const LevelInfo li = state->lv[level];
	uint32_t leaves = 0;
	for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < li.num; k += gridDim.x * blockDim.x) {
		const ulonglong2 a = reinterpret_cast<const ulonglong2 *>(sums)[k];
		const uint32_t n = (uint32_t)(a.y >> 32);
		if (n == 0) continue;
		const uint32_t r = (uint32_t)(a.x & 0xffffffffull) / n, g = (uint32_t)(a.x >> 32) / n;
		const uint32_t b = (uint32_t)(a.y & 0xffffffffull) / n;
		pool[li.begin + k] = 0xC0000000u | (min(n, 63u) << 24) | (b << 16) | (g << 8) | r;
		++leaves;
	}
	leaves = warp_sum(leaves);
	if (lane_id() == 0) s_warp[threadIdx.x >> 5] = leaves;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t t = 0;
		for (int i = 0; i < 256 / 32; ++i) t += s_warp[i];
		atomicAdd(&state->leaves, t);
		if (blockIdx.x == 0) state->range_words = li.begin + li.num;
	}
}

// ---------------------------------------------------------------------------------------------------
uint64_t build_pool_bound(uint32_t count, uint32_t level) {
	uint64_t words = 8, per = 1;
	for (uint32_t i = 1; i < level; ++i) {
		per = per >= (1ull << 40) ? per : per * 8; // 8^i (saturating)
		words += 8 * (per < count ? per : (uint64_t)count);
	}
	return words < SVO_MAX_POOL_WORDS ? words : SVO_MAX_POOL_WORDS;
}

// Largest word range of one depth: 8 * min(8^(i-1), count) over depths 1..level.
static uint64_t max_level_words(uint32_t count, uint32_t level) {
	uint64_t best = 8, per = 1;
	for (uint32_t i = 1; i <= level; ++i) {
		const uint64_t w = 8 * (per < count ? per : (uint64_t)count);
		best = w > best ? w : best;
		per = per >= (1ull << 40) ? per : per * 8;
	}
	return best < SVO_MAX_POOL_WORDS ? best : SVO_MAX_POOL_WORDS;
}

size_t build_workspace_bytes(uint32_t count, uint32_t level, uint64_t capacity) {
	BuildWorkspace w;
	build_workspace_layout(nullptr, count, level, capacity, w);
	return w.total_bytes;
}

// Layout: state | descriptors | per-fragment node cache | leaf accumulators (16 B per leaf word).
void build_workspace_layout(void *ws, uint32_t count, uint32_t level, uint64_t capacity, BuildWorkspace &w) {
	char *p = (char *)ws;
	size_t off = 0;
	w.state = (BuildState *)(p + off);
	off += align_up(sizeof(BuildState), 256);
	uint64_t lw = max_level_words(count, level);
	if (lw > capacity) lw = capacity;
	w.desc_count = (size_t)((lw + kAllocTile - 1) / kAllocTile + 1);
	w.descs = (unsigned long long *)(p + off);
	off += align_up(w.desc_count * sizeof(unsigned long long), 256);
	w.cache = (uint32_t *)(p + off);
	off += align_up((size_t)count * sizeof(uint32_t) + 16, 256);
	w.sums = (unsigned long long *)(p + off);
	w.sum_slots = (size_t)lw;
	off += align_up((size_t)lw * 16 + 16, 256);
	w.total_bytes = off;
}

cudaError_t build_launch(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool, uint64_t capacity,
                         const BuildWorkspace &w, cudaStream_t stream) {
	cudaError_t e = cudaMemsetAsync(w.descs, 0, w.desc_count * sizeof(unsigned long long), stream);
	if (e != cudaSuccess) return e;
	build_init<<<1, 256, 0, stream>>>(w.state, pool, w.sums, level);
	note_launch();
	const int sms = device_sm_count();
	const int vec_ok = ((uintptr_t)frags & 15u) == 0;
	const uint64_t nq = ((uint64_t)count + 3) / 4;
	const uint32_t tag_blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((nq + kTagTPB - 1) / kTagTPB,
	                                                                                   (uint64_t)sms * 16));
	const uint32_t alloc_blocks = (uint32_t)sms * 4;
	for (uint32_t depth = 1; depth <= level; ++depth) {
		if (depth < level) {
			build_tag<false><<<tag_blocks, kTagTPB, 0, stream>>>(frags, count, level, depth, pool, w.cache, w.sums,
			                                                     w.state, vec_ok);
			note_launch();
			build_alloc<<<alloc_blocks, kAllocTPB, 0, stream>>>(pool, capacity, depth, level, w.sums, w.state, w.descs);
			note_launch();
		} else {
			build_tag<true><<<tag_blocks, kTagTPB, 0, stream>>>(frags, count, level, depth, pool, w.cache, w.sums,
			                                                    w.state, vec_ok);
			note_launch();
		}
	}
	build_finalize<<<(uint32_t)sms * 4, 256, 0, stream>>>(pool, w.sums, w.state, level);
	note_launch();
	return cudaGetLastError();
}

} // namespace svo

namespace svo {

// Writes svo_build_info followed by the status word to `out` (device) from the build state.
__global__ void build_export(const BuildState *state, uint32_t level, uint32_t count, uint32_t *out) {
	if (threadIdx.x != 0) return;
	svo_build_info *info = reinterpret_cast<svo_build_info *>(out);
	info->level = level;
	info->fragments = count;
	info->range_words = state->range_words;
	info->leaves = state->leaves;
	for (uint32_t d = 1; d <= SVO_LEVEL_MAX; ++d)
		info->level_nodes[d - 1] = d < level ? state->lv[d].nodes : (d == level ? state->leaves : 0u);
	out[sizeof(svo_build_info) / 4] = state->status;
}

cudaError_t build_launch_export(const BuildWorkspace &w, uint32_t level, uint32_t count, void *out,
                                cudaStream_t stream) {
	build_export<<<1, 32, 0, stream>>>(w.state, level, count, (uint32_t *)out);
	note_launch();
	return cudaGetLastError();
}

} // namespace svo
