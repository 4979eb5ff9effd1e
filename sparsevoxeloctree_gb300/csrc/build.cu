// build.cu — fragments -> octree node pool (replaces OctreeBuilder::CmdBuild, src/OctreeBuilder.cpp:142-210,
// and the shaders shader/octree_{init,tag,alloc}_node.comp, shader/octree_modify_arg.comp).
//
// The reference builds level by level: at depth i every fragment tags its node (0x80000000, or the leaf
// colour at depth L, shader/octree_tag_node.comp:33-60), then every tagged word gets a child block
// ((b+1)<<3 | 0x80000000, shader/octree_alloc_node.comp:21) whose words are zeroed for the next level
// (shader/octree_init_node.comp:7-11).  Blocks handed out in word order (the engine's canonical order)
// make the result a pure function of the set of occupied cells at each depth:
//   * the depth-d word of occupied cell m (Morton code of its d-bit prefix) holds
//     0x80000000 | 8 * (1 + grank(d, m)), where grank counts occupied cells of depths 1..d-1 plus the
//     occupied depth-d cells whose Morton code is below m (breadth-first order = Morton order per depth);
//   * that word sits at 8 * (1 + grank(d-1, m >> 3)) + (m & 7), i.e. in its parent's child block.
// GB300 design, in four stages:
//   dense   depths 1..D (D = min(L-1, 9); 8^9 bits = 16 MB stays in L2): one sweep over the fragments sets
//           the occupancy bits of depth D (warp-deduplicated atomicOr), coarser depths are OR-reductions of
//           8-bit groups, one single-pass look-back scan of popcounts over all depths gives every grank,
//           and one pass writes all interior words of depths 1..D;
//   buckets the same sweep counts fragments per bucket of 32^3 voxels; a look-back scan and one scatter
//           copy the fragments into bucket order (8 B per fragment), which every later sweep reads;
//   sparse  depths D+1..L-1 (only when L > 10): the reference's tag / prefix-sum alloc per level with a
//           per-fragment cached node index (4 B per fragment), so tag reads one parent word;
//   leaf    one block per bucket: the bucket's leaf blocks are contiguous in the pool, so the block
//           accumulates their colours in shared memory (r, g, b, n in 16-bit fields, one shared atomic
//           per fragment) and writes every leaf word, 0xC0000000 | min(n,63)<<24 | floor(sum/n) (the
//           channel-wise integer mean), with no accumulator array in device memory.  The packing is exact
//           up to 257 fragments per voxel; a window where a voxel exceeds that is redone with exact
//           64-bit sums in the same block.
// Sizes stay on the device (BuildState): no host round trip inside a stage.
#include "common.cuh"
#include "svo_internal.h"

namespace svo {

constexpr int kTPB = 256;
constexpr int kAllocIPT = 8;
constexpr int kAllocTile = kTPB * kAllocIPT;
constexpr int kScanIPT = 8;
constexpr int kScanTile = kTPB * kScanIPT;
constexpr unsigned long long kLeafOne = 1ull << 48; // count field of a packed leaf accumulator

// ------------------------------------------------------------------------------------------ helpers
SVO_DEV void frag_xyz(uint64_t f, uint32_t &x, uint32_t &y, uint32_t &z) {
	const uint32_t fx = (uint32_t)f, fy = (uint32_t)(f >> 32);
	x = fx & 0xfffu;
	y = (fx >> 12) & 0xfffu;
	z = (fx >> 24) | ((fy >> 28) << 8);
}

// Spreads the low 10 bits of v to every third bit (bit-interleave by shifts and masks).
SVO_DEV uint32_t spread3(uint32_t v) {
	v &= 0x3ffu;
	v = (v | (v << 16)) & 0x030000FFu;
	v = (v | (v << 8)) & 0x0300F00Fu;
	v = (v | (v << 4)) & 0x030C30C3u;
	v = (v | (v << 2)) & 0x09249249u;
	return v;
}

// Morton code of the depth-(level - shift) prefix of a voxel: octant bit order x, y, z.
SVO_DEV uint32_t morton(uint32_t x, uint32_t y, uint32_t z, uint32_t shift) {
	return spread3(x >> shift) | (spread3(y >> shift) << 1) | (spread3(z >> shift) << 2);
}

SVO_DEV uint32_t octant_at(uint32_t x, uint32_t y, uint32_t z, uint32_t shift) {
	return ((x >> shift) & 1u) | (((y >> shift) & 1u) << 1) | (((z >> shift) & 1u) << 2);
}

// grank of occupied cell m at dense depth d (see the file comment).
SVO_DEV uint32_t grank(const DenseView &dv, uint32_t d, uint32_t m) {
	const uint32_t w = dv.off[d] + (m >> 5);
	return __ldg(dv.prefix + w) + __popc(__ldg(dv.bits + w) & ((1u << (m & 31)) - 1u));
}

SVO_DEV bool dense_bit(const DenseView &dv, uint32_t d, uint32_t m) {
	return (__ldg(dv.bits + dv.off[d] + (m >> 5)) >> (m & 31)) & 1u;
}

// Word index of the depth-`depth` node of a voxel whose parent is dense (depth-1 <= D).
SVO_DEV uint32_t dense_child_word(const DenseView &dv, uint32_t x, uint32_t y, uint32_t z, uint32_t level,
                                  uint32_t depth) {
	const uint32_t oct = octant_at(x, y, z, level - depth);
	if (depth == 1) return oct;
	return 8u * (1u + grank(dv, depth - 1, morton(x, y, z, level - depth + 1))) + oct;
}

// ------------------------------------------------------------------------------------------ init
__global__ void build_init(BuildState *state) {
	uint32_t *s = reinterpret_cast<uint32_t *>(state);
	for (uint32_t k = threadIdx.x; k < sizeof(BuildState) / 4; k += blockDim.x) s[k] = 0u;
	__syncthreads();
	if (threadIdx.x == 0) state->lv[1] = LevelInfo{0u, 8u, 0u, 0u};
}

// ------------------------------------------------------------------------------------------ dense stage
// Sets the depth-D occupancy bit of every fragment and counts the fragments of every bucket.  Per warp,
// fragments that fall in the same bitmap word (or bucket) are merged first, so one atomic covers them.
__global__ void __launch_bounds__(kTPB) dense_mark(const uint64_t *__restrict__ frags, uint32_t n, uint32_t level,
                                                   DenseView dv, uint32_t bshift, uint32_t *__restrict__ bcount) {
	const uint32_t shift = level - dv.D;
	const uint32_t key_shift = 3 * (bshift - shift); // the bucket key is a prefix of the depth-D Morton code
	uint32_t *bits = dv.bits + dv.off[dv.D];
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	for (uint64_t f = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; f < ((n + 31ull) & ~31ull); f += stride) {
		uint32_t word = 0xffffffffu, bit = 0, key = 0xffffffffu;
		if (f < n) {
			uint32_t x, y, z;
			frag_xyz(__ldcs(frags + f), x, y, z);
			const uint32_t m = morton(x, y, z, shift);
			word = m >> 5;
			bit = 1u << (m & 31);
			key = m >> key_shift;
		}
		const uint32_t peers = __match_any_sync(kFullMask, word);
		const uint32_t merged = __reduce_or_sync(peers, bit);
		if (word != 0xffffffffu && lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicOr(bits + word, merged);
		// fragments per bucket (of 32^3 voxels), for the bucketed copy
		const uint32_t kpeers = __match_any_sync(kFullMask, key);
		if (key != 0xffffffffu && lane_id() == (uint32_t)(__ffs(kpeers) - 1)) atomicAdd(bcount + key, __popc(kpeers));
	}
}

// bitmap of depth d from depth d+1: bit p = (byte p of the child bitmap != 0).
__global__ void dense_reduce(DenseView dv, uint32_t d) {
	const uint32_t nbits = 1u << (3 * d);
	const uint32_t nwords = (nbits + 31) / 32;
	const uint8_t *child = reinterpret_cast<const uint8_t *>(dv.bits + dv.off[d + 1]);
	uint32_t *parent = dv.bits + dv.off[d];
	for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += gridDim.x * blockDim.x) {
		uint32_t out = 0;
		if (nbits >= 32) {
			const uint4 *c = reinterpret_cast<const uint4 *>(child + 32 * (size_t)w);
			const uint4 a = c[0], b = c[1];
			const uint32_t v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
			for (int i = 0; i < 8; ++i)
#pragma unroll
				for (int j = 0; j < 4; ++j) out |= (uint32_t)(((v[i] >> (8 * j)) & 0xffu) != 0u) << (4 * i + j);
		} else {
			for (uint32_t p = 0; p < nbits; ++p) out |= (uint32_t)(child[p] != 0) << p;
		}
		parent[w] = out;
	}
}

// Exclusive prefix of popcounts over the concatenated bitmaps of depths 1..D; prefix[total] = total
// occupied cells.  Persistent grid, tiles claimed in order by ticket.
__global__ void __launch_bounds__(kTPB) dense_scan(DenseView dv, uint32_t total_words, BuildState *state,
                                                   unsigned long long *descs) {
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kTPB / 32 + 1];
	__shared__ uint32_t s_prefix;
	const uint32_t ntiles = (total_words + kScanTile - 1) / kScanTile;
	for (;;) {
		if (threadIdx.x == 0) s_tile = atomicAdd(&state->tiles[0], 1u);
		__syncthreads();
		const uint32_t tile = s_tile;
		__syncthreads();
		if (tile >= ntiles) break;
		const uint32_t w0 = tile * kScanTile + threadIdx.x * kScanIPT;
		uint32_t c[kScanIPT], local = 0;
#pragma unroll
		for (int k = 0; k < kScanIPT; ++k) {
			c[k] = w0 + k < total_words ? __popc(dv.bits[w0 + k]) : 0u;
			local += c[k];
		}
		uint32_t total;
		uint32_t run = block_exclusive_sum<uint32_t, kTPB>(local, s_warp, total);
		if (threadIdx.x < 32) {
			const uint32_t p = (uint32_t)tile_lookback_warp(descs, tile, 15u, total, &state->status);
			if (threadIdx.x == 0) s_prefix = p;
		}
		__syncthreads();
		run += s_prefix;
#pragma unroll
		for (int k = 0; k < kScanIPT; ++k) {
			if (w0 + k < total_words) dv.prefix[w0 + k] = run;
			run += c[k];
		}
		if (tile == ntiles - 1 && threadIdx.x == 0) dv.prefix[total_words] = s_prefix + total;
		__syncthreads();
	}
}

// Level ranges of depths 1..D+1 from the scanned counts (BuildState.lv as the sparse stage keeps it).
__global__ void dense_finish(DenseView dv, BuildState *state) {
	if (threadIdx.x != 0) return;
	// occupied cells of depth d: N_d = prefix[off[d+1]] - prefix[off[d]]; cells of depths < d: prefix[off[d]]
	for (uint32_t d = 1; d <= dv.D + 1; ++d) {
		const uint32_t before_parent = d >= 2 ? dv.prefix[dv.off[d - 1]] : 0u; // occupied cells of depths < d-1
		const uint32_t parents = d >= 2 ? dv.prefix[dv.off[d]] - dv.prefix[dv.off[d - 1]] : 1u;
		LevelInfo li;
		li.begin = d == 1 ? 0u : 8u * (1u + before_parent);
		li.num = 8u * parents;
		li.blocks_before = d == 1 ? 0u : dv.prefix[dv.off[d]];
		li.nodes = d <= dv.D ? dv.prefix[dv.off[d + 1]] - dv.prefix[dv.off[d]] : 0u;
		state->lv[d] = li;
	}
}

// Writes the child blocks of every occupied cell of depths 0 (the root) .. D that has interior or
// sparse children: interior words of depths 1..D, and zeroed words of depth D+1 when sparse levels
// follow.  When depth D+1 is the leaf depth, depth-D cells are skipped: the leaf stage writes those
// blocks whole.  One bitmap word and one prefix word of the child depth serve all 8 children.
__global__ void __launch_bounds__(kTPB) dense_write(uint32_t *__restrict__ pool, uint64_t capacity, DenseView dv,
                                                    uint32_t level, BuildState *state) {
	const uint32_t D = dv.D;
	const bool leaf_next = D + 1 == level;
	const uint32_t last_parent_depth = leaf_next ? D - 1 : D;
	const uint32_t parent_words = dv.off[last_parent_depth + 1]; // words of parent depths 1..last; item 0 = root
	for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item <= parent_words; item += gridDim.x * blockDim.x) {
		uint32_t bits, e, base_m, r;
		if (item == 0) { // the root: a single occupied cell whose block (words 0..7) holds the depth-1 nodes
			bits = 1u, e = 0, base_m = 0, r = 0;
		} else {
			const uint32_t gw = item - 1; // global word of a parent depth e in 1..last
			e = 1;
			while (gw >= dv.off[e + 1]) ++e;
			bits = __ldg(dv.bits + gw);
			base_m = (gw - dv.off[e]) << 5;
			r = __ldg(dv.prefix + gw); // grank of the first set bit of this word
		}
		const uint32_t d = e + 1; // depth of the words being written
		while (bits) {
			const uint32_t b = __ffs(bits) - 1;
			bits &= bits - 1;
			const uint32_t q = base_m + b; // parent cell (depth e)
			const uint64_t blk = e == 0 ? 0ull : 8ull * (1u + r++);
			if (blk + 8 > capacity || blk + 8 > SVO_MAX_POOL_WORDS) {
				atomicOr(&state->status, kStatusCapacity);
				continue;
			}
			uint32_t w[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
			if (d <= D) { // children are interior nodes: one byte of the depth-d bitmap
				const uint32_t cw = dv.off[d] + (q >> 2), shift = (q & 3u) * 8u;
				const uint32_t word = __ldg(dv.bits + cw);
				const uint32_t kids = (word >> shift) & 0xffu;
				const uint32_t rank0 = __ldg(dv.prefix + cw) + __popc(word & ((1u << shift) - 1u));
#pragma unroll
				for (int o = 0; o < 8; ++o)
					if ((kids >> o) & 1u) w[o] = 0x80000000u | (8u * (1u + rank0 + __popc(kids & ((1u << o) - 1u))));
			}
			uint4 *dst = reinterpret_cast<uint4 *>(pool + blk);
			dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
			dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
		}
	}
}

// ------------------------------------------------------------------------------------------ tag (sparse levels)
// Marks the depth-`depth` node of every fragment (0x80000000), reading its parent through the node index
// cached by the previous sparse depth (or the dense bitmaps when the parent depth is dense).
SVO_DEV void tag_one(uint64_t frag, uint32_t &node, uint32_t level, uint32_t depth, bool parent_dense,
                     const DenseView &dv, uint32_t *__restrict__ pool) {
	uint32_t x, y, z;
	frag_xyz(frag, x, y, z);
	uint32_t idx;
	if (parent_dense)
		idx = dense_child_word(dv, x, y, z, level, depth);
	else
		idx = (pool[node] & 0x3fffffffu) + octant_at(x, y, z, level - depth);
	if ((pool[idx] & 0x80000000u) == 0u) pool[idx] = 0x80000000u;
	node = idx;
}

__global__ void __launch_bounds__(kTPB) build_tag(const uint64_t *__restrict__ frags, uint32_t n, uint32_t level,
                                                  uint32_t depth, uint32_t *__restrict__ pool,
                                                  uint32_t *__restrict__ cache, DenseView dv, BuildState *state) {
	if (state->status & kStatusCapacity) return;
	const bool parent_dense = depth == 1 || depth - 1 <= dv.D;
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t nq = (n + 3ull) / 4ull;
	for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
		const uint64_t f0 = q * 4;
		if (f0 + 4 <= n) { // the sorted copy is 256-byte aligned: 16-byte loads
			const ulonglong2 a = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0));
			const ulonglong2 b = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0 + 2));
			uint4 c = make_uint4(0, 0, 0, 0);
			if (!parent_dense) c = __ldcs(reinterpret_cast<const uint4 *>(cache + f0));
			tag_one(a.x, c.x, level, depth, parent_dense, dv, pool);
			tag_one(a.y, c.y, level, depth, parent_dense, dv, pool);
			tag_one(b.x, c.z, level, depth, parent_dense, dv, pool);
			tag_one(b.y, c.w, level, depth, parent_dense, dv, pool);
			__stcs(reinterpret_cast<uint4 *>(cache + f0), c);
		} else {
			for (uint64_t f = f0; f < n; ++f) {
				uint32_t c = parent_dense ? 0u : cache[f];
				tag_one(frags[f], c, level, depth, parent_dense, dv, pool);
				cache[f] = c;
			}
		}
	}
}


// Prefix-sum allocation of child blocks for the marked words of a sparse depth (persistent grid, tiles
// claimed in order by ticket so the look-back always waits on a running or finished tile).  The block
// of a node is zeroed (the next depth's init) unless the next depth is the leaf depth.
__global__ void __launch_bounds__(kTPB) build_alloc(uint32_t *__restrict__ pool, uint64_t capacity, uint32_t depth,
                                                    uint32_t level, BuildState *state, unsigned long long *descs) {
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kTPB / 32 + 1];
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
		const uint32_t rank0 = block_exclusive_sum<uint32_t, kTPB>(cnt, s_warp, total);
		if (threadIdx.x < 32) {
			const uint32_t p = (uint32_t)tile_lookback_warp(descs, tile, depth, total, &state->status);
			if (threadIdx.x == 0) s_prefix = p;
		}
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
			if (!next_is_leaf) { // the next depth's init; leaf blocks are written whole by the leaf stage
				uint4 *child = reinterpret_cast<uint4 *>(pool + ptr);
				child[0] = make_uint4(0, 0, 0, 0);
				child[1] = make_uint4(0, 0, 0, 0);
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

// ------------------------------------------------------------------------------------------ buckets
// The fragments are copied once into buckets of 32^3 voxels (Morton order of the bucket, any order
// inside one).  All later sweeps read the bucketed copy: the sparse tag passes then touch the pool
// region by region, and the leaf stage gives each bucket to one block, which accumulates its leaf
// colours in shared memory.  The leaf blocks (8 words per depth L-1 node) of one bucket are contiguous
// in the pool (breadth-first order is Morton order within a depth), so that block writes them whole.
constexpr uint32_t kBucketVoxelBits = 5; // bucket edge: 32 voxels

SVO_DEV uint32_t bucket_of(uint32_t x, uint32_t y, uint32_t z, uint32_t bshift) { return morton(x, y, z, bshift); }

// Fragment counts per bucket (used when the dense stage does not run: level 1).
__global__ void __launch_bounds__(kTPB) bucket_hist(const uint64_t *__restrict__ frags, uint32_t n, uint32_t bshift,
                                                    uint32_t *__restrict__ bcount) {
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	for (uint64_t f = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; f < ((n + 31ull) & ~31ull); f += stride) {
		uint32_t key = 0xffffffffu;
		if (f < n) {
			uint32_t x, y, z;
			frag_xyz(frags[f], x, y, z);
			key = bucket_of(x, y, z, bshift);
		}
		const uint32_t peers = __match_any_sync(kFullMask, key);
		if (key != 0xffffffffu && lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicAdd(bcount + key, __popc(peers));
	}
}

// Exclusive prefix of the bucket counts (boff[nb] = total) and the list of non-empty buckets in order;
// two single-pass look-back scans, tiles claimed in order by ticket.
__global__ void __launch_bounds__(kTPB) bucket_scan(const uint32_t *__restrict__ bcount, uint32_t nb,
                                                    uint32_t *__restrict__ boff, uint32_t *__restrict__ blist,
                                                    BuildState *state, unsigned long long *descs) {
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kTPB / 32 + 1];
	__shared__ uint32_t s_prefix[2];
	if (threadIdx.x == 0) s_tile = atomicAdd(&state->tiles[1], 1u);
	__syncthreads();
	const uint32_t tile = s_tile;
	const uint32_t ntiles = (nb + kScanTile - 1) / kScanTile;
	const uint32_t b0 = tile * kScanTile + threadIdx.x * kScanIPT;
	uint32_t c[kScanIPT], local = 0, nonempty = 0;
#pragma unroll
	for (int k = 0; k < kScanIPT; ++k) {
		c[k] = b0 + k < nb ? bcount[b0 + k] : 0u;
		local += c[k];
		nonempty += c[k] != 0u;
	}
	uint32_t total, total_ne;
	uint32_t run = block_exclusive_sum<uint32_t, kTPB>(local, s_warp, total);
	__syncthreads();
	uint32_t run_ne = block_exclusive_sum<uint32_t, kTPB>(nonempty, s_warp, total_ne);
	if (threadIdx.x < 32) {
		const uint32_t p = (uint32_t)tile_lookback_warp(descs, tile, 1u, total, &state->status);
		const uint32_t q = (uint32_t)tile_lookback_warp(descs + ntiles, tile, 1u, total_ne, &state->status);
		if (threadIdx.x == 0) s_prefix[0] = p, s_prefix[1] = q;
	}
	__syncthreads();
	run += s_prefix[0];
	run_ne += s_prefix[1];
#pragma unroll
	for (int k = 0; k < kScanIPT; ++k) {
		if (b0 + k < nb) {
			boff[b0 + k] = run;
			if (c[k]) blist[run_ne++] = b0 + k;
		}
		run += c[k];
	}
	if (tile == ntiles - 1 && threadIdx.x == 0) {
		boff[nb] = s_prefix[0] + total;
		state->buckets = s_prefix[1] + total_ne;
	}
}

// Copies every fragment into its bucket; lanes of a warp with the same bucket take one cursor step.
// When the leaf depth's parents are dense (level <= 10), the copy holds leaf items instead of fragments:
// the leaf word slot (from the dense bitmap of depth level-1) in the high word and the colour in the low
// one, so the leaf stage needs no lookups.
__global__ void __launch_bounds__(kTPB) bucket_scatter(const uint64_t *__restrict__ frags, uint32_t n,
                                                       uint32_t bshift, const uint32_t *__restrict__ boff,
                                                       uint32_t *__restrict__ bfill, uint64_t *__restrict__ sorted,
                                                       bool items, DenseView dv, uint32_t level,
                                                       const BuildState *state) {
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint32_t lane = lane_id();
	const uint32_t *pbits = items && level > 1 ? dv.bits + dv.off[level - 1] : nullptr;
	const uint32_t *pprefix = items && level > 1 ? dv.prefix + dv.off[level - 1] : nullptr;
	const uint32_t leaf_begin = items ? state->lv[level].begin : 0u;
	for (uint64_t f = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; f < ((n + 31ull) & ~31ull); f += stride) {
		uint32_t key = 0xffffffffu;
		uint64_t out = 0;
		if (f < n) {
			const uint64_t frag = __ldcs(frags + f);
			uint32_t x, y, z;
			frag_xyz(frag, x, y, z);
			out = frag;
			if (pbits) { // parent cell m (depth level-1); the bucket key is its prefix
				const uint32_t m = morton(x, y, z, 1), w = m >> 5;
				key = m >> (3 * (bshift - 1));
				out = ((uint64_t)(octant_at(x, y, z, 0) + 8u * (1u + __ldg(pprefix + w) +
				                                                 __popc(__ldg(pbits + w) & ((1u << (m & 31)) - 1u))) -
				                  leaf_begin)
				       << 32) |
				      ((frag >> 32) & 0xffffffu);
			} else {
				key = bucket_of(x, y, z, bshift);
			}
			if (items && !pbits) {
				const uint32_t idx = octant_at(x, y, z, 0);
				out = ((uint64_t)(idx - leaf_begin) << 32) | ((frag >> 32) & 0xffffffu);
			}
		}
		const uint32_t peers = __match_any_sync(kFullMask, key);
		const uint32_t leader = __ffs(peers) - 1;
		uint32_t base = 0;
		if (key != 0xffffffffu && lane == leader) base = atomicAdd(bfill + key, __popc(peers));
		base = __shfl_sync(kFullMask, base, leader);
		if (key != 0xffffffffu) sorted[boff[key] + base + __popc(peers & ((1u << lane) - 1u))] = out;
	}
}

// ------------------------------------------------------------------------------------------ leaf stage
// Leaf word from exact 64-bit colour sums (the overflow path; integer division).
SVO_DEV uint32_t leaf_word_wide(uint32_t n, uint64_t sr, uint64_t sg, uint64_t sb) {
	return 0xC0000000u | (min(n, 63u) << 24) | ((uint32_t)(sb / n) << 16) | ((uint32_t)(sg / n) << 8) |
	       (uint32_t)(sr / n);
}

// Leaf word from packed sums (1 <= n <= 257, every sum < 2^16).  floor(s / n) = trunc(s * (1/n) + 2^-10):
// the float product is within 4e-5 of s / n, a non-integer s / n lies at least 1/257 below the next
// integer, and an integer one is lifted clear of the truncation by the 2^-10.
SVO_DEV uint32_t leaf_word(uint32_t n, uint32_t sr, uint32_t sg, uint32_t sb) {
	const float inv = __frcp_rn((float)n);
	const uint32_t r = (uint32_t)fmaf((float)sr, inv, 0.0009765625f);
	const uint32_t g = (uint32_t)fmaf((float)sg, inv, 0.0009765625f);
	const uint32_t b = (uint32_t)fmaf((float)sb, inv, 0.0009765625f);
	return 0xC0000000u | (min(n, 63u) << 24) | (b << 16) | (g << 8) | r;
}

// Where the leaf stage finds the parent of a leaf: the dense bitmap of depth level-1 (its words at
// bits/prefix) or, below the dense depths, the node index cached per fragment by the last sparse tag.
struct LeafParent {
	const uint32_t *bits, *prefix; // dense depth level-1 (null at level 1: the parent is the root)
	const uint32_t *pool, *cache;  // sparse parent
	uint32_t leaf_begin;
};

// Leaf word slot (index from the start of the leaf range) of fragment f of the bucketed copy.
SVO_DEV uint32_t leaf_slot(uint64_t frag, uint64_t f, const LeafParent &lp) {
	uint32_t x, y, z;
	frag_xyz(frag, x, y, z);
	const uint32_t oct = octant_at(x, y, z, 0);
	uint32_t idx;
	if (lp.cache) {
		idx = (__ldg(lp.pool + __ldg(lp.cache + f)) & 0x3fffffffu) + oct;
	} else if (lp.bits) { // 8 * (1 + grank(level-1, parent)) + octant
		const uint32_t m = morton(x, y, z, 1);
		const uint32_t w = m >> 5;
		idx = 8u * (1u + __ldg(lp.prefix + w) + __popc(__ldg(lp.bits + w) & ((1u << (m & 31)) - 1u))) + oct;
	} else {
		idx = oct;
	}
	return idx - lp.leaf_begin;
}

constexpr uint32_t kLeafSlots = 4096;         // packed accumulators in shared memory (8 B each)
constexpr uint32_t kWideSlots = kLeafSlots / 4; // exact accumulators (4 x 8 B each) of the overflow path

// Extent of every non-empty bucket, in list order: first and last item, first and last leaf slot
// (lo = 0xffffffff, hi = 0 when the leaf stage reduces the span over the bucket's fragments).
//   one bucket (level <= 5): the whole leaf range;
//   dense parents: bucket b is 4096 parent cells = 128 words of the depth level-1 bitmap, and the prefix
//     entries at its first word and at the next bucket's give its first and last leaf block.
__global__ void bucket_meta(const uint32_t *__restrict__ boff, const uint32_t *__restrict__ blist, uint32_t nb,
                            DenseView dv, uint32_t level, const BuildState *state, uint4 *__restrict__ meta) {
	const uint32_t nbuckets = state->buckets;
	const bool items = level == 1 || level - 1 <= dv.D;
	const uint32_t leaf_begin = state->lv[level].begin, leaf_num = state->lv[level].num;
	const uint32_t *pprefix = items && level > 1 ? dv.prefix + dv.off[level - 1] : nullptr;
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nbuckets; t += gridDim.x * blockDim.x) {
		const uint32_t b = blist[t];
		uint4 m = make_uint4(boff[b], boff[b + 1], 0xffffffffu, 0u);
		if (nb == 1) {
			m.z = 0, m.w = leaf_num - 1;
		} else if (pprefix) {
			const uint32_t before = leaf_begin / 8u - 1u; // occupied cells of depths below the parents
			m.z = 8u * (pprefix[128u * b] - before);
			m.w = 8u * (pprefix[128u * (b + 1)] - before) - 1u;
		}
		meta[t] = m;
	}
}

// One bucket per block at a time, buckets taken grid-stride from the list (the next bucket's extent is
// loaded while the block works on the current one).  For each window of kLeafSlots slots of the
// bucket's span: zero the shared accumulators, add every item of the window, and write the window's
// leaf words (empty slots as 0).  An accumulator is two 32-bit words, (r | g << 16) and (b | n << 16):
// a field can carry only when a voxel has more than 257 fragments (257 x 255 = 65535), so an add that
// sees a count of 257 or more marks the window, which is then redone exactly with 64-bit r, g, b and n
// sums, kWideSlots slots at a time.
//   items (dense parents): the bucketed copy holds (slot << 32 | rgb);
//   otherwise: fragments, slots through the cached parent index, span reduced over the bucket.
__global__ void __launch_bounds__(kTPB) build_leaf(const uint64_t *__restrict__ sorted, uint32_t level,
                                                   uint32_t *__restrict__ pool, uint64_t capacity,
                                                   const uint32_t *__restrict__ cache, DenseView dv,
                                                   const uint4 *__restrict__ meta, BuildState *state) {
	extern __shared__ unsigned long long s_acc[];
	uint32_t *s_acc32 = reinterpret_cast<uint32_t *>(s_acc);
	__shared__ uint32_t s_lo, s_hi, s_over, s_leaves;
	if (state->status & kStatusCapacity) return;
	const uint64_t leaf_end = (uint64_t)state->lv[level].begin + state->lv[level].num;
	if (leaf_end > capacity || leaf_end > SVO_MAX_POOL_WORDS) { // leaf blocks of dense parents: checked here
		if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&state->status, kStatusCapacity);
		return;
	}
	const bool items = level == 1 || level - 1 <= dv.D;
	const uint32_t leaf_begin = state->lv[level].begin;
	LeafParent lp;
	lp.bits = nullptr, lp.prefix = nullptr;
	lp.pool = pool;
	lp.cache = cache;
	lp.leaf_begin = leaf_begin;
	const uint32_t nbuckets = state->buckets;
	if (threadIdx.x == 0) s_leaves = 0;
	uint4 next = blockIdx.x < nbuckets ? meta[blockIdx.x] : make_uint4(0, 0, 0, 0);
	for (uint32_t t = blockIdx.x; t < nbuckets; t += gridDim.x) {
		const uint4 m = next;
		if (t + gridDim.x < nbuckets) next = meta[t + gridDim.x];
		const uint32_t f0 = m.x, f1 = m.y;
		uint32_t span_lo = m.z & ~7u, span_hi = (m.w | 7u) + 1u;
		if (m.z > m.w) { // span reduced over the bucket's fragments
			if (threadIdx.x == 0) s_lo = 0xffffffffu, s_hi = 0u;
			__syncthreads();
			uint32_t lo = 0xffffffffu, hi = 0u;
			for (uint32_t fb = f0 + threadIdx.x; fb < f1; fb += 4 * kTPB) {
				uint64_t fr[4];
#pragma unroll
				for (int k = 0; k < 4; ++k) fr[k] = fb + k * kTPB < f1 ? sorted[fb + k * kTPB] : 0ull;
#pragma unroll
				for (int k = 0; k < 4; ++k)
					if (fb + k * kTPB < f1) {
						const uint32_t sl = leaf_slot(fr[k], fb + k * kTPB, lp);
						lo = min(lo, sl), hi = max(hi, sl);
					}
			}
			lo = __reduce_min_sync(kFullMask, lo), hi = __reduce_max_sync(kFullMask, hi);
			if (lane_id() == 0) atomicMin(&s_lo, lo), atomicMax(&s_hi, hi);
			__syncthreads();
			span_lo = s_lo & ~7u, span_hi = (s_hi | 7u) + 1u;
		}
		for (uint32_t w0 = span_lo; w0 < span_hi; w0 += kLeafSlots) {
			const uint32_t wn = min(kLeafSlots, span_hi - w0);
			for (uint32_t i = threadIdx.x; i < wn; i += kTPB) s_acc[i] = 0ull;
			if (threadIdx.x == 0) s_over = 0;
			__syncthreads();
			bool over = false;
			for (uint32_t fb = f0 + threadIdx.x; fb < f1; fb += 4 * kTPB) {
				uint64_t fr[4];
				uint32_t sl[4], rgb[4];
#pragma unroll
				for (int k = 0; k < 4; ++k) fr[k] = fb + k * kTPB < f1 ? sorted[fb + k * kTPB] : 0ull;
#pragma unroll
				for (int k = 0; k < 4; ++k) {
					const bool in = fb + k * kTPB < f1;
					sl[k] = !in ? 0xffffffffu : (items ? (uint32_t)(fr[k] >> 32) : leaf_slot(fr[k], fb + k * kTPB, lp)) - w0;
					rgb[k] = items ? (uint32_t)fr[k] : (uint32_t)(fr[k] >> 32);
				}
#pragma unroll
				for (int k = 0; k < 4; ++k)
					if (sl[k] < wn) {
						atomicAdd(s_acc32 + 2 * sl[k], (rgb[k] & 0xffu) | (((rgb[k] >> 8) & 0xffu) << 16));
						over |= (atomicAdd(s_acc32 + 2 * sl[k] + 1, ((rgb[k] >> 16) & 0xffu) | (1u << 16)) >> 16) >= 257u;
					}
			}
			if (__any_sync(kFullMask, over) && lane_id() == 0) s_over = 1;
			__syncthreads();
			uint32_t leaves = 0;
			if (!s_over) {
				for (uint32_t i = 4 * threadIdx.x; i < wn; i += 4 * kTPB) {
					const uint4 a = *reinterpret_cast<const uint4 *>(s_acc32 + 2 * i);
					const uint4 c = *reinterpret_cast<const uint4 *>(s_acc32 + 2 * i + 4);
					const uint32_t rg[4] = {a.x, a.z, c.x, c.z}, bn[4] = {a.y, a.w, c.y, c.w};
					uint32_t word[4];
#pragma unroll
					for (int j = 0; j < 4; ++j) {
						const uint32_t n = bn[j] >> 16;
						word[j] = n ? leaf_word(n, rg[j] & 0xffffu, rg[j] >> 16, bn[j] & 0xffffu) : 0u;
						leaves += word[j] != 0u;
					}
					*reinterpret_cast<uint4 *>(pool + leaf_begin + w0 + i) = make_uint4(word[0], word[1], word[2], word[3]);
				}
			} else {
				// exact sums for this window, kWideSlots slots at a time
				unsigned long long *acc4 = s_acc;
				for (uint32_t v0 = 0; v0 < wn; v0 += kWideSlots) {
					const uint32_t vn = min(kWideSlots, wn - v0);
					__syncthreads();
					for (uint32_t i = threadIdx.x; i < 4 * vn; i += kTPB) acc4[i] = 0ull;
					__syncthreads();
					for (uint32_t f = f0 + threadIdx.x; f < f1; f += kTPB) {
						const uint64_t item = sorted[f];
						const uint32_t sl = (items ? (uint32_t)(item >> 32) : leaf_slot(item, f, lp)) - w0 - v0;
						const uint32_t c = items ? (uint32_t)item : (uint32_t)(item >> 32);
						if (sl < vn) {
							atomicAdd(acc4 + 4 * sl, (unsigned long long)(c & 0xffu));
							atomicAdd(acc4 + 4 * sl + 1, (unsigned long long)((c >> 8) & 0xffu));
							atomicAdd(acc4 + 4 * sl + 2, (unsigned long long)((c >> 16) & 0xffu));
							atomicAdd(acc4 + 4 * sl + 3, 1ull);
						}
					}
					__syncthreads();
					for (uint32_t i = threadIdx.x; i < vn; i += kTPB) {
						const unsigned long long n = acc4[4 * i + 3];
						// n < 2^32 (fragment counts are 32-bit)
						const uint32_t word = n ? leaf_word_wide((uint32_t)n, acc4[4 * i], acc4[4 * i + 1], acc4[4 * i + 2]) : 0u;
						pool[leaf_begin + w0 + v0 + i] = word;
						leaves += word != 0u;
					}
				}
			}
			leaves = warp_sum(leaves);
			if (lane_id() == 0 && leaves) atomicAdd(&s_leaves, leaves);
			__syncthreads();
		}
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		if (s_leaves) atomicAdd(&state->leaves, s_leaves);
		if (blockIdx.x == 0) state->range_words = leaf_end;
	}
}

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

// ------------------------------------------------------------------------------------------ host side
uint64_t build_pool_bound(uint32_t count, uint32_t level) {
	uint64_t words = 8, per = 1;
	for (uint32_t i = 1; i < level; ++i) {
		per = per >= (1ull << 40) ? per : per * 8; // 8^i (saturating)
		words += 8 * (per < count ? per : (uint64_t)count);
	}
	return words < SVO_MAX_POOL_WORDS ? words : SVO_MAX_POOL_WORDS;
}

uint32_t dense_depth(uint32_t level) { return level - 1 < kDenseMaxDepth ? level - 1 : kDenseMaxDepth; }

static uint32_t dense_words_of(uint32_t d) { return d <= 1 ? 1u : (1u << (3 * d)) / 32u; }

// Largest word range of one sparse depth: 8 * min(8^(i-1), count) over depths D+2..level-1.
static uint64_t max_sparse_level_words(uint32_t count, uint32_t level, uint32_t D) {
	uint64_t best = 8, per = 1;
	for (uint32_t i = 1; i < level; ++i) {
		if (i >= D + 2) {
			const uint64_t w = 8 * (per < count ? per : (uint64_t)count);
			best = w > best ? w : best;
		}
		per = per >= (1ull << 40) ? per : per * 8;
	}
	return best;
}

// Layout: state | dense-scan descriptors | dense bitmaps | dense prefix | bucket counts, offsets,
// cursors, list and scan descriptors | bucketed fragment copy (8 B per fragment) | node cache (4 B per
// fragment, sparse levels only).  The leaf stage needs nothing more: its accumulators live in shared
// memory.
void build_workspace_layout(void *ws, uint32_t count, uint32_t level, uint64_t capacity, BuildWorkspace &w) {
	char *p = (char *)ws;
	size_t off = 0;
	auto take = [&](size_t bytes) {
		char *q = p + off;
		off += align_up(bytes, 256);
		return q;
	};
	const uint32_t D = dense_depth(level);
	w.dv.D = D;
	uint32_t o = 0;
	w.dv.off[0] = 0;
	for (uint32_t d = 1; d <= kDenseMaxDepth + 1; ++d) {
		w.dv.off[d] = o;
		if (d <= D) o += (dense_words_of(d) + 7u) & ~7u; // 32-byte aligned levels (16-byte vector loads)
	}
	w.dense_words = o;
	w.state = (BuildState *)take(sizeof(BuildState));
	uint64_t sparse_words = max_sparse_level_words(count, level, D);
	if (sparse_words > capacity) sparse_words = capacity;
	const uint64_t scan_items = std::max<uint64_t>(o, sparse_words);
	w.desc_count = (size_t)((scan_items + kScanTile - 1) / kScanTile + 2);
	w.descs = (unsigned long long *)take(w.desc_count * sizeof(unsigned long long));
	w.dv.bits = (uint32_t *)take((size_t)o * 4 + 32);
	w.dv.prefix = (uint32_t *)take(((size_t)o + 1) * 4);
	w.bshift = std::min<uint32_t>(level, kBucketVoxelBits);
	w.nb = 1u << (3 * (level - w.bshift));
	w.bcount = (uint32_t *)take((size_t)w.nb * 4);
	w.bfill = (uint32_t *)take((size_t)w.nb * 4);
	w.boff = (uint32_t *)take(((size_t)w.nb + 1) * 4);
	w.blist = (uint32_t *)take((size_t)w.nb * 4);
	w.bmeta = (uint4 *)take((size_t)w.nb * 16);
	w.bdesc_count = 2 * ((size_t)(w.nb + kScanTile - 1) / kScanTile + 1);
	w.bdescs = (unsigned long long *)take(w.bdesc_count * sizeof(unsigned long long));
	w.sorted = (uint64_t *)take((size_t)count * 8 + 32);
	w.cache = (uint32_t *)take(level > D + 1 ? (size_t)count * 4 + 16 : 16);
	w.total_bytes = off;
}

static uint32_t grid_for(uint64_t items, uint32_t per_block, uint32_t cap) {
	const uint64_t b = (items + per_block - 1) / per_block;
	return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(b, cap));
}

cudaError_t build_launch_interior(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool,
                                  uint64_t capacity, const BuildWorkspace &w, cudaStream_t stream) {
	cudaError_t e = cudaMemsetAsync(w.descs, 0, w.desc_count * sizeof(unsigned long long), stream);
	if (e == cudaSuccess && w.dense_words) e = cudaMemsetAsync(w.dv.bits, 0, (size_t)w.dense_words * 4, stream);
	// bucket counts and cursors are adjacent: one memset
	if (e == cudaSuccess) e = cudaMemsetAsync(w.bcount, 0, (char *)w.boff - (char *)w.bcount, stream);
	if (e == cudaSuccess) e = cudaMemsetAsync(w.bdescs, 0, w.bdesc_count * sizeof(unsigned long long), stream);
	if (e != cudaSuccess) return e;
	const int sms = device_sm_count();
	const uint32_t D = w.dv.D;
	SVO_LAUNCH("build_init", stream, build_init<<<1, 256, 0, stream>>>(w.state););
	if (D >= 1) {
		SVO_LAUNCH("dense_mark", stream,
		           dense_mark<<<grid_for(count, kTPB, (uint32_t)sms * 16), kTPB, 0, stream>>>(frags, count, level, w.dv,
		                                                                                      w.bshift, w.bcount););
	} else {
		SVO_LAUNCH("bucket_hist", stream,
		           bucket_hist<<<grid_for(count, kTPB, (uint32_t)sms * 16), kTPB, 0, stream>>>(frags, count, w.bshift,
		                                                                                       w.bcount););
	}
	SVO_LAUNCH("bucket_scan", stream,
	           bucket_scan<<<(w.nb + kScanTile - 1) / kScanTile, kTPB, 0, stream>>>(w.bcount, w.nb, w.boff, w.blist,
	                                                                               w.state, w.bdescs););
	if (D >= 1) {
		for (uint32_t d = D - 1; d >= 1; --d)
			SVO_LAUNCH("dense_reduce", stream,
			           dense_reduce<<<grid_for(dense_words_of(d), kTPB, (uint32_t)sms * 8), kTPB, 0, stream>>>(w.dv, d););
		SVO_LAUNCH("dense_scan", stream,
		           dense_scan<<<grid_for(w.dense_words, kScanTile, (uint32_t)sms * 4), kTPB, 0, stream>>>(
		               w.dv, w.dense_words, w.state, w.descs););
		SVO_LAUNCH("dense_finish", stream, dense_finish<<<1, 32, 0, stream>>>(w.dv, w.state););
		SVO_LAUNCH("dense_write", stream,
		           dense_write<<<grid_for((uint64_t)w.dense_words + 1, kTPB, (uint32_t)sms * 16), kTPB, 0, stream>>>(
		               pool, capacity, w.dv, level, w.state););
	}
	// the bucketed copy: leaf items when the leaf parents are dense (their bitmap is final now), fragments
	// for the sparse levels otherwise
	const bool items = level == 1 || level - 1 <= D;
	SVO_LAUNCH("bucket_scatter", stream,
	           bucket_scatter<<<grid_for(count, kTPB, (uint32_t)sms * 16), kTPB, 0, stream>>>(
	               frags, count, w.bshift, w.boff, w.bfill, w.sorted, items, w.dv, level, w.state););
	const uint32_t tag_blocks = grid_for(((uint64_t)count + 3) / 4, kTPB, (uint32_t)sms * 16);
	for (uint32_t depth = D + 1; depth < level; ++depth) {
		SVO_LAUNCH("build_tag", stream,
		           build_tag<<<tag_blocks, kTPB, 0, stream>>>(w.sorted, count, level, depth, pool, w.cache, w.dv,
		                                                      w.state););
		SVO_LAUNCH("build_alloc", stream,
		           build_alloc<<<(uint32_t)sms * 4, kTPB, 0, stream>>>(pool, capacity, depth, level, w.state, w.descs););
	}
	return cudaGetLastError();
}

cudaError_t build_launch_leaf(uint32_t count, uint32_t level, uint32_t *pool, uint64_t capacity,
                              const BuildWorkspace &w, cudaStream_t stream) {
	(void)count;
	const int sms = device_sm_count();
	const size_t smem = kLeafSlots * sizeof(unsigned long long); // 32 KB: below the default dynamic limit
	SVO_LAUNCH("bucket_meta", stream,
	           bucket_meta<<<grid_for(w.nb, kTPB, (uint32_t)sms * 4), kTPB, 0, stream>>>(w.boff, w.blist, w.nb, w.dv, level,
	                                                                                w.state, w.bmeta););
	SVO_LAUNCH("build_leaf", stream,
	           build_leaf<<<(uint32_t)sms * 6, kTPB, smem, stream>>>(w.sorted, level, pool, capacity, w.cache, w.dv,
	                                                                  w.bmeta, w.state););
	return cudaGetLastError();
}

cudaError_t build_launch_export(const BuildWorkspace &w, uint32_t level, uint32_t count, void *out,
                                cudaStream_t stream) {
	SVO_LAUNCH("build_export", stream, build_export<<<1, 32, 0, stream>>>(w.state, level, count, (uint32_t *)out););
	return cudaGetLastError();
}

} // namespace svo
