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
// GB300 design, in three stages:
//   dense   depths 1..D (D = min(L-1, 9); 8^9 bits = 16 MB stays in L2): one sweep over the fragments sets
//           the occupancy bits of depth D (warp-deduplicated atomicOr), coarser depths are OR-reductions of
//           8-bit groups, one single-pass look-back scan of popcounts over all depths gives every grank,
//           and one pass writes all interior words of depths 1..D;
//   sparse  depths D+1..L-1 (only when L > 10): the reference's tag / prefix-sum alloc per level with a
//           per-fragment cached node index (4 B per fragment), so tag reads one parent word;
//   leaf    one sweep: each fragment finds its leaf word and adds its colour to a packed 64-bit
//           accumulator (r, g, b, n in 16-bit fields: one atomic per fragment); a finalize pass writes
//           every leaf word as 0xC0000000 | min(n,63)<<24 | floor(sum/n) (the channel-wise integer mean).
//           The packing is exact up to 257 fragments per voxel; a voxel beyond that raises a flag and a
//           flag-gated second leaf pass redoes the colours with 2 x 64-bit accumulators per voxel.
// Sizes stay on the device (BuildState): no host round trip inside a stage.
#include "common.cuh"
#include "svo_internal.h"

namespace svo {

constexpr int kTPB = 256;
constexpr int kAllocIPT = 8;
constexpr int kAllocTile = kTPB * kAllocIPT;
constexpr int kScanIPT = 8;
constexpr int kScanTile = kTPB * kScanIPT;
constexpr unsigned long long kLeafOne = 1ull << 48;

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
// Sets the depth-D occupancy bit of every fragment.  Per warp, fragments that fall in the same bitmap
// word are merged first (match + reduce), so one atomicOr covers them.
__global__ void __launch_bounds__(kTPB) dense_mark(const uint64_t *__restrict__ frags, uint32_t n, uint32_t level,
                                                   DenseView dv) {
	const uint32_t shift = level - dv.D;
	uint32_t *bits = dv.bits + dv.off[dv.D];
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	for (uint64_t f = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; f < ((n + 31ull) & ~31ull); f += stride) {
		uint32_t word = 0xffffffffu, bit = 0;
		if (f < n) {
			uint32_t x, y, z;
			frag_xyz(__ldcs(frags + f), x, y, z);
			const uint32_t m = morton(x, y, z, shift);
			word = m >> 5;
			bit = 1u << (m & 31);
		}
		const uint32_t peers = __match_any_sync(kFullMask, word);
		const uint32_t merged = __reduce_or_sync(peers, bit);
		if (word != 0xffffffffu && lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicOr(bits + word, merged);
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
// follow.  When depth D+1 is the leaf depth, depth-D cells are skipped: the leaf finalize writes those
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

// ------------------------------------------------------------------------------------------ tag (sparse levels, leaf)
enum TagMode { kTagInterior = 0, kTagLeaf = 1, kTagLeafWide = 2 };

template <int MODE>
SVO_DEV void tag_one(uint64_t frag, uint32_t &node, uint32_t level, uint32_t depth, bool parent_dense,
                     const DenseView &dv, uint32_t *__restrict__ pool, unsigned long long *__restrict__ acc,
                     uint32_t leaf_begin, uint32_t leaf_num, uint32_t *status) {
	uint32_t x, y, z;
	frag_xyz(frag, x, y, z);
	uint32_t idx;
	if (parent_dense)
		idx = dense_child_word(dv, x, y, z, level, depth);
	else
		idx = (pool[node] & 0x3fffffffu) + octant_at(x, y, z, level - depth);
	if (MODE == kTagInterior) {
		if ((pool[idx] & 0x80000000u) == 0u) pool[idx] = 0x80000000u;
		node = idx;
	} else {
		const uint32_t slot = idx - leaf_begin;
		if (slot >= leaf_num) return;
		const uint32_t rgb = (uint32_t)(frag >> 32);
		const uint32_t r = rgb & 0xffu, g = (rgb >> 8) & 0xffu, b = (rgb >> 16) & 0xffu;
		if (MODE == kTagLeaf) {
			const unsigned long long v = r | ((unsigned long long)g << 16) | ((unsigned long long)b << 32) | kLeafOne;
			const unsigned long long old = atomicAdd(acc + slot, v);
			if ((old >> 48) >= 257ull) atomicOr(status, kStatusLeafWide); // the packed sums may have carried
		} else {
			atomicAdd(acc + 2 * (size_t)slot, r | ((unsigned long long)g << 32));
			atomicAdd(acc + 2 * (size_t)slot + 1, b | (1ull << 32));
		}
	}
}

template <int MODE>
__global__ void __launch_bounds__(kTPB) build_tag(const uint64_t *__restrict__ frags, uint32_t n, uint32_t level,
                                                  uint32_t depth, uint32_t *__restrict__ pool,
                                                  uint32_t *__restrict__ cache, unsigned long long *__restrict__ acc,
                                                  DenseView dv, BuildState *state, int vec_ok) {
	const uint32_t status = state->status;
	if (status & kStatusCapacity) return;
	if (MODE == kTagLeafWide && !(status & kStatusLeafWide)) return;
	const bool parent_dense = depth == 1 || depth - 1 <= dv.D;
	const bool store_cache = MODE == kTagInterior;
	const uint32_t leaf_begin = MODE != kTagInterior ? state->lv[depth].begin : 0u;
	const uint32_t leaf_num = MODE != kTagInterior ? state->lv[depth].num : 0u;
	uint32_t *st = &state->status;
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t nq = (n + 3ull) / 4ull;
	for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
		const uint64_t f0 = q * 4;
		if (vec_ok && f0 + 4 <= n) {
			const ulonglong2 a = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0));
			const ulonglong2 b = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0 + 2));
			uint4 c = make_uint4(0, 0, 0, 0);
			if (!parent_dense) c = __ldcs(reinterpret_cast<const uint4 *>(cache + f0));
			tag_one<MODE>(a.x, c.x, level, depth, parent_dense, dv, pool, acc, leaf_begin, leaf_num, st);
			tag_one<MODE>(a.y, c.y, level, depth, parent_dense, dv, pool, acc, leaf_begin, leaf_num, st);
			tag_one<MODE>(b.x, c.z, level, depth, parent_dense, dv, pool, acc, leaf_begin, leaf_num, st);
			tag_one<MODE>(b.y, c.w, level, depth, parent_dense, dv, pool, acc, leaf_begin, leaf_num, st);
			if (store_cache) __stcs(reinterpret_cast<uint4 *>(cache + f0), c);
		} else {
			for (uint64_t f = f0; f < f0 + 4 && f < n; ++f) {
				uint32_t c = parent_dense ? 0u : cache[f];
				tag_one<MODE>(frags[f], c, level, depth, parent_dense, dv, pool, acc, leaf_begin, leaf_num, st);
				if (store_cache) cache[f] = c;
			}
		}
	}
}

// Leaf sweep: 4 fragments per thread, in phases so their loads and atomics overlap: fragment loads,
// leaf-word lookups (dense ranks or the cached parent), then the four accumulator updates.
__global__ void __launch_bounds__(kTPB) build_leaf(const uint64_t *__restrict__ frags, uint32_t n, uint32_t level,
                                                   const uint32_t *__restrict__ pool,
                                                   const uint32_t *__restrict__ cache,
                                                   unsigned long long *__restrict__ acc, DenseView dv,
                                                   BuildState *state) {
	const uint32_t status = state->status;
	if (status & kStatusCapacity) return;
	const bool parent_dense = level == 1 || level - 1 <= dv.D;
	const uint32_t leaf_begin = state->lv[level].begin, leaf_num = state->lv[level].num;
	uint32_t *st = &state->status;
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t nq = (n + 3ull) / 4ull;
	for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
		const uint64_t f0 = q * 4;
		uint64_t f[4];
		uint32_t c[4] = {0u, 0u, 0u, 0u};
		const bool full = f0 + 4 <= n && ((uintptr_t)(frags + f0) & 15u) == 0;
		if (full) {
			const ulonglong2 a = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0));
			const ulonglong2 b = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0 + 2));
			f[0] = a.x, f[1] = a.y, f[2] = b.x, f[3] = b.y;
			if (!parent_dense) {
				const uint4 cc = __ldcs(reinterpret_cast<const uint4 *>(cache + f0));
				c[0] = cc.x, c[1] = cc.y, c[2] = cc.z, c[3] = cc.w;
			}
		} else {
#pragma unroll
			for (int k = 0; k < 4; ++k) {
				f[k] = f0 + k < n ? frags[f0 + k] : 0ull;
				c[k] = (!parent_dense && f0 + k < n) ? cache[f0 + k] : 0u;
			}
		}
		uint32_t slot[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			uint32_t x, y, z;
			frag_xyz(f[k], x, y, z);
			const uint32_t idx = parent_dense ? dense_child_word(dv, x, y, z, level, level)
			                                  : (__ldg(pool + c[k]) & 0x3fffffffu) + octant_at(x, y, z, 0);
			slot[k] = f0 + k < n ? idx - leaf_begin : 0xffffffffu;
		}
		unsigned long long old[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			old[k] = 0ull;
			if (slot[k] < leaf_num) {
				const uint32_t rgb = (uint32_t)(f[k] >> 32);
				const unsigned long long v = (rgb & 0xffu) | ((unsigned long long)((rgb >> 8) & 0xffu) << 16) |
				                             ((unsigned long long)((rgb >> 16) & 0xffu) << 32) | kLeafOne;
				old[k] = atomicAdd(acc + slot[k], v);
			}
		}
		if ((old[0] >> 48) >= 257ull || (old[1] >> 48) >= 257ull || (old[2] >> 48) >= 257ull || (old[3] >> 48) >= 257ull)
			atomicOr(st, kStatusLeafWide); // a packed sum may have carried: the wide pass redoes the colours
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
			if (!next_is_leaf) { // the next depth's init; leaf blocks are written whole by the finalize
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

// ------------------------------------------------------------------------------------------ leaf finalize
SVO_DEV uint32_t leaf_word(uint32_t n, uint32_t sr, uint32_t sg, uint32_t sb) {
	return 0xC0000000u | (min(n, 63u) << 24) | ((sb / n) << 16) | ((sg / n) << 8) | (sr / n);
}

// Writes every leaf word (empty ones as 0) from the packed accumulators; the packed pass is skipped
// when the wide pass must redo the colours, and the wide pass only runs then.
template <bool WIDE>
__global__ void __launch_bounds__(kTPB) build_finalize(uint32_t *__restrict__ pool,
                                                       const unsigned long long *__restrict__ acc, BuildState *state,
                                                       uint32_t level) {
	__shared__ uint32_t s_warp[kTPB / 32];
	__shared__ uint32_t s_skip;
	if (threadIdx.x == 0) {
		const uint32_t st = state->status;
		s_skip = (st & kStatusCapacity) || (WIDE ? !(st & kStatusLeafWide) : (st & kStatusLeafWide));
	}
	__syncthreads();
	if (s_skip) return;
	const LevelInfo li = state->lv[level];
	uint32_t leaves = 0;
	// 4 leaf words per thread (num and begin are multiples of 8: 16-byte stores, 32-byte packed loads)
	for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < li.num / 4u; g += gridDim.x * blockDim.x) {
		uint32_t word[4];
#pragma unroll
		for (int j = 0; j < 4; ++j) word[j] = 0u;
		if (WIDE) {
			const ulonglong2 *a = reinterpret_cast<const ulonglong2 *>(acc) + 4u * g;
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				const ulonglong2 v = a[j];
				const uint32_t n = (uint32_t)(v.y >> 32);
				if (n) word[j] = leaf_word(n, (uint32_t)v.x, (uint32_t)(v.x >> 32), (uint32_t)v.y);
			}
		} else {
			const ulonglong2 *a = reinterpret_cast<const ulonglong2 *>(acc) + 2u * g;
			const ulonglong2 v0 = __ldcs(a), v1 = __ldcs(a + 1);
			const unsigned long long v[4] = {v0.x, v0.y, v1.x, v1.y};
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				const uint32_t n = (uint32_t)(v[j] >> 48);
				if (n)
					word[j] = leaf_word(n, (uint32_t)(v[j] & 0xffffu), (uint32_t)((v[j] >> 16) & 0xffffu),
					                    (uint32_t)((v[j] >> 32) & 0xffffu));
			}
		}
		reinterpret_cast<uint4 *>(pool + li.begin)[g] = make_uint4(word[0], word[1], word[2], word[3]);
#pragma unroll
		for (int j = 0; j < 4; ++j) leaves += word[j] != 0u;
	}
	leaves = warp_sum(leaves);
	if (lane_id() == 0) s_warp[threadIdx.x >> 5] = leaves;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t t = 0;
		for (int i = 0; i < kTPB / 32; ++i) t += s_warp[i];
		atomicAdd(&state->leaves, t);
		if (blockIdx.x == 0) state->range_words = li.begin + li.num;
	}
}

// Zeroes the packed leaf accumulators of the leaf depth; a leaf range larger than the accumulator
// array is a capacity error.
__global__ void build_leaf_zero(unsigned long long *acc, uint64_t acc_slots, BuildState *state, uint32_t level) {
	if (state->status & kStatusCapacity) return;
	const uint32_t num = state->lv[level].num;
	if (num > acc_slots) {
		if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&state->status, kStatusCapacity);
		return;
	}
	ulonglong2 *a = reinterpret_cast<ulonglong2 *>(acc);
	for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < num / 2u; k += (uint64_t)gridDim.x * blockDim.x)
		a[k] = make_ulonglong2(0ull, 0ull);
}

// Zeroes the wide accumulators (only when a voxel overflowed the packed ones).
__global__ void build_wide_zero(unsigned long long *acc, BuildState *state, uint32_t level) {
	if (!(state->status & kStatusLeafWide) || (state->status & kStatusCapacity)) return;
	const uint32_t num = state->lv[level].num;
	for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < 2ull * num; k += (uint64_t)gridDim.x * blockDim.x)
		acc[k] = 0ull;
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
	out[sizeof(svo_build_info) / 4] = state->status & ~kStatusLeafWide; // the wide pass resolved it
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

uint64_t build_leaf_slot_bound(uint32_t count, uint32_t level, uint64_t capacity) {
	uint64_t per = 1;
	for (uint32_t i = 1; i < level; ++i) per = per >= (1ull << 40) ? per : per * 8;
	uint64_t b = 8 * (per < count ? per : (uint64_t)count);
	if (b < 8) b = 8;
	return b < capacity ? b : capacity;
}

// Layout: state | descriptors | dense bitmaps | dense prefix | node cache | packed leaf accumulators
// (leaf_slots x 8 B) | wide leaf accumulators (leaf_slots x 16 B).  leaf_slots = 0 lays out the
// interior part only (the accumulators are then placed separately by the caller).
void build_workspace_layout(void *ws, uint32_t count, uint32_t level, uint64_t capacity, uint64_t leaf_slots,
                            BuildWorkspace &w) {
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
	w.cache = (uint32_t *)take(level > D + 1 ? (size_t)count * 4 + 16 : 16);
	w.interior_bytes = off;
	w.leaf_slots = leaf_slots;
	w.acc = leaf_slots ? (unsigned long long *)take(leaf_slots * 8 + 16) : nullptr;
	w.acc_wide = leaf_slots ? (unsigned long long *)take(leaf_slots * 16 + 16) : nullptr;
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
	if (e != cudaSuccess) return e;
	const int sms = device_sm_count();
	const uint32_t D = w.dv.D;
	SVO_LAUNCH("build_init", stream, build_init<<<1, 256, 0, stream>>>(w.state););
	if (D >= 1) {
		SVO_LAUNCH("dense_mark", stream,
		           dense_mark<<<grid_for(count, kTPB, (uint32_t)sms * 16), kTPB, 0, stream>>>(frags, count, level, w.dv););
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
	const int vec_ok = ((uintptr_t)frags & 15u) == 0;
	const uint32_t tag_blocks = grid_for(((uint64_t)count + 3) / 4, kTPB, (uint32_t)sms * 16);
	for (uint32_t depth = D + 1; depth < level; ++depth) {
		SVO_LAUNCH("build_tag", stream,
		           build_tag<kTagInterior><<<tag_blocks, kTPB, 0, stream>>>(frags, count, level, depth, pool, w.cache,
		                                                                    w.acc, w.dv, w.state, vec_ok););
		SVO_LAUNCH("build_alloc", stream,
		           build_alloc<<<(uint32_t)sms * 4, kTPB, 0, stream>>>(pool, capacity, depth, level, w.state, w.descs););
	}
	return cudaGetLastError();
}

cudaError_t build_launch_leaf(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool,
                              const BuildWorkspace &w, bool wide, cudaStream_t stream) {
	const int sms = device_sm_count();
	const int vec_ok = ((uintptr_t)frags & 15u) == 0;
	const uint32_t tag_blocks = grid_for(((uint64_t)count + 3) / 4, kTPB, (uint32_t)sms * 16);
	if (w.acc) {
		SVO_LAUNCH("build_leaf_zero", stream,
		           build_leaf_zero<<<(uint32_t)sms * 8, kTPB, 0, stream>>>(w.acc, w.leaf_slots, w.state, level););
		SVO_LAUNCH("build_leaf", stream,
		           build_leaf<<<tag_blocks, kTPB, 0, stream>>>(frags, count, level, pool, w.cache, w.acc, w.dv, w.state););
		SVO_LAUNCH("build_finalize", stream,
		           build_finalize<false><<<(uint32_t)sms * 8, kTPB, 0, stream>>>(pool, w.acc, w.state, level););
	}
	if (wide && w.acc_wide) {
		// exact colours for voxels with more than 257 fragments; these launches return at once otherwise
		SVO_LAUNCH("build_wide_zero", stream,
		           build_wide_zero<<<(uint32_t)sms * 4, kTPB, 0, stream>>>(w.acc_wide, w.state, level););
		SVO_LAUNCH("build_leaf_wide", stream,
		           build_tag<kTagLeafWide><<<tag_blocks, kTPB, 0, stream>>>(frags, count, level, level, pool, w.cache,
		                                                                    w.acc_wide, w.dv, w.state, vec_ok););
		SVO_LAUNCH("build_finalize_wide", stream,
		           build_finalize<true><<<(uint32_t)sms * 8, kTPB, 0, stream>>>(pool, w.acc_wide, w.state, level););
	}
	return cudaGetLastError();
}

cudaError_t build_launch_export(const BuildWorkspace &w, uint32_t level, uint32_t count, void *out,
                                cudaStream_t stream) {
	SVO_LAUNCH("build_export", stream, build_export<<<1, 32, 0, stream>>>(w.state, level, count, (uint32_t *)out););
	return cudaGetLastError();
}

} // namespace svo
