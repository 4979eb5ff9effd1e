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
//   dense   depths 1..D (D = min(L-1, 9), or 10 for L >= 11 from 2^24 fragments; 8^9 bits = 16 MB stays in
//           L2, 8^10 bits = 128 MB about fills it): one sweep over the fragments sets
//           the occupancy bits of depth D (run-merged atomicOr), coarser depths are OR-reductions of
//           8-bit groups, one single-pass look-back scan of popcounts over all depths gives every grank,
//           and one pass writes all interior words of depths 1..D;
//   buckets the same sweep counts fragments per bucket (16^3 voxels while the leaf parents are dense,
//           L - 1 <= D; 32^3 voxels otherwise); a look-back scan and one scatter copy the fragments into
//           bucket order (8 B each: a leaf item, slot << 32 | rgb, when the leaf parents are dense, else
//           the fragment), which every later sweep reads;
//   sparse  depths D+1..L-1 (only when L > 10): the reference's tag / prefix-sum alloc per level with a
//           per-fragment cached node index (4 B per fragment), so tag reads one parent word; after the
//           last depth, the pass that measures each bucket's leaf span turns its fragments into leaf items;
//   leaf    one block per leaf window (4096 consecutive words of the leaf range) at a time: the window's
//           items come from the run of buckets whose leaf spans meet it (each item is read at most
//           twice), the block accumulates their colours in shared memory (r, g, b, n in 16-bit fields,
//           two 32-bit shared atomics per item) and writes every leaf word of the window,
//           0xC0000000 | min(n,63)<<24 | floor(sum/n) (the channel-wise integer mean), with no
//           accumulator array in device memory.  The packing is exact up to 257 fragments per voxel; a
//           window where a voxel exceeds that is redone with exact 64-bit sums in the same block.
// Sizes stay on the device (BuildState): no host round trip inside a stage.
#include <cstring>

#include "common.cuh"
#include "svo_internal.h"

namespace svo {

constexpr int kTPB = 256;
constexpr int kAllocIPT = 32; // words per thread of an alloc tile (large tiles: short look-back distances)
static_assert(kAllocIPT == 32, "an alloc thread's words are one word of the tag bitmap");
constexpr int kAllocTile = kTPB * kAllocIPT;
constexpr int kScanIPT = 8;
constexpr int kScanTile = kTPB * kScanIPT;

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

// The fragment sweeps spread coordinates through a 1024-entry table in shared memory (three loads
// instead of three 4-step bit spreads); the table holds spread3(i) for every 10-bit i.
constexpr uint32_t kSpreadEntries = 1024;
SVO_DEV void spread_table_init(uint32_t *tab) {
	for (uint32_t i = threadIdx.x; i < kSpreadEntries; i += blockDim.x) tab[i] = spread3(i);
	__syncthreads();
}
SVO_DEV uint32_t morton_tab(const uint32_t *tab, uint32_t x, uint32_t y, uint32_t z, uint32_t shift) {
	return tab[(x >> shift) & 0x3ffu] | (tab[(y >> shift) & 0x3ffu] << 1) | (tab[(z >> shift) & 0x3ffu] << 2);
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

// ------------------------------------------------------------------------------------------ batches
// Every stage runs over all meshes of a batch in one launch.  Work items are flat over the batch
// (fragments, buckets, dense_write items) and find their mesh by a binary search over the [M+1] offsets;
// a single build (B = false) takes its one mesh by value and searches nothing.
template <typename T> SVO_DEV uint32_t mesh_search(const T *__restrict__ a, uint32_t M, T x) {
	uint32_t lo = 0, hi = M; // a[lo] <= x < a[hi]
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (__ldg(a + mid) <= x)
			lo = mid;
		else
			hi = mid;
	}
	return lo;
}

// The mesh of fragment f in a sweep pass whose fragments start at `first` (f >= first), given m0, the mesh
// of `first` (searched once per pass: a pass covers a few runs of 32 consecutive fragments, which rarely
// cross a mesh boundary).  a = frag_base, so a[M] is the batch total and the step ends there.
SVO_DEV uint32_t mesh_from(const unsigned long long *__restrict__ a, uint32_t m0, unsigned long long f) {
	while (__ldg(a + m0 + 1) <= f) ++m0;
	return m0;
}

template <bool B> SVO_DEV BuildMesh mesh_at(const BuildBatch &bb, uint32_t m) {
	if constexpr (B)
		return bb.table[m];
	else
		return bb.one;
}

template <bool B> SVO_DEV uint32_t batch_size(const BuildBatch &bb) { return B ? bb.M : 1u; }

// Internal bounds checks, compiled in with -DSVO_CHECKED: a failed check records its id (first one
// wins, in the batch state's pad word), sets kStatusCheck and skips the access it guards.
#ifdef SVO_CHECKED
SVO_DEV bool check_ok(bool ok, uint32_t id, BuildState *g) {
	if (!ok) {
		atomicCAS(&g->pad, 0u, id);
		atomicOr(&g->status, kStatusCheck);
	}
	return ok;
}
#define SVO_CHECK(cond, id, g) check_ok((cond), (id), (g))
#define SVO_CHECK_FAIL(id, g) (void)check_ok(false, (id), (g))
#else
#define SVO_CHECK(cond, id, g) true
#define SVO_CHECK_FAIL(id, g) ((void)0)
#endif

// A fragment of a level-L octree has every coordinate below 2^L; the build skips any other (a caller's
// malformed list) and reports it, and no later stage of the build (or batch) runs on it.
// Conditions of the batch (or single build) state after which no later stage may trust the scans or the
// fragment list: every stage that writes through scanned offsets skips its work and the call reports it.
constexpr uint32_t kStatusAbort = kStatusTimeout | kStatusBadFragment;

SVO_DEV bool frag_in_level(uint32_t x, uint32_t y, uint32_t z, uint32_t level) { return ((x | y | z) >> level) == 0u; }
SVO_DEV void flag_bad_fragment(BuildState *state, BuildState *g) {
	atomicOr(&state->status, kStatusBadFragment);
	if (g != state) atomicOr(&g->status, kStatusBadFragment);
}

// ------------------------------------------------------------------------------------------ init
// The scratch a build zeroes before its first sweep (scan descriptors, dense bitmaps, bucket counters):
// up to four 16-byte-aligned ranges whose sizes are multiples of 4 bytes.
struct ClearList {
	void *p[4];
	size_t bytes[4];
};

// Zeroes the ranges (every block, grid-stride, 16-byte stores), and block m < M clears mesh m's state
// (block 0 also the batch-wide state of a batch): one launch instead of a memset per range.
template <bool B> __global__ void build_init(BuildBatch bb, BuildState *gstate, ClearList cl) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (uint64_t)gridDim.x * blockDim.x;
#pragma unroll
	for (int r = 0; r < 4; ++r) {
		uint4 *d4 = reinterpret_cast<uint4 *>(cl.p[r]);
		const uint64_t n4 = cl.bytes[r] / 16;
		for (uint64_t i = tid; i < n4; i += nth) d4[i] = make_uint4(0u, 0u, 0u, 0u);
		uint32_t *d = reinterpret_cast<uint32_t *>(cl.p[r]);
		for (uint64_t i = 4 * n4 + tid; i < cl.bytes[r] / 4; i += nth) d[i] = 0u;
	}
	if (blockIdx.x >= batch_size<B>(bb)) return;
	BuildState *state = mesh_at<B>(bb, blockIdx.x).state;
	uint32_t *s = reinterpret_cast<uint32_t *>(state);
	for (uint32_t k = threadIdx.x; k < sizeof(BuildState) / 4; k += blockDim.x) s[k] = 0u;
	if (B && blockIdx.x == 0) {
		uint32_t *g = reinterpret_cast<uint32_t *>(gstate);
		for (uint32_t k = threadIdx.x; k < sizeof(BuildState) / 4; k += blockDim.x) g[k] = 0u;
	}
	__syncthreads();
	if (threadIdx.x == 0) state->lv[1] = LevelInfo{0u, 8u, 0u, 0u};
}

// ------------------------------------------------------------------------------------------ dense stage
// The fragment sweeps (dense_mark, bucket_scatter) take kSweepRuns warp-sized runs of fragments per warp
// and pass, loading all of them before any is processed: each fragment's work is a short dependent chain
// (load, bitmap lookups, one atomic per group of a warp), so independent loads in flight set the rate.
constexpr uint32_t kSweepRuns = 4;   // dense_mark
constexpr uint32_t kScatterRuns = 2; // bucket_scatter (more state per fragment: fewer runs, more warps)

// First run of warp w's pass and the run stride of a sweep taking R runs per warp and pass.
template <uint32_t R> SVO_DEV uint64_t sweep_first_run() {
	return ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * R;
}
template <uint32_t R> SVO_DEV uint64_t sweep_run_stride() { return (uint64_t)gridDim.x * (blockDim.x >> 5) * R; }

// Sets the depth-D occupancy bit of every fragment and counts the fragments of every bucket.  Per warp,
// consecutive fragments that fall in the same bitmap word (or bucket) are merged first, so one atomic
// covers them (a triangle's fragments are consecutive in the list).  Bitmap words and buckets are
// numbered over the whole batch, so merging never mixes meshes.
template <bool B>
__global__ void __launch_bounds__(kTPB) dense_mark(const uint64_t *__restrict__ frags, uint64_t n, BuildBatch bb,
                                                   uint32_t *__restrict__ bcount) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_spread[kSpreadEntries];
	spread_table_init(s_spread);
	const uint64_t runs = (n + 31ull) >> 5;
	const uint32_t lane = lane_id();
	for (uint64_t r = sweep_first_run<kSweepRuns>(); r < runs; r += sweep_run_stride<kSweepRuns>()) {
		const uint32_t m0 = B ? mesh_search(bb.frag_base, bb.M, (unsigned long long)(r << 5)) : 0u;
		uint64_t fr[kSweepRuns];
#pragma unroll
		for (uint32_t k = 0; k < kSweepRuns; ++k) {
			const uint64_t f = ((r + k) << 5) + lane;
			fr[k] = f < n ? __ldcs(frags + f) : 0ull;
		}
#pragma unroll
		for (uint32_t k = 0; k < kSweepRuns; ++k) {
			const uint64_t f = ((r + k) << 5) + lane;
			uint32_t word = 0xffffffffu, bit = 0, key = 0xffffffffu;
			if (f < n) {
				const uint32_t mi = B ? mesh_from(bb.frag_base, m0, f) : 0u;
				const BuildMesh md = mesh_at<B>(bb, mi);
				uint32_t x, y, z;
				frag_xyz(fr[k], x, y, z);
				const uint32_t D = md.dv.D;
				if (!frag_in_level(x, y, z, md.level)) {
					flag_bad_fragment(md.state, bb.gstate);
				} else if (D >= 1) {
					const uint32_t shift = md.level - D;
					const uint32_t m = morton_tab(s_spread, x, y, z, shift);
					word = md.mark_word + (m >> 5);
					bit = 1u << (m & 31);
					key = md.bucket_base + (m >> (3 * (md.bshift - shift))); // a prefix of the depth-D code
				} else {
					key = md.bucket_base + morton_tab(s_spread, x, y, z, md.bshift);
				}
				if (word != 0xffffffffu && !SVO_CHECK(word < bb.dense_total, 1u, bb.gstate)) word = 0xffffffffu, bit = 0;
				if (key != 0xffffffffu && !SVO_CHECK(key < bb.nb_total, 2u, bb.gstate)) key = 0xffffffffu;
			}
			uint32_t first, last;
			lane_run(word, lane, first, last);
			const uint32_t merged = run_or(bit, lane, last);
			// fragments per bucket, for the bucketed copy: equal bitmap words have equal bucket keys (the key
			// is a coarser prefix of the same Morton code, and both are numbered over the batch), so a
			// word's run adds its length to its bucket; keys without a word (no dense depth) run alone
			if (word != 0xffffffffu && lane == first) {
				atomicOr(bb.dense_bits + word, merged);
				if (key != 0xffffffffu) atomicAdd(bcount + key, last - first + 1u);
			}
			const bool loose = word == 0xffffffffu && key != 0xffffffffu;
			if (__any_sync(kFullMask, loose)) {
				lane_run(loose ? key : 0xffffffffu, lane, first, last);
				if (loose && lane == first) atomicAdd(bcount + key, last - first + 1u);
			}
		}
	}
}

// Bitmaps of depths D-1 .. 1 from depth D in one launch (bit p of depth d = byte p of depth d+1 is
// nonzero).  Work items are chunks of kReduceChunk words of a mesh's depth-D bitmap, listed over the batch
// (reduce_base) and taken grid-stride, so no block is spent on a mesh without that chunk.  A block
// reduces its chunk level by level in shared memory: the words of a level that the chunk covers whole are
// written directly, and once the chunk's image is smaller than a word its bits are ORed into place
// (atomicOr), so higher levels collect every chunk's contribution.  The bitmaps were zeroed before the
// build.
constexpr uint32_t kReduceChunk = 8192;

SVO_DEV uint32_t byte_bits(uint32_t v) { // bit j = byte j of v is nonzero
	return (uint32_t)((v & 0xffu) != 0u) | ((uint32_t)((v & 0xff00u) != 0u) << 1) |
	       ((uint32_t)((v & 0xff0000u) != 0u) << 2) | ((uint32_t)((v & 0xff000000u) != 0u) << 3);
}

// One chunk (called by the whole block; D >= 2).
SVO_DEV void reduce_chunk(const DenseView &dv, uint32_t chunk_idx, uint32_t (*s_buf)[kReduceChunk / 8]) {
	const uint32_t D = dv.D;
	const uint32_t words_D = (1u << (3 * D)) / 32u; // D >= 2: at least 2 words
	const uint32_t chunk = min(words_D, kReduceChunk);
	const uint32_t first = chunk_idx * chunk;
	uint32_t nbits = chunk * 32u, bit0 = first * 32u; // the chunk's image at the current level
	const uint32_t *src = dv.bits + dv.off[D] + first;
	bool src_shared = false;
	int cur = 0;
	for (uint32_t c = D; c >= 2; --c) {
		uint32_t *parent = dv.bits + dv.off[c - 1];
		const uint32_t nb_out = nbits / 8u, out0 = bit0 / 8u;
		if (nb_out >= 32u) { // whole words, owned by this block
			const uint32_t nw = nb_out / 32u;
			for (uint32_t w = threadIdx.x; w < nw; w += blockDim.x) {
				uint32_t out = 0;
				if (src_shared) {
#pragma unroll
					for (int i = 0; i < 8; ++i) out |= byte_bits(src[8 * w + i]) << (4 * i);
				} else {
					const uint4 *c4 = reinterpret_cast<const uint4 *>(src + 8 * w);
					const uint4 p = __ldcs(c4), q = __ldcs(c4 + 1);
					const uint32_t v[8] = {p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w};
#pragma unroll
					for (int i = 0; i < 8; ++i) out |= byte_bits(v[i]) << (4 * i);
				}
				parent[out0 / 32u + w] = out;
				s_buf[cur][w] = out;
			}
		} else { // fewer than 32 bits: OR them into the parent word
			if (threadIdx.x == 0) {
				uint32_t out = 0;
				for (uint32_t p = 0; p < nb_out; ++p) out |= (uint32_t)(((src[p >> 2] >> (8 * (p & 3u))) & 0xffu) != 0u) << p;
				if (out) atomicOr(parent + out0 / 32u, out << (out0 % 32u));
				s_buf[cur][0] = out;
			}
		}
		__syncthreads();
		src = s_buf[cur];
		src_shared = true;
		cur ^= 1;
		nbits = nb_out, bit0 = out0;
		if (nbits < 8u) { // the chunk's image is one bit or less: it ORs one bit into each level above
			const bool any = s_buf[cur ^ 1][0] != 0u;
			if (threadIdx.x == 0 && any)
				for (uint32_t d = c - 2; d >= 1; --d) {
					bit0 /= 8u;
					atomicOr(dv.bits + dv.off[d] + bit0 / 32u, 1u << (bit0 % 32u));
				}
			return;
		}
	}
}

uint32_t dense_reduce_chunks(uint32_t D) {
	if (D < 2) return 0;
	const uint32_t words_D = (1u << (3 * D)) / 32u;
	return (words_D + kReduceChunk - 1) / kReduceChunk;
}

template <bool B> __global__ void __launch_bounds__(256) dense_reduce(BuildBatch bb) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_buf[2][kReduceChunk / 8];
	const uint32_t total = bb.reduce_total;
	for (uint32_t item = blockIdx.x; item < total; item += gridDim.x) {
		const uint32_t mi = B ? mesh_search(bb.reduce_base, bb.M, item) : 0u;
		const uint32_t chunk_idx = item - (B ? __ldg(bb.reduce_base + mi) : 0u);
		const DenseView dv = mesh_at<B>(bb, mi).dv;
		reduce_chunk(dv, chunk_idx, s_buf);
		__syncthreads(); // s_buf is reused by the next item
	}
}

// Exclusive prefix of popcounts over the concatenated bitmaps of depths 1..D, segmented per mesh (a
// mesh's region is whole tiles, the first of which starts a segment); prefix[W] = occupied cells of the
// mesh for its region of W bitmap words (the padding words are zero).  Persistent grid, tiles claimed in
// order by ticket.  A tile is kDenseTile words, 32 per thread read and written as 16-byte vectors: large
// tiles keep the number of tiles in flight (and so the look-back distance) small against the work.
constexpr int kDenseIPT = 32;
constexpr uint32_t kDenseTile = kTPB * kDenseIPT;
static_assert(kDenseTile == kBuildScanTile, "dense regions are padded to whole scan tiles");

template <bool B>
__global__ void __launch_bounds__(kTPB) dense_scan(BuildBatch bb, uint32_t total_words, BuildState *gstate,
                                                   unsigned long long *descs) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kTPB / 32 + 1];
	__shared__ uint32_t s_prefix;
	const uint32_t *bits = bb.dense_bits;
	uint32_t *prefix = bb.dense_prefix;
	const uint32_t ntiles = total_words / kDenseTile; // regions are whole tiles
	// the pending tile (pipelined as the voxelize scans: aggregate published, look-back and prefixes one
	// tile later); its word popcounts (at most 32 each) kept four to a register
	uint32_t p_tile = 0xffffffffu, p_run = 0, p_total = 0, p_c[kDenseIPT / 4];
	for (;;) {
		if (threadIdx.x == 0) s_tile = atomicAdd(&gstate->tiles[0], 1u);
		__syncthreads();
		const uint32_t tile = s_tile;
		__syncthreads();
		uint32_t c[kDenseIPT / 4], run = 0, total = 0;
		if (tile < ntiles) {
			const uint32_t first = tile * kDenseTile;
			bool seg_start = tile == 0;
			if constexpr (B) seg_start = __ldg(bb.dense_base + mesh_search(bb.dense_base, bb.M, first)) == first;
			const uint4 *src = reinterpret_cast<const uint4 *>(bits + first + threadIdx.x * kDenseIPT);
			uint32_t local = 0;
#pragma unroll
			for (int k = 0; k < kDenseIPT / 4; ++k) {
				const uint4 v = __ldcs(src + k);
				const uint32_t a = __popc(v.x), b = __popc(v.y), d = __popc(v.z), e = __popc(v.w);
				c[k] = a | (b << 8) | (d << 16) | (e << 24);
				local += a + b + d + e;
			}
			run = block_exclusive_sum<uint32_t, kTPB>(local, s_warp, total);
			if (threadIdx.x == 0) tile_publish_aggregate(descs, tile, 15u, total, seg_start);
		}
		if (p_tile != 0xffffffffu) {
			if (threadIdx.x < 32) {
				bool seg_start = p_tile == 0;
				if constexpr (B) {
					const uint32_t first = p_tile * kDenseTile;
					seg_start = __ldg(bb.dense_base + mesh_search(bb.dense_base, bb.M, first)) == first;
				}
				const uint32_t p = (uint32_t)tile_lookback_warp(descs, p_tile, 15u, p_total, &gstate->status, seg_start, true);
				if (threadIdx.x == 0) s_prefix = p;
			}
			__syncthreads();
			uint32_t r = p_run + s_prefix;
			uint4 *dst = reinterpret_cast<uint4 *>(prefix + p_tile * kDenseTile + threadIdx.x * kDenseIPT);
#pragma unroll
			for (int k = 0; k < kDenseIPT / 4; ++k) {
				uint4 o;
				o.x = r, r += p_c[k] & 0xffu;
				o.y = r, r += (p_c[k] >> 8) & 0xffu;
				o.z = r, r += (p_c[k] >> 16) & 0xffu;
				o.w = r, r += p_c[k] >> 24;
				dst[k] = o;
			}
			__syncthreads();
		}
		if (tile >= ntiles) break;
		p_tile = tile, p_run = run, p_total = total;
#pragma unroll
		for (int k = 0; k < kDenseIPT / 4; ++k) p_c[k] = c[k];
	}
}

// Level ranges of depths 1..D+1 from the scanned counts (BuildState.lv as the sparse stage keeps it);
// one thread per mesh.
template <bool B> __global__ void dense_finish(BuildBatch bb) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	for (uint32_t mi = blockIdx.x * blockDim.x + threadIdx.x; mi < batch_size<B>(bb); mi += gridDim.x * blockDim.x) {
		const BuildMesh md = mesh_at<B>(bb, mi);
		const DenseView &dv = md.dv;
		if (dv.D == 0) continue;
		// occupied cells of depth d: N_d = prefix[off[d+1]] - prefix[off[d]]; cells of depths < d: prefix[off[d]]
		for (uint32_t d = 1; d <= dv.D + 1; ++d) {
			const uint32_t before_parent = d >= 2 ? dv.prefix[dv.off[d - 1]] : 0u; // occupied cells of depths < d-1
			const uint32_t parents = d >= 2 ? dv.prefix[dv.off[d]] - dv.prefix[dv.off[d - 1]] : 1u;
			LevelInfo li;
			li.begin = d == 1 ? 0u : 8u * (1u + before_parent);
			li.num = 8u * parents;
			li.blocks_before = d == 1 ? 0u : dv.prefix[dv.off[d]];
			li.nodes = d <= dv.D ? dv.prefix[dv.off[d + 1]] - dv.prefix[dv.off[d]] : 0u;
			md.state->lv[d] = li;
		}
	}
}

// Writes the child blocks of every occupied cell of depths 0 (the root) .. D-1: the interior words of
// depths 1..D.  The blocks of depth-D cells are the leaf stage's when depth D+1 is the leaf depth, and
// the first sparse alloc's when sparse depths follow.  One bitmap word and one prefix word of the child depth serve
// all 8 children.
template <bool B>
__global__ void __launch_bounds__(kTPB) dense_write(BuildBatch bb, uint32_t total_items) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	if (bb.gstate->status & kStatusAbort) return; // the prefix is not a complete scan: write nothing
	for (uint32_t gitem = blockIdx.x * blockDim.x + threadIdx.x; gitem < total_items; gitem += gridDim.x * blockDim.x) {
		const uint32_t mi = B ? mesh_search(bb.item_base, bb.M, gitem) : 0u;
		const BuildMesh md = mesh_at<B>(bb, mi);
		const DenseView &dv = md.dv;
		const uint32_t item = gitem - md.item_base;
		const uint32_t D = dv.D;
		uint32_t bits, e, base_m, r;
		if (item == 0) { // the root: a single occupied cell whose block (words 0..7) holds the depth-1 nodes
			bits = 1u, e = 0, base_m = 0, r = 0;
		} else {
			const uint32_t gw = item - 1; // word of a parent depth e in 1..last
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
			if (blk + 8 > md.capacity || blk + 8 > SVO_MAX_POOL_WORDS) {
				atomicOr(&md.state->status, kStatusCapacity);
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
			uint4 *dst = reinterpret_cast<uint4 *>(md.pool + blk);
			dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
			dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
		}
	}
}

// Clears the tag bitmap of sparse depth `depth`: one bit per word of the depth's range, set by the tag
// pass for every occupied node.  (The words themselves are written whole by the alloc, so the pool needs
// no init pass, shader/octree_init_node.comp:7-11.)  A range beyond the pool or the bitmap is reported as
// a capacity overflow and nothing is cleared.
__global__ void __launch_bounds__(kTPB) tag_clear(uint32_t *__restrict__ tagbits, uint64_t tag_words,
                                                  uint64_t capacity, BuildState *state, uint32_t depth,
                                                  const BuildState *gstate) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	if ((state->status & kStatusCapacity) || (gstate->status & kStatusAbort)) return;
	const LevelInfo li = state->lv[depth];
	const uint64_t end = (uint64_t)li.begin + li.num, n4 = ((uint64_t)li.num + 127) / 128; // 4 words each
	if (end > capacity || end > SVO_MAX_POOL_WORDS || 4 * n4 > tag_words) {
		if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&state->status, kStatusCapacity);
		return;
	}
	uint4 *dst = reinterpret_cast<uint4 *>(tagbits);
	for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (uint64_t)gridDim.x * blockDim.x)
		dst[i] = make_uint4(0u, 0u, 0u, 0u);
}

// ------------------------------------------------------------------------------------------ tag (sparse levels)
// The depth-`depth` node of a fragment, through its parent: the node index cached by the previous sparse
// depth, or the dense bitmaps when the parent depth is dense.
SVO_DEV uint32_t tag_node(uint64_t frag, uint32_t node, uint32_t level, uint32_t depth, bool parent_dense,
                          const DenseView &dv, const uint32_t *__restrict__ pool) {
	uint32_t x, y, z;
	frag_xyz(frag, x, y, z);
	if (parent_dense) return dense_child_word(dv, x, y, z, level, depth);
	return (pool[node] & 0x3fffffffu) + octant_at(x, y, z, level - depth);
}

// Sets the tag bits of nodes idx[0..3] (words of the depth's range [begin, begin + num)), one atomicOr per
// run of equal bitmap words.
SVO_DEV void tag_set(uint32_t *__restrict__ tagbits, uint32_t begin, uint32_t num, const uint32_t idx[4],
                     BuildState *gstate) {
	uint32_t word = 0xffffffffu, bits = 0u;
#pragma unroll
	for (int k = 0; k < 4; ++k) {
		const uint32_t rel = idx[k] - begin;
		if (rel >= num) { // a child of an allocated node lies in the range: cannot happen
			SVO_CHECK_FAIL(10u, gstate);
			continue;
		}
		if ((rel >> 5) != word) {
			if (bits) atomicOr(tagbits + word, bits);
			word = rel >> 5, bits = 0u;
		}
		bits |= 1u << (rel & 31u);
	}
	if (bits) atomicOr(tagbits + word, bits);
	(void)gstate;
}

// Marks the depth-`depth` node of every fragment in the depth's tag bitmap (the tag of
// shader/octree_tag_node.comp:33-60 for interior nodes) and caches the node index per fragment for the
// next depth and the leaf stage.
__global__ void __launch_bounds__(kTPB) build_tag(const uint64_t *__restrict__ frags, uint32_t n, uint32_t level,
                                                  uint32_t depth, const uint32_t *__restrict__ pool,
                                                  uint32_t *__restrict__ tagbits, uint32_t *__restrict__ cache,
                                                  DenseView dv, BuildState *state, BuildState *gstate) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	if ((state->status & kStatusCapacity) || (gstate->status & kStatusAbort)) return;
	const bool parent_dense = depth == 1 || depth - 1 <= dv.D;
	const uint32_t begin = state->lv[depth].begin, num = state->lv[depth].num;
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t nq = (n + 3ull) / 4ull;
	for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += stride) {
		const uint64_t f0 = q * 4;
		if (f0 + 4 <= n) { // the sorted copy of a mesh is 32-byte aligned: 16-byte loads
			const ulonglong2 a = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0));
			const ulonglong2 b = __ldcs(reinterpret_cast<const ulonglong2 *>(frags + f0 + 2));
			uint4 c = make_uint4(0, 0, 0, 0);
			if (!parent_dense) c = __ldcs(reinterpret_cast<const uint4 *>(cache + f0));
			const uint32_t idx[4] = {tag_node(a.x, c.x, level, depth, parent_dense, dv, pool),
			                         tag_node(a.y, c.y, level, depth, parent_dense, dv, pool),
			                         tag_node(b.x, c.z, level, depth, parent_dense, dv, pool),
			                         tag_node(b.y, c.w, level, depth, parent_dense, dv, pool)};
			tag_set(tagbits, begin, num, idx, gstate);
			__stcs(reinterpret_cast<uint4 *>(cache + f0), make_uint4(idx[0], idx[1], idx[2], idx[3]));
		} else {
			for (uint64_t f = f0; f < n; ++f) {
				const uint32_t node = tag_node(frags[f], parent_dense ? 0u : cache[f], level, depth, parent_dense, dv, pool);
				const uint32_t idx[4] = {node, node, node, node};
				tag_set(tagbits, begin, num, idx, gstate);
				cache[f] = node;
			}
		}
	}
}

// Prefix-sum allocation of child blocks for the tagged words of a sparse depth (persistent grid, tiles
// claimed in order by ticket so the look-back always waits on a running or finished tile).  Every word of
// the depth's range is written: a child pointer for a tagged word, 0 for the others.
__global__ void __launch_bounds__(kTPB) build_alloc(uint32_t *__restrict__ pool, uint64_t capacity, uint32_t depth,
                                                    const uint32_t *__restrict__ tagbits, BuildState *state,
                                                    unsigned long long *descs, BuildState *gstate) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kTPB / 32 + 1];
	__shared__ uint32_t s_prefix;
	__shared__ uint32_t s_abort;
	// other blocks of this launch may set the capacity flag: decide once per block
	if (threadIdx.x == 0)
		s_abort = (atomicOr(&state->status, 0u) & kStatusCapacity) | (gstate->status & kStatusAbort);
	__syncthreads();
	if (s_abort) return;
	const LevelInfo li = state->lv[depth];
	const uint32_t ntiles = (li.num + kAllocTile - 1) / kAllocTile;
	const uint32_t next_begin = li.begin + li.num;
	if (ntiles == 0) {
		if (blockIdx.x == 0 && threadIdx.x == 0) {
			state->lv[depth].nodes = 0;
			state->lv[depth + 1] = LevelInfo{next_begin, 0u, li.blocks_before, 0u};
		}
		return;
	}
	// pipelined as the voxelize scans: a tile's count is published at once, its look-back and its
	// pointers follow after the block has counted its next tile.  A thread's kAllocIPT = 32 words are
	// one word of the tag bitmap.
	uint32_t p_tile = 0xffffffffu, p_mask = 0, p_rank0 = 0, p_total = 0;
	for (;;) {
		if (threadIdx.x == 0) s_tile = atomicAdd(&state->tiles[depth], 1u);
		__syncthreads();
		const uint32_t tile = s_tile;
		__syncthreads();
		uint32_t mask = 0, rank0 = 0, total = 0;
		if (tile < ntiles) {
			const uint32_t w0 = tile * kAllocTile + threadIdx.x * kAllocIPT; // offset inside the level
			if (w0 < li.num) mask = tagbits[w0 / kAllocIPT]; // bits past the range are clear
			rank0 = block_exclusive_sum<uint32_t, kTPB>((uint32_t)__popc(mask), s_warp, total);
			if (threadIdx.x == 0) tile_publish_aggregate(descs, tile, depth, total);
		}
		if (p_tile != 0xffffffffu) {
			if (threadIdx.x < 32) {
				// a timeout goes to the batch-wide status, which every later stage of every mesh checks
				const uint32_t p =
				    (uint32_t)tile_lookback_warp(descs, p_tile, depth, p_total, &gstate->status, false, true);
				if (threadIdx.x == 0) s_prefix = p;
			}
			__syncthreads();
			const uint32_t prefix = s_prefix;
			const uint32_t w0 = p_tile * kAllocTile + threadIdx.x * kAllocIPT;
			uint32_t w[kAllocIPT], rank = p_rank0;
#pragma unroll
			for (int k = 0; k < kAllocIPT; ++k) {
				w[k] = 0u;
				if (!((p_mask >> k) & 1u)) continue;
				const uint64_t b = (uint64_t)li.blocks_before + prefix + rank++; // 0-based child block number
				const uint64_t ptr = (b + 1) * 8;
				if (ptr + 8 > capacity || ptr + 8 > SVO_MAX_POOL_WORDS) {
					atomicOr(&state->status, kStatusCapacity);
					w[k] = 0x80000000u; // leave unallocated; the build reports SVO_ERR_CAPACITY
					continue;
				}
				w[k] = (uint32_t)ptr | 0x80000000u;
			}
			if (w0 + kAllocIPT <= li.num) {
				uint4 *dst = reinterpret_cast<uint4 *>(pool + li.begin + w0);
#pragma unroll
				for (int k = 0; k < kAllocIPT / 4; ++k)
					dst[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
			} else {
#pragma unroll
				for (int k = 0; k < kAllocIPT; ++k)
					if (w0 + k < li.num) pool[li.begin + w0 + k] = w[k];
			}
			if (p_tile == ntiles - 1 && threadIdx.x == 0) {
				const uint32_t nodes = prefix + p_total;
				state->lv[depth].nodes = nodes;
				state->lv[depth + 1] = LevelInfo{next_begin, nodes * 8u, li.blocks_before + nodes, 0u};
			}
			__syncthreads();
		}
		if (tile >= ntiles) break;
		p_tile = tile, p_mask = mask, p_rank0 = rank0, p_total = total;
	}
}

// ------------------------------------------------------------------------------------------ buckets
// The fragments are copied once into buckets of voxels (Morton order of the bucket, any order
// inside one).  All later sweeps read the bucketed copy: the sparse tag passes then touch the pool
// region by region, and the leaf stage gives each bucket to one block, which accumulates its leaf
// colours in shared memory.  The leaf blocks (8 words per depth L-1 node) of one bucket are contiguous
// in the pool (breadth-first order is Morton order within a depth), so that block writes them whole.
// In a batch the buckets of all meshes are concatenated in mesh order, so one scan over all of them
// places every mesh's bucketed copy after the previous mesh's.
// Bucket edge: 16 voxels while the leaf parents are dense (level <= D + 1): a bucket then spans at most
// one leaf window's worth of leaf words (8^3 parents x 8), which the windowed leaf stage relies on; 32
// voxels when they are sparse, where 16-voxel buckets would need 8^8 bucket counters at level 12.  (A
// 32-voxel bucket may meet more windows, each reading all its items; 16-voxel buckets at level 12 made
// the leaf stage 3% faster and the bucket scan, scatter and span passes 0.4 ms slower on a 2^12 scene.)
uint32_t bucket_shift(uint32_t level, uint32_t D) { return std::min<uint32_t>(level, level <= D + 1 ? 4u : 5u); }

// Leaf windows a dense-parent mesh can need: its leaf range is at most 8 words per possible parent.
uint64_t leaf_window_bound(uint32_t count, uint32_t level) {
	const uint64_t parents = level == 1 ? 1ull : std::min<uint64_t>(1ull << (3 * (level - 1)), std::max<uint32_t>(count, 1u));
	return (8ull * parents + 4095) / 4096;
}


// Exclusive prefix of the bucket counts (boff[nb] = total) and the list of non-empty buckets in order;
// two single-pass look-back scans, tiles claimed in order by ticket.
__global__ void __launch_bounds__(kTPB) bucket_scan(const uint32_t *__restrict__ bcount, uint32_t nb,
                                                    uint32_t *__restrict__ boff, uint32_t *__restrict__ blist,
                                                    BuildState *state, unsigned long long *descs) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kTPB / 32 + 1];
	__shared__ uint32_t s_prefix[2];
	if (threadIdx.x == 0) s_tile = atomicAdd(&state->tiles[1], 1u);
	__syncthreads();
	const uint32_t tile = s_tile;
	const uint32_t ntiles = (nb + kScanTile - 1) / kScanTile;
	if (tile >= ntiles) return; // one tile per block: only an uncleared ticket goes past the grid
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
template <bool B>
__global__ void __launch_bounds__(kTPB) bucket_scatter(const uint64_t *__restrict__ frags, uint64_t n, BuildBatch bb,
                                                       const uint32_t *__restrict__ boff, uint32_t *__restrict__ bfill,
                                                       uint64_t *__restrict__ sorted) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_spread[kSpreadEntries];
	spread_table_init(s_spread);
	const uint64_t runs = (n + 31ull) >> 5;
	const uint32_t lane = lane_id();
	for (uint64_t r = sweep_first_run<kScatterRuns>(); r < runs; r += sweep_run_stride<kScatterRuns>()) {
		const uint32_t m0 = B ? mesh_search(bb.frag_base, bb.M, (unsigned long long)(r << 5)) : 0u;
		uint64_t out[kScatterRuns], send[kScatterRuns];
		uint32_t key[kScatterRuns], pad[kScatterRuns], first[kScatterRuns], base[kScatterRuns];
#pragma unroll
		for (uint32_t k = 0; k < kScatterRuns; ++k) {
			const uint64_t f = ((r + k) << 5) + lane;
			out[k] = f < n ? __ldcs(frags + f) : 0ull;
		}
#pragma unroll
		for (uint32_t k = 0; k < kScatterRuns; ++k) {
			const uint64_t f = ((r + k) << 5) + lane;
			key[k] = 0xffffffffu, pad[k] = 0, send[k] = 0;
			if (f < n) {
				const uint32_t mi = B ? mesh_from(bb.frag_base, m0, f) : 0u;
				const BuildMesh md = mesh_at<B>(bb, mi);
				const uint32_t level = md.level;
				const bool items = level == 1 || level - 1 <= md.dv.D;
				const uint64_t frag = out[k];
				uint32_t x, y, z;
				frag_xyz(frag, x, y, z);
				if (!frag_in_level(x, y, z, level)) {
					// skipped (dense_mark reported it)
				} else if (items && level > 1) { // parent cell m (depth level-1); the bucket key is its prefix
					const uint32_t *pbits = md.dv.bits + md.parent_off;
					const uint32_t *pprefix = md.dv.prefix + md.parent_off;
					// the leaf range starts after the blocks of every occupied cell above the parents'
					// depth (dense_finish's level table, which may still be in flight on the other stream)
					const uint32_t leaf_begin = 8u * (1u + __ldg(pprefix));
					const uint32_t m = morton_tab(s_spread, x, y, z, 1), w = m >> 5;
					key[k] = m >> (3 * (md.bshift - 1));
					out[k] = ((uint64_t)(octant_at(x, y, z, 0) +
					                     8u * (1u + __ldg(pprefix + w) +
					                           __popc(__ldg(pbits + w) & ((1u << (m & 31)) - 1u))) -
					                     leaf_begin)
					          << 32) |
					         ((frag >> 32) & 0xffffffu);
				} else {
					key[k] = morton_tab(s_spread, x, y, z, md.bshift);
					if (items) // level 1: the leaf words are the root block
						out[k] = ((uint64_t)octant_at(x, y, z, 0) << 32) | ((frag >> 32) & 0xffffffu);
				}
				if (key[k] != 0xffffffffu) {
					key[k] += md.bucket_base;
					if (!SVO_CHECK(key[k] < bb.nb_total, 3u, bb.gstate)) key[k] = 0xffffffffu;
				}
				pad[k] = md.sorted_pad;
				send[k] = md.frag_base + md.sorted_pad + md.count;
			}
		}
		// one cursor atomic per run of equal keys in consecutive lanes; the atomics of all runs of
		// fragments are in flight together
#pragma unroll
		for (uint32_t k = 0; k < kScatterRuns; ++k) {
			uint32_t last;
			lane_run(key[k], lane, first[k], last);
			base[k] = 0;
			if (key[k] != 0xffffffffu && lane == first[k]) base[k] = atomicAdd(bfill + key[k], last - first[k] + 1u);
		}
#pragma unroll
		for (uint32_t k = 0; k < kScatterRuns; ++k) {
			const uint32_t b = __shfl_sync(kFullMask, base[k], first[k]);
			if (key[k] != 0xffffffffu) {
				const uint64_t at = (uint64_t)__ldg(boff + key[k]) + pad[k] + b + (lane - first[k]);
				if (at < send[k]) // always true after a complete bucket scan (a timed-out scan is reported)
					sorted[at] = out[k];
				else
					SVO_CHECK_FAIL(4u, bb.gstate);
			}
		}
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

constexpr uint32_t kLeafSlots = 4096;         // packed accumulators in shared memory (8 B each)
constexpr uint32_t kWideSlots = kLeafSlots / 4; // exact accumulators (4 x 8 B each) of the overflow path

// Leaf windows.  A mesh has its leaf stage cut into windows of kLeafSlots words of its leaf range;
// window k is built by one block from the buckets whose leaf spans meet it.  Consecutive non-empty
// buckets of a mesh have adjacent spans (breadth-first order is Morton order), so those buckets are one
// run of the bucket list and their items one range of the bucketed copy; a 16^3-voxel bucket spans at
// most 512 parents = kLeafSlots words, so it meets at most two windows and every item is read at most
// twice (a 32^3-voxel bucket of a sparse-parent mesh spans at most 4096 parents, eight windows).
constexpr uint32_t kWinBits = 12;
static_assert((1u << kWinBits) == kLeafSlots, "a leaf window is one shared-memory accumulator window");

SVO_DEV bool dense_parents(const BuildMesh &md) { return md.level == 1 || md.level - 1 <= md.dv.D; }

// Leaf words [first, last] of local bucket bl of a dense-parent mesh: the prefix entries at its first
// parent-bitmap word and at the next bucket's give its first and last leaf block.
SVO_DEV uint2 bucket_span(const BuildMesh &md, uint32_t bl, uint32_t leaf_begin, uint32_t leaf_num) {
	if (md.nb == 1) return make_uint2(0u, leaf_num - 1u);
	const uint32_t *pprefix = md.dv.prefix + md.parent_off;
	const uint32_t before = leaf_begin / 8u - 1u;              // occupied cells of depths below the parents
	const uint32_t wpb = (1u << (3 * (md.bshift - 1))) >> 5;  // parent-bitmap words per bucket
	return make_uint2(8u * (__ldg(pprefix + wpb * bl) - before), 8u * (__ldg(pprefix + wpb * (bl + 1)) - before) - 1u);
}

// Exclusive prefix of the meshes' window counts (one block); win_base[M] = windows of the batch.
template <bool B> __global__ void __launch_bounds__(kTPB) leaf_window_scan(BuildBatch bb, uint32_t *__restrict__ win_base) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_warp[kTPB / 32 + 1];
	uint32_t carry = 0;
	const uint32_t M = batch_size<B>(bb);
	for (uint32_t base = 0; base < M; base += kTPB) {
		const uint32_t mi = base + threadIdx.x;
		uint32_t c = 0;
		if (mi < M && !(bb.gstate->status & kStatusAbort)) { // no windows after an aborted scan
			const BuildMesh md = mesh_at<B>(bb, mi);
			c = (md.state->lv[md.level].num + kLeafSlots - 1) >> kWinBits;
		}
		uint32_t total;
		const uint32_t excl = block_exclusive_sum<uint32_t, kTPB>(c, s_warp, total);
		if (mi < M) win_base[mi] = carry + excl;
		carry += total;
	}
	if (threadIdx.x == 0) win_base[M] = carry;
}

// Extent of every non-empty bucket, in list order: first and last item and first and last leaf word.
// Dense-parent meshes: the span comes from the parent bitmap's prefix; sparse-parent meshes: it is
// reduced over the bucket's fragments by bucket_span_sparse.  Also writes every mesh's range (final once
// the interior levels are built).
template <bool B>
__global__ void bucket_meta(BuildBatch bb, const uint32_t *__restrict__ boff, const uint32_t *__restrict__ blist,
                            const BuildState *gstate, uint4 *__restrict__ meta) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	// after an aborted scan the bucket list may hold entries no tile wrote: nothing is read through it
	const uint32_t nbuckets = (gstate->status & kStatusAbort) ? 0u : gstate->buckets;
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nbuckets; t += gridDim.x * blockDim.x) {
		const uint32_t b = blist[t];
		const uint32_t mi = B ? mesh_search(bb.bucket_base, bb.M, b) : 0u;
		const BuildMesh md = mesh_at<B>(bb, mi);
		const uint32_t level = md.level, bl = b - md.bucket_base;
		const uint32_t leaf_begin = md.state->lv[level].begin, leaf_num = md.state->lv[level].num;
		uint4 m = make_uint4(boff[b] + md.sorted_pad, boff[b + 1] + md.sorted_pad, 0u, 0u);
		if (dense_parents(md)) {
			const uint2 sp = bucket_span(md, bl, leaf_begin, leaf_num);
			m.z = sp.x, m.w = sp.y;
			if (!SVO_CHECK(sp.y < leaf_num && sp.x <= sp.y, 6u, bb.gstate)) m.y = m.x, m.z = 1, m.w = 0;
		}
		if (!SVO_CHECK(m.y <= bb.sorted_total && m.x <= m.y, 5u, bb.gstate)) m.y = m.x;
		meta[t] = m;
	}
	for (uint32_t mi = blockIdx.x * blockDim.x + threadIdx.x; mi < batch_size<B>(bb); mi += gridDim.x * blockDim.x) {
		const BuildMesh md = mesh_at<B>(bb, mi);
		md.state->range_words = md.state->lv[md.level].begin + md.state->lv[md.level].num;
	}
}

// Leaf span of each bucket of a sparse-parent mesh, one warp per bucket: the least and greatest leaf
// slot of its fragments (through the node index the last sparse tag cached), widened to whole blocks.
// A bucket holds all fragments of its parents, so its blocks are exactly those parents' blocks.  Each
// fragment of the bucketed copy is replaced by its leaf item (slot << 32 | rgb), the form the copy of a
// dense-parent mesh has from the start, so the leaf stage reads no node words.
template <bool B>
__global__ void __launch_bounds__(kTPB) bucket_span_sparse(uint64_t *__restrict__ sorted, BuildBatch bb,
                                                           const uint32_t *__restrict__ blist,
                                                           const uint32_t *__restrict__ cache,
                                                           const BuildState *gstate, uint4 *__restrict__ meta) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	const uint32_t nbuckets = (gstate->status & kStatusAbort) ? 0u : gstate->buckets, lane = lane_id();
	const uint32_t warps = gridDim.x * (blockDim.x / 32);
	for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) / 32; t < nbuckets; t += warps) {
		const uint32_t mi = B ? mesh_search(bb.bucket_base, bb.M, blist[t]) : 0u;
		const BuildMesh md = mesh_at<B>(bb, mi);
		if (dense_parents(md)) continue; // warp-uniform
		// the node cache is only complete when every sparse depth ran (no capacity, timeout or bad fragment)
		if ((md.state->status & kStatusCapacity) || (gstate->status & kStatusAbort)) continue;
		const uint4 m = meta[t];
		const uint32_t leaf_begin = md.state->lv[md.level].begin, leaf_num = md.state->lv[md.level].num;
		uint32_t lo = 0xffffffffu, hi = 0u;
		// four fragments per lane and pass, their loads issued together (a fragment's slot is a chain of
		// two dependent loads)
		for (uint32_t f = m.x + lane; f < m.y; f += 4 * 32) {
			uint64_t frag[4];
			uint32_t node[4];
#pragma unroll
			for (uint32_t k = 0; k < 4; ++k) {
				const uint32_t g = f + 32 * k;
				frag[k] = g < m.y ? sorted[g] : 0ull;
				node[k] = g < m.y ? __ldg(cache + g) : 0u;
			}
#pragma unroll
			for (uint32_t k = 0; k < 4; ++k) {
				const uint32_t g = f + 32 * k;
				if (g < m.y) {
					uint32_t x, y, z;
					frag_xyz(frag[k], x, y, z);
					const uint32_t sl = (__ldg(md.pool + node[k]) & 0x3fffffffu) + octant_at(x, y, z, 0) - leaf_begin;
					lo = min(lo, sl), hi = max(hi, sl);
					sorted[g] = ((uint64_t)sl << 32) | ((frag[k] >> 32) & 0xffffffu);
				}
			}
		}
		lo = __reduce_min_sync(kFullMask, lo), hi = __reduce_max_sync(kFullMask, hi);
		if (lane == 0) {
			uint4 out = m;
			if (lo <= hi && (hi | 7u) < leaf_num) { // always, after a complete tag (a failed one is reported)
				out.z = lo & ~7u, out.w = hi | 7u;
			} else {
				SVO_CHECK_FAIL(9u, bb.gstate);
				out.y = out.x, out.z = 1u, out.w = 0u;
			}
			meta[t] = out;
		}
	}
}

// First and last bucket of every leaf window from the buckets' spans: bucket t is a window's first when
// the previous bucket of its mesh ends before the window, its last when the next one starts after it.
// Consecutive buckets of a mesh have adjacent spans, so every window of the leaf range gets both.
template <bool B>
__global__ void bucket_windows(BuildBatch bb, const uint32_t *__restrict__ blist, const BuildState *gstate,
                               const uint4 *__restrict__ meta, const uint32_t *__restrict__ win_base,
                               uint32_t *__restrict__ wfirst, uint32_t *__restrict__ wlast) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	const uint32_t nbuckets = (gstate->status & kStatusAbort) ? 0u : gstate->buckets; // as in bucket_meta
	for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nbuckets; t += gridDim.x * blockDim.x) {
		const uint32_t mi = B ? mesh_search(bb.bucket_base, bb.M, blist[t]) : 0u;
		const uint32_t b_lo = B ? __ldg(bb.bucket_base + mi) : 0u, b_hi = B ? __ldg(bb.bucket_base + mi + 1) : bb.one.nb;
		const uint4 m = meta[t];
		if (m.z > m.w) continue; // span rejected by a check
		const bool prev_in = t > 0 && (!B || blist[t - 1] >= b_lo);
		const bool next_in = t + 1 < nbuckets && blist[t + 1] < b_hi;
		const uint32_t prev_end = prev_in ? meta[t - 1].w : 0u, next_start = next_in ? meta[t + 1].z : 0u;
		const uint32_t wb = win_base[mi];
		for (uint32_t k = m.z >> kWinBits; k <= (m.w >> kWinBits); ++k) {
			if (!prev_in || (prev_end >> kWinBits) < k) wfirst[wb + k] = t;
			if (!next_in || (next_start >> kWinBits) > k) wlast[wb + k] = t;
		}
	}
}

// Packed-accumulator window of the leaf stage, shared by both leaf kernels: adds items f0..f1 of the
// bucketed copy whose slot (relative to the window start w0) is below wn, then writes the window's wn
// leaf words to dst (empty slots as 0) and returns the block's count of non-empty words.  An
// accumulator is two 32-bit words, (r | g << 16) and (b | n << 16): a field can carry only when a voxel
// has more than 257 fragments (257 x 255 = 65535), so an add that sees a count of 257 or more marks the
// window, which is then redone exactly with 64-bit r, g, b and n sums, kWideSlots slots at a time.
// SLOT(item, f) gives an item's slot relative to the leaf range and RGB(item) its colour.
template <typename SlotFn, typename RgbFn>
SVO_DEV uint32_t leaf_window(const uint64_t *__restrict__ sorted, uint32_t f0, uint32_t f1, uint32_t w0, uint32_t wn,
                             uint32_t *dst, unsigned long long *s_acc, uint32_t *s_over, SlotFn SLOT, RgbFn RGB) {
	uint32_t *s_acc32 = reinterpret_cast<uint32_t *>(s_acc);
	// the accumulators are zero here: cleared once per block, then by each window's write-out
	if (threadIdx.x == 0) *s_over = 0;
	__syncthreads();
	bool over = false;
	for (uint32_t fb = f0 + threadIdx.x; fb < f1; fb += 4 * kTPB) {
		uint64_t fr[4];
		uint32_t sl[4], rgb[4];
#pragma unroll
		for (int k = 0; k < 4; ++k) fr[k] = fb + k * kTPB < f1 ? __ldcs(sorted + fb + k * kTPB) : 0ull;
#pragma unroll
		for (int k = 0; k < 4; ++k) {
			sl[k] = fb + k * kTPB < f1 ? SLOT(fr[k], fb + k * kTPB) - w0 : 0xffffffffu;
			rgb[k] = RGB(fr[k]);
		}
#pragma unroll
		for (int k = 0; k < 4; ++k)
			if (sl[k] < wn) {
				atomicAdd(s_acc32 + 2 * sl[k], (rgb[k] & 0xffu) | (((rgb[k] >> 8) & 0xffu) << 16));
				over |= (atomicAdd(s_acc32 + 2 * sl[k] + 1, ((rgb[k] >> 16) & 0xffu) | (1u << 16)) >> 16) >= 257u;
			}
	}
	if (__any_sync(kFullMask, over) && lane_id() == 0) *s_over = 1;
	__syncthreads();
	uint32_t leaves = 0;
	if (!*s_over) {
		for (uint32_t i = 4 * threadIdx.x; i < wn; i += 4 * kTPB) {
			const uint4 a = *reinterpret_cast<const uint4 *>(s_acc32 + 2 * i);
			const uint4 c = *reinterpret_cast<const uint4 *>(s_acc32 + 2 * i + 4);
			*reinterpret_cast<uint4 *>(s_acc32 + 2 * i) = make_uint4(0u, 0u, 0u, 0u); // ready for the next window
			*reinterpret_cast<uint4 *>(s_acc32 + 2 * i + 4) = make_uint4(0u, 0u, 0u, 0u);
			const uint32_t rg[4] = {a.x, a.z, c.x, c.z}, bn[4] = {a.y, a.w, c.y, c.w};
			uint32_t word[4];
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				const uint32_t n = bn[j] >> 16;
				word[j] = n ? leaf_word(n, rg[j] & 0xffffu, rg[j] >> 16, bn[j] & 0xffffu) : 0u;
				leaves += word[j] != 0u;
			}
			*reinterpret_cast<uint4 *>(dst + i) = make_uint4(word[0], word[1], word[2], word[3]);
		}
	} else {
		unsigned long long *acc4 = s_acc;
		for (uint32_t v0 = 0; v0 < wn; v0 += kWideSlots) {
			const uint32_t vn = min(kWideSlots, wn - v0);
			__syncthreads();
			for (uint32_t i = threadIdx.x; i < 4 * vn; i += kTPB) acc4[i] = 0ull;
			__syncthreads();
			for (uint32_t f = f0 + threadIdx.x; f < f1; f += kTPB) {
				const uint64_t item = sorted[f];
				const uint32_t sl = SLOT(item, f) - w0 - v0;
				const uint32_t c = RGB(item);
				if (sl < vn) {
					atomicAdd(acc4 + 4 * sl, (unsigned long long)(c & 0xffu));
					atomicAdd(acc4 + 4 * sl + 1, (unsigned long long)((c >> 8) & 0xffu));
					atomicAdd(acc4 + 4 * sl + 2, (unsigned long long)((c >> 16) & 0xffu));
					atomicAdd(acc4 + 4 * sl + 3, 1ull);
				}
			}
			__syncthreads();
			for (uint32_t i = threadIdx.x; i < vn; i += kTPB) {
				const unsigned long long n = acc4[4 * i + 3]; // < 2^32 (fragment counts are 32-bit)
				const uint32_t word = n ? leaf_word_wide((uint32_t)n, acc4[4 * i], acc4[4 * i + 1], acc4[4 * i + 2]) : 0u;
				dst[v0 + i] = word;
				leaves += word != 0u;
			}
		}
		__syncthreads();
		for (uint32_t i = threadIdx.x; i < kLeafSlots; i += kTPB) s_acc[i] = 0ull; // the next window starts at zero
	}
	__syncthreads(); // the accumulators are reused by the next window
	return leaves;
}

// Leaf stage: one leaf window per block at a time, windows of all meshes taken grid-stride.  The bucketed
// copy holds (slot << 32 | rgb) items: from the scatter for dense-parent meshes, from bucket_span_sparse
// for sparse-parent ones.
template <bool B>
__global__ void __launch_bounds__(kTPB) build_leaf_windows(const uint64_t *__restrict__ sorted, BuildBatch bb,
                                                           const uint4 *__restrict__ meta,
                                                           const uint32_t *__restrict__ win_base,
                                                           const uint32_t *__restrict__ wfirst,
                                                           const uint32_t *__restrict__ wlast, BuildState *gstate) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	extern __shared__ unsigned long long s_acc[];
	__shared__ uint32_t s_over, s_leaves, s_skip;
	const uint32_t M = batch_size<B>(bb);
	if (gstate->status & kStatusAbort) return; // no window bookkeeping was made (leaf_window_scan)
	const uint32_t total = win_base[M], nbuckets = gstate->buckets;
	for (uint32_t i = threadIdx.x; i < kLeafSlots; i += kTPB) s_acc[i] = 0ull; // leaf_window keeps them zero after
	__syncthreads();
	for (uint32_t gw = blockIdx.x; gw < total; gw += gridDim.x) {
		const uint32_t mi = B ? mesh_search(win_base, M, gw) : 0u;
		const BuildMesh md = mesh_at<B>(bb, mi);
		const uint32_t level = md.level;
		const uint32_t leaf_begin = md.state->lv[level].begin, leaf_num = md.state->lv[level].num;
		const uint32_t w0 = (gw - win_base[mi]) << kWinBits;
		const uint32_t t0 = wfirst[gw], t1 = wlast[gw];
		if (threadIdx.x == 0) {
			const uint64_t leaf_end = (uint64_t)leaf_begin + leaf_num;
			uint32_t skip = (md.state->status & kStatusCapacity) | (gstate->status & kStatusAbort);
			if (!skip && (leaf_end > md.capacity || leaf_end > SVO_MAX_POOL_WORDS)) { // leaf blocks: checked here
				atomicOr(&md.state->status, kStatusCapacity);
				skip = 1;
			}
			if (!skip && !(t0 <= t1 && t1 < nbuckets)) { // only after a reported scan failure
				SVO_CHECK_FAIL(8u, gstate);
				skip = 1;
			}
			s_skip = skip;
			s_leaves = 0;
		}
		__syncthreads();
		if (s_skip) {
			__syncthreads();
			continue;
		}
		const uint32_t f0 = meta[t0].x, f1 = meta[t1].y;
		const uint32_t wn = min(kLeafSlots, leaf_num - w0);
		const uint32_t leaves = leaf_window(
		    sorted, f0, f1, w0, wn, md.pool + leaf_begin + w0, s_acc, &s_over,
		    [](uint64_t item, uint32_t) { return (uint32_t)(item >> 32); }, [](uint64_t item) { return (uint32_t)item; });
		const uint32_t wl = warp_sum(leaves);
		if (lane_id() == 0 && wl) atomicAdd(&s_leaves, wl);
		__syncthreads();
		if (threadIdx.x == 0 && s_leaves) atomicAdd(&md.state->leaves, s_leaves);
		__syncthreads();
	}
}

// Writes svo_build_info followed by the status word of every mesh to `out` (device), one record of
// sizeof(svo_build_info) + 4 bytes per mesh.
template <bool B> __global__ void build_export(BuildBatch bb, const BuildState *gstate, uint32_t *out) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	constexpr uint32_t kRec = sizeof(svo_build_info) / 4 + 1;
	for (uint32_t mi = blockIdx.x * blockDim.x + threadIdx.x; mi < batch_size<B>(bb); mi += gridDim.x * blockDim.x) {
		const BuildMesh md = mesh_at<B>(bb, mi);
		const BuildState *state = md.state;
		svo_build_info *info = reinterpret_cast<svo_build_info *>(out + kRec * mi);
		info->level = md.level;
		info->fragments = md.count;
		info->range_words = state->range_words;
		info->leaves = state->leaves;
		for (uint32_t d = 1; d <= SVO_LEVEL_MAX; ++d)
			info->level_nodes[d - 1] = d < md.level ? state->lv[d].nodes : (d == md.level ? state->leaves : 0u);
#ifdef SVO_CHECKED
		out[kRec * mi + kRec - 1] = state->status | gstate->status | (gstate->pad << 16);
#else
		out[kRec * mi + kRec - 1] = state->status | gstate->status;
#endif
	}
}

// ------------------------------------------------------------------------------------------ host side
cudaError_t build_set_wait_fault(uint32_t limit, uint32_t withheld) { return set_wait_fault_here(limit, withheld); }

uint64_t build_pool_bound(uint32_t count, uint32_t level) {
	uint64_t words = 8, per = 1;
	for (uint32_t i = 1; i < level; ++i) {
		per = per >= (1ull << 40) ? per : per * 8; // 8^i (saturating)
		words += 8 * (per < count ? per : (uint64_t)count);
	}
	return words < SVO_MAX_POOL_WORDS ? words : SVO_MAX_POOL_WORDS;
}

uint32_t dense_depth(uint32_t level, uint32_t count) {
	const uint32_t D = level - 1 < 9u ? level - 1 : 9u;
	return level >= 11 && count >= kDeepDenseMinFragments ? 10u : D;
}

uint32_t dense_words_of(uint32_t d) { return d <= 1 ? 1u : (1u << (3 * d)) / 32u; }

uint32_t dense_layout(uint32_t D, uint32_t off[kDenseMaxDepth + 2]) {
	uint32_t o = 0;
	off[0] = 0;
	for (uint32_t d = 1; d <= kDenseMaxDepth + 1; ++d) {
		off[d] = o;
		if (d <= D) o += (dense_words_of(d) + 7u) & ~7u; // 32-byte aligned levels (16-byte vector loads)
	}
	return o;
}

uint32_t dense_items(uint32_t level, uint32_t D, const uint32_t off[kDenseMaxDepth + 2]) {
	(void)level;
	if (D == 0) return 0;
	return off[D] + 1; // parent words of depths 1..D-1, and the root
}

// Words of a mesh's dense scan region: its bitmap words and the total entry, padded to whole tiles.
static uint32_t dense_region(uint32_t D, uint32_t words) {
	return D ? (words + 1 + kBuildScanTile - 1) / kBuildScanTile * kBuildScanTile : 0u;
}

// Largest word range of one sparse depth: depth i spans 8 words per occupied cell of depth i-1, at most
// 8 * min(8^(i-1), count), over the sparse depths D+1..level-1.
uint64_t max_sparse_level_words(uint32_t count, uint32_t level, uint32_t D) {
	uint64_t best = 8, per = 1;
	for (uint32_t i = 1; i < level; ++i) {
		if (i >= D + 1) {
			const uint64_t w = 8 * (per < count ? per : (uint64_t)count);
			best = w > best ? w : best;
		}
		per = per >= (1ull << 40) ? per : per * 8;
	}
	return best;
}

// Words of a tag bitmap for a sparse depth of up to `level_words` words (whole 16-byte groups).
uint64_t tag_bitmap_words(uint64_t level_words) { return (level_words + 127) / 128 * 4 + 4; }

// Layout: state | dense-scan descriptors | dense bitmaps | dense prefix | bucket counts, offsets,
// cursors, list and scan descriptors | bucketed fragment copy (8 B per fragment) | node cache (4 B per
// fragment) and tag bitmap (1 bit per word of the largest sparse depth), sparse levels only.  The leaf
// stage needs nothing more: its accumulators live in shared memory.
void build_workspace_layout(void *ws, uint32_t count, uint32_t level, uint64_t capacity, BuildWorkspace &w) {
	char *p = (char *)ws;
	size_t off = 0;
	auto take = [&](size_t bytes) {
		char *q = p + off;
		off += align_up(bytes, 256);
		return q;
	};
	const uint32_t D = dense_depth(level, count);
	w.dv.D = D;
	const uint32_t o = dense_layout(D, w.dv.off);
	w.dense_words = dense_region(D, o);
	w.state = (BuildState *)take(sizeof(BuildState));
	uint64_t sparse_words = max_sparse_level_words(count, level, D);
	if (sparse_words > capacity) sparse_words = capacity;
	const uint64_t scan_items = std::max<uint64_t>(w.dense_words, sparse_words);
	w.desc_count = (size_t)((scan_items + kScanTile - 1) / kScanTile + 2);
	w.descs = (unsigned long long *)take(w.desc_count * sizeof(unsigned long long));
	w.dv.bits = (uint32_t *)take((size_t)w.dense_words * 4 + 32);
	w.dv.prefix = (uint32_t *)take((size_t)w.dense_words * 4 + 32);
	w.bshift = bucket_shift(level, D);
	w.nb = 1u << (3 * (level - w.bshift));
	w.bcount = (uint32_t *)take((size_t)w.nb * 4);
	w.bfill = (uint32_t *)take((size_t)w.nb * 4);
	w.boff = (uint32_t *)take(((size_t)w.nb + 1) * 4);
	w.blist = (uint32_t *)take((size_t)w.nb * 4);
	w.bmeta = (uint4 *)take((size_t)w.nb * 16);
	w.bdesc_count = 2 * ((size_t)(w.nb + kScanTile - 1) / kScanTile + 1);
	w.bdescs = (unsigned long long *)take(w.bdesc_count * sizeof(unsigned long long));
	w.win_base = (uint32_t *)take(2 * 4);
	const uint64_t wins = leaf_window_bound(count, level);
	w.wfirst = (uint32_t *)take(wins * 4 + 4);
	w.wlast = (uint32_t *)take(wins * 4 + 4);
	w.sorted = (uint64_t *)take((size_t)count * 8 + 32);
	w.cache = (uint32_t *)take(level > D + 1 ? (size_t)count * 4 + 16 : 16);
	w.tag_words = level > D + 1 ? tag_bitmap_words(sparse_words) : 4;
	w.tagbits = (uint32_t *)take(w.tag_words * 4);
	w.total_bytes = off;
}

static uint32_t grid_for(uint64_t items, uint32_t per_block, uint32_t cap) {
	const uint64_t b = (items + per_block - 1) / per_block;
	return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(b, cap));
}

static BuildBatch single_batch(const BuildWorkspace &w, uint32_t count, uint32_t level, uint32_t *pool,
                               uint64_t capacity) {
	BuildBatch bb;
	memset(&bb, 0, sizeof(bb));
	bb.M = 1;
	bb.dense_bits = w.dv.bits;
	bb.dense_prefix = w.dv.prefix;
	bb.gstate = w.state;
	bb.sorted_total = count;
	bb.dense_total = w.dense_words;
	bb.nb_total = w.nb;
	bb.reduce_total = dense_reduce_chunks(w.dv.D);
	BuildMesh &m = bb.one;
	m.pool = pool;
	m.capacity = capacity;
	m.state = w.state;
	m.dv = w.dv;
	m.frag_base = 0;
	m.count = count;
	m.level = level;
	m.bshift = w.bshift;
	m.nb = w.nb;
	m.bucket_base = 0;
	m.dense_base = 0;
	m.item_base = 0;
	m.sorted_pad = 0;
	m.mark_word = w.dv.off[w.dv.D];
	m.parent_off = level > 1 ? w.dv.off[std::min(level - 1, kDenseMaxDepth + 1)] : 0u;
	return bb;
}

// The leaf windows' bookkeeping: windows per mesh, each listed bucket's item range and leaf span, the
// first and last bucket of every window.  Without sparse depths none of it reads the bucketed copy, so it
// runs on the build's second stream beside the bucketed copy.
struct LeafTables {
	uint4 *bmeta;
	uint32_t *win_base, *wfirst, *wlast;
};

template <bool B>
static void launch_leaf_prep(const BuildBatch &bb, uint32_t M, uint32_t nb_total, const uint32_t *boff,
                             const uint32_t *blist, const BuildState *gstate, const LeafTables &lt, bool any_sparse,
                             uint64_t *sorted, const uint32_t *cache, cudaStream_t stream) {
	const int sms = device_sm_count();
	const uint32_t meta_items = std::max<uint32_t>(nb_total, M);
	SVO_LAUNCH("leaf_window_scan", stream, ::svo::launch_k(leaf_window_scan<B>, 1, kTPB, 0, stream, bb, lt.win_base););
	SVO_LAUNCH("bucket_meta", stream,
	           ::svo::launch_k(bucket_meta<B>, grid_for(meta_items, kTPB, (uint32_t)sms * 4), kTPB, 0, stream, bb, boff, blist, gstate, lt.bmeta););
	if (any_sparse)
		SVO_LAUNCH("bucket_span_sparse", stream,
		           ::svo::launch_k(bucket_span_sparse<B>, grid_for((uint64_t)nb_total * 32, kTPB, (uint32_t)sms * 8), kTPB, 0, stream, sorted, bb, blist, cache, gstate, lt.bmeta););
	SVO_LAUNCH("bucket_windows", stream,
	           ::svo::launch_k(bucket_windows<B>, grid_for(nb_total, kTPB, (uint32_t)sms * 4), kTPB, 0, stream, bb, blist, gstate, lt.bmeta, lt.win_base, lt.wfirst, lt.wlast););
}

// The stages shared by a single build and a batch.  `maxD` = deepest dense depth of any mesh.
template <bool B>
static void launch_dense_and_scatter(const uint64_t *frags, uint64_t n, uint32_t tune_level, const BuildBatch &bb,
                                     uint32_t M, uint32_t maxD,
                                     uint32_t dense_words, uint32_t items_total, uint32_t nb_total, BuildState *gstate,
                                     unsigned long long *descs, uint32_t *bcount, uint32_t *boff, uint32_t *bfill,
                                     uint32_t *blist, unsigned long long *bdescs, uint64_t *sorted,
                                     const LeafTables *early_leaf_prep, const ClearList &clear, cudaStream_t stream) {
	const int sms = device_sm_count();
	const uint32_t sweep = (uint32_t)sms * (uint32_t)tune_value(kTuneSweepBlocks, tune_level, n);
	SVO_LAUNCH("build_init", stream,
	           ::svo::launch_k(build_init<B>, std::max<uint32_t>(M, (uint32_t)sms * 4), 256, 0, stream, bb, gstate, clear););
	SVO_LAUNCH("dense_mark", stream,
	           ::svo::launch_k(dense_mark<B>, grid_for(n, kTPB * kSweepRuns, sweep), kTPB, 0, stream, frags, n, bb, bcount););
	// Two independent chains after the sweep: the bucket scan (then, once the dense prefix is final, the
	// level table, the interior words and, without sparse depths, the leaf windows' bookkeeping) on a
	// second stream, the dense reduce / scan and then the bucketed copy on the caller's stream; the copy
	// needs the bucket offsets and the dense prefix, and the caller's later work waits for both.
	SideFork fork(stream, tune_value(kTuneBuildStreams, tune_level, n) == 2);
	cudaStream_t aux = fork.side();
	SVO_LAUNCH("bucket_scan", aux,
	           ::svo::launch_k(bucket_scan, (nb_total + kScanTile - 1) / kScanTile, kTPB, 0, aux, bcount, nb_total, boff, blist, gstate, bdescs););
	fork.mark_side(0);
	if (maxD >= 1) {
		if (maxD >= 2 && bb.reduce_total)
			SVO_LAUNCH("dense_reduce", stream,
			           ::svo::launch_k(dense_reduce<B>, std::min<uint32_t>(bb.reduce_total, (uint32_t)sms * 8), 256, 0, stream, bb););
		SVO_LAUNCH("dense_scan", stream,
		           ::svo::launch_k(dense_scan<B>, grid_for(dense_words, kDenseTile, (uint32_t)sms * 4), kTPB, 0, stream, bb, dense_words, gstate, descs););
		fork.side_waits_main();
		// the level table, the interior words and (without sparse depths) the leaf bookkeeping on the
		// second stream; the bucketed copy needs none of them
		SVO_LAUNCH("dense_finish", aux, ::svo::launch_k(dense_finish<B>, (M + 127) / 128, 128, 0, aux, bb););
		SVO_LAUNCH("dense_write", aux,
		           ::svo::launch_k(dense_write<B>, grid_for(items_total, kTPB, (uint32_t)sms * 16), kTPB, 0, aux, bb, items_total););
	} else {
		fork.side_waits_main(); // the leaf ranges of the level tables
	}
	if (early_leaf_prep) // no sparse depths: the leaf windows' bookkeeping beside the bucketed copy
		launch_leaf_prep<B>(bb, M, nb_total, boff, blist, gstate, *early_leaf_prep, false, sorted, nullptr, aux);
	fork.mark_side(1);
	fork.main_waits(0); // bucket offsets
	// the bucketed copy: leaf items when the leaf parents are dense (their bitmap is final now), fragments
	// for the sparse levels otherwise
	SVO_LAUNCH("bucket_scatter", stream,
	           ::svo::launch_k(bucket_scatter<B>, grid_for(n, kTPB * kScatterRuns, sweep), kTPB, 0, stream, frags, n, bb, boff, bfill, sorted););
	fork.main_waits(1); // interior words
}

static void launch_sparse(const uint64_t *sorted, uint32_t count, uint32_t level, const DenseView &dv, uint32_t *pool,
                          uint64_t capacity, uint32_t *cache, uint32_t *tagbits, uint64_t tag_words, BuildState *state,
                          unsigned long long *descs, BuildState *gstate, cudaStream_t stream) {
	const int sms = device_sm_count();
	const uint32_t tag_blocks =
	    grid_for(((uint64_t)count + 3) / 4, kTPB, (uint32_t)sms * (uint32_t)tune_value(kTuneSweepBlocks, level, count));
	for (uint32_t depth = dv.D + 1; depth < level; ++depth) {
		SVO_LAUNCH("tag_clear", stream,
		           ::svo::launch_k(tag_clear, (uint32_t)sms * 4, kTPB, 0, stream, tagbits, tag_words, capacity, state, depth, gstate););
		SVO_LAUNCH("build_tag", stream,
		           ::svo::launch_k(build_tag, tag_blocks, kTPB, 0, stream, sorted, count, level, depth, pool, tagbits, cache, dv, state, gstate););
		SVO_LAUNCH("build_alloc", stream,
		           ::svo::launch_k(build_alloc, (uint32_t)sms * 4, kTPB, 0, stream, pool, capacity, depth, tagbits, state, descs, gstate););
	}
}

// The leaf stage; `prepared`: the windows' bookkeeping already ran beside the bucketed copy.
template <bool B>
static void launch_leaf_stage(const BuildBatch &bb, uint32_t M, uint32_t tune_level, uint64_t n, uint32_t nb_total,
                              const uint32_t *boff, const uint32_t *blist, const BuildState *gstate, const LeafTables &lt,
                              bool any_sparse, bool prepared, uint64_t *sorted, const uint32_t *cache, cudaStream_t stream) {
	const int sms = device_sm_count();
	const size_t smem = kLeafSlots * sizeof(unsigned long long); // 32 KB: below the default dynamic limit
	const uint32_t blocks = (uint32_t)sms * (uint32_t)tune_value(kTuneLeafBlocks, tune_level, n);
	if (!prepared) launch_leaf_prep<B>(bb, M, nb_total, boff, blist, gstate, lt, any_sparse, sorted, cache, stream);
	SVO_LAUNCH("build_leaf_windows", stream,
	           ::svo::launch_k(build_leaf_windows<B>, blocks, kTPB, smem, stream, sorted, bb, lt.bmeta, lt.win_base, lt.wfirst, lt.wlast, const_cast<BuildState *>(gstate)););
}

cudaError_t build_launch_interior(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool,
                                  uint64_t capacity, const BuildWorkspace &w, cudaStream_t stream) {
	// scan descriptors, dense bitmaps, bucket counts and cursors (adjacent), bucket-scan descriptors
	const ClearList clear{{w.descs, w.dv.bits, w.bcount, w.bdescs},
	                      {w.desc_count * sizeof(unsigned long long), (size_t)w.dense_words * 4,
	                       (size_t)((char *)w.boff - (char *)w.bcount), w.bdesc_count * sizeof(unsigned long long)}};
	const BuildBatch bb = single_batch(w, count, level, pool, capacity);
	const uint32_t items = dense_items(level, w.dv.D, w.dv.off);
	const LeafTables lt{w.bmeta, w.win_base, w.wfirst, w.wlast};
	const bool sparse = level > w.dv.D + 1;
	launch_dense_and_scatter<false>(frags, count, level, bb, 1, w.dv.D, w.dense_words, items, w.nb, w.state, w.descs, w.bcount,
	                                w.boff, w.bfill, w.blist, w.bdescs, w.sorted, sparse ? nullptr : &lt, clear, stream);
	if (sparse)
		launch_sparse(w.sorted, count, level, w.dv, pool, capacity, w.cache, w.tagbits, w.tag_words, w.state, w.descs,
		              w.state, stream);
	return cudaGetLastError();
}

cudaError_t build_launch_leaf(uint32_t count, uint32_t level, uint32_t *pool, uint64_t capacity,
                              const BuildWorkspace &w, cudaStream_t stream) {
	const BuildBatch bb = single_batch(w, count, level, pool, capacity);
	const LeafTables lt{w.bmeta, w.win_base, w.wfirst, w.wlast};
	const bool sparse = level > w.dv.D + 1; // without sparse depths build_launch_interior prepared the windows
	launch_leaf_stage<false>(bb, 1, level, count, w.nb, w.boff, w.blist, w.state, lt, sparse, !sparse, w.sorted, w.cache,
	                         stream);
	return cudaGetLastError();
}

cudaError_t build_launch_export(const BuildWorkspace &w, uint32_t level, uint32_t count, void *out,
                                cudaStream_t stream) {
	const BuildBatch bb = single_batch(w, count, level, nullptr, 0);
	SVO_LAUNCH("build_export", stream, ::svo::launch_k(build_export<false>, 1, 32, 0, stream, bb, w.state, (uint32_t *)out););
	return cudaGetLastError();
}

// The whole build of a batch: clears, dense and bucket stages over all meshes, the sparse depths of the
// meshes that have them (one mesh at a time), the leaf stage over all buckets, and one export record per
// mesh to result_dev.
cudaError_t build_launch_batch(const uint64_t *frags, const BuildBatchPlan &p, void *result_dev, cudaStream_t stream) {
	// scan descriptors, dense bitmaps, bucket counts and cursors (adjacent), bucket-scan descriptors
	const ClearList clear{{p.descs, p.bb.dense_bits, p.bcount, p.bdescs},
	                      {p.desc_count * sizeof(unsigned long long), (size_t)p.dense_total * 4,
	                       (size_t)((char *)p.boff - (char *)p.bcount), p.bdesc_count * sizeof(unsigned long long)}};
	cudaError_t e = cudaSuccess;
	const LeafTables lt{p.bmeta, p.win_base, p.wfirst, p.wlast};
	launch_dense_and_scatter<true>(frags, p.frags_total, p.max_level, p.bb, p.M, p.max_D, p.dense_total, p.items_total,
	                               p.nb_total, p.gstate, p.descs, p.bcount, p.boff, p.bfill, p.blist, p.bdescs, p.sorted,
	                               p.any_sparse ? nullptr : &lt, clear, stream);
	for (uint32_t m = 0; m < p.M; ++m) {
		const BuildMesh &md = p.meshes[m];
		if (md.level <= md.dv.D + 1) continue; // no sparse depths (an empty mesh still sets its leaf range)
		e = cudaMemsetAsync(p.descs, 0, p.desc_count * sizeof(unsigned long long), stream);
		if (e != cudaSuccess) return e;
		const uint64_t sb = md.frag_base + md.sorted_pad;
		launch_sparse(p.sorted + sb, md.count, md.level, md.dv, md.pool, md.capacity, p.cache + sb, p.tagbits, p.tag_words,
		              md.state, p.descs, p.gstate, stream);
	}
	launch_leaf_stage<true>(p.bb, p.M, p.max_level, p.frags_total, p.nb_total, p.boff, p.blist, p.gstate, lt,
	                        p.any_sparse, !p.any_sparse, p.sorted, p.cache, stream);
	SVO_LAUNCH("build_export", stream,
	           ::svo::launch_k(build_export<true>, (p.M + 127) / 128, 128, 0, stream, p.bb, p.gstate, (uint32_t *)result_dev););
	return cudaGetLastError();
}

} // namespace svo
