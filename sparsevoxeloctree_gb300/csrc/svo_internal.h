// svo_internal.h — declarations shared by the engine's translation units (not part of the ABI).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/svo.h"

namespace svo {

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Device status word bits (one word per call; the host turns them into svo_status codes).
enum : uint32_t {
	kStatusTimeout = 1u,  // a bounded look-back wait gave up
	kStatusCapacity = 2u, // an output buffer or the 30-bit pointer range would overflow
	kStatusMalformed = 4u  // a march met a pointer outside the pool or a tree deeper than its level
};

void note_launch();      // counts kernel launches (svo_kernel_launches)
int svo_fail(int code, const char *fmt, ...); // sets the calling thread's svo_last_error message

// Brackets one kernel launch with CUDA events on its stream while profiling is enabled.
struct ProfScope {
	ProfScope(const char *name, cudaStream_t stream);
	~ProfScope();
	int slot;
	cudaStream_t stream;
};
#define SVO_LAUNCH(name, stream, ...)                                                                       \
	do {                                                                                                \
		::svo::ProfScope prof_scope_(name, stream);                                                 \
		__VA_ARGS__;                                                                                \
		::svo::note_launch();                                                                       \
	} while (0)
int device_sm_count();   // SMs of the current device (cached per device)

// ---------------------------------------------------------------- voxelize
enum : uint32_t { kCtrTicketA = 0, kCtrTicketB = 1, kCtrStatus = 2, kCtrCount = 8 };
enum : uint32_t { kStatusUnits = 8u }; // the unit arrays of the workspace are too small (caller retries)

struct VoxWorkspace {
	uint32_t n;
	uint64_t unit_cap;             // units the unit arrays hold
	uint64_t *small_off;           // [n+1] fragment offsets of small triangles
	uint32_t *unit_off;            // [n+1] unit offsets of large triangles
	unsigned long long *unit_frag; // [unit_cap+1] fragment offset of each unit inside the large region
	uint32_t *unit_tri;            // [unit_cap+1] triangle of each unit
	unsigned long long *descs, *descs2, *descs3; // look-back descriptors of the three scans
	size_t desc_bytes;
	uint32_t *counters;            // tile tickets, status
	unsigned long long *totals;    // [0] fragments, [1] units, [2] status (written by vox_launch_totals)
};
uint64_t vox_default_unit_cap(uint32_t n);
size_t vox_workspace_bytes(uint32_t n, uint64_t unit_cap);
size_t vox_workspace_layout(void *ws, uint32_t n, uint64_t unit_cap, VoxWorkspace &w);
cudaError_t vox_launch_count(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                             cudaStream_t stream);
cudaError_t vox_launch_totals(const VoxWorkspace &w, cudaStream_t stream);
cudaError_t vox_launch_emit(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                            uint64_t *frags, uint64_t capacity, cudaStream_t stream);

// ---------------------------------------------------------------- build
struct LevelInfo {
	uint32_t begin;         // first word of this depth's node range
	uint32_t num;           // words in the range (8 per parent node)
	uint32_t blocks_before; // child blocks allocated before this depth's alloc
	uint32_t nodes;         // non-empty words at this depth (written by its alloc)
};

struct BuildState {
	uint32_t status;
	uint32_t range_words;
	uint32_t leaves;
	uint32_t pad;
	uint32_t tiles[16];                 // tile tickets of each depth's alloc scan
	LevelInfo lv[SVO_LEVEL_MAX + 2];    // lv[d] for depth d (1-based)
	uint32_t buckets;                   // non-empty fragment buckets (bucket_scan)
	uint32_t leaf_ticket;               // buckets claimed by the leaf stage
};

constexpr uint32_t kDenseMaxDepth = 9; // deepest depth held as a dense occupancy bitmap (8^9 bits)

// Dense occupancy bitmaps of depths 1..D, concatenated (level d at word off[d]), and the exclusive
// prefix of their popcounts over the concatenation (prefix[off[D+1]] = occupied cells of depths 1..D).
struct DenseView {
	uint32_t *bits;
	uint32_t *prefix;
	uint32_t off[kDenseMaxDepth + 2];
	uint32_t D;
};

struct BuildWorkspace {
	BuildState *state;
	unsigned long long *descs;
	size_t desc_count;
	DenseView dv;
	uint32_t dense_words;
	uint32_t bshift;                // bucket key = Morton code of the voxel >> bshift bits per axis
	uint32_t nb;                    // buckets (8^(level - bshift))
	uint32_t *bcount;               // [nb] fragments per bucket
	uint32_t *boff;                 // [nb+1] first fragment of each bucket in `sorted`
	uint32_t *bfill;                // [nb] scatter cursors
	uint32_t *blist;                // [nb] non-empty buckets in order
	uint4 *bmeta;                   // [nb] per listed bucket: first/last item, first/last leaf slot
	unsigned long long *bdescs;     // look-back descriptors of the bucket scan (2 scans)
	size_t bdesc_count;
	uint64_t *sorted;               // [count] the fragments, bucketed
	uint32_t *cache;                // [count] node index of the previous sparse depth, per sorted fragment
	size_t total_bytes;
};
uint64_t build_pool_bound(uint32_t count, uint32_t level);
uint32_t dense_depth(uint32_t level);
void build_workspace_layout(void *ws, uint32_t count, uint32_t level, uint64_t capacity, BuildWorkspace &w);
// Interior levels (dense bitmaps, then sparse tag/alloc); the leaf range ends up in state->lv[level].
cudaError_t build_launch_interior(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool,
                                  uint64_t capacity, const BuildWorkspace &w, cudaStream_t stream);
// Leaf words of the deepest level from the bucketed fragments.
cudaError_t build_launch_leaf(uint32_t count, uint32_t level, uint32_t *pool, uint64_t capacity,
                              const BuildWorkspace &w, cudaStream_t stream);
// svo_build_info followed by the uint32 status word, written to device memory `out`.
cudaError_t build_launch_export(const BuildWorkspace &w, uint32_t level, uint32_t count, void *out,
                                cudaStream_t stream);

// ---------------------------------------------------------------- march
struct MarchArgs {
	const uint32_t *pool;
	uint32_t range;
	uint32_t level;
	const svo_ray *rays;
	svo_camera cam;
	uint32_t width, height;
	uint32_t n;
	svo_hit *hits;
	unsigned long long *ticket;   // device work-slot ticket (zeroed by march_launch)
	unsigned long long *fetches;  // optional node-load total
	uint32_t *status;             // device status word
};
cudaError_t march_launch(const MarchArgs &a, bool camera, cudaStream_t stream);
cudaError_t bounce_launch(const svo_hit *hits, uint32_t n, uint64_t seed, svo_ray *rays, cudaStream_t stream);

} // namespace svo
