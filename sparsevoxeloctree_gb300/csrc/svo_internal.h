// svo_internal.h — declarations shared by the engine's translation units (not part of the ABI).
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#include "../../include/svo.h"

namespace svo {

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Device status word bits (one word per call; the host turns them into svo_status codes).
enum : uint32_t {
	kStatusTimeout = 1u,  // a bounded look-back wait gave up
	kStatusCapacity = 2u, // an output buffer or the 30-bit pointer range would overflow
	kStatusMalformed = 4u, // a march met a pointer outside the pool or a tree deeper than its level
	kStatusBadFragment = 16u, // a build met a fragment whose coordinates lie outside its octree level
	kStatusCheck = 32u     // an internal bounds check failed (builds compiled with SVO_CHECKED; id in bits 16+)
};

void note_launch();      // counts kernel launches (svo_kernel_launches)
void note_allocation();  // counts memory allocation calls the library makes (svo_allocation_calls)
// The wait-fault test hook (svo_debug_wait_fault) of each translation unit with bounded device waits.
cudaError_t vox_set_wait_fault(uint32_t limit, uint32_t withheld);
cudaError_t build_set_wait_fault(uint32_t limit, uint32_t withheld);
cudaError_t march_set_wait_fault(uint32_t limit, uint32_t withheld);
cudaError_t texture_set_wait_fault(uint32_t limit, uint32_t withheld);
int svo_fail(int code, const char *fmt, ...); // sets the calling thread's svo_last_error message

// Every memory allocation the library makes goes through these (counted by svo_allocation_calls).
template <typename T> cudaError_t counted_malloc(T **p, size_t bytes) {
	note_allocation();
	return cudaMalloc((void **)p, bytes);
}
template <typename T> cudaError_t counted_malloc_async(T **p, size_t bytes, cudaStream_t s) {
	note_allocation();
	return cudaMallocAsync((void **)p, bytes, s);
}
template <typename T> cudaError_t counted_malloc_host(T **p, size_t bytes) {
	note_allocation();
	return cudaMallocHost((void **)p, bytes);
}

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

// A fork of the caller's stream onto a second stream of the calling thread (one per thread, device and
// stream priority, so concurrent callers and stream captures never share it, and the side work keeps
// the caller's priority) and back, with events made per call.  When a stream or event cannot be had,
// every "side" launch runs on the caller's stream instead.
class SideFork {
public:
	explicit SideFork(cudaStream_t main, bool enabled = true) : main_(main) {
		if (!enabled) return;
		constexpr int kSlots = 8; // priority levels kept apart (the device's range is smaller)
		thread_local cudaStream_t sides[kSlots] = {};
		thread_local int side_dev[kSlots] = {-1, -1, -1, -1, -1, -1, -1, -1};
		int dev = 0, prio = 0, least = 0, greatest = 0;
		if (cudaGetDevice(&dev) != cudaSuccess) return;
		if (cudaStreamGetPriority(main, &prio) != cudaSuccess ||
		    cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess)
			prio = least = greatest = 0;
		const int slot = std::min(std::max(least - prio, 0), kSlots - 1);
		cudaStream_t &side = sides[slot];
		if (!side || side_dev[slot] != dev) {
			if (cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, prio) != cudaSuccess) {
				side = nullptr;
				return;
			}
			side_dev[slot] = dev;
		}
		for (cudaEvent_t &e : ev_)
			if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return;
		if (cudaEventRecord(ev_[2], main_) != cudaSuccess || cudaStreamWaitEvent(side, ev_[2], 0) != cudaSuccess) return;
		side_ = side;
	}
	~SideFork() {
		for (cudaEvent_t e : ev_)
			if (e) cudaEventDestroy(e);
	}
	cudaStream_t side() const { return side_ ? side_ : main_; }
	void mark_side(int k) {
		if (side_) cudaEventRecord(ev_[k], side_);
	}
	void main_waits(int k) {
		if (side_) cudaStreamWaitEvent(main_, ev_[k], 0);
	}
	void side_waits_main() {
		if (side_ && cudaEventRecord(ev_[3], main_) == cudaSuccess) cudaStreamWaitEvent(side_, ev_[3], 0);
	}

private:
	cudaStream_t main_, side_ = nullptr;
	cudaEvent_t ev_[4] = {nullptr, nullptr, nullptr, nullptr};
};


// Launch parameters set by the autotuner (svo_tune_set), per (level, size class of the launch's work).
enum : uint32_t {
	kTuneMarchBlock = 0,   // threads per march block: 64, 128, 256
	kTuneMarchRays = 1,    // rays a lane takes per ticket: 1, 2; 0 = persistent refill
	kTuneMarchShared = 2,  // traversal stack in shared (1) or local (0) memory
	kTuneSweepBlocks = 3,  // blocks per SM of the fragment sweeps
	kTuneLeafBlocks = 4,   // blocks per SM of the leaf stage
	kTuneEmitBlocks = 5,   // blocks per SM of the voxelizer's emission
	kTuneBuildStreams = 6, // streams of the build's bucket / dense stages: 1, or 2 (a second stream overlaps them)
	kTuneMarchBufferRays = 7, // as kTuneMarchRays, for marches of a ray buffer (svo_raycast); tuned separately
	kTuneDownloadBands = 8,   // row bands of svo_raycast_camera_download (traced and copied to the host in turn)
	kTuneParams = 9
};
int tune_value(uint32_t param, uint32_t level, uint64_t items);

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

// One mesh of a voxelize batch.  The batch's triangles are indexed flat: mesh m owns flat triangles
// [tri_base[m], tri_base[m+1]), read from its own buffer.
struct VoxMesh {
	const svo_triangle *tris; // (device)
	uint32_t level;
	uint32_t pad;
};

struct VoxBatch {
	const VoxMesh *table;         // [M] (device; unused for a single mesh)
	const uint32_t *tri_base;     // [M+1] (device)
	unsigned long long *shifts;   // [2M] output shift of small / large fragments (vox_launch_batch_totals)
	unsigned long long *mesh_out; // [4M] per mesh: fragments, first fragment, units, 0 (for the host)
	uint32_t M;
	uint32_t max_level;           // deepest level of the batch (selects its launch parameters)
	VoxMesh one;                  // the mesh of a single voxelization
};

uint64_t vox_default_unit_cap(uint32_t n);
size_t vox_workspace_bytes(uint32_t n, uint64_t unit_cap);
size_t vox_workspace_layout(void *ws, uint32_t n, uint64_t unit_cap, VoxWorkspace &w);
cudaError_t vox_launch_count(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                             cudaStream_t stream);
cudaError_t vox_launch_totals(const VoxWorkspace &w, cudaStream_t stream);
// Count, totals and emission into `frags` (capacity fragments) in one stream-ordered sequence; the
// small-triangle emission overlaps the unit scan on a second stream.
cudaError_t vox_launch_count_emit(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                                  uint64_t *frags, uint64_t capacity, cudaStream_t stream);
// two_streams = false: every launch on `stream`, no side stream or event is made (svo_voxelize_static)
cudaError_t vox_launch_emit(const svo_triangle *tris, uint32_t n, uint32_t level, const VoxWorkspace &w,
                            uint64_t *frags, uint64_t capacity, cudaStream_t stream,
                            bool two_streams = true);
// Batched forms: n = flat triangles of all meshes.  The batch totals write per-mesh counts and the
// output shifts that make every mesh's fragments contiguous (mesh order; inside a mesh the order of a
// single voxelization of that mesh).
cudaError_t vox_launch_count_batch(const VoxBatch &vb, uint32_t n, const VoxWorkspace &w, cudaStream_t stream);
cudaError_t vox_launch_batch_totals(const VoxBatch &vb, uint32_t n, const VoxWorkspace &w, cudaStream_t stream);
cudaError_t vox_launch_emit_batch(const VoxBatch &vb, uint32_t n, const VoxWorkspace &w, uint64_t *frags,
                                  uint64_t capacity, cudaStream_t stream);

// Texture-sampled fragment colour (texture.cu).  One texture of a set: its size, mip levels and the
// first texel of every level in the set's linear float texel array.
struct TexDesc {
	uint64_t level_off[16];
	uint32_t width, height, levels, pad;
};
// Samples the textured candidates (colour, alpha test) and compacts the survivors in order into `out`;
// scratch (vox_texture_scratch_bytes, device) returns the survivor count in its first word.
cudaError_t vox_texture_launch(const uint64_t *cand, uint64_t n_cand, const svo_triangle *tris,
                               const svo_triangle_uv *uvs, uint32_t n_tris, uint32_t level, const VoxWorkspace &w,
                               const svo_texture_set *set, uint64_t *out, unsigned long long *scratch,
                               cudaStream_t stream);
size_t vox_texture_scratch_bytes(uint64_t n_cand);

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

constexpr uint32_t kDenseMaxDepth = 10; // deepest depth held as a dense occupancy bitmap (8^10 bits, 128 MiB)
// Fragments from which an octree of level >= 11 keeps depth 10 dense too: its 8^10-bit bitmap and prefix
// (256 MiB, scanned once) cost about what one sparse tag + alloc pass over that many fragments does.
constexpr uint32_t kDeepDenseMinFragments = 1u << 24;
constexpr uint32_t kBuildScanTile = 8192; // words per tile of the dense scan (a mesh's dense region is a multiple)

// Dense occupancy bitmaps of depths 1..D, concatenated (level d at word off[d]), and the exclusive
// prefix of their popcounts over the concatenation (prefix[off[D+1]] = occupied cells of depths 1..D).
struct DenseView {
	uint32_t *bits;
	uint32_t *prefix;
	uint32_t off[kDenseMaxDepth + 2];
	uint32_t D;
};

// One mesh of a build batch.  Fragments of mesh m are [frag_base, frag_base + count) of the batch's
// fragment list; its bucketed copy starts at frag_base + sorted_pad (16-byte aligned); its buckets,
// dense region and dense_write items are slices of the batch's concatenated arrays.
struct BuildMesh {
	uint32_t *pool;         // (device) the mesh's node pool
	uint64_t capacity;      // words
	BuildState *state;      // (device) the mesh's level table, counters and status
	DenseView dv;           // the mesh's dense region (prefix values count from the mesh's first word)
	uint64_t frag_base;
	uint32_t count;
	uint32_t level;
	uint32_t bshift, nb;    // bucket key shift, buckets of the mesh
	uint32_t bucket_base;   // first bucket in the concatenated bucket arrays
	uint32_t dense_base;    // first word of the dense region in the concatenated bitmaps
	uint32_t item_base;     // first dense_write item
	uint32_t sorted_pad;    // padding of the mesh's bucketed copy before it (fragments)
	// scalar copies of dv.off entries the per-fragment sweeps need (no runtime-indexed array in a loop)
	uint32_t mark_word;     // dense_base + dv.off[D]: first word of the depth-D bitmap in the concatenation
	uint32_t parent_off;    // dv.off[level-1]: depth level-1 bitmap (leaf parents) inside the mesh region
};

// Kernel view of a build: one mesh by value, or a table of M meshes in device memory with the flat
// offsets the kernels search (each [M+1], non-decreasing).
struct BuildBatch {
	const BuildMesh *table;
	const unsigned long long *frag_base;
	const uint32_t *bucket_base;
	const uint32_t *item_base;
	const uint32_t *dense_base;
	const uint32_t *reduce_base; // [M+1] dense_reduce chunks before each mesh (chunks of meshes with D >= 2)
	uint32_t *dense_bits;   // base of the concatenated bitmaps
	uint32_t *dense_prefix; // base of the concatenated prefixes
	BuildState *gstate;     // batch-wide tickets and status (the mesh's own state for a single build)
	unsigned long long sorted_total; // entries of the bucketed copy (bounds checks)
	uint32_t dense_total, nb_total;  // dense words and buckets of all meshes (bounds checks)
	uint32_t reduce_total;           // dense_reduce chunks of all meshes
	uint32_t M;
	BuildMesh one;
};

struct BuildWorkspace {
	BuildState *state;
	unsigned long long *descs;
	size_t desc_count;
	DenseView dv;
	uint32_t dense_words;           // words of the dense scan (the region, padded to whole tiles)
	uint32_t bshift;                // bucket key = Morton code of the voxel >> bshift bits per axis
	uint32_t nb;                    // buckets (8^(level - bshift))
	uint32_t *bcount;               // [nb] fragments per bucket
	uint32_t *boff;                 // [nb+1] first fragment of each bucket in `sorted`
	uint32_t *bfill;                // [nb] scatter cursors
	uint32_t *blist;                // [nb] non-empty buckets in order
	uint4 *bmeta;                   // [nb] per listed bucket: first/last item, first/last leaf slot
	unsigned long long *bdescs;     // look-back descriptors of the bucket scan (2 scans)
	size_t bdesc_count;
	uint32_t *win_base;             // [2] leaf windows before / after the mesh (leaf_window_scan)
	uint32_t *wfirst, *wlast;       // [leaf_window_bound] first and last listed bucket of each leaf window
	uint64_t *sorted;               // [count] the fragments, bucketed
	uint32_t *cache;                // [count] node index of the previous sparse depth, per sorted fragment
	uint32_t *tagbits;              // [tag_words] tag bit per word of the sparse depth being built
	uint64_t tag_words;
	size_t total_bytes;
};
uint64_t build_pool_bound(uint32_t count, uint32_t level);
uint32_t dense_depth(uint32_t level, uint32_t count); // deepest dense depth D of a build of `count` fragments
uint32_t bucket_shift(uint32_t level, uint32_t D);   // bucket edge of the build's fragment buckets: 2^shift voxels
uint64_t leaf_window_bound(uint32_t count, uint32_t level); // leaf windows a dense-parent mesh can need
uint32_t dense_words_of(uint32_t d);
uint32_t dense_reduce_chunks(uint32_t D); // work items of dense_reduce for a mesh whose dense depth is D
// Words of the dense bitmaps of depths 1..D (32-byte aligned levels) and their offsets.
uint32_t dense_layout(uint32_t D, uint32_t off[kDenseMaxDepth + 2]);
// dense_write items of a mesh (parent words of the depths whose child blocks it writes, plus the root).
uint32_t dense_items(uint32_t level, uint32_t D, const uint32_t off[kDenseMaxDepth + 2]);
uint64_t max_sparse_level_words(uint32_t count, uint32_t level, uint32_t D);
uint64_t tag_bitmap_words(uint64_t level_words); // words of a sparse depth's tag bitmap
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

// A build batch: the host plan and the device views of its shared arrays.
struct BuildBatchPlan {
	BuildBatch bb;                  // device table view (bb.table etc. point into the plan buffer)
	std::vector<BuildMesh> meshes;  // host copy of the table
	uint32_t M;
	uint64_t frags_total;           // fragments of all meshes
	uint32_t nb_total;              // buckets of all meshes
	uint32_t dense_total;           // dense words of all meshes (whole scan tiles per mesh)
	uint32_t items_total;           // dense_write items of all meshes
	uint32_t max_level, max_D;
	uint64_t sorted_total;          // fragments of the bucketed copy, with per-mesh padding
	BuildState *gstate;             // batch-wide tickets, bucket total and scan status
	unsigned long long *descs;      // dense-scan / sparse-alloc descriptors
	size_t desc_count;
	uint32_t *bcount, *bfill, *boff, *blist;
	uint4 *bmeta;
	unsigned long long *bdescs;
	size_t bdesc_count;
	uint32_t *dense_prefix;
	uint64_t *sorted;
	uint32_t *cache;                // only when a mesh has sparse levels (level > 10)
	uint32_t *tagbits;              // tag bitmap of the sparse depth being built (one mesh at a time)
	uint64_t tag_words;
	uint32_t *win_base;             // [M+1] leaf windows before each mesh (leaf_window_scan)
	uint32_t *wfirst, *wlast;       // [sum of leaf_window_bound] first and last listed bucket per window
	bool any_sparse;                // a mesh's leaf parents are sparse (level > 10)
};
cudaError_t build_launch_batch(const uint64_t *frags, const BuildBatchPlan &p, void *result_dev, cudaStream_t stream);

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
	const float *beam;            // camera rays: beam texels to advance each ray by (null: none)
	uint32_t row0, rows;          // camera rays: trace image rows [row0, row0 + rows) only (rows = 0: to the end)
};
cudaError_t march_launch(const MarchArgs &a, bool camera, cudaStream_t stream);
// Beam pre-pass texels ((width + 7) / 8 + 1) x ((height + 7) / 8 + 1) for camera `a.cam`.
cudaError_t beam_launch(const MarchArgs &a, float *beam, cudaStream_t stream);
// Beam pre-pass + beam-advanced camera march in one launch (hits as march_launch with a.beam, and the
// beam image written to `beam`).
cudaError_t march_beam_fused_launch(const MarchArgs &a, float *beam, cudaStream_t stream);
// Octree_RayMarchOcclude for a.n rays: occluded[i] = 1 when ray i hits a leaf.
cudaError_t occlude_launch(const MarchArgs &a, uint32_t *occluded, cudaStream_t stream);
cudaError_t bounce_launch(const svo_hit *hits, uint32_t n, uint64_t seed, svo_ray *rays, cudaStream_t stream);

// Path tracer (shader/path_tracer.comp as PathTracer::CmdRender dispatches it, src/PathTracer.cpp:205-227).
// The environment map as shader/environment_map.glsl samples it: texels = (radiance rgb, pdf weight) and
// the alias table (prob, alias) per texel, both row-major width x height.
struct EnvMapView {
	const float4 *texels;
	const uint2 *alias;
	uint32_t width, height;
};
// A path between the wavefront launches of one sample: throughput, radiance, current vertex (position,
// normal code: axis | negative << 2), and the first hit's albedo and normal code (kPathNoNormal: none).
constexpr uint32_t kPathNoNormal = 0xffu;
struct PathState {
	float acc[3], rad[3], pos[3], dalb[3];
	uint32_t nrm, first_nrm;
};
// Tickets (one per launch of a sample) and surviving-path counts (one per vertex), zeroed per sample.
constexpr uint32_t kPtMaxVertices = 32;
constexpr size_t kPtScratchBytes = kPtMaxVertices * sizeof(unsigned long long) + (kPtMaxVertices + 1) * sizeof(uint32_t);
struct PtArgs {
	const uint32_t *pool;
	uint32_t range, level;
	svo_camera cam;
	uint32_t width, height;
	uint32_t bounce;     // uBounce: path vertices per sample
	uint32_t light_type; // uLightType: 0 constant colour, 1 environment map
	float const_color[3];
	float env_rotation, env_multiplier;
	EnvMapView env;
	const uint32_t *sobol; // Sobol state: 2 * (bounce + 1) dimensions, then the sample index
	const uint8_t *noise;  // 256 x 256 RG8 noise texture
	float4 *color;         // accumulated radiance (rgba32f)
	uint32_t *albedo;      // accumulated first-hit albedo (rgba8 unorm)
	uint32_t *normal;      // accumulated first-hit normal (rgba8 snorm)
	PathState *paths;      // one per pixel
	uint32_t *queue[2];    // surviving paths of the current / next vertex
	unsigned long long *tickets; // kPtScratchBytes: tickets[kPtMaxVertices], then counts[kPtMaxVertices + 1]
	uint32_t *counts;
	uint32_t *status;
};
cudaError_t pt_render_launch(const PtArgs &a, cudaStream_t stream);
// Sobol::CmdNext (sobol.comp): advances the first `dim` dimensions by the Gray-code step.
cudaError_t sobol_next_launch(uint32_t *sobol, const uint32_t *matrices, uint32_t dim, cudaStream_t stream);

// One request's share of a shared march launch: its octree, its rays (a ray buffer, or camera rays for
// the first n pixels, row-major, of a width x height image) and its hit buffer.  Work slots of the
// launch are numbered job after job; slot_begin is the job's first.
struct MarchJob {
	const uint32_t *pool;
	uint32_t range, level;
	const svo_ray *rays;   // null: camera rays
	svo_camera cam;
	uint32_t width, height;
	uint32_t n;
	uint32_t req; // the job's request in its batch: its rays report a malformed pool in status[req]
	svo_hit *hits;
	unsigned long long slot_begin;
};
// Work slots of a job (camera jobs: 32 per 8x4 tile of the rows holding its n pixels).
uint64_t march_job_slots(const MarchJob &j);
// Device-side address of page-locked host memory mapped into the device's address space (cudaHostAlloc;
// cudaHostRegister with the mapped flag), when it is aligned to `align` bytes; null otherwise.
inline void *mapped_host_ptr(const void *p, size_t align) {
	if (!p) return nullptr;
	cudaPointerAttributes attr;
	if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
		cudaGetLastError(); // not a CUDA-known pointer: clear the error
		return nullptr;
	}
	if (attr.type != cudaMemoryTypeHost || !attr.devicePointer) return nullptr;
	return ((uintptr_t)attr.devicePointer % align) == 0 ? attr.devicePointer : nullptr;
}
// `jobs` (device) holds njobs jobs whose slot_begin are set; total = slots of all jobs.  ticket (device,
// 8 B) is zeroed here; status (device) gets kStatusMalformed for a malformed pool.
// fetches (may be null) accumulates the node words the jobs' rays read.
cudaError_t march_jobs_launch(const MarchJob *jobs, uint32_t njobs, uint64_t total, unsigned long long *ticket,
                              uint32_t *status, unsigned long long *fetches, cudaStream_t stream);

// One request's bounce rays: n hits in, n rays out, seeded per request (ray index local to the job).
struct BounceJob {
	const svo_hit *hits;
	svo_ray *rays;
	unsigned long long seed;
	unsigned long long begin; // first flat index of the job in the launch
};
cudaError_t bounce_jobs_launch(const BounceJob *jobs, uint32_t njobs, uint64_t total, cudaStream_t stream);

} // namespace svo
