/*
 * svo.h — C ABI of the GB300 sparse-voxel-octree engine.
 *
 * Three stages, each a stream-ordered call on one CUDA device:
 *   svo_voxelize  triangles  -> voxel-fragment list   (replaces Voxelizer, src/Voxelizer.cpp:5-179)
 *   svo_build     fragments  -> octree node pool      (replaces OctreeBuilder, src/OctreeBuilder.cpp:8-214,
 *                                                       and Octree::Update, src/Octree.cpp:22-35)
 *   svo_raycast   octree+rays -> hits                 (replaces Octree_RayMarchLeaf, shader/octree.glsl:179-340,
 *                                                       as called by shader/octree_tracer.frag:23-37)
 *
 * Formats kept bit-for-bit from the reference:
 *   fragment  uint32 x: vx | vy<<12 | (vz&0xff)<<24 ; uint32 y: (vz>>8)<<28 | rgb24   (shader/voxelizer.frag:40-42)
 *   node word 0 = empty; bit31 = non-empty; interior: bits0-29 = word index of the first of 8 children;
 *             leaf: 0xC0000000 | min(count,63)<<24 | B<<16 | G<<8 | R       (shader/octree_tag_node.comp:10-16,59;
 *                                                                             shader/octree_alloc_node.comp:21)
 *   the root's 8 children are words 0..7; a child block occupies 8 consecutive words.
 *
 * Differences from the reference, all deliberate and documented in the design notes:
 *   - fragment order is deterministic (triangle order, then span order), the multiset is what is compared;
 *   - child blocks are numbered by a prefix sum in word order (breadth-first, canonical) instead of racing atomics;
 *   - leaf colour is the channel-wise integer mean floor(sum/n) (order independent) instead of a CAS running mean.
 *
 * Pointers marked (device) are CUDA device pointers; `stream` is a cudaStream_t (NULL = legacy default stream).
 * Every call returns an svo_status; svo_last_error() gives a readable message for the calling thread.
 */
#ifndef SVO_H
#define SVO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
typedef enum svo_status {
	SVO_OK = 0,
	SVO_ERR_INVALID = 1,  /* bad argument (level out of range, null pointer, misaligned buffer) */
	SVO_ERR_CAPACITY = 2, /* an output would exceed its buffer or the format (detected; nothing written out of bounds) */
	SVO_ERR_OOM = 3,      /* device allocation failed */
	SVO_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up (status word set by the kernel) */
	SVO_ERR_CUDA = 5      /* a CUDA runtime call failed */
} svo_status;

/* ------------------------------------------------------------------ limits (src/Config.hpp:18-22) */
#define SVO_LEVEL_MIN 1u                 /* kOctreeLevelMin */
#define SVO_LEVEL_MAX 12u                /* kOctreeLevelMax: 12-bit fragment coordinates */
#define SVO_MAX_POOL_WORDS (1u << 30)    /* 30-bit child pointers (0x3fffffff mask) */
#define SVO_SUBVOXEL_BITS 8u             /* fixed-point vertex snapping: 1/256 voxel */
#define SVO_STACK_SIZE 23u               /* STACK_SIZE of the ray march (shader/octree.glsl:43) */
#define SVO_MARCH_MAX_ITER (1u << 20)    /* march iteration bound (malformed pools only; a valid octree needs far fewer) */

/* ------------------------------------------------------------------ data types */

/* One input triangle, 48 bytes, 16-byte aligned.  Vertex k is v[3k..3k+2] in the unit cube [0,1]^3
 * (the reference's [-1,1] normalised scene maps as p = (p_ref + 1) / 2, src/Scene.cpp:90-99).
 * rgb[k] = 0x00BBGGRR colour of vertex k; the triangle's colour is floor((c0+c1+c2)/3) per channel. */
typedef struct svo_triangle {
	float v[9];
	uint32_t rgb[3];
} svo_triangle;

/* A ray in octree space: the octree occupies [1,2]^3 exactly as in shader/octree.glsl:53. */
typedef struct svo_ray {
	float o[3];
	float d[3];
} svo_ray;

/* Camera uniform block (shader/camera.glsl:8): position, look, side, up as vec4 (w ignored). */
typedef struct svo_camera {
	float pos[4];
	float look[4];
	float side[4];
	float up[4];
} svo_camera;

/* Result of one ray, 32 bytes.
 *   t        t_min when the march stopped
 *   pos      o_pos of Octree_RayMarchLeaf (octree space, clamped to the hit cube and nudged by EPS)
 *   node     the leaf word that was hit (0 on a miss); colour = node & 0xffffff (R low byte)
 *   iter     loop iterations (o_iter of the reference)
 *   voxel    leaf coordinates at the octree level (0xffff on a miss)
 *   flags    bit0 hit; bits1-2 normal axis (0=x,1=y,2=z); bit3 normal points to -axis;
 *            bit4 the march was aborted (a child pointer outside the pool's range, an interior word
 *            below the octree level, or SVO_MARCH_MAX_ITER iterations): the pool is malformed and the
 *            ray counts as a miss.  A pool made by svo_build never sets it;
 *            bit5 (beam march without a beam image only) the wait for one of the ray's tile's beam
 *            texels gave up, so the ray was marched from the camera: apart from this bit its result is
 *            svo_raycast_camera's.  A correct run never sets it. */
typedef struct svo_hit {
	float t;
	float pos[3];
	uint32_t node;
	uint32_t iter;
	uint16_t voxel[3];
	uint16_t flags;
} svo_hit;

#define SVO_HIT_FLAG_HIT 1u
#define SVO_HIT_NORMAL_AXIS(f) (((f) >> 1) & 3u)
#define SVO_HIT_NORMAL_NEG 8u
#define SVO_HIT_FLAG_ABORTED 16u
#define SVO_HIT_FLAG_BEAM_WAIT 32u

/* A voxel-fragment list (device memory). data holds `count` uint64 fragments: low word = fragment.x,
 * high word = fragment.y (the reference's uvec2 layout). */
typedef struct svo_fraglist {
	uint64_t *data;    /* (device) */
	uint32_t count;    /* fragments written */
	uint32_t level;    /* octree level the fragments were voxelized at */
	uint64_t capacity; /* fragments the buffer can hold */
	uint32_t owned;    /* 1 if allocated by the library (freed by svo_fraglist_destroy) */
	uint32_t units;    /* raster units of the large triangles (sizes svo_voxelize_into's workspace) */
} svo_fraglist;

/* An octree node pool (device memory). */
typedef struct svo_octree {
	uint32_t *words;        /* (device) node words; the used range is [0, range_words) */
	uint64_t capacity;      /* words the buffer can hold */
	uint32_t range_words;   /* words in use = (blocks + 1) * 8 (src/OctreeBuilder.cpp:213, in words) */
	uint32_t level;         /* octree level (resolution 2^level) */
	uint32_t owned;         /* 1 if allocated by the library (freed by svo_octree_destroy) */
	uint32_t reserved;
} svo_octree;

/* Per-level and per-stage counters a build reports (read back once, at the end of the build). */
typedef struct svo_build_info {
	uint32_t level;
	uint32_t fragments;
	uint32_t range_words;
	uint32_t leaves;                     /* non-empty leaf words */
	uint32_t level_nodes[SVO_LEVEL_MAX]; /* non-empty node words at depth 1..level */
} svo_build_info;

/* Caller-supplied device allocator.  alloc(user, bytes) returns device memory (256-byte aligned) or
 * NULL; release(user, ptr) gives back memory the library asked for.  Buffers handed to the caller in an
 * output (fragment list data, octree words) are never released by the library: the caller owns them
 * (svo_fraglist.owned / svo_octree.owned = 0).  Scratch buffers are released before the call returns,
 * after the work that uses them has been ordered on the call's stream. */
typedef struct svo_allocator {
	void *(*alloc)(void *user, size_t bytes);
	void (*release)(void *user, void *ptr);
	void *user;
} svo_allocator;

/* ------------------------------------------------------------------ library */
const char *svo_last_error(void);
const char *svo_version(void);
/* Number of kernels this library launched since load (all devices); a cheap sanity counter for callers. */
uint64_t svo_kernel_launches(void);
/* Number of memory allocation calls (device, stream-ordered, pinned host, or through a caller's
 * svo_allocator) this library made since load; lets a caller check that a path allocates nothing. */
uint64_t svo_allocation_calls(void);
/* Test hook for the failure path of the bounded device waits; no counterpart in the reference, whose
 * shaders wait on nothing.  With spin_limit > 0 every wait of the single-pass scans (voxelize, build,
 * textured compaction) and of the fused beam march gives up after spin_limit iterations, and the scan tile
 * or beam texel numbered `withheld` never publishes its value, so the waits on it run out: scans then
 * report SVO_ERR_TIMEOUT (no later stage writes through their offsets) and beam marches set
 * SVO_HIT_FLAG_BEAM_WAIT on the rays concerned.  spin_limit = 0 restores the defaults.  It applies to the
 * current device, process-wide, to calls launched after it returns; not for production use. */
int svo_debug_wait_fault(uint32_t spin_limit, uint32_t withheld);

/* Device memory and transfers for callers without the CUDA headers (C, C++, FFI bindings).  Allocation
 * is stream-ordered (freed memory stays pooled for reuse); copies are asynchronous on `stream` except
 * svo_download with sync = 1, which returns once the data is in host memory.  Copies go through
 * unified addressing, so either side may also be device memory (a device-to-device copy). */
int svo_device_alloc(void **ptr, size_t bytes, void *stream);
void svo_device_free(void *ptr, void *stream);
int svo_upload(void *dst_device, const void *src_host, size_t bytes, void *stream);
int svo_download(void *dst_host, const void *src_device, size_t bytes, int sync, void *stream);
int svo_stream_synchronize(void *stream);

/* Per-kernel timing (the GPU-timestamp instrument of src/LoaderThread.cpp:57-97, per kernel instead of
 * per stage).  While enabled, every launch of this library is bracketed by two CUDA events recorded on
 * its own stream.  svo_profile_summary synchronizes on those events and writes a JSON object
 * {"kernel": {"launches": n, "ms": total}, ...} into buf; it returns the length it needed (excluding
 * the terminating NUL).  Enabling clears earlier records. */
void svo_profile_enable(int on);
size_t svo_profile_summary(char *buf, size_t cap);

/* Launch parameters (an autotuner's table: sparsevoxeloctree_gb300/autotune.py measures the candidates and
 * sets the best).  A value is kept per (parameter, octree level, size class), the size class of a launch
 * being that of its work items (fragments, triangles or rays): class 0 below 65,536, then one class per
 * factor 4, class 7 from 2^30.  Results do not depend on these values, only the speed does. */
#define SVO_TUNE_MARCH_BLOCK 0u         /* threads per march block: 64, 128 (default), 256 */
#define SVO_TUNE_MARCH_RAYS_PER_LANE 1u /* rays a lane takes per warp ticket: 1 (default), 2; or 0: persistent
                                           refill (each lane takes a new ray as soon as its ray ends) */
#define SVO_TUNE_MARCH_STACK_SHARED 2u  /* traversal stack in shared memory (1, default) or local memory (0) */
#define SVO_TUNE_SWEEP_BLOCKS 3u        /* blocks per SM of the build's fragment sweeps (default 16) */
#define SVO_TUNE_LEAF_BLOCKS 4u         /* blocks per SM of the build's leaf stage (default 6) */
#define SVO_TUNE_EMIT_BLOCKS 5u         /* blocks per SM of the voxelizer's emission (default 16) */
#define SVO_TUNE_BUILD_STREAMS 6u       /* streams of the build's bucket and dense stages: 1, or 2 (default: a second
                                           stream of the calling thread overlaps them) */
#define SVO_TUNE_MARCH_BUFFER_RAYS 7u   /* as SVO_TUNE_MARCH_RAYS_PER_LANE for svo_raycast's ray buffers (default 1) */
#define SVO_TUNE_DOWNLOAD_BANDS 8u      /* svo_raycast_camera_download: 0 (default): the march writes into a mapped
                                         * host buffer; 1, 2, 4, 8, 16: row bands traced and copied in turn */
#define SVO_TUNE_PARAMS 9u
/* level 0: every level; size_class -1: every class.  Rejects values a parameter does not allow. */
int svo_tune_set(uint32_t param, uint32_t level, int32_t size_class, int32_t value);
/* The value a launch of `items` work items at `level` uses. */
int svo_tune_get(uint32_t param, uint32_t level, uint64_t items);
uint32_t svo_tune_size_class(uint64_t items);
void svo_tune_reset(void);

/* ------------------------------------------------------------------ voxelize (Voxelizer) */

/* Voxelizer::Create + CmdVoxelize (src/Voxelizer.cpp:5-26, 134-179): count pass, exact allocation,
 * emit pass.  `tris` (device) holds n_tris triangles.  On success *out owns a new device buffer holding
 * out->count fragments (out->capacity >= out->count: when the same triangle buffer, count and level
 * were voxelized recently, the list is sized by that earlier count and the emission is queued before
 * the count is read back).  Blocks the calling thread once to read the fragment count, as the
 * reference does (src/Voxelizer.cpp:151-155). */
int svo_voxelize(const svo_triangle *tris, uint32_t n_tris, uint32_t level, svo_fraglist *out, void *stream);

/* The count pass alone (src/Voxelizer.cpp:134-158, uCountOnly = 1): writes the fragment count to
 * *count_host (blocking). */
int svo_voxelize_count(const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint64_t *count_host,
                       void *stream);

/* Count and emit into a caller buffer (no allocation, no host synchronisation): frags (device) holds
 * `capacity` fragments; count_dev (device, 2 x uint64) receives [0] the number of fragments the
 * triangles produce and [1] a status word (0 = complete).  Fragments beyond `capacity` are not written
 * (count_dev[0] > capacity tells the caller to retry with a larger buffer).  Scratch comes from
 * `workspace` (device, 256-byte aligned, `workspace_bytes` long), at least
 * svo_voxelize_workspace_size(n_tris, units) with `units` from an earlier count of the same mesh
 * (svo_fraglist.units) or 0 for a guess; when the mesh's large triangles need more raster units than
 * the workspace holds, their fragments are skipped and count_dev[1] is non-zero. */
size_t svo_voxelize_workspace_size(uint32_t n_tris, uint64_t units);
int svo_voxelize_into(const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint64_t *frags, uint64_t capacity,
                      uint64_t *count_dev, void *workspace, size_t workspace_bytes, void *stream);

/* svo_voxelize with every device allocation made through `alloc` (NULL = the library's stream-ordered
 * pool, exactly svo_voxelize). */
int svo_voxelize_ex(const svo_triangle *tris, uint32_t n_tris, uint32_t level, const svo_allocator *alloc,
                    svo_fraglist *out, void *stream);

void svo_fraglist_destroy(svo_fraglist *f, void *stream);

/* svo_voxelize_into for callers that cannot allocate device memory (a frame loop that forbids
 * allocation after start-up, a thread holding an allocator lock, a fully pre-partitioned device).
 * No counterpart in the reference.  The caller passes the triangles, the fragment buffer (`capacity`
 * fragments) and count_dev (device, 2 x uint64: [0] fragments produced, [1] status, 0 = complete); the
 * engine's scratch is a fixed 16 MiB array in device memory that every GPU loading this library holds
 * until the process exits.  It takes at most 262,144 triangles (more: SVO_ERR_CAPACITY, nothing
 * launched) whose large triangles split into at most about 1 million raster units (1,047,808 at the
 * triangle limit, up to 1.29 million for small meshes; a 1024 x 1024 wall is 4,096; beyond the limit count_dev[1] is non-zero and svo_voxelize must be used).  No
 * allocation call is made.  The first call on a device looks up that array's address; make that first
 * call before any stream capture.  All calls share the array: calls whose work overlaps on the GPU
 * (other streams, other host threads) race and must be serialized by the caller. */
int svo_voxelize_static(const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint64_t *frags, uint64_t capacity,
                        uint64_t *count_dev, void *stream);

/* ------------------------------------------------------------------ build (OctreeBuilder + Octree) */

/* OctreeBuilder::Create + CmdBuild + GetOctreeRange + Octree::Update (src/OctreeBuilder.cpp:8-50,142-214,
 * src/Octree.cpp:22-35).  Builds the octree of `frags` (device, count fragments at `level`).  On success
 * *out owns a device pool of exactly out->range_words words.  Blocks once at the end to read the range,
 * as GetOctreeRange does.  `info` (host, may be NULL) receives the per-level counters. */
int svo_build(const uint64_t *frags, uint32_t count, uint32_t level, svo_octree *out, svo_build_info *info,
              void *stream);

/* Convenience: svo_build on a fragment list. */
int svo_build_fraglist(const svo_fraglist *f, svo_octree *out, svo_build_info *info, void *stream);

/* Build into a caller pool (no allocation, no host synchronisation).  pool (device, 16-byte aligned)
 * holds `capacity` words (svo_build_pool_bound(count, level) always suffices); `workspace` (device,
 * 256-byte aligned) holds `workspace_bytes` bytes, at least svo_build_workspace_size(count, level,
 * capacity, leaf_words) (about 12 bytes per fragment plus the dense bitmaps; `leaf_words` is accepted
 * for compatibility and no longer changes the size: the leaf level accumulates in on-chip memory).
 * The result (svo_build_info followed by a uint32 status word, 0 = complete) is written to
 * `result_dev` (device).  A pool too small for the octree reports SVO_ERR_CAPACITY through the status
 * word; a workspace below svo_build_workspace_size is rejected before any launch. */
size_t svo_build_workspace_size(uint32_t count, uint32_t level, uint64_t capacity, uint64_t leaf_words);
uint64_t svo_build_pool_bound(uint32_t count, uint32_t level);
int svo_build_into(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool, uint64_t capacity,
                   void *workspace, size_t workspace_bytes, void *result_dev, void *stream);

/* svo_build with every device allocation made through `alloc` (NULL = svo_build). */
int svo_build_ex(const uint64_t *frags, uint32_t count, uint32_t level, const svo_allocator *alloc, svo_octree *out,
                 svo_build_info *info, void *stream);

void svo_octree_destroy(svo_octree *o, void *stream);

/* ------------------------------------------------------------------ batched voxelize + build */

/* One mesh of a batch: its triangles (device, 16-byte aligned) and the octree level it is built at. */
typedef struct svo_batch_mesh {
	const svo_triangle *tris;
	uint32_t n_tris;
	uint32_t level;
} svo_batch_mesh;

/* A batcher builds many meshes together (the reference builds one mesh per Voxelizer::CmdVoxelize +
 * OctreeBuilder::CmdBuild, src/Voxelizer.cpp:134-179, src/OctreeBuilder.cpp:142-210; LoaderThread
 * drives one at a time, src/LoaderThread.cpp:43-116).  It owns device arenas that only grow (a repeated
 * batch allocates nothing) and the CUDA graphs of its launch sequences.  Not thread-safe: one caller at
 * a time per batcher. */
typedef struct svo_batcher svo_batcher;

int svo_batcher_create(svo_batcher **out);
void svo_batcher_destroy(svo_batcher *b);

/* Voxelizes and builds every mesh: one count pass over all triangles, one blocking readback of the
 * per-mesh fragment counts, then the emit pass, every build level and the result export as launches
 * that each cover all meshes (depths below level 10 of meshes finer than 2^10 run per mesh), recorded
 * as a CUDA graph that is replayed while the batch's sizes and buffers are unchanged, and one blocking
 * readback of the per-mesh results.  Per mesh, fragments and octree are identical to svo_voxelize +
 * svo_build of that mesh alone.  Results are read with svo_batcher_result and stay valid until the
 * next svo_batcher_build on this batcher or its destruction. */
int svo_batcher_build(svo_batcher *b, const svo_batch_mesh *meshes, uint32_t n_meshes, void *stream);

/* Number of meshes of the last batch. */
uint32_t svo_batcher_meshes(const svo_batcher *b);

/* Views of mesh `mesh` of the last batch (any output may be NULL): its fragment list and octree inside
 * the batcher's shared fragment list and node pool (owned = 0: never destroy them), and its counters. */
int svo_batcher_result(const svo_batcher *b, uint32_t mesh, svo_fraglist *frags, svo_octree *octree,
                       svo_build_info *info);

/* Graph recording on (default) or off (every launch issued directly). */
int svo_batcher_set_graph(svo_batcher *b, int on);

/* Graphs captured and replays since creation. */
void svo_batcher_stats(const svo_batcher *b, uint64_t *graph_captures, uint64_t *graph_replays);

/* ------------------------------------------------------------------ march (OctreeTracer) */

/* Octree_RayMarchLeaf (shader/octree.glsl:179-340) for n rays (device) -> n hits (device).
 * `fetches_dev` (device, may be NULL) accumulates the number of node words the march loaded. */
int svo_raycast(const svo_octree *o, const svo_ray *rays, uint32_t n, svo_hit *hits, uint64_t *fetches_dev,
                void *stream);

/* OctreeTracer::CmdDrawPipeline (src/OctreeTracer.cpp:213-246) with shader/octree_tracer.frag:24,37:
 * one primary ray per pixel of a width x height image, d = Camera_GenRay(ivec2(pixel) / size)
 * (shader/camera.glsl:11-14), origin = cam->pos.  Hit of pixel (x, y) goes to hits[y * width + x]. */
int svo_raycast_camera(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height, svo_hit *hits,
                       uint64_t *fetches_dev, void *stream);

/* svo_raycast_camera with the hits delivered into host memory (`hits_host`, width * height hits, 16-byte
 * aligned) as they are produced.  When `hits_host` is page-locked and mapped into the device's address space
 * (cudaHostAlloc; cudaHostRegister with cudaHostRegisterMapped) the march stores the hits straight into it
 * and `hits` may be NULL.  Otherwise (or with SVO_TUNE_DOWNLOAD_BANDS set to a band count) the image is
 * traced in bands of rows into `hits` (device, the whole image) and each band is copied to `hits_host` on a
 * second stream while the next band is traced.  Either way the hits are in host memory once `stream`
 * reaches this point, and they are those of svo_raycast_camera (OctreeTracer::CmdDrawPipeline + reading
 * the image back). */
int svo_raycast_camera_download(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height,
                                svo_hit *hits, svo_hit *hits_host, uint64_t *fetches_dev, void *stream);

/* Beam optimisation of the tracer (OctreeTracer::CmdBeamRenderPass, src/OctreeTracer.cpp:183-211, with
 * shader/octree_tracer_beam.frag and Octree_RayMarchCoarse, shader/octree.glsl:47-177): one start distance
 * per corner of each SVO_BEAM_SIZE x SVO_BEAM_SIZE pixel tile, written to `beam` (device floats,
 * svo_beam_texels(width, height) of them, row-major with (width + 7) / 8 + 1 per row); 1e10 where the
 * tile's cone misses the octree. */
#define SVO_BEAM_SIZE 8u /* kBeamSize (src/Config.hpp:22) */
uint64_t svo_beam_texels(uint32_t width, uint32_t height);
int svo_beam_prepass(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height, float *beam,
                     void *stream);

/* svo_raycast_camera with the beam enabled (shader/octree_tracer.frag:27-33): each primary ray starts at
 * o + d * (the least of the 4 beam texels at the corners of its tile), then Octree_RayMarchLeaf.  `beam`
 * (device) from svo_beam_prepass for the same octree, camera and size, or NULL to run the pre-pass here
 * (on stream-ordered scratch).  hit.t counts from the advanced origin. */
int svo_raycast_camera_beam(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height,
                            const float *beam, svo_hit *hits, uint64_t *fetches_dev, void *stream);

/* Octree_RayMarchOcclude (shader/octree.glsl:504-629), the shadow-ray march of the path tracer:
 * occluded[i] (device uint32) = 1 when ray i hits a leaf, else 0.  A ray with d = 0 is not occluded. */
int svo_occlude(const svo_octree *o, const svo_ray *rays, uint32_t n, uint32_t *occluded, void *stream);

/* Secondary rays for hits: o = hit pos, d = cosine-weighted direction about the hit normal
 * (shader/diffuse.glsl:7-14, shader/util.glsl:5-9, shader/path_tracer.comp:44-47) with (u1,u2) from a
 * counter hash of (seed, ray index).  Misses produce a ray with d = 0 that svo_raycast reports as a miss
 * without touching the octree. */
int svo_bounce_rays(const svo_hit *hits, uint32_t n, uint64_t seed, svo_ray *rays, void *stream);

/* ------------------------------------------------------------------ serving */

/* A server keeps many octrees resident and traces requests from many callers in shared launches
 * (continuous batching).  The reference renders one octree per frame (Application::draw_frame,
 * src/Application.cpp:130-159; PathTracer::CmdRender, src/PathTracer.cpp:192-215) and rebuilds on its
 * loader thread (src/LoaderThread.cpp:43-116); this is the multi-request form of that path.  A scheduler
 * thread takes pending requests in arrival order into a batch while the batch's rays, request count and
 * the device bytes in flight stay within the limits below, and issues it on a free lane (stream): one
 * march launch for all primary rays, one bounce launch, one march launch for all bounce rays, one copy
 * of each request's hits.  Up to `lanes` batches run at once; requests that arrive meanwhile are admitted
 * as lanes and memory free up.  A request's hits are those of svo_raycast_camera / svo_bounce_rays /
 * svo_raycast run for it alone. */
typedef struct svo_server svo_server;

typedef struct svo_server_config {
	uint64_t hbm_budget_bytes;   /* resident octrees + buffers of requests in flight (0: 40 GiB) */
	uint32_t lanes;              /* batches in flight at once (0: 3) */
	uint32_t max_batch_rays;     /* hits per batch (0: 8 Mi); a larger request runs alone */
	uint32_t max_batch_requests; /* requests per batch (0: 256) */
	uint32_t flags;              /* SVO_SERVER_COUNT_FETCHES: count the node words the march reads */
} svo_server_config;

/* svo_server_config.flags: count node fetches into svo_server_stats.node_fetches (for a roofline;
 * costs the served march about 7%). */
#define SVO_SERVER_COUNT_FETCHES 1u

#define SVO_REQUEST_CAMERA 0u /* primary camera rays, then one diffuse bounce ray per primary ray */
#define SVO_REQUEST_RAYS 1u   /* caller-given rays */

typedef struct svo_trace_request {
	uint32_t scene;
	uint32_t mode;          /* SVO_REQUEST_CAMERA or SVO_REQUEST_RAYS */
	svo_camera camera;      /* camera mode: Camera_GenRay of the first n_primary pixels (row-major) of a */
	uint32_t width, height; /*   width x height image, as svo_raycast_camera traces them */
	uint32_t n_primary;
	uint32_t n_rays;        /* rays mode */
	const svo_ray *rays;    /* rays mode: host memory, read while the request runs */
	svo_hit *hits;          /* host memory (page-locked and mapped, as cudaHostAlloc gives it: the march stores
	                           the final hits there directly; otherwise copied): camera mode 2 * n_primary hits,
	                           primary then bounce (bounce i from primary hit i, svo_bounce_rays with `seed`);
	                           rays mode n_rays hits.  Written when the request completes. */
	uint64_t seed;
} svo_trace_request;

typedef struct svo_request_result {
	int status;              /* svo_status of the request */
	uint32_t batch_requests; /* requests in the batch it ran in */
	double submit_us, launch_us, done_us; /* server clock: microseconds since svo_server_create */
} svo_request_result;

typedef struct svo_server_stats {
	uint64_t submitted, completed, failed;
	uint64_t batches, batched_requests; /* shared launches issued and the requests they carried */
	uint64_t rays;                      /* hits produced */
	uint64_t rebuilds;
	uint64_t resident_bytes, inflight_bytes, pending;
	uint64_t node_fetches;              /* node words the served rays read (with SVO_SERVER_COUNT_FETCHES) */
} svo_server_stats;

int svo_server_create(const svo_server_config *cfg, svo_server **out);
/* Finishes every submitted request, then releases the server's streams, buffers and owned octrees. */
void svo_server_destroy(svo_server *s);
/* Makes a caller-owned octree resident as a new scene (kept valid by the caller while the server uses it). */
int svo_server_add_octree(svo_server *s, const svo_octree *o, uint32_t *scene);
/* Voxelizes and builds `tris` (device) into a server-owned scene, pool shrunk to its range (blocking). */
int svo_server_build_scene(svo_server *s, const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint32_t *scene);
/* View of a scene's current octree.  The view stays valid until the scene is rebuilt: a rebuild frees the
 * server-owned octree it replaces once the batches that use it have completed. */
int svo_server_scene(svo_server *s, uint32_t scene, svo_octree *view);
/* Queues a trace request (thread-safe, does not block on the GPU); the request traces the scene's
 * octree current at submission. */
int svo_server_submit_trace(svo_server *s, const svo_trace_request *r, uint64_t *ticket);
/* Queues a rebuild of `scene` from `tris` (device, valid until the request completes) on the server's
 * rebuild thread and stream; the new octree replaces the scene's when done. */
int svo_server_submit_rebuild(svo_server *s, uint32_t scene, const svo_triangle *tris, uint32_t n_tris, uint32_t level,
                              uint64_t *ticket);
/* Blocks until the request completes (timeout_ms < 0: no limit; otherwise SVO_ERR_TIMEOUT after it),
 * fills `res` (may be NULL), releases the ticket and returns the request's status. */
int svo_server_wait(svo_server *s, uint64_t ticket, int timeout_ms, svo_request_result *res);
void svo_server_get_stats(svo_server *s, svo_server_stats *out);

/* ------------------------------------------------------------------ files */

/* Scene::Create's mesh loading (Scene::load_meshes, src/Scene.cpp:36-147) for the engine's triangle
 * format: an OBJ file's faces (polygons as triangle fans; "v", "v/t", "v//n", "v/t/n" and negative
 * indices), its materials' Kd from the mtllib beside it packed like packUnorm4x8 (src/Scene.cpp:164), the
 * vertices the faces use normalised to [-1, 1] as the reference does ((p - centre) / (largest extent /
 * 2), src/Scene.cpp:90-99) and mapped to [0, 1] by p = (p_ref + 1) / 2.  Like the reference, a file
 * without materials is rejected; faces before the first usemtl, or naming an undefined material, take
 * the library's first material.  Textures are not read.  *tris_host is allocated here: release it with svo_free_host. */
int svo_load_obj(const char *path, svo_triangle **tris_host, uint32_t *n_tris);
void svo_free_host(void *p);

/* Octree files: a 32-byte header ("SVOOCT01", uint32 level, uint32 range_words, uint32 header size 32,
 * 12 reserved bytes) followed by the range_words node words, little-endian.  Reading checks the header,
 * the size and that every child pointer lies inside the range at a whole block. */
int svo_octree_write_host(const uint32_t *words, uint32_t range_words, uint32_t level, const char *path);
/* *words allocated here: release it with svo_free_host. */
int svo_octree_read_host(const char *path, uint32_t **words, uint32_t *range_words, uint32_t *level);
/* Device forms: save downloads the used range (blocking); load allocates an owned pool of exactly the
 * range from the stream-ordered pool (free it with svo_octree_destroy). */
int svo_octree_save(const svo_octree *o, const char *path, void *stream);
int svo_octree_load(const char *path, svo_octree *out, void *stream);

/* Host helper: Camera::fetch_uniform_data (src/Camera.cpp:77-95) for a position, yaw, pitch, fov and
 * aspect ratio (radians; the reference's default fov is pi/3, src/Camera.hpp:17). */
void svo_camera_from_angles(const float pos[3], float yaw, float pitch, float fov, float aspect, svo_camera *cam);

/* ------------------------------------------------------------------ textured voxelization
 * shader/voxelizer.frag:27-36: a textured triangle's fragment takes its texture's colour at the pixel
 * centre (packUnorm4x8 of the sRGB-decoded, trilinearly filtered sample) and is discarded where the
 * sampled alpha is below 0.5.  Textures are RGBA8 with sRGB colour and linear alpha
 * (VK_FORMAT_R8G8B8A8_SRGB, src/Scene.cpp:262), repeat addressing, linear filtering between and
 * within mip levels (src/Scene.cpp:409-411); the mip chain is built on the host.  The level of detail
 * comes from the exact screen-space derivatives of the triangle's affine texture mapping. */
typedef struct svo_texture_set svo_texture_set;

/* Texture coordinates of one triangle's vertices and its texture (an index into the set; 0xffffffff or
 * an index beyond the set: the triangle's own colour, as for a draw without a texture). */
typedef struct svo_triangle_uv {
	float uv[6];
	uint32_t texture;
	uint32_t reserved;
} svo_triangle_uv;

/* Scene::load_textures minus the file decoding: `count` RGBA8 images (host, row-major, as stb_image loads
 * them with 4 channels), each up to 32768 x 32768. */
int svo_texture_set_create(const uint8_t *const *rgba, const uint32_t *width, const uint32_t *height, uint32_t count,
                           svo_texture_set **out);
/* One mip level's RGBA8 bytes (host copy; rgba may be null to query the size). */
int svo_texture_set_level(const svo_texture_set *s, uint32_t texture, uint32_t level, uint8_t *rgba, uint32_t *width,
                          uint32_t *height);
void svo_texture_set_destroy(svo_texture_set *s);
/* svo_voxelize with texture-sampled colour and the alpha discard: uvs[i] belongs to tris[i] (device,
 * 8-byte aligned).  The list's capacity is the untextured fragment count; count = the survivors, in the
 * order svo_voxelize emits them. */
int svo_voxelize_textured(const svo_triangle *tris, const svo_triangle_uv *uvs, uint32_t n_tris, uint32_t level,
                          const svo_texture_set *textures, svo_fraglist *out, void *stream);

/* ------------------------------------------------------------------ path tracer
 * PathTracer (src/PathTracer.hpp:15-75; shader/path_tracer.comp): per pixel and sample, the camera ray
 * with a Sobol sub-pixel offset, up to `bounce` path vertices of leaf marches with cosine-weighted
 * diffuse bounces, and the light: a constant colour, or an environment map sampled with multiple
 * importance sampling (light sample with a shadow march + bsdf sample).  Radiance, first-hit albedo and
 * normal accumulate as running means over samples in an rgba32f, an rgba8 unorm and an rgba8 snorm
 * image.  The whole path runs in one kernel; the Sobol state advances on the device after each sample
 * (Sobol::CmdNext).  Transcendentals are the engine's own float restatements (sin/cos, atan, acos),
 * so results are bit-identical to the oracle's. */
typedef struct svo_envmap svo_envmap;
typedef struct svo_path_tracer svo_path_tracer;

/* Lighting (src/Lighting.hpp:7-20) with EnvironmentMap::m_rotation / m_multiplier. */
typedef struct svo_lighting {
	uint32_t type;            /* 0 constant colour, 1 environment map (LightTypes) */
	float sun_radiance[3];    /* m_sun_radiance; the reference's default is 5 (kDefaultConstantColor) */
	float envmap_rotation;    /* radians, default 0 */
	float envmap_multiplier;  /* default 1 */
	const svo_envmap *envmap; /* type 1 with a null map renders with the constant colour (GetFinalLightType) */
} svo_lighting;

/* EnvironmentMap::Reset minus the file decoding (src/EnvironmentMap.cpp:44-52): rgba = width x height
 * float texels (host, row-major; alpha ignored).  Builds the pdf weights (alpha channel) and the alias
 * table on the host and uploads both.  SVO_ERR_INVALID for an image with no positive luminance. */
int svo_envmap_create(const float *rgba, uint32_t width, uint32_t height, svo_envmap **out);
/* Host copies of the tables: rgba (4 floats per texel, alpha = pdf weight), alias (prob, alias per
 * texel).  Either may be null. */
int svo_envmap_tables(const svo_envmap *e, float *rgba, uint32_t *alias);
void svo_envmap_destroy(svo_envmap *e);

/* The engine's default Sobol direction numbers: 64 dimensions x 32 (see svo_path_tracer_set_sobol_matrices). */
int svo_sobol_default_matrices(uint32_t *out);

/* PathTracer::Create + Reset: targets of width x height, `bounce` path vertices (1..31; the reference
 * offers 2..16, default 4), default Sobol numbers and noise texture. */
int svo_path_tracer_create(uint32_t width, uint32_t height, uint32_t bounce, svo_path_tracer **out);
/* PathTracer::Reset: (re)sizes and clears the targets and the Sobol state. */
int svo_path_tracer_reset(svo_path_tracer *pt, uint32_t width, uint32_t height, uint32_t bounce, void *stream);
/* The 256 x 256 RG8 noise texture (uNoise, src/PathTracer.cpp set_noise_image); host or device memory. */
int svo_path_tracer_set_noise(svo_path_tracer *pt, const uint8_t *rg, void *stream);
/* Sobol direction numbers, 64 x 32 words (kMatrices of shader/sobol.comp); host or device memory. */
int svo_path_tracer_set_sobol_matrices(svo_path_tracer *pt, const uint32_t *matrices, void *stream);
/* PathTracer::CmdRender, `samples` times (stream-ordered, no host synchronisation). */
int svo_path_tracer_render(svo_path_tracer *pt, const svo_octree *o, const svo_camera *cam, const svo_lighting *light,
                           uint32_t samples, void *stream);
/* Samples accumulated since the last reset; the device status word (blocking read; nonzero bits as in
 * the march: a malformed pool). */
int svo_path_tracer_info(const svo_path_tracer *pt, uint32_t *spp, uint32_t *status);
/* Device pointers of the targets (float4 colour, uint32 rgba8 albedo and normal words) and of the Sobol
 * state (65 words). */
int svo_path_tracer_images(const svo_path_tracer *pt, void **color, void **albedo, void **normal, void **sobol);
/* ExtractColorImage / ExtractAlbedoImage / ExtractNormalImage (src/PathTracer.cpp:229-298): image 0, 1
 * or 2 as width x height x 3 floats on the host (blocking). */
int svo_path_tracer_extract(const svo_path_tracer *pt, uint32_t image, float *rgb, void *stream);
void svo_path_tracer_destroy(svo_path_tracer *pt);

#ifdef __cplusplus
}
#endif

#endif /* SVO_H */
