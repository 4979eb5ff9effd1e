// batch.cu — many meshes voxelized and built together (the batched form of Voxelizer::CmdVoxelize +
// OctreeBuilder::CmdBuild, src/Voxelizer.cpp:134-179, src/OctreeBuilder.cpp:142-210, which build one
// mesh per call).
//
// A batch is one count pass over the triangles of every mesh, one blocking readback of the per-mesh
// fragment counts (the reference reads its one count the same way, src/Voxelizer.cpp:151-155), then
// the emit pass and every build stage as single launches over all meshes, with per-mesh offsets into
// one shared fragment list and one shared node pool, and one readback of the per-mesh results (the
// reference's GetOctreeRange, src/OctreeBuilder.cpp:212-214, once per batch).  The launch sequence after
// the count (emit, the fixed level loop of the build, export) is captured as a CUDA graph and replayed
// while the batch's sizes and buffers stay the same.  Buffers live in arenas owned by the batcher that
// only grow, so repeated batches allocate nothing.
#include <cstring>
#include <vector>

#include "svo_internal.h"

namespace svo {

int svo_fail(int code, const char *fmt, ...);

namespace {

struct DevArena {
	void *ptr = nullptr;
	size_t cap = 0;
	cudaError_t ensure(size_t bytes) {
		if (bytes <= cap) return cudaSuccess;
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		cap = 0;
		const size_t want = bytes + bytes / 4 + 4096;
		cudaError_t e = counted_malloc(&ptr, want);
		if (e != cudaSuccess) {
			ptr = nullptr;
			return e;
		}
		cap = want;
		return cudaSuccess;
	}
	void release() {
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		cap = 0;
	}
};

struct HostArena {
	void *ptr = nullptr;
	size_t cap = 0;
	cudaError_t ensure(size_t bytes) {
		if (bytes <= cap) return cudaSuccess;
		if (ptr) cudaFreeHost(ptr);
		ptr = nullptr;
		cap = 0;
		const size_t want = bytes + bytes / 4 + 4096;
		cudaError_t e = counted_malloc_host(&ptr, want);
		if (e != cudaSuccess) {
			ptr = nullptr;
			return e;
		}
		cap = want;
		return cudaSuccess;
	}
	void release() {
		if (ptr) cudaFreeHost(ptr);
		ptr = nullptr;
		cap = 0;
	}
};

// Offsets of the plan buffer (device) and of its pinned host mirror; every part 256-byte aligned.
struct PlanLayout {
	size_t vox_mesh, tri_base, shifts, mesh_out, build_mesh, frag_base, bucket_base, item_base, dense_base, reduce_base,
	    results;
	size_t total;
	PlanLayout(uint32_t M) {
		size_t off = 0;
		auto take = [&](size_t bytes) {
			const size_t o = off;
			off += align_up(bytes, 256);
			return o;
		};
		vox_mesh = take(sizeof(VoxMesh) * M);
		tri_base = take(4ull * (M + 1));
		shifts = take(8ull * 2 * M);
		mesh_out = take(8ull * 4 * M);
		build_mesh = take(sizeof(BuildMesh) * M);
		frag_base = take(8ull * (M + 1));
		bucket_base = take(4ull * (M + 1));
		item_base = take(4ull * (M + 1));
		dense_base = take(4ull * (M + 1));
		reduce_base = take(4ull * (M + 1));
		results = take(kResultRec * 4ull * M);
		total = off;
	}
	static constexpr size_t kResultRec = sizeof(svo_build_info) / 4 + 1; // words per mesh result record
};

struct MeshResult {
	uint64_t frag_base = 0, frag_count = 0, units = 0;
	uint64_t pool_base = 0, capacity = 0;
	svo_build_info info;
	uint32_t status = 0;
};

// One captured launch sequence and the key it was captured for.
struct GraphSlot {
	std::vector<uint64_t> key;
	cudaGraphExec_t exec = nullptr;
	void reset() {
		if (exec) cudaGraphExecDestroy(exec);
		exec = nullptr;
		key.clear();
	}
};

} // namespace

struct Batcher {
	DevArena plan, vox_ws, frags, pool, build_ws;
	HostArena staging;
	GraphSlot count_graph, build_graph;
	bool use_graph = true;
	cudaStream_t capture_stream = nullptr;
	uint64_t unit_hint = 0; // raster units of the last batch (first guess for the next one)
	uint64_t graph_replays = 0, graph_captures = 0;
	std::vector<MeshResult> results;
	~Batcher() {
		if (capture_stream) cudaStreamDestroy(capture_stream);
		count_graph.reset();
		build_graph.reset();
		plan.release();
		vox_ws.release();
		frags.release();
		pool.release();
		build_ws.release();
		staging.release();
	}
};

// Runs `record(stream)` (which enqueues work on the stream it is given) through a graph captured for
// `key`, launched on `s`; re-captures when the key differs.  Capture happens on the batcher's own stream
// (the legacy default stream cannot be captured); the graph then runs on the caller's stream.  Without
// graphs, `record` enqueues on `s` directly.
template <typename F>
static cudaError_t run_recorded(Batcher &b, GraphSlot &slot, const std::vector<uint64_t> &key, cudaStream_t s,
                                F &&record) {
	if (!b.use_graph) return record(s);
	if (slot.exec == nullptr || slot.key != key) {
		slot.reset();
		if (!b.capture_stream) {
			cudaError_t e = cudaStreamCreateWithFlags(&b.capture_stream, cudaStreamNonBlocking);
			if (e != cudaSuccess) {
				b.capture_stream = nullptr;
				return e;
			}
		}
		cudaStream_t cs = b.capture_stream;
		cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
		if (e != cudaSuccess) return e;
		cudaError_t er = record(cs);
		cudaGraph_t g = nullptr;
		e = cudaStreamEndCapture(cs, &g);
		if (er != cudaSuccess) {
			if (g) cudaGraphDestroy(g);
			return er;
		}
		if (e != cudaSuccess) return e;
		e = cudaGraphInstantiate(&slot.exec, g, 0);
		cudaGraphDestroy(g);
		if (e != cudaSuccess) {
			slot.exec = nullptr;
			return e;
		}
		slot.key = key;
		++b.graph_captures;
	} else {
		++b.graph_replays;
	}
	return cudaGraphLaunch(slot.exec, s);
}

static int ck(cudaError_t e, const char *what) {
	if (e == cudaSuccess) return SVO_OK;
	cudaGetLastError();
	return svo_fail(e == cudaErrorMemoryAllocation ? SVO_ERR_OOM : SVO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SVO_BCK(call, what)                                                                                 \
	do {                                                                                                \
		const int rc_ = ck((call), what);                                                           \
		if (rc_) return rc_;                                                                        \
	} while (0)

static int batch_build(Batcher &b, const svo_batch_mesh *meshes, uint32_t M, cudaStream_t s) {
	if (M == 0) return svo_fail(SVO_ERR_INVALID, "empty batch");
	if (!meshes) return svo_fail(SVO_ERR_INVALID, "null mesh array");
	uint64_t N = 0;
	for (uint32_t m = 0; m < M; ++m) {
		const svo_batch_mesh &bm = meshes[m];
		if (bm.level < SVO_LEVEL_MIN || bm.level > SVO_LEVEL_MAX)
			return svo_fail(SVO_ERR_INVALID, "mesh %u: level %u outside [%u, %u]", m, bm.level, SVO_LEVEL_MIN, SVO_LEVEL_MAX);
		if (bm.n_tris && !bm.tris) return svo_fail(SVO_ERR_INVALID, "mesh %u: null triangle buffer", m);
		if ((uintptr_t)bm.tris % 16) return svo_fail(SVO_ERR_INVALID, "mesh %u: triangle buffer must be 16-byte aligned", m);
		N += bm.n_tris;
	}
	if (N >= 0xffffffffull) return svo_fail(SVO_ERR_CAPACITY, "a batch holds fewer than 2^32 triangles");
	const PlanLayout pl(M);
	SVO_BCK(b.plan.ensure(pl.total), "batch plan allocation");
	SVO_BCK(b.staging.ensure(pl.total), "batch staging allocation");
	char *hs = (char *)b.staging.ptr, *ds = (char *)b.plan.ptr;

	// ---- voxelize count over every mesh
	VoxMesh *hvm = (VoxMesh *)(hs + pl.vox_mesh);
	uint32_t *htb = (uint32_t *)(hs + pl.tri_base);
	htb[0] = 0;
	for (uint32_t m = 0; m < M; ++m) {
		hvm[m].tris = meshes[m].tris;
		hvm[m].level = meshes[m].level;
		hvm[m].pad = 0;
		htb[m + 1] = htb[m] + meshes[m].n_tris;
	}
	// one copy covers the mesh table and the triangle offsets (adjacent in the layout)
	SVO_BCK(cudaMemcpyAsync(ds, hs, pl.shifts, cudaMemcpyHostToDevice, s), "batch table upload");
	VoxBatch vb;
	memset(&vb, 0, sizeof(vb));
	vb.table = (const VoxMesh *)(ds + pl.vox_mesh);
	vb.tri_base = (const uint32_t *)(ds + pl.tri_base);
	vb.shifts = (unsigned long long *)(ds + pl.shifts);
	vb.mesh_out = (unsigned long long *)(ds + pl.mesh_out);
	vb.M = M;
	vb.max_level = 1;
	for (uint32_t m = 0; m < M; ++m) vb.max_level = std::max(vb.max_level, meshes[m].level);
	const uint32_t n = (uint32_t)N;
	uint64_t unit_cap = std::max<uint64_t>(vox_default_unit_cap(n), b.unit_hint);
	VoxWorkspace vw;
	uint64_t totals[3] = {0, 0, 0};
	for (int attempt = 0;; ++attempt) {
		SVO_BCK(b.vox_ws.ensure(vox_workspace_bytes(n, unit_cap)), "voxelize workspace allocation");
		vox_workspace_layout(b.vox_ws.ptr, n, unit_cap, vw);
		const std::vector<uint64_t> key = {1, M, n, unit_cap, (uint64_t)b.vox_ws.ptr, (uint64_t)b.plan.ptr};
		SVO_BCK(run_recorded(b, b.count_graph, key, s, [&](cudaStream_t rs) -> cudaError_t {
			        cudaError_t e = vox_launch_count_batch(vb, n, vw, rs);
			        if (e == cudaSuccess) e = vox_launch_batch_totals(vb, n, vw, rs);
			        return e;
		        }),
		        "batch voxelize count");
		SVO_BCK(cudaMemcpyAsync(hs + pl.mesh_out, ds + pl.mesh_out, 8ull * 4 * M, cudaMemcpyDeviceToHost, s),
		        "batch count readback");
		SVO_BCK(cudaMemcpyAsync(totals, vw.totals, sizeof(totals), cudaMemcpyDeviceToHost, s), "batch count readback");
		SVO_BCK(cudaStreamSynchronize(s), "batch count");
		if ((totals[2] & kStatusUnits) && attempt == 0) {
			if (totals[1] >= 0xffffffffull) return svo_fail(SVO_ERR_CAPACITY, "too many raster units");
			unit_cap = totals[1];
			continue;
		}
		break;
	}
	if (totals[2] & kStatusTimeout) return svo_fail(SVO_ERR_TIMEOUT, "batch voxelize: a device-side wait gave up");
	if (totals[2]) return svo_fail(SVO_ERR_CAPACITY, "batch voxelize: unit workspace retry failed (status 0x%llx)",
	                               (unsigned long long)totals[2]);
	b.unit_hint = totals[1];
	const uint64_t F = totals[0];
	if (F >= 0xffffffffull) return svo_fail(SVO_ERR_CAPACITY, "%llu fragments exceed the 32-bit batch fragment count",
	                                        (unsigned long long)F);

	// ---- plan: per-mesh offsets into the shared fragment list, node pool and build arrays
	const unsigned long long *hmo = (const unsigned long long *)(hs + pl.mesh_out);
	b.results.assign(M, MeshResult());
	BuildMesh *hbm = (BuildMesh *)(hs + pl.build_mesh);
	unsigned long long *hfb = (unsigned long long *)(hs + pl.frag_base);
	uint32_t *hbb = (uint32_t *)(hs + pl.bucket_base), *hib = (uint32_t *)(hs + pl.item_base),
	         *hdb = (uint32_t *)(hs + pl.dense_base), *hrb = (uint32_t *)(hs + pl.reduce_base);
	BuildBatchPlan p;
	p.M = M;
	p.frags_total = F;
	p.max_level = 0, p.max_D = 0;
	uint64_t pool_words = 0, sorted_total = 0, max_scan = 0, max_sparse = 0;
	uint32_t nb_total = 0, dense_total = 0, items_total = 0;
	bool any_sparse = false;
	uint64_t windows = 0;
	hfb[0] = 0, hbb[0] = 0, hib[0] = 0, hdb[0] = 0, hrb[0] = 0;
	uint32_t reduce_total = 0;
	for (uint32_t m = 0; m < M; ++m) {
		MeshResult &r = b.results[m];
		r.frag_count = hmo[4 * m];
		r.frag_base = hmo[4 * m + 1];
		r.units = hmo[4 * m + 2];
		const uint32_t level = meshes[m].level, count = (uint32_t)r.frag_count;
		BuildMesh &bm = hbm[m];
		memset(&bm, 0, sizeof(bm));
		bm.level = level;
		bm.count = count;
		bm.frag_base = r.frag_base;
		bm.dv.D = dense_depth(level, count);
		const uint32_t words = dense_layout(bm.dv.D, bm.dv.off);
		const uint32_t region = bm.dv.D ? (words + 1 + kBuildScanTile - 1) / kBuildScanTile * kBuildScanTile : 0u;
		bm.dense_base = dense_total;
		bm.mark_word = dense_total + bm.dv.off[bm.dv.D];
		bm.parent_off = level > 1 ? bm.dv.off[std::min(level - 1, kDenseMaxDepth + 1)] : 0u;
		bm.item_base = items_total;
		bm.bucket_base = nb_total;
		bm.bshift = bucket_shift(level, bm.dv.D);
		bm.nb = 1u << (3 * (level - bm.bshift));
		const uint64_t sorted_base = (sorted_total + 3) & ~3ull; // 32-byte aligned per mesh (vector loads)
		bm.sorted_pad = (uint32_t)(sorted_base - r.frag_base);
		sorted_total = sorted_base + count;
		r.capacity = build_pool_bound(count, level);
		r.pool_base = pool_words;
		pool_words += (r.capacity + 63) & ~63ull; // 256-byte aligned pools
		dense_total += region;
		items_total += dense_items(level, bm.dv.D, bm.dv.off);
		nb_total += bm.nb;
		hfb[m + 1] = r.frag_base + count;
		hbb[m + 1] = nb_total;
		hib[m + 1] = items_total;
		hdb[m + 1] = dense_total;
		reduce_total += dense_reduce_chunks(bm.dv.D);
		hrb[m + 1] = reduce_total;
		p.max_level = std::max(p.max_level, level);
		p.max_D = std::max(p.max_D, bm.dv.D);
		windows += leaf_window_bound(count, level);
		if (level > bm.dv.D + 1) {
			any_sparse = true;
			const uint64_t sw = std::min<uint64_t>(max_sparse_level_words(count, level, bm.dv.D), r.capacity);
			max_scan = std::max<uint64_t>(max_scan, sw);
			max_sparse = std::max<uint64_t>(max_sparse, sw);
		}
	}
	if (hfb[M] != F) return svo_fail(SVO_ERR_CUDA, "batch voxelize: per-mesh counts do not add up");
	max_scan = std::max<uint64_t>(max_scan, dense_total);
	p.nb_total = nb_total;
	p.dense_total = dense_total;
	p.items_total = items_total;
	p.sorted_total = sorted_total;

	// ---- buffers
	SVO_BCK(b.frags.ensure(F * 8 + 64), "batch fragment list allocation");
	SVO_BCK(b.pool.ensure(pool_words * 4 + 64), "batch node pool allocation");
	size_t off = 0;
	auto take = [&](size_t bytes) {
		const size_t o = off;
		off += align_up(bytes, 256);
		return o;
	};
	const size_t o_gstate = take(sizeof(BuildState));
	const size_t o_states = take(sizeof(BuildState) * M);
	p.desc_count = (size_t)((max_scan + 2047) / 2048 + 2);
	const size_t o_descs = take(p.desc_count * 8);
	const size_t o_bits = take((size_t)dense_total * 4 + 32);
	const size_t o_prefix = take((size_t)dense_total * 4 + 32);
	const size_t o_bcount = take((size_t)nb_total * 4);
	const size_t o_bfill = take((size_t)nb_total * 4);
	const size_t o_boff = take(((size_t)nb_total + 1) * 4);
	const size_t o_blist = take((size_t)nb_total * 4);
	const size_t o_bmeta = take((size_t)nb_total * 16);
	p.bdesc_count = 2 * ((size_t)(nb_total + 2047) / 2048 + 1);
	const size_t o_bdescs = take(p.bdesc_count * 8);
	const size_t o_win_base = take(4ull * (M + 1));
	const size_t o_wfirst = take(windows * 4 + 4);
	const size_t o_wlast = take(windows * 4 + 4);
	const size_t o_sorted = take(sorted_total * 8 + 32);
	const size_t o_cache = take(any_sparse ? sorted_total * 4 + 16 : 16);
	p.tag_words = any_sparse ? tag_bitmap_words(max_sparse) : 4;
	const size_t o_tagbits = take(p.tag_words * 4);
	SVO_BCK(b.build_ws.ensure(off), "batch build workspace allocation");
	char *ws = (char *)b.build_ws.ptr;
	p.gstate = (BuildState *)(ws + o_gstate);
	BuildState *states = (BuildState *)(ws + o_states);
	p.descs = (unsigned long long *)(ws + o_descs);
	uint32_t *bits = (uint32_t *)(ws + o_bits), *prefix = (uint32_t *)(ws + o_prefix);
	p.bcount = (uint32_t *)(ws + o_bcount);
	p.bfill = (uint32_t *)(ws + o_bfill);
	p.boff = (uint32_t *)(ws + o_boff);
	p.blist = (uint32_t *)(ws + o_blist);
	p.bmeta = (uint4 *)(ws + o_bmeta);
	p.bdescs = (unsigned long long *)(ws + o_bdescs);
	p.dense_prefix = prefix;
	p.win_base = (uint32_t *)(ws + o_win_base);
	p.wfirst = (uint32_t *)(ws + o_wfirst);
	p.wlast = (uint32_t *)(ws + o_wlast);
	p.any_sparse = any_sparse;
	p.sorted = (uint64_t *)(ws + o_sorted);
	p.cache = (uint32_t *)(ws + o_cache);
	p.tagbits = (uint32_t *)(ws + o_tagbits);
	uint32_t *pool = (uint32_t *)b.pool.ptr;
	for (uint32_t m = 0; m < M; ++m) {
		BuildMesh &bm = hbm[m];
		bm.pool = pool + b.results[m].pool_base;
		bm.capacity = b.results[m].capacity;
		bm.state = states + m;
		bm.dv.bits = bits + bm.dense_base;
		bm.dv.prefix = prefix + bm.dense_base;
	}
	p.meshes.assign(hbm, hbm + M);
	memset(&p.bb, 0, sizeof(p.bb));
	p.bb.table = (const BuildMesh *)(ds + pl.build_mesh);
	p.bb.frag_base = (const unsigned long long *)(ds + pl.frag_base);
	p.bb.bucket_base = (const uint32_t *)(ds + pl.bucket_base);
	p.bb.item_base = (const uint32_t *)(ds + pl.item_base);
	p.bb.dense_base = (const uint32_t *)(ds + pl.dense_base);
	p.bb.reduce_base = (const uint32_t *)(ds + pl.reduce_base);
	p.bb.reduce_total = reduce_total;
	p.bb.dense_bits = bits;
	p.bb.dense_prefix = prefix;
	p.bb.gstate = p.gstate;
	p.bb.sorted_total = sorted_total;
	p.bb.dense_total = dense_total;
	p.bb.nb_total = nb_total;
	p.bb.M = M;
	// build tables: BuildMesh[M] .. dense_base[M+1] are adjacent in the layout
	SVO_BCK(cudaMemcpyAsync(ds + pl.build_mesh, hs + pl.build_mesh, pl.results - pl.build_mesh, cudaMemcpyHostToDevice, s),
	        "batch build table upload");

	// ---- emit + build + export: one recorded sequence
	uint64_t *frags = (uint64_t *)b.frags.ptr;
	std::vector<uint64_t> key = {2, M, n, unit_cap, F, (uint64_t)b.plan.ptr, (uint64_t)b.vox_ws.ptr,
	                             (uint64_t)b.frags.ptr, (uint64_t)b.pool.ptr, (uint64_t)b.build_ws.ptr, pool_words};
	for (uint32_t m = 0; m < M; ++m) {
		key.push_back(meshes[m].level);
		key.push_back(b.results[m].frag_count);
		key.push_back(b.results[m].frag_base);
	}
	uint32_t *results_dev = (uint32_t *)(ds + pl.results);
	SVO_BCK(run_recorded(b, b.build_graph, key, s, [&](cudaStream_t rs) -> cudaError_t {
		        cudaError_t e = vox_launch_emit_batch(vb, n, vw, frags, F, rs);
		        if (e == cudaSuccess) e = build_launch_batch(frags, p, results_dev, rs);
		        return e;
	        }),
	        "batch emit and build");
	SVO_BCK(cudaMemcpyAsync(hs + pl.results, ds + pl.results, PlanLayout::kResultRec * 4ull * M, cudaMemcpyDeviceToHost, s),
	        "batch result readback");
	SVO_BCK(cudaStreamSynchronize(s), "batch build");
	const uint32_t *hres = (const uint32_t *)(hs + pl.results);
	int rc = SVO_OK;
	for (uint32_t m = 0; m < M; ++m) {
		MeshResult &r = b.results[m];
		memcpy(&r.info, hres + PlanLayout::kResultRec * m, sizeof(svo_build_info));
		r.status = hres[PlanLayout::kResultRec * m + PlanLayout::kResultRec - 1];
		if (rc == SVO_OK && r.status) {
			if (r.status & kStatusCheck)
				rc = svo_fail(SVO_ERR_CUDA, "batch mesh %u: internal bounds check %u failed (status 0x%x)", m,
				              r.status >> 16, r.status);
			else if (r.status & kStatusBadFragment)
				rc = svo_fail(SVO_ERR_INVALID, "batch mesh %u: fragment coordinates outside the octree level "
				              "(status 0x%x)", m, r.status);
			else if (r.status & kStatusCapacity)
				rc = svo_fail(SVO_ERR_CAPACITY, "batch mesh %u: octree exceeds its pool or the 30-bit pointer range", m);
			else if (r.status & kStatusTimeout)
				rc = svo_fail(SVO_ERR_TIMEOUT, "batch mesh %u: a device-side wait gave up", m);
			else
				rc = svo_fail(SVO_ERR_CUDA, "batch mesh %u: build status 0x%x", m, r.status);
		}
	}
	return rc;
}

} // namespace svo

using namespace svo;

struct svo_batcher {
	Batcher b;
};

extern "C" {

int svo_batcher_create(svo_batcher **out) {
	if (!out) return svo_fail(SVO_ERR_INVALID, "null output");
	*out = new (std::nothrow) svo_batcher();
	return *out ? SVO_OK : svo_fail(SVO_ERR_OOM, "batcher allocation");
}

void svo_batcher_destroy(svo_batcher *b) { delete b; }

int svo_batcher_set_graph(svo_batcher *b, int on) {
	if (!b) return svo_fail(SVO_ERR_INVALID, "null batcher");
	b->b.use_graph = on != 0;
	if (!on) {
		b->b.count_graph.reset();
		b->b.build_graph.reset();
	}
	return SVO_OK;
}

int svo_batcher_build(svo_batcher *b, const svo_batch_mesh *meshes, uint32_t n_meshes, void *stream) {
	if (!b) return svo_fail(SVO_ERR_INVALID, "null batcher");
	b->b.results.clear();
	const int rc = batch_build(b->b, meshes, n_meshes, (cudaStream_t)stream);
	if (rc != SVO_OK) b->b.results.clear();
	return rc;
}

uint32_t svo_batcher_meshes(const svo_batcher *b) { return b ? (uint32_t)b->b.results.size() : 0u; }

int svo_batcher_result(const svo_batcher *b, uint32_t mesh, svo_fraglist *frags, svo_octree *octree,
                       svo_build_info *info) {
	if (!b) return svo_fail(SVO_ERR_INVALID, "null batcher");
	if (mesh >= b->b.results.size()) return svo_fail(SVO_ERR_INVALID, "mesh %u outside the last batch", mesh);
	const MeshResult &r = b->b.results[mesh];
	if (frags) {
		memset(frags, 0, sizeof(*frags));
		frags->data = (uint64_t *)b->b.frags.ptr + r.frag_base;
		frags->count = (uint32_t)r.frag_count;
		frags->level = r.info.level;
		frags->capacity = r.frag_count;
		frags->owned = 0;
		frags->units = (uint32_t)r.units;
	}
	if (octree) {
		memset(octree, 0, sizeof(*octree));
		octree->words = (uint32_t *)b->b.pool.ptr + r.pool_base;
		octree->capacity = r.capacity;
		octree->range_words = r.info.range_words;
		octree->level = r.info.level;
		octree->owned = 0;
	}
	if (info) *info = r.info;
	return SVO_OK;
}

void svo_batcher_stats(const svo_batcher *b, uint64_t *graph_captures, uint64_t *graph_replays) {
	if (graph_captures) *graph_captures = b ? b->b.graph_captures : 0;
	if (graph_replays) *graph_replays = b ? b->b.graph_replays : 0;
}

} // extern "C"
