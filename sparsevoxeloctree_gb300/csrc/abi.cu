// abi.cu — the C ABI of include/svo.h: argument checks, stream-ordered allocation, launches and the
// few blocking readbacks the reference also performs (fragment count, octree range).
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include <algorithm>

#include "svo_internal.h"

namespace svo {

static std::atomic<uint64_t> g_launches{0};
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
static std::atomic<uint64_t> g_allocations{0};
void note_allocation() { g_allocations.fetch_add(1, std::memory_order_relaxed); }

static thread_local std::string g_error;

// ---------------------------------------------------------------- profiling
struct ProfRecord {
	const char *name;
	cudaEvent_t begin, end;
};
static std::mutex g_prof_mu;
static std::atomic<bool> g_prof_on{false};
static std::vector<ProfRecord> g_prof;
static std::vector<cudaEvent_t> g_prof_free;

static cudaEvent_t prof_event() {
	if (!g_prof_free.empty()) {
		cudaEvent_t e = g_prof_free.back();
		g_prof_free.pop_back();
		return e;
	}
	cudaEvent_t e = nullptr;
	cudaEventCreate(&e);
	return e;
}

ProfScope::ProfScope(const char *name, cudaStream_t s) : slot(-1), stream(s) {
	if (!g_prof_on.load(std::memory_order_relaxed)) return;
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return; // graph replays are timed whole
	std::lock_guard<std::mutex> lk(g_prof_mu);
	ProfRecord r{name, prof_event(), prof_event()};
	cudaEventRecord(r.begin, s);
	g_prof.push_back(r);
	slot = (int)g_prof.size() - 1;
}

ProfScope::~ProfScope() {
	if (slot < 0) return;
	std::lock_guard<std::mutex> lk(g_prof_mu);
	if (slot < (int)g_prof.size()) cudaEventRecord(g_prof[slot].end, stream);
}

static int fail(int code, const char *fmt, ...) {
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_error = buf;
	return code;
}

int svo_fail(int code, const char *fmt, ...) {
	char buf[512];
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(buf, sizeof(buf), fmt, ap);
	va_end(ap);
	g_error = buf;
	return code;
}

static int cuda_fail(cudaError_t e, const char *what) {
	cudaGetLastError(); // clear a sticky launch error of this thread
	return fail(e == cudaErrorMemoryAllocation ? SVO_ERR_OOM : SVO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SVO_CK(call, what)                                                                                  \
	do {                                                                                                \
		cudaError_t e_ = (call);                                                                    \
		if (e_ != cudaSuccess) return cuda_fail(e_, what);                                          \
	} while (0)

constexpr int kMaxDevices = 64;
static int g_sm_count[kMaxDevices];
static std::once_flag g_pool_once[kMaxDevices];

static int current_device() {
	int dev = 0;
	cudaGetDevice(&dev);
	return dev < kMaxDevices ? dev : 0;
}

int device_sm_count() {
	const int dev = current_device();
	if (g_sm_count[dev] == 0) {
		int n = 0;
		cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
		g_sm_count[dev] = n > 0 ? n : 1;
	}
	return g_sm_count[dev];
}

// ---------------------------------------------------------------- launch-parameter table
// Entry [param][level][size class]; level 0 is unused (a set with level 0 writes every level).
constexpr uint32_t kTuneClasses = 8;
static const int kTuneDefault[kTuneParams] = {128, 1, 1, 16, 6, 16, 2, 1, 0};
static std::atomic<int> g_tune[kTuneParams][SVO_LEVEL_MAX + 1][kTuneClasses];
static std::once_flag g_tune_once;

static void tune_init() {
	std::call_once(g_tune_once, [] {
		for (uint32_t p = 0; p < kTuneParams; ++p)
			for (uint32_t l = 0; l <= SVO_LEVEL_MAX; ++l)
				for (uint32_t c = 0; c < kTuneClasses; ++c) g_tune[p][l][c].store(kTuneDefault[p]);
	});
}

static bool tune_valid(uint32_t param, int v) {
	switch (param) {
	case kTuneMarchBlock: return v == 64 || v == 128 || v == 256;
	case kTuneMarchRays:
	case kTuneMarchBufferRays: return v == 0 || v == 1 || v == 2;
	case kTuneMarchShared: return v == 0 || v == 1;
	case kTuneBuildStreams: return v == 1 || v == 2;
	case kTuneDownloadBands: return v == 0 || v == 1 || v == 2 || v == 4 || v == 8 || v == 16;
	default: return v >= 1 && v <= 64;
	}
}

static uint32_t size_class_of(uint64_t items) {
	uint32_t c = 0; // < 64k items: class 0; then one class per factor 4, up to class 7 (>= 1G)
	for (uint64_t lim = 1ull << 16; items >= lim && c + 1 < kTuneClasses; lim <<= 2) ++c;
	return c;
}

int tune_value(uint32_t param, uint32_t level, uint64_t items) {
	tune_init();
	if (param >= kTuneParams) return 0;
	if (level > SVO_LEVEL_MAX) level = SVO_LEVEL_MAX;
	return g_tune[param][level][size_class_of(items)].load(std::memory_order_relaxed);
}

// Stream-ordered allocations come from the device's default memory pool; keeping freed memory in the
// pool (release threshold = max) makes repeated builds allocation-free after the first one.
static void prepare_pool() {
	const int dev = current_device();
	std::call_once(g_pool_once[dev], [dev] {
		cudaMemPool_t pool;
		if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
			uint64_t threshold = UINT64_MAX;
			cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
		}
	});
}

template <typename T> static cudaError_t alloc_async(T **p, size_t bytes, cudaStream_t s) {
	prepare_pool();
	return counted_malloc_async(p, bytes ? bytes : 16, s);
}

static bool aligned(const void *p, size_t a) { return ((uintptr_t)p % a) == 0; }

// Device memory from the caller's allocator, or from the stream-ordered pool when there is none.
struct Mem {
	const svo_allocator *a;
	cudaStream_t s;
	cudaError_t get(void **p, size_t bytes) {
		if (a && a->alloc) {
			note_allocation();
			*p = a->alloc(a->user, bytes ? bytes : 16);
			return *p ? cudaSuccess : cudaErrorMemoryAllocation;
		}
		return alloc_async(p, bytes, s);
	}
	void put(void *p) {
		if (!p) return;
		if (a && a->alloc) {
			if (a->release) a->release(a->user, p);
		} else {
			cudaFreeAsync(p, s);
		}
	}
	uint32_t owned() const { return (a && a->alloc) ? 0u : 1u; }
};

static int check_level(uint32_t level) {
	if (level < SVO_LEVEL_MIN || level > SVO_LEVEL_MAX)
		return fail(SVO_ERR_INVALID, "level %u outside [%u, %u]", level, SVO_LEVEL_MIN, SVO_LEVEL_MAX);
	return SVO_OK;
}

static int status_to_error(uint32_t status, const char *what) {
	if (status & kStatusCheck) return fail(SVO_ERR_CUDA, "%s: internal bounds check %u failed", what, status >> 16);
	if (status & kStatusBadFragment)
		return fail(SVO_ERR_INVALID, "%s: fragment coordinates outside the octree level", what);
	if (status & kStatusCapacity) return fail(SVO_ERR_CAPACITY, "%s: output exceeds its buffer or the 30-bit pointer range", what);
	if (status & kStatusTimeout) return fail(SVO_ERR_TIMEOUT, "%s: a device-side wait gave up", what);
	if (status & kStatusMalformed) return fail(SVO_ERR_INVALID, "%s: malformed octree pool", what);
	return SVO_OK;
}

} // namespace svo

using namespace svo;

extern "C" {

const char *svo_last_error(void) { return g_error.c_str(); }

int svo_device_alloc(void **ptr, size_t bytes, void *stream) {
	if (!ptr) return fail(SVO_ERR_INVALID, "null pointer");
	SVO_CK(alloc_async(ptr, bytes, (cudaStream_t)stream), "device allocation");
	return SVO_OK;
}

void svo_device_free(void *ptr, void *stream) {
	if (ptr) cudaFreeAsync(ptr, (cudaStream_t)stream);
}

int svo_upload(void *dst_device, const void *src_host, size_t bytes, void *stream) {
	if (bytes && (!dst_device || !src_host)) return fail(SVO_ERR_INVALID, "null pointer");
	SVO_CK(cudaMemcpyAsync(dst_device, src_host, bytes, cudaMemcpyDefault, (cudaStream_t)stream), "upload");
	return SVO_OK;
}

int svo_download(void *dst_host, const void *src_device, size_t bytes, int sync, void *stream) {
	if (bytes && (!dst_host || !src_device)) return fail(SVO_ERR_INVALID, "null pointer");
	SVO_CK(cudaMemcpyAsync(dst_host, src_device, bytes, cudaMemcpyDefault, (cudaStream_t)stream), "download");
	if (sync) SVO_CK(cudaStreamSynchronize((cudaStream_t)stream), "download synchronize");
	return SVO_OK;
}

int svo_stream_synchronize(void *stream) {
	SVO_CK(cudaStreamSynchronize((cudaStream_t)stream), "stream synchronize");
	return SVO_OK;
}

void svo_profile_enable(int on) {
	std::lock_guard<std::mutex> lk(g_prof_mu);
	if (on) {
		for (auto &r : g_prof) {
			g_prof_free.push_back(r.begin);
			g_prof_free.push_back(r.end);
		}
		g_prof.clear();
	}
	g_prof_on.store(on != 0);
}

size_t svo_profile_summary(char *buf, size_t cap) {
	std::lock_guard<std::mutex> lk(g_prof_mu);
	std::vector<std::pair<std::string, std::pair<int, double>>> agg;
	for (auto &r : g_prof) {
		cudaEventSynchronize(r.end);
		float ms = 0.0f;
		if (cudaEventElapsedTime(&ms, r.begin, r.end) != cudaSuccess) ms = 0.0f;
		auto it = std::find_if(agg.begin(), agg.end(), [&](const auto &a) { return a.first == r.name; });
		if (it == agg.end()) {
			agg.push_back({r.name, {1, (double)ms}});
		} else {
			it->second.first += 1;
			it->second.second += ms;
		}
	}
	std::string out = "{";
	for (size_t i = 0; i < agg.size(); ++i) {
		char item[256];
		snprintf(item, sizeof(item), "%s\"%s\": {\"launches\": %d, \"ms\": %.6f}", i ? ", " : "", agg[i].first.c_str(),
		         agg[i].second.first, agg[i].second.second);
		out += item;
	}
	out += "}";
	if (buf && cap) {
		const size_t n = std::min(cap - 1, out.size());
		memcpy(buf, out.data(), n);
		buf[n] = 0;
	}
	return out.size();
}
const char *svo_version(void) { return "svo-gb300 0.1 (sm_103a)"; }

uint32_t svo_tune_size_class(uint64_t items) { return size_class_of(items); }

int svo_tune_set(uint32_t param, uint32_t level, int32_t size_class, int32_t value) {
	tune_init();
	if (param >= kTuneParams) return fail(SVO_ERR_INVALID, "unknown launch parameter %u", param);
	if (level > SVO_LEVEL_MAX) return fail(SVO_ERR_INVALID, "level %u outside [0, %u]", level, SVO_LEVEL_MAX);
	if (size_class >= (int32_t)kTuneClasses || size_class < -1)
		return fail(SVO_ERR_INVALID, "size class %d outside [-1, %u]", size_class, kTuneClasses - 1);
	if (!tune_valid(param, value)) return fail(SVO_ERR_INVALID, "value %d not allowed for parameter %u", value, param);
	for (uint32_t l = level ? level : 1; l <= (level ? level : SVO_LEVEL_MAX); ++l)
		for (uint32_t c = size_class < 0 ? 0 : (uint32_t)size_class; c <= (size_class < 0 ? kTuneClasses - 1 : (uint32_t)size_class); ++c)
			g_tune[param][l][c].store(value);
	return SVO_OK;
}

int svo_tune_get(uint32_t param, uint32_t level, uint64_t items) { return tune_value(param, level ? level : 1, items); }

void svo_tune_reset(void) {
	tune_init();
	for (uint32_t p = 0; p < kTuneParams; ++p)
		for (uint32_t l = 0; l <= SVO_LEVEL_MAX; ++l)
			for (uint32_t c = 0; c < kTuneClasses; ++c) g_tune[p][l][c].store(kTuneDefault[p]);
}
uint64_t svo_kernel_launches(void) { return g_launches.load(); }
uint64_t svo_allocation_calls(void) { return g_allocations.load(); }

int svo_debug_wait_fault(uint32_t spin_limit, uint32_t withheld) {
	cudaError_t e = vox_set_wait_fault(spin_limit, withheld);
	if (e == cudaSuccess) e = build_set_wait_fault(spin_limit, withheld);
	if (e == cudaSuccess) e = march_set_wait_fault(spin_limit, withheld);
	if (e == cudaSuccess) e = texture_set_wait_fault(spin_limit, withheld);
	if (e != cudaSuccess) return cuda_fail(e, "wait-fault hook");
	return SVO_OK;
}

// ------------------------------------------------------------------------------------------ voxelize
static int check_tris(const svo_triangle *tris, uint32_t n) {
	if (n && !tris) return fail(SVO_ERR_INVALID, "null triangle buffer");
	if (!aligned(tris, 16)) return fail(SVO_ERR_INVALID, "triangle buffer must be 16-byte aligned");
	return SVO_OK;
}

size_t svo_voxelize_workspace_size(uint32_t n_tris, uint64_t units) {
	return vox_workspace_bytes(n_tris, units ? units : vox_default_unit_cap(n_tris));
}

// Count pass with a workspace from `mem`; retries once with exact unit arrays when the first guess is
// short.  On success *ws_out (still owned by the caller) holds the counted workspace.
// The most raster units a count of this process has met (a high-water mark).  The unit scratch of a
// count's first attempt covers it, so a mesh with more large-triangle units than the default guess is
// not counted twice on every call (the first attempt would overflow and report the exact number).  It
// only sizes scratch: every call still runs its whole count.
static std::atomic<uint64_t> g_units_seen{0};

static void note_units(uint64_t units) {
	uint64_t cur = g_units_seen.load(std::memory_order_relaxed);
	while (units > cur && !g_units_seen.compare_exchange_weak(cur, units, std::memory_order_relaxed)) {
	}
}

static int voxelize_count_pass(const svo_triangle *tris, uint32_t n_tris, uint32_t level, Mem &mem, void **ws_out,
                               VoxWorkspace &w, uint64_t &total, uint64_t &units) {
	uint64_t cap = std::max<uint64_t>(vox_default_unit_cap(n_tris), g_units_seen.load(std::memory_order_relaxed));
	for (int attempt = 0; attempt < 2; ++attempt) {
		void *ws = nullptr;
		SVO_CK(mem.get(&ws, vox_workspace_bytes(n_tris, cap)), "voxelize workspace");
		vox_workspace_layout(ws, n_tris, cap, w);
		unsigned long long tot[3] = {0, 0, 0};
		cudaError_t e = vox_launch_count(tris, n_tris, level, w, mem.s);
		if (e == cudaSuccess) e = vox_launch_totals(w, mem.s);
		if (e == cudaSuccess) e = cudaMemcpyAsync(tot, w.totals, sizeof(tot), cudaMemcpyDeviceToHost, mem.s);
		if (e == cudaSuccess) e = cudaStreamSynchronize(mem.s);
		if (e != cudaSuccess) {
			mem.put(ws);
			return cuda_fail(e, "voxelize count");
		}
		const uint32_t status = (uint32_t)tot[2];
		if (tot[1] < 0xffffffffull) note_units(tot[1]);
		if (status & kStatusUnits) {
			mem.put(ws);
			if (tot[1] >= 0xffffffffull) return fail(SVO_ERR_CAPACITY, "too many raster units");
			cap = tot[1];
			continue;
		}
		int rc = status_to_error(status, "voxelize count");
		if (rc) {
			mem.put(ws);
			return rc;
		}
		*ws_out = ws;
		total = tot[0];
		units = tot[1];
		return SVO_OK;
	}
	return fail(SVO_ERR_CAPACITY, "voxelize workspace retry failed");
}

// The fragment counts of the meshes this process voxelized last (their triangle buffer, triangle count and
// level).  A repeated call with the library's own memory emits into a list of that size right after the
// count pass, so the count's readback overlaps the emission instead of the device idling while the host
// reads the count and launches it; a count that turns out larger is emitted again into an exact list.
struct RecentVox {
	const void *tris;
	uint32_t n, level;
	uint64_t total;
};
static std::mutex g_recent_mu;
static RecentVox g_recent[8];
static uint32_t g_recent_next = 0;

static uint64_t recent_total(const void *tris, uint32_t n, uint32_t level) {
	std::lock_guard<std::mutex> lock(g_recent_mu);
	for (const RecentVox &r : g_recent)
		if (r.tris == tris && r.n == n && r.level == level) return r.total;
	return 0;
}

static void note_recent(const void *tris, uint32_t n, uint32_t level, uint64_t total) {
	std::lock_guard<std::mutex> lock(g_recent_mu);
	for (RecentVox &r : g_recent)
		if (r.tris == tris && r.n == n && r.level == level) {
			r.total = total;
			return;
		}
	g_recent[g_recent_next++ % 8] = RecentVox{tris, n, level, total};
}

// svo_voxelize_ex's path for a mesh whose count is known from an earlier call (`guess` fragments, the
// library's stream-ordered memory): count, emission into `guess` slots, then the count's readback.
// Returns SVO_OK with *done = false when the count pass needs a larger unit scratch (the caller runs the
// ordinary path, which counts again).
static int voxelize_overlapped(const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint64_t guess, Mem &mem,
                               svo_fraglist *out, bool *done) {
	*done = false;
	thread_local unsigned long long *tot = nullptr; // page-locked, so the copy is asynchronous
	thread_local cudaEvent_t ready = nullptr;
	thread_local int ready_dev = -1; // the event belongs to the device current when it was made
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || (ready && ready_dev != dev)) return SVO_OK; // the ordinary path
	if (!tot) {
		note_allocation();
		if (cudaHostAlloc((void **)&tot, 4 * sizeof(unsigned long long), cudaHostAllocDefault) != cudaSuccess) {
			tot = nullptr;
			return SVO_OK; // the ordinary path
		}
	}
	if (!ready) {
		if (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess) {
			ready = nullptr;
			return SVO_OK;
		}
		ready_dev = dev;
	}
	const uint64_t cap = std::max<uint64_t>(vox_default_unit_cap(n_tris), g_units_seen.load(std::memory_order_relaxed));
	void *ws = nullptr, *frags = nullptr;
	VoxWorkspace w;
	SVO_CK(mem.get(&ws, vox_workspace_bytes(n_tris, cap)), "voxelize workspace");
	vox_workspace_layout(ws, n_tris, cap, w);
	cudaError_t e = vox_launch_count(tris, n_tris, level, w, mem.s);
	if (e == cudaSuccess) e = vox_launch_totals(w, mem.s);
	if (e == cudaSuccess) e = cudaMemcpyAsync(tot, w.totals, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, mem.s);
	if (e == cudaSuccess) e = cudaEventRecord(ready, mem.s);
	if (e == cudaSuccess) e = mem.get(&frags, guess * sizeof(uint64_t));
	if (e == cudaSuccess) e = vox_launch_emit(tris, n_tris, level, w, (uint64_t *)frags, guess, mem.s);
	if (e == cudaSuccess) e = cudaEventSynchronize(ready);
	if (e != cudaSuccess) {
		mem.put(frags);
		mem.put(ws);
		return cuda_fail(e, "voxelize");
	}
	const uint64_t total = tot[0], units = tot[1];
	const uint32_t status = (uint32_t)tot[2];
	if (units < 0xffffffffull) note_units(units);
	if (status & kStatusUnits) { // the units did not fit the scratch: nothing of them was emitted
		mem.put(frags);
		mem.put(ws);
		return SVO_OK;
	}
	int rc = status_to_error(status, "voxelize count");
	if (!rc && total > 0xffffffffull)
		rc = fail(SVO_ERR_CAPACITY, "%llu fragments exceed the 32-bit fragment count", (unsigned long long)total);
	if (rc) {
		mem.put(frags);
		mem.put(ws);
		return rc;
	}
	uint64_t capacity = guess;
	if (total > guess) { // the list was short: emit again into an exact one (the scans are unchanged)
		mem.put(frags);
		frags = nullptr;
		e = mem.get(&frags, total * sizeof(uint64_t));
		if (e == cudaSuccess) e = vox_launch_emit(tris, n_tris, level, w, (uint64_t *)frags, total, mem.s);
		if (e != cudaSuccess) {
			mem.put(frags);
			mem.put(ws);
			return cuda_fail(e, "voxelize emit");
		}
		capacity = total;
	}
	mem.put(ws);
	note_recent(tris, n_tris, level, total);
	out->data = (uint64_t *)frags;
	out->count = (uint32_t)total;
	out->level = level;
	out->capacity = capacity;
	out->owned = mem.owned();
	out->units = (uint32_t)units;
	*done = true;
	return SVO_OK;
}

int svo_voxelize_count(const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint64_t *count_host,
                       void *stream) {
	int rc;
	if ((rc = check_level(level)) || (rc = check_tris(tris, n_tris))) return rc;
	if (!count_host) return fail(SVO_ERR_INVALID, "null count pointer");
	Mem mem{nullptr, (cudaStream_t)stream};
	void *ws = nullptr;
	VoxWorkspace w;
	uint64_t total = 0, units = 0;
	if ((rc = voxelize_count_pass(tris, n_tris, level, mem, &ws, w, total, units))) return rc;
	mem.put(ws);
	*count_host = total;
	return SVO_OK;
}

int svo_voxelize_ex(const svo_triangle *tris, uint32_t n_tris, uint32_t level, const svo_allocator *alloc,
                    svo_fraglist *out, void *stream) {
	int rc;
	if ((rc = check_level(level)) || (rc = check_tris(tris, n_tris))) return rc;
	if (!out) return fail(SVO_ERR_INVALID, "null output fragment list");
	cudaStream_t s = (cudaStream_t)stream;
	Mem mem{alloc, s};
	if (!(alloc && alloc->alloc) && n_tris) { // a caller's allocator may reuse a released list at once
		const uint64_t guess = recent_total(tris, n_tris, level);
		bool done = false;
		if (guess && (rc = voxelize_overlapped(tris, n_tris, level, guess, mem, out, &done))) return rc;
		if (done) return SVO_OK;
	}
	void *ws = nullptr;
	VoxWorkspace w;
	uint64_t total = 0, units = 0;
	if ((rc = voxelize_count_pass(tris, n_tris, level, mem, &ws, w, total, units))) return rc;
	if (total > 0xffffffffull) { // the reference's fragment count is a uint32 (src/Voxelizer.hpp:33)
		mem.put(ws);
		return fail(SVO_ERR_CAPACITY, "%llu fragments exceed the 32-bit fragment count", (unsigned long long)total);
	}
	void *frags = nullptr;
	cudaError_t e = mem.get(&frags, total * sizeof(uint64_t));
	if (e != cudaSuccess) {
		mem.put(ws);
		return cuda_fail(e, "fragment list allocation");
	}
	e = vox_launch_emit(tris, n_tris, level, w, (uint64_t *)frags, total, s);
	mem.put(ws);
	if (e != cudaSuccess) {
		mem.put(frags);
		return cuda_fail(e, "voxelize emit");
	}
	if (!(alloc && alloc->alloc)) note_recent(tris, n_tris, level, total);
	out->data = (uint64_t *)frags;
	out->count = (uint32_t)total;
	out->level = level;
	out->capacity = total;
	out->owned = mem.owned();
	out->units = (uint32_t)units;
	return SVO_OK;
}

int svo_voxelize(const svo_triangle *tris, uint32_t n_tris, uint32_t level, svo_fraglist *out, void *stream) {
	return svo_voxelize_ex(tris, n_tris, level, nullptr, out, stream);
}

int svo_voxelize_textured(const svo_triangle *tris, const svo_triangle_uv *uvs, uint32_t n_tris, uint32_t level,
                          const svo_texture_set *textures, svo_fraglist *out, void *stream) {
	int rc;
	if ((rc = check_level(level)) || (rc = check_tris(tris, n_tris))) return rc;
	if (!out || (n_tris && !uvs)) return fail(SVO_ERR_INVALID, "null argument");
	if (!aligned(uvs, 8)) return fail(SVO_ERR_INVALID, "texture coordinates must be 8-byte aligned");
	cudaStream_t s = (cudaStream_t)stream;
	Mem mem{nullptr, s};
	void *ws = nullptr;
	VoxWorkspace w;
	uint64_t total = 0, units = 0;
	if ((rc = voxelize_count_pass(tris, n_tris, level, mem, &ws, w, total, units))) return rc;
	if (total > 0xffffffffull) {
		mem.put(ws);
		return fail(SVO_ERR_CAPACITY, "%llu fragments exceed the 32-bit fragment count", (unsigned long long)total);
	}
	void *cand = nullptr, *frags = nullptr, *scratch = nullptr;
	cudaError_t e = mem.get(&cand, total * sizeof(uint64_t));
	if (e == cudaSuccess) e = mem.get(&frags, total * sizeof(uint64_t));
	if (e == cudaSuccess) e = mem.get(&scratch, vox_texture_scratch_bytes(total));
	if (e == cudaSuccess) e = vox_launch_emit(tris, n_tris, level, w, (uint64_t *)cand, total, s);
	if (e == cudaSuccess)
		e = vox_texture_launch((const uint64_t *)cand, total, tris, uvs, n_tris, level, w, textures, (uint64_t *)frags,
		                       (unsigned long long *)scratch, s);
	unsigned long long res[2] = {0, 0};
	if (e == cudaSuccess && total) e = cudaMemcpyAsync(res, scratch, sizeof(res), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	mem.put(ws);
	mem.put(cand);
	mem.put(scratch);
	if (e != cudaSuccess) {
		mem.put(frags);
		return cuda_fail(e, "textured voxelize");
	}
	if ((rc = status_to_error((uint32_t)(res[1] >> 32), "textured voxelize"))) {
		mem.put(frags);
		return rc;
	}
	out->data = (uint64_t *)frags;
	out->count = (uint32_t)res[0];
	out->level = level;
	out->capacity = total;
	out->owned = mem.owned();
	out->units = (uint32_t)units;
	return SVO_OK;
}

int svo_voxelize_into(const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint64_t *frags, uint64_t capacity,
                      uint64_t *count_dev, void *workspace, size_t workspace_bytes, void *stream) {
	int rc;
	if ((rc = check_level(level)) || (rc = check_tris(tris, n_tris))) return rc;
	if (!count_dev || !workspace || (capacity && !frags)) return fail(SVO_ERR_INVALID, "null argument");
	if (!aligned(workspace, 256)) return fail(SVO_ERR_INVALID, "workspace must be 256-byte aligned");
	VoxWorkspace w;
	const size_t fixed = vox_workspace_layout(nullptr, n_tris, 0, w);
	if (workspace_bytes < fixed)
		return fail(SVO_ERR_CAPACITY, "workspace of %zu bytes is below the %zu this mesh needs", workspace_bytes, fixed);
	// the most raster units whose layout fits in workspace_bytes (the layout grows with the capacity)
	uint64_t lo = 0, hi = (workspace_bytes - fixed) / 8 + 1;
	while (hi - lo > 1) {
		const uint64_t mid = lo + (hi - lo) / 2;
		if (vox_workspace_layout(nullptr, n_tris, mid, w) <= workspace_bytes)
			lo = mid;
		else
			hi = mid;
	}
	const uint64_t cap = lo;
	cudaStream_t s = (cudaStream_t)stream;
	vox_workspace_layout(workspace, n_tris, cap, w);
	SVO_CK(vox_launch_count_emit(tris, n_tris, level, w, frags, capacity, s), "voxelize count and emit");
	// count_dev[0] = fragments, count_dev[1] = status bits (totals[2])
	SVO_CK(cudaMemcpyAsync(count_dev, w.totals, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s), "voxelize count copy");
	SVO_CK(cudaMemcpyAsync(count_dev + 1, w.totals + 2, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s),
	       "voxelize status copy");
	return SVO_OK;
}

void svo_fraglist_destroy(svo_fraglist *f, void *stream) {
	if (!f) return;
	if (f->owned && f->data) cudaFreeAsync(f->data, (cudaStream_t)stream);
	memset(f, 0, sizeof(*f));
}

// ------------------------------------------------------------------------------------------ build
uint64_t svo_build_pool_bound(uint32_t count, uint32_t level) { return build_pool_bound(count, level); }

size_t svo_build_workspace_size(uint32_t count, uint32_t level, uint64_t capacity, uint64_t leaf_words) {
	(void)leaf_words; // the leaf level accumulates in shared memory: its size does not matter
	BuildWorkspace w;
	build_workspace_layout(nullptr, count, level, capacity, w);
	return w.total_bytes;
}

static int check_frags(const uint64_t *frags, uint32_t count) {
	if (count && !frags) return fail(SVO_ERR_INVALID, "null fragment buffer");
	if (!aligned(frags, 8)) return fail(SVO_ERR_INVALID, "fragment buffer must be 8-byte aligned");
	return SVO_OK;
}

// Reads the build state back (blocking).
static cudaError_t read_state(const BuildWorkspace &w, BuildState &st, cudaStream_t s) {
	cudaError_t e = cudaMemcpyAsync(&st, w.state, sizeof(st), cudaMemcpyDeviceToHost, s);
	return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
}

int svo_build_ex(const uint64_t *frags, uint32_t count, uint32_t level, const svo_allocator *alloc, svo_octree *out,
                 svo_build_info *info, void *stream) {
	int rc;
	if ((rc = check_level(level)) || (rc = check_frags(frags, count))) return rc;
	if (!out) return fail(SVO_ERR_INVALID, "null output octree");
	cudaStream_t s = (cudaStream_t)stream;
	Mem mem{alloc, s};
	const uint64_t capacity = build_pool_bound(count, level);
	void *pool = nullptr, *ws = nullptr;
	SVO_CK(mem.get(&pool, capacity * sizeof(uint32_t)), "octree pool allocation");
	BuildWorkspace w;
	build_workspace_layout(nullptr, count, level, capacity, w);
	cudaError_t e = mem.get(&ws, w.total_bytes);
	if (e != cudaSuccess) {
		mem.put(pool);
		return cuda_fail(e, "build workspace allocation");
	}
	build_workspace_layout(ws, count, level, capacity, w);
	e = build_launch_interior(frags, count, level, (uint32_t *)pool, capacity, w, s);
	if (e == cudaSuccess) e = build_launch_leaf(count, level, (uint32_t *)pool, capacity, w, s);
	// the range is read back once, as GetOctreeRange reads the counter (src/OctreeBuilder.cpp:212-214)
	BuildState st;
	if (e == cudaSuccess) e = read_state(w, st, s);
	mem.put(ws);
	if (e != cudaSuccess) {
		mem.put(pool);
		return cuda_fail(e, "build");
	}
	if ((rc = status_to_error(st.status, "build"))) {
		mem.put(pool);
		return rc;
	}
	out->words = (uint32_t *)pool;
	out->capacity = capacity;
	out->range_words = st.range_words;
	out->level = level;
	out->owned = mem.owned();
	out->reserved = 0;
	if (info) {
		memset(info, 0, sizeof(*info));
		info->level = level;
		info->fragments = count;
		info->range_words = st.range_words;
		info->leaves = st.leaves;
		for (uint32_t d = 1; d <= level; ++d) info->level_nodes[d - 1] = d < level ? st.lv[d].nodes : st.leaves;
	}
	return SVO_OK;
}

int svo_build(const uint64_t *frags, uint32_t count, uint32_t level, svo_octree *out, svo_build_info *info,
              void *stream) {
	return svo_build_ex(frags, count, level, nullptr, out, info, stream);
}

int svo_build_fraglist(const svo_fraglist *f, svo_octree *out, svo_build_info *info, void *stream) {
	if (!f) return fail(SVO_ERR_INVALID, "null fragment list");
	return svo_build(f->data, f->count, f->level, out, info, stream);
}

int svo_build_into(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool, uint64_t capacity,
                   void *workspace, size_t workspace_bytes, void *result_dev, void *stream) {
	int rc;
	if ((rc = check_level(level)) || (rc = check_frags(frags, count))) return rc;
	if (!pool || !workspace || !result_dev) return fail(SVO_ERR_INVALID, "null argument");
	if (capacity < 8) return fail(SVO_ERR_CAPACITY, "pool smaller than the root block");
	if (!aligned(pool, 16) || !aligned(workspace, 256) || !aligned(result_dev, 4))
		return fail(SVO_ERR_INVALID, "pool must be 16-byte and workspace 256-byte aligned");
	BuildWorkspace w;
	build_workspace_layout(nullptr, count, level, capacity, w);
	if (workspace_bytes < w.total_bytes)
		return fail(SVO_ERR_CAPACITY, "workspace of %zu bytes is below the %zu this build needs", workspace_bytes,
		            w.total_bytes);
	build_workspace_layout(workspace, count, level, capacity, w);
	cudaStream_t s = (cudaStream_t)stream;
	SVO_CK(build_launch_interior(frags, count, level, pool, capacity, w, s), "build interior levels");
	SVO_CK(build_launch_leaf(count, level, pool, capacity, w, s), "build leaf level");
	SVO_CK(build_launch_export(w, level, count, result_dev, s), "build info export");
	return SVO_OK;
}

void svo_octree_destroy(svo_octree *o, void *stream) {
	if (!o) return;
	if (o->owned && o->words) cudaFreeAsync(o->words, (cudaStream_t)stream);
	memset(o, 0, sizeof(*o));
}

// ------------------------------------------------------------------------------------------ march
static int check_octree(const svo_octree *o) {
	if (!o || !o->words) return fail(SVO_ERR_INVALID, "null octree");
	int rc = check_level(o->level);
	if (rc) return rc;
	if (o->range_words < 8 || o->range_words % 8) return fail(SVO_ERR_INVALID, "octree range must be a positive multiple of 8");
	return SVO_OK;
}

static int raycast_common(const svo_octree *o, const svo_ray *rays, const svo_camera *cam, uint32_t width,
                          uint32_t height, uint32_t n, svo_hit *hits, uint64_t *fetches_dev, void *stream,
                          const float *beam = nullptr) {
	int rc;
	if ((rc = check_octree(o))) return rc;
	if (n && !hits) return fail(SVO_ERR_INVALID, "null hit buffer");
	if (!aligned(hits, 16)) return fail(SVO_ERR_INVALID, "hit buffer must be 16-byte aligned");
	if (!cam && n && (!rays || !aligned(rays, 8))) return fail(SVO_ERR_INVALID, "ray buffer must be 8-byte aligned");
	cudaStream_t s = (cudaStream_t)stream;
	unsigned long long *scratch = nullptr;
	SVO_CK(alloc_async(&scratch, 2 * sizeof(unsigned long long), s), "ray ticket allocation");
	MarchArgs a;
	memset(&a, 0, sizeof(a));
	a.pool = o->words;
	a.range = o->range_words;
	a.level = o->level;
	a.rays = rays;
	if (cam) a.cam = *cam;
	a.width = width;
	a.height = height;
	a.n = n;
	a.hits = hits;
	a.ticket = scratch;
	a.status = reinterpret_cast<uint32_t *>(scratch + 1);
	a.fetches = (unsigned long long *)fetches_dev;
	a.beam = beam;
	cudaError_t e = march_launch(a, cam != nullptr, s);
	cudaFreeAsync(scratch, s);
	if (e != cudaSuccess) return cuda_fail(e, "raycast");
	return SVO_OK;
}

int svo_raycast(const svo_octree *o, const svo_ray *rays, uint32_t n, svo_hit *hits, uint64_t *fetches_dev,
                void *stream) {
	return raycast_common(o, rays, nullptr, 0, 0, n, hits, fetches_dev, stream);
}

int svo_raycast_camera(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height, svo_hit *hits,
                       uint64_t *fetches_dev, void *stream) {
	if (!cam) return fail(SVO_ERR_INVALID, "null camera");
	const uint64_t n = (uint64_t)width * height;
	if (n > 0xffffffffull) return fail(SVO_ERR_INVALID, "image too large");
	return raycast_common(o, nullptr, cam, width, height, (uint32_t)n, hits, fetches_dev, stream);
}

static svo_hit *mapped_host(svo_hit *p) { return static_cast<svo_hit *>(svo::mapped_host_ptr(p, 16)); }

// Mode 0 (mapped host buffer): the march stores each hit straight into host memory over the GPU-CPU link,
// so the download runs inside the march.  Otherwise the image in row bands (multiples of 4 rows, the
// camera launch's tile height): each band is traced on `stream`, then copied to the host on a second
// stream while the next band is traced; `stream` waits for the copies at the end.  Per pixel the march is
// svo_raycast_camera's, so the hits are identical either way.
int svo_raycast_camera_download(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height,
                                svo_hit *hits, svo_hit *hits_host, uint64_t *fetches_dev, void *stream) {
	if (!cam) return fail(SVO_ERR_INVALID, "null camera");
	const uint64_t n = (uint64_t)width * height;
	if (n > 0xffffffffull) return fail(SVO_ERR_INVALID, "image too large");
	int rc;
	if ((rc = check_octree(o))) return rc;
	if (n == 0) return SVO_OK;
	if (!hits_host) return fail(SVO_ERR_INVALID, "null host hit buffer");
	if (!aligned(hits_host, 16)) return fail(SVO_ERR_INVALID, "host hit buffer must be 16-byte aligned");
	uint32_t bands = (uint32_t)tune_value(kTuneDownloadBands, o->level, n);
	if (bands == 0) {
		if (svo_hit *direct = mapped_host(hits_host))
			return raycast_common(o, nullptr, cam, width, height, (uint32_t)n, direct, fetches_dev, stream);
		bands = 2; // not mapped: copies
	}
	if (!hits) return fail(SVO_ERR_INVALID, "null hit buffer (the host buffer is not mapped)");
	if (!aligned(hits, 16)) return fail(SVO_ERR_INVALID, "hit buffer must be 16-byte aligned");
	cudaStream_t s = (cudaStream_t)stream;
	const uint32_t band_rows = std::max<uint32_t>(4u, (height + bands - 1) / bands + 3u) / 4u * 4u;
	unsigned long long *scratch = nullptr;
	SVO_CK(alloc_async(&scratch, 2 * sizeof(unsigned long long), s), "ray ticket allocation");
	SVO_CK(cudaMemsetAsync(scratch + 1, 0, sizeof(unsigned long long), s), "ray status");
	MarchArgs a;
	memset(&a, 0, sizeof(a));
	a.pool = o->words;
	a.range = o->range_words;
	a.level = o->level;
	a.cam = *cam;
	a.width = width;
	a.height = height;
	a.n = (uint32_t)n; // launch shape and launch parameters of the whole image
	a.hits = hits;
	a.ticket = scratch;
	a.status = reinterpret_cast<uint32_t *>(scratch + 1);
	a.fetches = (unsigned long long *)fetches_dev;
	cudaError_t e = cudaSuccess;
	{
		SideFork fork(s, bands > 1);
		for (uint32_t row0 = 0; row0 < height && e == cudaSuccess; row0 += band_rows) {
			a.row0 = row0;
			a.rows = std::min(band_rows, height - row0);
			e = march_launch(a, true, s);
			if (e != cudaSuccess) break;
			fork.side_waits_main();
			const size_t off = (size_t)row0 * width, bytes = (size_t)a.rows * width * sizeof(svo_hit);
			e = cudaMemcpyAsync(hits_host + off, hits + off, bytes, cudaMemcpyDeviceToHost, fork.side());
		}
		fork.mark_side(0);
		fork.main_waits(0);
	}
	cudaFreeAsync(scratch, s);
	if (e != cudaSuccess) return cuda_fail(e, "raycast download");
	return SVO_OK;
}

uint64_t svo_beam_texels(uint32_t width, uint32_t height) {
	return (uint64_t)((width + SVO_BEAM_SIZE - 1) / SVO_BEAM_SIZE + 1) * ((height + SVO_BEAM_SIZE - 1) / SVO_BEAM_SIZE + 1);
}

// MarchArgs with a 16-byte scratch (ticket + status) from the stream-ordered pool.
static int march_args(const svo_octree *o, cudaStream_t s, MarchArgs &a, unsigned long long **scratch) {
	int rc;
	if ((rc = check_octree(o))) return rc;
	SVO_CK(alloc_async(scratch, 2 * sizeof(unsigned long long), s), "march scratch allocation");
	SVO_CK(cudaMemsetAsync(*scratch, 0, 2 * sizeof(unsigned long long), s), "march scratch");
	memset(&a, 0, sizeof(a));
	a.pool = o->words;
	a.range = o->range_words;
	a.level = o->level;
	a.ticket = *scratch;
	a.status = reinterpret_cast<uint32_t *>(*scratch + 1);
	return SVO_OK;
}

int svo_beam_prepass(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height, float *beam,
                     void *stream) {
	if (!cam || !beam) return fail(SVO_ERR_INVALID, "null argument");
	if (!width || !height) return fail(SVO_ERR_INVALID, "empty image");
	if (!aligned(beam, 4)) return fail(SVO_ERR_INVALID, "beam buffer must be 4-byte aligned");
	cudaStream_t s = (cudaStream_t)stream;
	MarchArgs a;
	unsigned long long *scratch = nullptr;
	int rc = march_args(o, s, a, &scratch);
	if (rc) return rc;
	a.cam = *cam;
	a.width = width;
	a.height = height;
	cudaError_t e = beam_launch(a, beam, s);
	cudaFreeAsync(scratch, s);
	if (e != cudaSuccess) return cuda_fail(e, "beam pre-pass");
	return SVO_OK;
}

int svo_raycast_camera_beam(const svo_octree *o, const svo_camera *cam, uint32_t width, uint32_t height,
                            const float *beam, svo_hit *hits, uint64_t *fetches_dev, void *stream) {
	if (!cam) return fail(SVO_ERR_INVALID, "null camera");
	const uint64_t n = (uint64_t)width * height;
	if (n > 0xffffffffull) return fail(SVO_ERR_INVALID, "image too large");
	if (n == 0) return raycast_common(o, nullptr, cam, width, height, 0, hits, fetches_dev, stream);
	if (beam) return raycast_common(o, nullptr, cam, width, height, (uint32_t)n, hits, fetches_dev, stream, beam);
	// no beam image given: pre-pass and march in one launch (the same texels and hits)
	if (!hits || !aligned(hits, 16)) return fail(SVO_ERR_INVALID, "hit buffer must be 16-byte aligned");
	cudaStream_t s = (cudaStream_t)stream;
	MarchArgs a;
	unsigned long long *scratch = nullptr;
	int rc = march_args(o, s, a, &scratch);
	if (rc) return rc;
	float *own = nullptr;
	cudaError_t e = alloc_async(&own, svo_beam_texels(width, height) * sizeof(float), s);
	if (e == cudaSuccess) {
		a.cam = *cam;
		a.width = width;
		a.height = height;
		a.n = (uint32_t)n;
		a.hits = hits;
		a.fetches = (unsigned long long *)fetches_dev;
		e = march_beam_fused_launch(a, own, s);
		cudaFreeAsync(own, s);
	}
	cudaFreeAsync(scratch, s);
	if (e != cudaSuccess) return cuda_fail(e, "beam march");
	return SVO_OK;
}

int svo_occlude(const svo_octree *o, const svo_ray *rays, uint32_t n, uint32_t *occluded, void *stream) {
	if (n && (!rays || !occluded)) return fail(SVO_ERR_INVALID, "null argument");
	if (!aligned(rays, 8) || !aligned(occluded, 4)) return fail(SVO_ERR_INVALID, "misaligned buffer");
	cudaStream_t s = (cudaStream_t)stream;
	MarchArgs a;
	unsigned long long *scratch = nullptr;
	int rc = march_args(o, s, a, &scratch);
	if (rc) return rc;
	a.rays = rays;
	a.n = n;
	cudaError_t e = occlude_launch(a, occluded, s);
	cudaFreeAsync(scratch, s);
	if (e != cudaSuccess) return cuda_fail(e, "occlude");
	return SVO_OK;
}

int svo_bounce_rays(const svo_hit *hits, uint32_t n, uint64_t seed, svo_ray *rays, void *stream) {
	if (n && (!hits || !rays)) return fail(SVO_ERR_INVALID, "null argument");
	SVO_CK(bounce_launch(hits, n, seed, rays, (cudaStream_t)stream), "bounce rays");
	return SVO_OK;
}

void svo_camera_from_angles(const float pos[3], float yaw, float pitch, float fov, float aspect, svo_camera *cam) {
	// trans = rotate(yaw about +y) * rotate(pitch about -x); look = trans*(0,0,1), side = trans*(1,0,0)
	const float cy = cosf(yaw), sy = sinf(yaw), cp = cosf(pitch), sp = sinf(pitch);
	const float tg = tanf(fov * 0.5f);
	float look[3] = {sy * cp, sp, cy * cp};
	float ll = sqrtf(look[0] * look[0] + look[1] * look[1] + look[2] * look[2]);
	float side[3] = {cy, 0.0f, -sy};
	float sl = sqrtf(side[0] * side[0] + side[2] * side[2]);
	for (int k = 0; k < 3; ++k) {
		look[k] /= ll;
		side[k] = side[k] / sl * tg * aspect;
	}
	float up[3] = {look[1] * side[2] - look[2] * side[1], look[2] * side[0] - look[0] * side[2],
	               look[0] * side[1] - look[1] * side[0]};
	float ul = sqrtf(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
	for (int k = 0; k < 3; ++k) {
		cam->pos[k] = pos[k];
		cam->look[k] = look[k];
		cam->side[k] = side[k];
		cam->up[k] = up[k] / ul * tg;
	}
	cam->pos[3] = cam->look[3] = cam->side[3] = cam->up[3] = 1.0f;
}

} // extern "C"
