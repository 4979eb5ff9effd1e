// noalloc.cu — svo_voxelize_static: the voxelizer's count + emit with its scratch in a fixed device array,
// for callers that cannot allocate device memory.
//
// Who needs this: code that runs where a cudaMalloc is not allowed or not safe — a renderer's frame loop
// that forbids allocation after start-up, a host thread holding a memory-pool lock, or an embedding
// whose device memory is fully carved up in advance.  They bring their own triangle and fragment
// buffers; the engine's own scratch (fragment offsets, large-triangle units, scan descriptors,
// counters) then has to live somewhere that needs no allocation call: a file-scope __device__ array
// that the module loader places when the library is loaded and that stays resident on every GPU that
// loads the library until the process exits.
#include <cstring>
#include <mutex>

#include <cuda.h>

#include "svo_internal.h"

namespace svo {

// Scratch for up to kStaticMaxTris triangles: (n+1) fragment offsets (8 B), (n+1) unit offsets (4 B),
// scan descriptors and counters; everything left over holds raster units of large triangles (12 B
// each; a room wall at level 10 is 4,096 units, the 262,144-triangle room scene 963,479 of the 1,047,808
// that fit beside 262,144 triangles).
constexpr uint32_t kStaticMaxTris = 262144;
constexpr size_t kStaticScratchBytes = 16u << 20; // 16 MiB

// Largest unit capacity whose workspace layout for n triangles fits the static scratch.
static uint64_t static_unit_cap(uint32_t n) {
	VoxWorkspace w;
	const size_t fixed = vox_workspace_layout(nullptr, n, 0, w);
	uint64_t cap = (kStaticScratchBytes - fixed) / 13;
	while (cap > 0 && vox_workspace_layout(nullptr, n, cap, w) > kStaticScratchBytes) cap -= cap > 4096 ? 4096 : cap;
	return cap;
}

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
struct ScratchAddr {
	unsigned long long ctx_id; // the driver's unique id of the context the address belongs to (0 = none)
	void *ptr;
};
static ScratchAddr g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mu;

// Unique id of the calling thread's current context (never reused within a process, so a context
// re-created after cudaDeviceReset gets a new one), through the driver entry points the runtime hands
// out; 0 when there is no current context or the driver lacks the calls.
static unsigned long long current_context_id() {
	using GetCurrentFn = CUresult (*)(CUcontext *);
	using GetIdFn = CUresult (*)(CUcontext, unsigned long long *);
	static GetCurrentFn get_current = nullptr;
	static GetIdFn get_id = nullptr;
	static std::once_flag once;
	std::call_once(once, [] {
		cudaDriverEntryPointQueryResult q;
		void *f = nullptr;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			get_current = (GetCurrentFn)f;
		f = nullptr;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
		    q == cudaDriverEntryPointSuccess)
			get_id = (GetIdFn)f;
	});
	CUcontext ctx = nullptr;
	unsigned long long id = 0;
	if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
		return 0;
	return id;
}

// Device address of g_static_scratch in the current device's context, looked up with the device
// current the first time a context uses it, and again whenever that context has been replaced (after a
// cudaDeviceReset the module is loaded anew and the array may move).  In host code the array's name
// only stands in for it; kernels must be given this address.
static cudaError_t static_scratch(void **out) {
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return e;
	if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
	std::lock_guard<std::mutex> lk(g_scratch_mu);
	const unsigned long long id = current_context_id();
	ScratchAddr &c = g_scratch_addr[dev];
	if (!c.ptr || id == 0 || c.ctx_id != id) {
		void *p = nullptr;
		e = cudaGetSymbolAddress(&p, g_static_scratch); // also brings up the device's context if needed
		if (e != cudaSuccess) return e;
		c.ptr = p;
		c.ctx_id = id ? id : current_context_id();
	}
	*out = c.ptr;
	return cudaSuccess;
}

} // namespace svo

using namespace svo;

extern "C" int svo_voxelize_static(const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint64_t *frags,
                                   uint64_t capacity, uint64_t *count_dev, void *stream) {
	if (level < SVO_LEVEL_MIN || level > SVO_LEVEL_MAX) return svo_fail(SVO_ERR_INVALID, "level %u outside [1, 12]", level);
	if (n_tris > kStaticMaxTris)
		return svo_fail(SVO_ERR_CAPACITY,
		                "svo_voxelize_static handles at most %u triangles (got %u); use svo_voxelize for larger meshes",
		                kStaticMaxTris, n_tris);
	if ((n_tris && !tris) || ((uintptr_t)tris % 16) != 0) return svo_fail(SVO_ERR_INVALID, "triangle buffer must be 16-byte aligned");
	if (!count_dev || (capacity && !frags)) return svo_fail(SVO_ERR_INVALID, "null argument");
	void *scratch = nullptr;
	cudaError_t e = static_scratch(&scratch);
	if (e != cudaSuccess) return svo_fail(SVO_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
	cudaStream_t s = (cudaStream_t)stream;
	VoxWorkspace w;
	vox_workspace_layout(scratch, n_tris, static_unit_cap(n_tris), w);
	// vox_launch_count clears the scan descriptors and counters the previous call left behind
	e = vox_launch_count(tris, n_tris, level, w, s);
	if (e == cudaSuccess) e = vox_launch_totals(w, s);
	if (e == cudaSuccess) e = vox_launch_emit(tris, n_tris, level, w, frags, capacity, s, false);
	if (e == cudaSuccess) e = cudaMemcpyAsync(count_dev, w.totals, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(count_dev + 1, w.totals + 2, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
	if (e != cudaSuccess) return svo_fail(SVO_ERR_CUDA, "svo_voxelize_static: %s", cudaGetErrorString(e));
	return SVO_OK;
}
