// common.cuh — device helpers shared by the voxelize, build and march kernels (sm_103a).
#pragma once

#include <atomic>
#include <cstdint>
#include <utility>
#include <cuda_runtime.h>

#include "../../include/svo.h"
#include "svo_internal.h"

#define SVO_DEV __device__ __forceinline__

namespace svo {

constexpr unsigned kFullMask = 0xffffffffu;

// Iterations a tile waits for its predecessor's descriptor before giving up.  Tiles are claimed in
// order by an atomic ticket, so the predecessor is always running or done; the bound only guards
// against a broken invariant and is never reached in a correct run.
constexpr uint32_t kSpinLimit = 1u << 22;

// Programmatic dependent launch.  Every engine kernel is launched with programmatic stream
// serialization, so the launch and set-up of a kernel overlap the last blocks of the kernel before it
// on the same stream; each kernel's first statement waits (`griddepcontrol.wait`) until that
// predecessor has completed and its memory operations are visible, which keeps the ordering of a plain
// stream launch.  No kernel triggers its dependents early, so a dependent's blocks take SM resources
// only as the predecessor's blocks retire.  Without the launch attribute the wait is a no-op.
SVO_DEV void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                            Args &&...args) {
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	attr[0].val.programmaticStreamSerializationAllowed = 1;
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = smem;
	cfg.stream = stream;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Grid of a persistent kernel: the blocks of `kernel` that are resident on the current device at once
// (its occupancy at `threads` threads and `smem` bytes of dynamic shared memory, measured once per device).
template <typename... KArgs>
inline uint32_t resident_grid(void (*kernel)(KArgs...), int threads, size_t smem = 0) {
	constexpr int kDevices = 16;
	static std::atomic<int> per_sm[kDevices];
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevices) dev = 0;
	int b = per_sm[dev].load(std::memory_order_relaxed);
	if (b == 0) {
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem) != cudaSuccess || b < 1) {
			cudaGetLastError();
			b = 1;
		}
		per_sm[dev].store(b, std::memory_order_relaxed);
	}
	return (uint32_t)(b * device_sm_count());
}

// Test hook of the bounded waits (svo_debug_wait_fault): `limit` bounds every wait's iterations, and the
// look-back tile or beam texel numbered `withheld` never publishes, so the waits on it run out and take
// their timeout path (a status bit, never a trap).  The defaults, kSpinLimit and no tile, leave the
// kernels' behaviour unchanged.  Each translation unit holds its own copy, set by its own setter.
struct WaitFault {
	uint32_t limit;
	uint32_t withheld;
};
static __constant__ WaitFault c_wait_fault = {kSpinLimit, 0xffffffffu};
static inline cudaError_t set_wait_fault_here(uint32_t limit, uint32_t withheld) {
	const WaitFault f = {limit ? limit : kSpinLimit, limit ? withheld : 0xffffffffu};
	return cudaMemcpyToSymbol(c_wait_fault, &f, sizeof(f));
}

// ------------------------------------------------------------------------------- warp / block scans
SVO_DEV uint32_t lane_id() { return threadIdx.x & 31u; }

template <typename T> SVO_DEV T warp_inclusive_sum(T v) {
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		T o = __shfl_up_sync(kFullMask, v, d);
		if ((int)lane_id() >= d) v += o;
	}
	return v;
}

template <typename T> SVO_DEV T warp_sum(T v) {
#pragma unroll
	for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFullMask, v, d);
	return v;
}

// Runs of equal keys in consecutive lanes (called by the full warp): the first and last lane of this
// lane's run.  Equal keys in separate runs form separate runs.  A shuffle and a ballot instead of
// __match_any_sync, whose throughput limits warp-merging sweeps.
SVO_DEV void lane_run(uint32_t key, uint32_t lane, uint32_t &first, uint32_t &last) {
	const uint32_t prev = __shfl_up_sync(kFullMask, key, 1);
	const uint32_t heads = __ballot_sync(kFullMask, lane == 0u || key != prev);
	const uint32_t upto = lane == 31u ? kFullMask : ((2u << lane) - 1u); // lanes 0..lane
	first = 31u - (uint32_t)__clz(heads & upto);
	const uint32_t after = heads & ~upto;
	last = after ? (uint32_t)__ffs(after) - 2u : 31u;
}

// OR of v over lanes lane..last (called by the full warp); at a run's first lane, the OR of its run.
SVO_DEV uint32_t run_or(uint32_t v, uint32_t lane, uint32_t last) {
#pragma unroll
	for (uint32_t d = 1; d < 32; d <<= 1) {
		const uint32_t o = __shfl_down_sync(kFullMask, v, d);
		if (lane + d <= last) v |= o;
	}
	return v;
}

// Exclusive block scan of one value per thread; returns the exclusive prefix and the block total.
// `warp_tmp` must hold blockDim.x / 32 + 1 elements.
template <typename T, int TPB> SVO_DEV T block_exclusive_sum(T v, T *warp_tmp, T &total) {
	const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
	T incl = warp_inclusive_sum(v);
	if (lane == 31) warp_tmp[warp] = incl;
	__syncthreads();
	if (warp == 0) {
		T w = lane < TPB / 32 ? warp_tmp[lane] : T(0);
		T wi = warp_inclusive_sum(w);
		if (lane < TPB / 32) warp_tmp[lane] = wi - w;
		if (lane == 31) warp_tmp[TPB / 32] = wi;
	}
	__syncthreads();
	T r = warp_tmp[warp] + incl - v;
	total = warp_tmp[TPB / 32];
	__syncthreads();
	return r;
}

// ------------------------------------------------------------------------------- decoupled look-back
// Tile descriptor (64 bits): epoch[56..63] | flag[54..55] | value[0..53]; flag 1 = tile aggregate,
// 2 = inclusive prefix.  A descriptor whose epoch differs from the caller's counts as unpublished, so
// one zeroed descriptor array serves several scans (levels) of one call.
constexpr unsigned long long kDescValueMask = (1ull << 54) - 1;

SVO_DEV void desc_publish(unsigned long long *d, uint32_t epoch, uint32_t flag, unsigned long long value) {
	unsigned long long w = ((unsigned long long)epoch << 56) | ((unsigned long long)flag << 54) | value;
	asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(d), "l"(w) : "memory");
}

SVO_DEV unsigned long long desc_load(const unsigned long long *d) {
	unsigned long long w;
	asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(w) : "l"(d) : "memory");
	return w;
}

// Decoupled look-back for tile `t` once its aggregate is known, called by all 32 lanes of one warp:
// each step inspects the 32 nearest unexamined predecessors at once and sums their aggregates up to
// the nearest inclusive prefix.  Returns the tile's exclusive prefix on every lane.  Waits are bounded
// (c_wait_fault.limit, kSpinLimit unless a test lowers it); on timeout the status word gets kStatusTimeout
// and the returned prefix is a partial sum of published aggregates, never above the true prefix, so
// offsets derived from it stay inside the buffers their totals size.  A tile with seg_start set begins a
// new segment (a segmented scan): its prefix is 0, and the look-back of later tiles stops there.
// published = true: the tile's aggregate was published earlier by tile_publish_aggregate.
SVO_DEV unsigned long long tile_lookback_warp(unsigned long long *descs, uint32_t t, uint32_t epoch,
                                              unsigned long long aggregate, uint32_t *status,
                                              bool seg_start = false, bool published = false) {
	const uint32_t lane = lane_id();
	const WaitFault wf = c_wait_fault;
	const bool publish = t != wf.withheld;
	if (t == 0 || seg_start) {
		if (lane == 0 && publish && !published) desc_publish(&descs[t], epoch, 2, aggregate);
		return 0;
	}
	if (lane == 0 && publish && !published) desc_publish(&descs[t], epoch, 1, aggregate);
	unsigned long long prefix = 0;
	int64_t end = (int64_t)t - 1; // window: descriptors end, end-1, ..., end-31 (lane k reads end-k)
	uint32_t spins = 0;
	for (;;) {
		const int64_t j = end - (int64_t)lane;
		unsigned long long w = 0;
		uint32_t flag = 2; // before tile 0: an inclusive prefix of 0
		if (j >= 0) {
			w = desc_load(&descs[j]);
			flag = ((uint32_t)(w >> 56) == epoch) ? (uint32_t)(w >> 54) & 3u : 0u;
		}
		const uint32_t incl = __ballot_sync(kFullMask, flag == 2);
		const uint32_t first = incl ? (uint32_t)(__ffs(incl) - 1) : 31u;
		const uint32_t need = first == 31u ? kFullMask : ((2u << first) - 1u);
		if (__ballot_sync(kFullMask, flag == 0) & need) { // a needed predecessor has not published yet
			if (++spins > wf.limit) { // prefix stays a partial sum of real aggregates: below the true one
				if (lane == 0) atomicOr(status, kStatusTimeout);
				break;
			}
			__nanosleep(20);
			continue;
		}
		prefix += warp_sum(((need >> lane) & 1u) && j >= 0 ? (w & kDescValueMask) : 0ull);
		if (incl) break;
		end -= 32;
	}
	if (lane == 0 && publish) desc_publish(&descs[t], epoch, 2, prefix + aggregate);
	return prefix;
}

// The first half of a deferred look-back (one thread): tile t publishes its aggregate (tile 0 or a
// segment start: its inclusive prefix) as soon as it is known, and looks back later
// (tile_lookback_warp(..., published = true)) after other work, when its predecessors have published.
SVO_DEV void tile_publish_aggregate(unsigned long long *descs, uint32_t t, uint32_t epoch,
                                    unsigned long long aggregate, bool seg_start = false) {
	if (t != c_wait_fault.withheld) desc_publish(&descs[t], epoch, (t == 0 || seg_start) ? 2u : 1u, aggregate);
}

// ------------------------------------------------------------------------------- integer helpers
// floor(num / den) for den > 0, exact whenever the exact quotient lies in [lo - 2, hi + 2]; outside
// that window the result lies outside [lo, hi] on the same side as the exact quotient, which is all a
// caller that clamps to [lo, hi] needs.  The estimate uses 32-bit arithmetic only (64-bit integer <->
// float conversions run on the FP64 pipe, which is narrow on this part): num and den are shifted right
// by the same amount until both fit 31 bits, which keeps their ratio.  Inside the window (|quotient| <
// 2^13) den then keeps at least 17 significant bits, so the float quotient is within 0.01 of the exact
// one; its floor is corrected by one exact int64 remainder.  (A den shifted to 0 means a quotient of
// magnitude >= 2^30: the infinite estimate clamps to the correct side.)
SVO_DEV int64_t floor_div_window(int64_t num, int64_t den, int32_t lo, int32_t hi) {
	const uint64_t mag = (uint64_t)(num < 0 ? -num : num) | (uint64_t)den;
	const int sh = max(0, 33 - __clzll((long long)mag)); // bits(mag) - 31
	const float nf = (float)(int32_t)(num >> sh), df = (float)(int32_t)(den >> sh);
	float est = floorf(__fdividef(nf, df));
	est = fminf(fmaxf(est, (float)(lo - 2)), (float)(hi + 2));
	int64_t q = (int32_t)est;
	const int64_t r = num - q * den;
	if (r < 0)
		q -= 1;
	else if (r >= den)
		q += 1;
	return q;
}

SVO_DEV int32_t clamp_i32(int64_t v, int32_t lo, int32_t hi) {
	return (int32_t)(v < lo ? lo : (v > hi ? hi : v));
}

} // namespace svo
