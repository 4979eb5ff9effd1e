// serve.cu — the serving loop: many octrees resident in HBM, ray-cast and rebuild requests of different
// sizes batched into shared launches (continuous batching), admitted against an HBM budget.
//
// The reference renders one frame of one octree at a time (Application::draw_frame, src/Application.cpp:
// 130-159, and PathTracer::CmdRender, src/PathTracer.cpp:192-215) and rebuilds on a loader thread that
// hands the new octree to the renderer (src/LoaderThread.cpp:43-116).  Here:
//   * a scheduler thread takes pending trace requests in arrival order into a batch while the batch's
//     rays, request count and the device bytes in flight stay within the configured limits, and issues
//     the batch on a free lane (a stream): one march launch for every request's primary rays, one bounce
//     launch, one march launch for the bounce rays, and one copy of each request's hits to its host
//     buffer (when that buffer is page-locked and mapped, the march stores the final hits there directly
//     and only a camera request's primary hits are copied);
//   * up to `lanes` batches are in flight at once, so requests that arrive while others run are admitted
//     as soon as a lane and memory free up, and their work overlaps on the device;
//   * a waiter thread per lane blocks on the lane's completion event and retires its requests (their
//     completion time is taken there);
//   * rebuild requests run on their own thread and stream (voxelize + build, then the pool is shrunk to
//     its range) and swap the scene's octree in; batches already issued keep the octree they started
//     with (shared ownership), later ones use the new one.
// A request's hits depend only on the request: every ray runs exactly the single-request march.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "svo_internal.h"

namespace svo {

int svo_fail(int code, const char *fmt, ...);

namespace {

using Clock = std::chrono::steady_clock;

struct Scene {
	svo_octree o;
	bool owned;
	~Scene() {
		if (owned && o.words) cudaFreeAsync(o.words, nullptr); // its last batch has completed
	}
};
using ScenePtr = std::shared_ptr<Scene>;

struct Req {
	uint64_t id = 0;
	bool rebuild = false;
	svo_trace_request tr;
	uint32_t scene = 0;
	const svo_triangle *tris = nullptr;
	uint32_t n_tris = 0, level = 0;
	ScenePtr sp;
	uint64_t hits = 0;  // hits the request produces
	uint64_t bytes = 0; // device bytes while in flight
	double t_submit = 0, t_launch = 0, t_done = 0;
	int status = -1;    // -1 while pending or running
	uint32_t batch = 0;
	std::string error;
};

struct Lane {
	cudaStream_t s = nullptr;
	cudaEvent_t done = nullptr;
	bool busy = false, armed = false;
	std::vector<Req *> reqs;
	uint64_t bytes = 0;
	void *arena = nullptr;
	size_t arena_cap = 0;
	char *staging = nullptr; // pinned: the batch's node-fetch count and one status word per request, then the job tables
	size_t staging_cap = 0;
	std::condition_variable cv;
	std::thread waiter;
};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

} // namespace

struct Server {
	svo_server_config cfg;
	int device = 0;
	std::mutex mu;
	std::condition_variable wake;    // scheduler: new requests, lanes or memory freed, stop
	std::condition_variable done_cv; // waiters: a request finished
	std::condition_variable rb_cv;   // rebuild thread
	std::deque<Req *> pending, rebuilds;
	std::unordered_map<uint64_t, Req *> reqs;
	std::vector<ScenePtr> scenes;
	std::vector<std::unique_ptr<Lane>> lanes;
	uint64_t next_id = 1, resident = 0, inflight = 0;
	svo_server_stats st;
	bool stop = false;
	std::thread sched, rebuilder;
	cudaStream_t rb_stream = nullptr;
	Clock::time_point t0;
	double now() const { return std::chrono::duration<double, std::micro>(Clock::now() - t0).count(); }
};

static uint64_t scene_bytes(const svo_octree &o) { return (uint64_t)o.capacity * 4; }

// Retires a completed batch (lock held).  Each request has its own status word, so a malformed pool
// (a scene added from a damaged file, say) fails only the requests that traced it.
static void retire(Server *S, Lane &L, double t) {
	S->st.node_fetches += *reinterpret_cast<const unsigned long long *>(L.staging);
	const uint32_t *status = reinterpret_cast<const uint32_t *>(L.staging + 8);
	for (size_t i = 0; i < L.reqs.size(); ++i) {
		Req *r = L.reqs[i];
		r->t_done = t;
		if (status[i] & kStatusMalformed) {
			r->status = SVO_ERR_INVALID;
			r->error = "malformed octree pool";
			++S->st.failed;
		} else {
			r->status = SVO_OK;
		}
		r->sp.reset();
		++S->st.completed;
		S->st.rays += r->hits;
	}
	S->inflight -= L.bytes;
	L.bytes = 0;
	L.reqs.clear();
	L.busy = false;
	L.armed = false;
	S->wake.notify_all();
	S->rb_cv.notify_all();
	S->done_cv.notify_all();
}

static void lane_waiter(Server *S, Lane *L) {
	cudaSetDevice(S->device);
	std::unique_lock<std::mutex> lk(S->mu);
	for (;;) {
		L->cv.wait(lk, [&] { return L->armed || (S->stop && !L->busy); });
		if (!L->armed) break;
		lk.unlock();
		cudaEventSynchronize(L->done);
		const double t = S->now();
		lk.lock();
		retire(S, *L, t);
	}
}

static cudaError_t grow_device(void **p, size_t *cap, size_t need, cudaStream_t s) {
	if (need <= *cap) return cudaSuccess;
	if (*p) cudaFreeAsync(*p, s);
	*p = nullptr;
	*cap = 0;
	const size_t want = need + need / 4 + 65536;
	cudaError_t e = counted_malloc_async(p, want, s);
	if (e == cudaSuccess) *cap = want;
	return e;
}

// Issues one batch on lane L (lock not held; L is marked busy and owned by the caller).
static cudaError_t issue(Server *S, Lane &L) {
	std::vector<Req *> &batch = L.reqs;
	uint32_t ncam = 0;
	for (Req *r : batch) ncam += r->tr.mode == SVO_REQUEST_CAMERA;
	const size_t nb = batch.size();
	size_t off = 0;
	const size_t o_jobs1 = off;
	off = align256(off + sizeof(MarchJob) * nb);
	const size_t o_bjobs = off;
	off = align256(off + sizeof(BounceJob) * ncam);
	const size_t o_jobs2 = off;
	off = align256(off + sizeof(MarchJob) * ncam);
	const size_t table_bytes = off;
	const size_t o_ticket = off; // the ticket (8 B), the node-fetch count (8 B), one status word per request
	off = align256(off + 16 + 4 * nb);
	std::vector<size_t> o_hits(nb), o_rays(nb);
	for (size_t i = 0; i < nb; ++i) {
		const svo_trace_request &t = batch[i]->tr;
		const uint64_t nr = t.mode == SVO_REQUEST_CAMERA ? t.n_primary : t.n_rays;
		o_hits[i] = off;
		off = align256(off + sizeof(svo_hit) * batch[i]->hits);
		o_rays[i] = off;
		off = align256(off + sizeof(svo_ray) * nr);
	}
	cudaError_t e = grow_device(&L.arena, &L.arena_cap, off, L.s);
	if (e != cudaSuccess) return e;
	const size_t status_bytes = align256(8 + 4 * nb); // the fetch count and the status words, read back
	if (table_bytes + status_bytes > L.staging_cap) {
		if (L.staging) cudaFreeHost(L.staging);
		L.staging = nullptr;
		L.staging_cap = 0;
		e = counted_malloc_host((void **)&L.staging, table_bytes + status_bytes + 4096);
		if (e != cudaSuccess) return e;
		L.staging_cap = table_bytes + status_bytes + 4096;
	}
	char *dev = (char *)L.arena, *host = L.staging + status_bytes; // staging: fetch count, status words
	MarchJob *j1 = (MarchJob *)(host + o_jobs1), *j2 = (MarchJob *)(host + o_jobs2);
	BounceJob *bj = (BounceJob *)(host + o_bjobs);
	uint64_t slots1 = 0, slots2 = 0, nbounce = 0;
	uint32_t k2 = 0;
	// A request whose hit buffer is page-locked and mapped gets its final hits stored in place by the march
	// over the GPU-CPU link (rays requests: all of them; camera requests: the bounce hits, while the primary
	// hits stay in the arena for the bounce launch to read and are copied).  Everything the kernels read
	// stays in device memory: reads over the link would stall the shared launches.
	std::vector<svo_hit *> hits_mapped(nb);
	for (size_t i = 0; i < nb; ++i) hits_mapped[i] = static_cast<svo_hit *>(mapped_host_ptr(batch[i]->tr.hits, 16));
	for (size_t i = 0; i < nb; ++i) {
		Req *r = batch[i];
		const svo_trace_request &t = r->tr;
		const svo_octree &o = r->sp->o;
		MarchJob j;
		memset(&j, 0, sizeof(j));
		j.pool = o.words;
		j.range = o.range_words;
		j.level = o.level;
		j.hits = hits_mapped[i] && t.mode == SVO_REQUEST_RAYS ? hits_mapped[i] : (svo_hit *)(dev + o_hits[i]);
		j.req = (uint32_t)i;
		if (t.mode == SVO_REQUEST_CAMERA) {
			j.rays = nullptr;
			j.cam = t.camera;
			j.width = t.width;
			j.height = t.height;
			j.n = t.n_primary;
			j.slot_begin = slots1;
			slots1 += march_job_slots(j);
			j1[i] = j;
			BounceJob b;
			b.hits = j.hits;
			b.rays = (svo_ray *)(dev + o_rays[i]);
			b.seed = t.seed;
			b.begin = nbounce;
			nbounce += t.n_primary;
			bj[k2] = b;
			MarchJob m2 = j;
			m2.rays = b.rays;
			m2.hits = (hits_mapped[i] ? hits_mapped[i] : j.hits) + t.n_primary;
			m2.slot_begin = slots2;
			slots2 += march_job_slots(m2);
			j2[k2++] = m2;
		} else {
			j.rays = (const svo_ray *)(dev + o_rays[i]);
			j.n = t.n_rays;
			j.slot_begin = slots1;
			slots1 += march_job_slots(j);
			j1[i] = j;
		}
	}
	unsigned long long *ticket = (unsigned long long *)(dev + o_ticket);
	// the node-fetch count is kept only when the server was asked to (it costs the march ~7%)
	unsigned long long *fetches = (S->cfg.flags & SVO_SERVER_COUNT_FETCHES) ? ticket + 1 : nullptr;
	uint32_t *status = (uint32_t *)(ticket + 2);
	e = cudaMemcpyAsync(dev, host, table_bytes, cudaMemcpyHostToDevice, L.s);
	if (e == cudaSuccess) e = cudaMemsetAsync(ticket + 1, 0, 8 + 4 * nb, L.s);
	for (size_t i = 0; i < nb && e == cudaSuccess; ++i)
		if (batch[i]->tr.mode == SVO_REQUEST_RAYS)
			e = cudaMemcpyAsync(dev + o_rays[i], batch[i]->tr.rays, sizeof(svo_ray) * batch[i]->tr.n_rays,
			                    cudaMemcpyHostToDevice, L.s);
	if (e == cudaSuccess)
		e = march_jobs_launch((const MarchJob *)(dev + o_jobs1), (uint32_t)nb, slots1, ticket, status, fetches, L.s);
	if (e == cudaSuccess && ncam) e = bounce_jobs_launch((const BounceJob *)(dev + o_bjobs), ncam, nbounce, L.s);
	if (e == cudaSuccess && ncam)
		e = march_jobs_launch((const MarchJob *)(dev + o_jobs2), ncam, slots2, ticket, status, fetches, L.s);
	for (size_t i = 0; i < nb && e == cudaSuccess; ++i) {
		const svo_trace_request &t = batch[i]->tr;
		// mapped: nothing for rays requests, the primary half for camera requests
		const uint64_t n = !hits_mapped[i] ? batch[i]->hits : (t.mode == SVO_REQUEST_CAMERA ? t.n_primary : 0);
		if (n) e = cudaMemcpyAsync(t.hits, dev + o_hits[i], sizeof(svo_hit) * n, cudaMemcpyDeviceToHost, L.s);
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(L.staging, ticket + 1, 8 + 4 * nb, cudaMemcpyDeviceToHost, L.s);
	if (e == cudaSuccess) e = cudaEventRecord(L.done, L.s);
	return e;
}

static void scheduler(Server *S) {
	cudaSetDevice(S->device);
	std::unique_lock<std::mutex> lk(S->mu);
	for (;;) {
		Lane *free_lane = nullptr;
		bool any_busy = false;
		for (auto &L : S->lanes) {
			if (L->busy)
				any_busy = true;
			else if (!free_lane)
				free_lane = L.get();
		}
		if (S->stop && S->pending.empty() && !any_busy) break;
		if (free_lane && !S->pending.empty()) {
			// FIFO batch within the ray, request and memory limits
			const uint64_t budget = S->cfg.hbm_budget_bytes;
			const uint64_t room = budget > S->resident + S->inflight ? budget - S->resident - S->inflight : 0;
			std::vector<Req *> batch;
			uint64_t rays = 0, bytes = 0;
			while (!S->pending.empty() && batch.size() < S->cfg.max_batch_requests) {
				Req *r = S->pending.front();
				if (!batch.empty() && rays + r->hits > S->cfg.max_batch_rays) break;
				if (bytes + r->bytes > room) {
					if (batch.empty() && !any_busy && r->bytes > (budget > S->resident ? budget - S->resident : 0)) {
						// can never fit: fail it rather than wait forever
						S->pending.pop_front();
						r->status = SVO_ERR_CAPACITY;
						r->error = "request exceeds the HBM budget left by the resident octrees";
						r->t_done = S->now();
						r->sp.reset();
						++S->st.failed;
						S->done_cv.notify_all();
						continue;
					}
					break;
				}
				S->pending.pop_front();
				rays += r->hits;
				bytes += r->bytes;
				batch.push_back(r);
			}
			if (!batch.empty()) {
				Lane &L = *free_lane;
				L.busy = true;
				L.reqs = batch;
				L.bytes = bytes;
				S->inflight += bytes;
				const double t = S->now();
				for (Req *r : batch) {
					r->t_launch = t;
					r->batch = (uint32_t)batch.size();
				}
				++S->st.batches;
				S->st.batched_requests += batch.size();
				lk.unlock();
				const cudaError_t e = issue(S, L);
				lk.lock();
				if (e != cudaSuccess) {
					cudaGetLastError();
					cudaStreamSynchronize(L.s);
					for (Req *r : L.reqs) {
						r->status = SVO_ERR_CUDA;
						r->error = cudaGetErrorString(e);
						r->t_done = S->now();
						r->sp.reset();
						++S->st.failed;
					}
					S->inflight -= L.bytes;
					L.bytes = 0;
					L.reqs.clear();
					L.busy = false;
					S->done_cv.notify_all();
				} else {
					L.armed = true;
					L.cv.notify_one();
				}
				continue;
			}
		}
		S->wake.wait(lk);
	}
}

// Voxelize + build on the given stream (blocking), then shrink the pool to its range.
static int build_scene(const svo_triangle *tris, uint32_t n, uint32_t level, cudaStream_t s, svo_octree *out) {
	svo_fraglist f;
	memset(&f, 0, sizeof(f));
	int rc = svo_voxelize(tris, n, level, &f, s);
	if (rc) return rc;
	svo_octree o;
	memset(&o, 0, sizeof(o));
	rc = svo_build_fraglist(&f, &o, nullptr, s);
	svo_fraglist_destroy(&f, s);
	if (rc) return rc;
	void *exact = nullptr;
	const uint32_t range = o.range_words;
	cudaError_t e = counted_malloc_async(&exact, (size_t)range * 4, s);
	if (e == cudaSuccess) e = cudaMemcpyAsync(exact, o.words, (size_t)range * 4, cudaMemcpyDeviceToDevice, s);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	svo_octree_destroy(&o, s); // (clears o)
	if (e != cudaSuccess) {
		if (exact) cudaFreeAsync(exact, s);
		cudaGetLastError();
		return svo_fail(e == cudaErrorMemoryAllocation ? SVO_ERR_OOM : SVO_ERR_CUDA, "scene build: %s",
		                cudaGetErrorString(e));
	}
	memset(out, 0, sizeof(*out));
	out->words = (uint32_t *)exact;
	out->capacity = range;
	out->range_words = range;
	out->level = level;
	out->owned = 1;
	return SVO_OK;
}

static void rebuild_worker(Server *S) {
	cudaSetDevice(S->device);
	std::unique_lock<std::mutex> lk(S->mu);
	for (;;) {
		S->rb_cv.wait(lk, [&] { return S->stop || !S->rebuilds.empty(); });
		if (S->rebuilds.empty()) break; // stop with nothing left
		Req *r = S->rebuilds.front();
		// admission: the new octree may need up to 64 B per triangle of scratch and as much pool as the old
		const uint64_t need = 64ull * r->n_tris + (S->scenes[r->scene] ? scene_bytes(S->scenes[r->scene]->o) : 0);
		if (S->resident + S->inflight + need > S->cfg.hbm_budget_bytes && (S->inflight > 0)) {
			S->rb_cv.wait(lk); // memory frees up as batches retire
			continue;
		}
		S->rebuilds.pop_front();
		r->t_launch = S->now();
		lk.unlock();
		svo_octree o;
		const int rc = build_scene(r->tris, r->n_tris, r->level, S->rb_stream, &o);
		std::string err = rc ? svo_last_error() : "";
		lk.lock();
		r->t_done = S->now();
		r->status = rc;
		r->error = err;
		if (rc == SVO_OK) {
			auto sp = std::make_shared<Scene>();
			sp->o = o;
			sp->owned = true;
			ScenePtr &slot = S->scenes[r->scene];
			if (slot) S->resident -= scene_bytes(slot->o);
			slot = sp; // batches issued earlier keep the old octree alive until they retire
			S->resident += scene_bytes(o);
			++S->st.rebuilds;
			++S->st.completed;
		} else {
			++S->st.failed;
		}
		S->done_cv.notify_all();
		S->wake.notify_all();
	}
}

} // namespace svo

using namespace svo;

struct svo_server {
	Server s;
};

extern "C" {

int svo_server_create(const svo_server_config *cfg, svo_server **out) {
	if (!out) return svo_fail(SVO_ERR_INVALID, "null output");
	*out = nullptr;
	auto *h = new (std::nothrow) svo_server();
	if (!h) return svo_fail(SVO_ERR_OOM, "server allocation");
	Server *S = &h->s;
	svo_server_config c;
	memset(&c, 0, sizeof(c));
	if (cfg) c = *cfg;
	if (c.hbm_budget_bytes == 0) c.hbm_budget_bytes = 40ull << 30;
	if (c.lanes == 0) c.lanes = 3;
	if (c.lanes > 16) c.lanes = 16;
	if (c.max_batch_rays == 0) c.max_batch_rays = 8u << 20;
	if (c.max_batch_requests == 0) c.max_batch_requests = 256;
	S->cfg = c;
	memset(&S->st, 0, sizeof(S->st));
	cudaGetDevice(&S->device);
	S->t0 = Clock::now();
	// trace lanes at the device's highest stream priority, rebuilds at its lowest: when both have blocks
	// waiting for an SM, a trace batch's go first, so requests queued behind a rebuild wait less
	int least = 0, greatest = 0;
	cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
	if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&S->rb_stream, cudaStreamNonBlocking, least);
	for (uint32_t i = 0; i < c.lanes && e == cudaSuccess; ++i) {
		auto L = std::make_unique<Lane>();
		e = cudaStreamCreateWithPriority(&L->s, cudaStreamNonBlocking, greatest);
		if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming);
		S->lanes.push_back(std::move(L));
	}
	if (e != cudaSuccess) {
		cudaGetLastError();
		for (auto &L : S->lanes) {
			if (L->s) cudaStreamDestroy(L->s);
			if (L->done) cudaEventDestroy(L->done);
		}
		if (S->rb_stream) cudaStreamDestroy(S->rb_stream);
		delete h;
		return svo_fail(SVO_ERR_CUDA, "server streams: %s", cudaGetErrorString(e));
	}
	for (auto &L : S->lanes) L->waiter = std::thread(lane_waiter, S, L.get());
	S->sched = std::thread(scheduler, S);
	S->rebuilder = std::thread(rebuild_worker, S);
	*out = h;
	return SVO_OK;
}

void svo_server_destroy(svo_server *h) {
	if (!h) return;
	Server *S = &h->s;
	{
		std::lock_guard<std::mutex> lk(S->mu);
		S->stop = true;
	}
	S->wake.notify_all();
	S->rb_cv.notify_all();
	S->sched.join(); // drains the pending requests
	S->rebuilder.join();
	{
		std::lock_guard<std::mutex> lk(S->mu);
		for (auto &L : S->lanes) L->cv.notify_all();
	}
	for (auto &L : S->lanes) L->waiter.join();
	for (auto &L : S->lanes) {
		cudaStreamSynchronize(L->s);
		if (L->arena) cudaFreeAsync(L->arena, L->s);
		cudaStreamSynchronize(L->s);
		if (L->staging) cudaFreeHost(L->staging);
		cudaEventDestroy(L->done);
		cudaStreamDestroy(L->s);
	}
	S->scenes.clear();
	cudaStreamSynchronize(nullptr);
	cudaStreamDestroy(S->rb_stream);
	for (auto &kv : S->reqs) delete kv.second;
	delete h;
}

int svo_server_add_octree(svo_server *h, const svo_octree *o, uint32_t *scene) {
	if (!h || !o || !scene) return svo_fail(SVO_ERR_INVALID, "null argument");
	if (!o->words || o->level < SVO_LEVEL_MIN || o->level > SVO_LEVEL_MAX || o->range_words < 8 || o->range_words % 8)
		return svo_fail(SVO_ERR_INVALID, "malformed octree");
	Server *S = &h->s;
	auto sp = std::make_shared<Scene>();
	sp->o = *o;
	sp->o.owned = 0;
	sp->owned = false;
	std::lock_guard<std::mutex> lk(S->mu);
	S->scenes.push_back(sp);
	S->resident += scene_bytes(sp->o);
	*scene = (uint32_t)S->scenes.size() - 1;
	return SVO_OK;
}

int svo_server_build_scene(svo_server *h, const svo_triangle *tris, uint32_t n_tris, uint32_t level, uint32_t *scene) {
	if (!h || !scene) return svo_fail(SVO_ERR_INVALID, "null argument");
	Server *S = &h->s;
	cudaStream_t s = nullptr;
	if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
		return svo_fail(SVO_ERR_CUDA, "scene build stream");
	svo_octree o;
	const int rc = build_scene(tris, n_tris, level, s, &o);
	cudaStreamDestroy(s);
	if (rc) return rc;
	auto sp = std::make_shared<Scene>();
	sp->o = o;
	sp->owned = true;
	std::lock_guard<std::mutex> lk(S->mu);
	S->scenes.push_back(sp);
	S->resident += scene_bytes(o);
	*scene = (uint32_t)S->scenes.size() - 1;
	return SVO_OK;
}

int svo_server_scene(svo_server *h, uint32_t scene, svo_octree *view) {
	if (!h || !view) return svo_fail(SVO_ERR_INVALID, "null argument");
	Server *S = &h->s;
	std::lock_guard<std::mutex> lk(S->mu);
	if (scene >= S->scenes.size() || !S->scenes[scene]) return svo_fail(SVO_ERR_INVALID, "no scene %u", scene);
	*view = S->scenes[scene]->o;
	view->owned = 0;
	return SVO_OK;
}

int svo_server_submit_trace(svo_server *h, const svo_trace_request *t, uint64_t *ticket) {
	if (!h || !t || !ticket) return svo_fail(SVO_ERR_INVALID, "null argument");
	if (!t->hits) return svo_fail(SVO_ERR_INVALID, "null hit buffer");
	uint64_t hits;
	if (t->mode == SVO_REQUEST_CAMERA) {
		if (t->n_primary == 0 || t->width == 0 || t->height == 0 || (uint64_t)t->width * t->height < t->n_primary)
			return svo_fail(SVO_ERR_INVALID, "camera request: need 0 < n_primary <= width * height");
		hits = 2ull * t->n_primary;
	} else if (t->mode == SVO_REQUEST_RAYS) {
		if (t->n_rays == 0 || !t->rays) return svo_fail(SVO_ERR_INVALID, "ray request: need rays");
		hits = t->n_rays;
	} else {
		return svo_fail(SVO_ERR_INVALID, "unknown request mode %u", t->mode);
	}
	Server *S = &h->s;
	auto *r = new (std::nothrow) Req();
	if (!r) return svo_fail(SVO_ERR_OOM, "request allocation");
	r->tr = *t;
	r->hits = hits;
	r->bytes = hits * sizeof(svo_hit) + (t->mode == SVO_REQUEST_CAMERA ? t->n_primary : t->n_rays) * sizeof(svo_ray);
	{
		std::lock_guard<std::mutex> lk(S->mu);
		if (S->stop) {
			delete r;
			return svo_fail(SVO_ERR_INVALID, "server is shutting down");
		}
		if (t->scene >= S->scenes.size() || !S->scenes[t->scene]) {
			delete r;
			return svo_fail(SVO_ERR_INVALID, "no scene %u", t->scene);
		}
		r->sp = S->scenes[t->scene]; // the octree current at submission
		r->id = S->next_id++;
		r->t_submit = S->now();
		S->reqs[r->id] = r;
		S->pending.push_back(r);
		++S->st.submitted;
		*ticket = r->id;
	}
	S->wake.notify_one();
	return SVO_OK;
}

int svo_server_submit_rebuild(svo_server *h, uint32_t scene, const svo_triangle *tris, uint32_t n_tris, uint32_t level,
                              uint64_t *ticket) {
	if (!h || !ticket) return svo_fail(SVO_ERR_INVALID, "null argument");
	if (level < SVO_LEVEL_MIN || level > SVO_LEVEL_MAX) return svo_fail(SVO_ERR_INVALID, "level %u", level);
	if (n_tris && !tris) return svo_fail(SVO_ERR_INVALID, "null triangle buffer");
	Server *S = &h->s;
	auto *r = new (std::nothrow) Req();
	if (!r) return svo_fail(SVO_ERR_OOM, "request allocation");
	r->rebuild = true;
	r->scene = scene;
	r->tris = tris;
	r->n_tris = n_tris;
	r->level = level;
	{
		std::lock_guard<std::mutex> lk(S->mu);
		if (S->stop || scene >= S->scenes.size()) {
			delete r;
			return svo_fail(SVO_ERR_INVALID, "no scene %u", scene);
		}
		r->id = S->next_id++;
		r->t_submit = S->now();
		S->reqs[r->id] = r;
		S->rebuilds.push_back(r);
		++S->st.submitted;
		*ticket = r->id;
	}
	S->rb_cv.notify_one();
	return SVO_OK;
}

int svo_server_wait(svo_server *h, uint64_t ticket, int timeout_ms, svo_request_result *res) {
	if (!h) return svo_fail(SVO_ERR_INVALID, "null server");
	Server *S = &h->s;
	std::unique_lock<std::mutex> lk(S->mu);
	auto it = S->reqs.find(ticket);
	if (it == S->reqs.end()) return svo_fail(SVO_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
	Req *r = it->second;
	auto ready = [&] { return r->status >= 0; };
	if (timeout_ms < 0)
		S->done_cv.wait(lk, ready);
	else if (!S->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
		return svo_fail(SVO_ERR_TIMEOUT, "request %llu not done after %d ms", (unsigned long long)ticket, timeout_ms);
	if (res) {
		res->status = r->status;
		res->batch_requests = r->batch;
		res->submit_us = r->t_submit;
		res->launch_us = r->t_launch;
		res->done_us = r->t_done;
	}
	const int status = r->status;
	const std::string err = r->error;
	S->reqs.erase(it);
	delete r;
	if (status != SVO_OK) return svo_fail(status, "request %llu: %s", (unsigned long long)ticket, err.c_str());
	return SVO_OK;
}

void svo_server_get_stats(svo_server *h, svo_server_stats *out) {
	if (!h || !out) return;
	Server *S = &h->s;
	std::lock_guard<std::mutex> lk(S->mu);
	*out = S->st;
	out->resident_bytes = S->resident;
	out->inflight_bytes = S->inflight;
	out->pending = S->pending.size() + S->rebuilds.size();
}

} // extern "C"
