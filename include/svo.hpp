// svo.hpp — C++ host classes with the reference's names and call shapes, over the C ABI (svo.h).
//
//   reference (Vulkan)                                 here (CUDA streams, device pointers)
//   Scene::Create(queue, filename)   src/Scene.cpp:387   svo::Scene::Create(triangles)        (upload only)
//   Voxelizer::Create(scene, pool, level)  :5-26         svo::Voxelizer::Create(scene, level)
//   Voxelizer::CmdVoxelize(cb)             :167-179      svo::Voxelizer::CmdVoxelize(stream)
//   OctreeBuilder::Create(voxelizer, pool) src/OctreeBuilder.cpp:8-22
//                                                        svo::OctreeBuilder::Create(voxelizer)
//   OctreeBuilder::CmdBuild(cb)            :142-210      svo::OctreeBuilder::CmdBuild(stream)
//   OctreeBuilder::GetOctreeRange(pool)    :212-214      svo::OctreeBuilder::GetOctreeRange()  (bytes)
//   Octree::Update(pool, builder)   src/Octree.cpp:22-35 svo::Octree::Update(builder)
//   OctreeTracer::CmdDrawPipeline(cb, frame) src/OctreeTracer.cpp:213-246
//                                                        svo::OctreeTracer::CmdDrawPipeline(hits, stream)
//   (+ reading the frame back)                           svo::OctreeTracer::CmdDrawPipelineToHost(hits, host, stream)
//   OctreeTracer::CmdBeamRenderPass(cb, frame) :183-211  svo::OctreeTracer::CmdBeamRenderPass(beam, stream)
//                                                        (+ CmdDrawPipelineBeam, CmdOcclude)
//   Scene::load_meshes(filename)   src/Scene.cpp:36-147  svo::LoadObj(path)
//   (one mesh per loader run)  src/LoaderThread.cpp:43  svo::BatchBuilder (many meshes per launch)
//   (one octree per frame)  src/Application.cpp:130-159 svo::Server (resident octrees, batched requests)
//   EnvironmentMap::Reset(pool, filename) src/EnvironmentMap.cpp:44-52
//                                                        svo::EnvironmentMap::Reset(rgba, width, height)
//   Lighting (src/Lighting.hpp)                          svo::Lighting
//   PathTracer::Create / Reset / CmdRender / Extract*Image src/PathTracer.cpp:168-298
//                                                        svo::PathTracer (same names, stream-ordered)
//
// Header-only; needs no CUDA headers.  Link against libsvo.so.  Errors throw svo::Error (the reference
// logs and continues, e.g. src/Octree.cpp:30-33).  A `stream` is a cudaStream_t passed as void*.
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "svo.h"

namespace svo {

class Error : public std::runtime_error {
public:
	Error(int code, const char *msg) : std::runtime_error(std::string("svo error ") + std::to_string(code) + ": " + msg), code(code) {}
	int code;
};

inline void Check(int rc) {
	if (rc != SVO_OK) throw Error(rc, svo_last_error());
}

// Device buffer owned by a wrapper (stream-ordered allocation through the engine).
class DeviceBuffer {
public:
	DeviceBuffer() = default;
	DeviceBuffer(size_t bytes, void *stream) : bytes_(bytes), stream_(stream) { Check(svo_device_alloc(&ptr_, bytes, stream)); }
	~DeviceBuffer() { svo_device_free(ptr_, stream_); }
	DeviceBuffer(const DeviceBuffer &) = delete;
	DeviceBuffer &operator=(const DeviceBuffer &) = delete;
	void *get() const { return ptr_; }
	size_t size() const { return bytes_; }

private:
	void *ptr_ = nullptr;
	size_t bytes_ = 0;
	void *stream_ = nullptr;
};

// Triangle soup in device memory (the reference's Scene holds vertex/index buffers and per-material
// albedo; here every triangle carries its vertex colours, src/Scene.cpp:155-164).
class Scene {
public:
	static std::shared_ptr<Scene> Create(const std::vector<svo_triangle> &triangles, void *stream = nullptr) {
		auto s = std::make_shared<Scene>();
		s->count_ = (uint32_t)triangles.size();
		s->buffer_ = std::make_unique<DeviceBuffer>(triangles.size() * sizeof(svo_triangle), stream);
		Check(svo_upload(s->buffer_->get(), triangles.data(), triangles.size() * sizeof(svo_triangle), stream));
		return s;
	}
	const svo_triangle *GetTriangles() const { return (const svo_triangle *)buffer_->get(); }
	uint32_t GetTriangleCount() const { return count_; }

private:
	std::unique_ptr<DeviceBuffer> buffer_;
	uint32_t count_ = 0;
};

class Voxelizer {
public:
	// Count pass, exact allocation and emission (the reference records the emission in CmdVoxelize).
	static std::shared_ptr<Voxelizer> Create(const std::shared_ptr<Scene> &scene, uint32_t octree_level,
	                                         void *stream = nullptr) {
		auto v = std::make_shared<Voxelizer>();
		v->scene_ = scene;
		v->level_ = octree_level;
		v->stream_ = stream;
		Check(svo_voxelize(scene->GetTriangles(), scene->GetTriangleCount(), octree_level, &v->list_, stream));
		return v;
	}
	~Voxelizer() { svo_fraglist_destroy(&list_, stream_); }

	// Emits the fragments again into the existing list (same scene, same level).
	void CmdVoxelize(void *stream = nullptr) {
		if (!workspace_)
			workspace_ = std::make_unique<DeviceBuffer>(
			    svo_voxelize_workspace_size(scene_->GetTriangleCount(), list_.units), stream);
		if (!count_) count_ = std::make_unique<DeviceBuffer>(2 * sizeof(uint64_t), stream);
		Check(svo_voxelize_into(scene_->GetTriangles(), scene_->GetTriangleCount(), level_, list_.data, list_.capacity,
		                        (uint64_t *)count_->get(), workspace_->get(), workspace_->size(), stream));
		stream_ = stream;
	}

	// Throws unless the last CmdVoxelize produced every fragment (blocking read).
	void CheckEmission() const {
		uint64_t c[2] = {0, 0};
		Check(svo_download(c, count_->get(), sizeof(c), 1, stream_));
		if (c[1] != 0 || c[0] != list_.count) throw Error(SVO_ERR_CAPACITY, "voxelizer re-emission incomplete");
	}

	const std::shared_ptr<Scene> &GetScenePtr() const { return scene_; }
	uint32_t GetLevel() const { return level_; }
	uint32_t GetVoxelResolution() const { return 1u << level_; }
	uint32_t GetVoxelFragmentCount() const { return list_.count; }
	const uint64_t *GetVoxelFragmentList() const { return list_.data; }
	const svo_fraglist &GetFragmentList() const { return list_; }

private:
	std::shared_ptr<Scene> scene_;
	uint32_t level_ = 0;
	void *stream_ = nullptr;
	svo_fraglist list_{};
	std::unique_ptr<DeviceBuffer> workspace_, count_;
};

class OctreeBuilder {
public:
	// Allocates the node pool (the exact worst-case bound, so a build never overflows) and scratch.
	static std::shared_ptr<OctreeBuilder> Create(const std::shared_ptr<Voxelizer> &voxelizer, void *stream = nullptr) {
		auto b = std::make_shared<OctreeBuilder>();
		b->voxelizer_ = voxelizer;
		const uint32_t n = voxelizer->GetVoxelFragmentCount(), level = voxelizer->GetLevel();
		b->capacity_ = svo_build_pool_bound(n, level);
		b->pool_ = std::make_unique<DeviceBuffer>(b->capacity_ * sizeof(uint32_t), stream);
		b->workspace_ = std::make_unique<DeviceBuffer>(svo_build_workspace_size(n, level, b->capacity_, 0), stream);
		b->result_ = std::make_unique<DeviceBuffer>(sizeof(svo_build_info) + 16, stream);
		return b;
	}

	void CmdBuild(void *stream = nullptr) {
		have_info_ = false;
		Check(svo_build_into(voxelizer_->GetVoxelFragmentList(), voxelizer_->GetVoxelFragmentCount(),
		                     voxelizer_->GetLevel(), (uint32_t *)pool_->get(), capacity_, workspace_->get(),
		                     workspace_->size(), result_->get(), stream));
		stream_ = stream;
	}

	// Shrinks the node pool to the exact range of the last build (blocking); later CmdBuild calls on the
	// same fragments fit it exactly.
	void Reserve(void *stream = nullptr) {
		const uint64_t range = GetInfo().range_words;
		const uint32_t n = voxelizer_->GetVoxelFragmentCount(), level = voxelizer_->GetLevel();
		capacity_ = range;
		pool_ = std::make_unique<DeviceBuffer>(capacity_ * sizeof(uint32_t), stream);
		workspace_ = std::make_unique<DeviceBuffer>(svo_build_workspace_size(n, level, capacity_, 0), stream);
		have_info_ = false;
	}

	// Counters of the last build (blocking read, like Counter::Read, src/Counter.cpp:23-34).
	const svo_build_info &GetInfo() {
		if (!have_info_) {
			unsigned char buf[sizeof(svo_build_info) + 4];
			Check(svo_download(buf, result_->get(), sizeof(buf), 1, stream_));
			uint32_t status;
			std::memcpy(&info_, buf, sizeof(info_));
			std::memcpy(&status, buf + sizeof(info_), 4);
			if (status) throw Error(SVO_ERR_CAPACITY, "octree build did not complete (pool or workspace too small)");
			have_info_ = true;
		}
		return info_;
	}
	uint64_t GetOctreeRange() { return (uint64_t)GetInfo().range_words * 4u; } // bytes, as the reference
	uint32_t *GetOctree() const { return (uint32_t *)pool_->get(); }
	uint64_t GetCapacityWords() const { return capacity_; }
	uint32_t GetLevel() const { return voxelizer_->GetLevel(); }
	const std::shared_ptr<Voxelizer> &GetVoxelizerPtr() const { return voxelizer_; }

private:
	std::shared_ptr<Voxelizer> voxelizer_;
	std::unique_ptr<DeviceBuffer> pool_, workspace_, result_;
	uint64_t capacity_ = 0;
	void *stream_ = nullptr;
	svo_build_info info_{};
	bool have_info_ = false;
};

class Octree {
public:
	Octree() = default;
	Octree(const Octree &) = delete;
	Octree &operator=(const Octree &) = delete;
	~Octree() {
		if (owned_) svo_octree_destroy(&octree_, nullptr);
	}
	static std::shared_ptr<Octree> Create() { return std::make_shared<Octree>(); }
	// An octree file (svo_octree_load); the pool is owned and released with the object.
	static std::shared_ptr<Octree> Load(const std::string &path, void *stream = nullptr) {
		auto o = std::make_shared<Octree>();
		Check(svo_octree_load(path.c_str(), &o->octree_, stream));
		o->owned_ = true;
		return o;
	}
	// A view of a pool owned elsewhere (a batcher's or a server's); `keep` keeps its owner alive.
	static std::shared_ptr<Octree> FromView(const svo_octree &view, std::shared_ptr<void> keep = nullptr) {
		auto o = std::make_shared<Octree>();
		o->octree_ = view;
		o->octree_.owned = 0;
		o->keep_ = std::move(keep);
		return o;
	}
	void Save(const std::string &path, void *stream = nullptr) const { Check(svo_octree_save(&octree_, path.c_str(), stream)); }
	void Update(const std::shared_ptr<OctreeBuilder> &builder) {
		if (owned_) svo_octree_destroy(&octree_, nullptr);
		owned_ = false;
		const uint64_t range = builder->GetOctreeRange();
		builder_ = builder;
		octree_.words = builder->GetOctree();
		octree_.capacity = builder->GetCapacityWords();
		octree_.range_words = (uint32_t)(range / 4u);
		octree_.level = builder->GetLevel();
		octree_.owned = 0;
	}
	bool Empty() const { return octree_.words == nullptr; }
	uint32_t *GetBuffer() const { return octree_.words; }
	uint32_t GetLevel() const { return octree_.level; }
	uint64_t GetRange() const { return (uint64_t)octree_.range_words * 4u; }
	const svo_octree &Get() const { return octree_; }

private:
	std::shared_ptr<OctreeBuilder> builder_;
	std::shared_ptr<void> keep_;
	svo_octree octree_{};
	bool owned_ = false;
};

// The tracer without a swapchain: one hit (svo_hit, 32 B) per pixel in a device buffer.
class OctreeTracer {
public:
	static std::shared_ptr<OctreeTracer> Create(const std::shared_ptr<Octree> &octree, const svo_camera &camera,
	                                            uint32_t width, uint32_t height) {
		auto t = std::make_shared<OctreeTracer>();
		t->octree_ = octree;
		t->camera_ = camera;
		t->width_ = width;
		t->height_ = height;
		return t;
	}
	void Resize(uint32_t width, uint32_t height) { width_ = width, height_ = height; }
	void SetCamera(const svo_camera &camera) { camera_ = camera; }
	void CmdDrawPipeline(svo_hit *hits_device, void *stream = nullptr) const {
		Check(svo_raycast_camera(&octree_->Get(), &camera_, width_, height_, hits_device, nullptr, stream));
	}
	// CmdDrawPipeline and the read-back of the image, overlapped: hits_host (page-locked) receives the hits.
	void CmdDrawPipelineToHost(svo_hit *hits_device, svo_hit *hits_host, void *stream = nullptr) const {
		Check(svo_raycast_camera_download(&octree_->Get(), &camera_, width_, height_, hits_device, hits_host, nullptr,
		                                  stream));
	}
	void CmdTrace(const svo_ray *rays_device, uint32_t n, svo_hit *hits_device, void *stream = nullptr) const {
		Check(svo_raycast(&octree_->Get(), rays_device, n, hits_device, nullptr, stream));
	}
	// OctreeTracer::CmdBeamRenderPass (src/OctreeTracer.cpp:183-211): svo_beam_texels(width, height) floats.
	void CmdBeamRenderPass(float *beam_device, void *stream = nullptr) const {
		Check(svo_beam_prepass(&octree_->Get(), &camera_, width_, height_, beam_device, stream));
	}
	// CmdDrawPipeline with the beam enabled (beam_device NULL: the pre-pass runs inside).
	void CmdDrawPipelineBeam(const float *beam_device, svo_hit *hits_device, void *stream = nullptr) const {
		Check(svo_raycast_camera_beam(&octree_->Get(), &camera_, width_, height_, beam_device, hits_device, nullptr,
		                              stream));
	}
	// Octree_RayMarchOcclude per ray (shadow rays): occluded[i] = 1 when ray i hits a leaf.
	void CmdOcclude(const svo_ray *rays_device, uint32_t n, uint32_t *occluded_device, void *stream = nullptr) const {
		Check(svo_occlude(&octree_->Get(), rays_device, n, occluded_device, stream));
	}
	uint32_t GetWidth() const { return width_; }
	uint32_t GetHeight() const { return height_; }

private:
	std::shared_ptr<Octree> octree_;
	svo_camera camera_{};
	uint32_t width_ = 0, height_ = 0;
};

// EnvironmentMap (src/EnvironmentMap.hpp): decoded float rgba image -> device texels + alias table.
class EnvironmentMap {
public:
	float m_rotation = 0.0f, m_multiplier = 1.0f;
	static std::shared_ptr<EnvironmentMap> Create() { return std::make_shared<EnvironmentMap>(); }
	~EnvironmentMap() { Reset(); }
	void Reset() {
		if (map_) svo_envmap_destroy(map_);
		map_ = nullptr;
	}
	void Reset(const float *rgba_host, uint32_t width, uint32_t height) {
		Reset();
		Check(svo_envmap_create(rgba_host, width, height, &map_));
	}
	bool Empty() const { return map_ == nullptr; }
	const svo_envmap *Get() const { return map_; }

private:
	svo_envmap *map_ = nullptr;
};

// Lighting (src/Lighting.hpp:7-20).
class Lighting {
public:
	enum class LightTypes : uint32_t { kConstantColor = 0, kEnvironmentMap = 1 };
	LightTypes m_light_type = LightTypes::kConstantColor;
	float m_sun_radiance[3] = {5.0f, 5.0f, 5.0f}; // kDefaultConstantColor
	static std::shared_ptr<Lighting> Create(const std::shared_ptr<EnvironmentMap> &environment_map) {
		auto l = std::make_shared<Lighting>();
		l->env_ = environment_map;
		return l;
	}
	const std::shared_ptr<EnvironmentMap> &GetEnvironmentMapPtr() const { return env_; }
	LightTypes GetFinalLightType() const {
		return (m_light_type == LightTypes::kEnvironmentMap && (!env_ || env_->Empty())) ? LightTypes::kConstantColor
		                                                                               : m_light_type;
	}
	svo_lighting Get() const {
		svo_lighting l{};
		l.type = (uint32_t)GetFinalLightType();
		for (int k = 0; k < 3; ++k) l.sun_radiance[k] = m_sun_radiance[k];
		l.envmap_rotation = env_ ? env_->m_rotation : 0.0f;
		l.envmap_multiplier = env_ ? env_->m_multiplier : 1.0f;
		l.envmap = env_ ? env_->Get() : nullptr;
		return l;
	}

private:
	std::shared_ptr<EnvironmentMap> env_;
};

// PathTracer (src/PathTracer.hpp:15-75): progressive path tracing, one fused kernel per sample.
class PathTracer {
public:
	uint32_t m_width = 1280, m_height = 720; // kDefaultWidth, kDefaultHeight
	uint32_t m_bounce = 4;                   // kDefaultBounce
	static std::shared_ptr<PathTracer> Create(const std::shared_ptr<Octree> &octree, const svo_camera &camera,
	                                          const std::shared_ptr<Lighting> &lighting) {
		auto p = std::make_shared<PathTracer>();
		p->octree_ = octree;
		p->camera_ = camera;
		p->lighting_ = lighting;
		return p;
	}
	~PathTracer() {
		if (pt_) svo_path_tracer_destroy(pt_);
	}
	void SetCamera(const svo_camera &camera) { camera_ = camera; }
	// PathTracer::Reset: targets of m_width x m_height cleared, Sobol state cleared.
	void Reset(void *stream = nullptr) {
		if (!pt_)
			Check(svo_path_tracer_create(m_width, m_height, m_bounce, &pt_));
		else
			Check(svo_path_tracer_reset(pt_, m_width, m_height, m_bounce, stream));
	}
	void CmdRender(void *stream = nullptr, uint32_t samples = 1) {
		if (!pt_) Reset(stream);
		const svo_lighting l = lighting_->Get();
		Check(svo_path_tracer_render(pt_, &octree_->Get(), &camera_, &l, samples, stream));
	}
	uint32_t GetSPP() const {
		uint32_t spp = 0;
		if (pt_) Check(svo_path_tracer_info(pt_, &spp, nullptr));
		return spp;
	}
	std::vector<float> ExtractColorImage() const { return extract(0); }
	std::vector<float> ExtractAlbedoImage() const { return extract(1); }
	std::vector<float> ExtractNormalImage() const { return extract(2); }
	svo_path_tracer *Get() const { return pt_; }

private:
	std::vector<float> extract(uint32_t image) const {
		std::vector<float> out((size_t)m_width * m_height * 3);
		if (pt_) Check(svo_path_tracer_extract(pt_, image, out.data(), nullptr));
		return out;
	}
	std::shared_ptr<Octree> octree_;
	std::shared_ptr<Lighting> lighting_;
	svo_camera camera_{};
	svo_path_tracer *pt_ = nullptr;
};

// Scene::load_meshes for the engine's triangle format (svo_load_obj).
inline std::vector<svo_triangle> LoadObj(const std::string &path) {
	svo_triangle *t = nullptr;
	uint32_t n = 0;
	Check(svo_load_obj(path.c_str(), &t, &n));
	std::vector<svo_triangle> out(t, t + n);
	svo_free_host(t);
	return out;
}

// Many meshes voxelized and built together (svo_batcher); per mesh identical to Voxelizer + OctreeBuilder.
class BatchBuilder {
public:
	static std::shared_ptr<BatchBuilder> Create() {
		auto b = std::make_shared<BatchBuilder>();
		Check(svo_batcher_create(&b->h_));
		return b;
	}
	BatchBuilder() = default;
	BatchBuilder(const BatchBuilder &) = delete;
	BatchBuilder &operator=(const BatchBuilder &) = delete;
	~BatchBuilder() { svo_batcher_destroy(h_); }
	// meshes: device triangles and levels; blocks for the count and result readbacks.
	void Build(const std::vector<svo_batch_mesh> &meshes, void *stream = nullptr) {
		Check(svo_batcher_build(h_, meshes.data(), (uint32_t)meshes.size(), stream));
	}
	uint32_t GetMeshCount() const { return svo_batcher_meshes(h_); }
	// View of mesh i's octree in the shared pool, valid until the next Build (holds the batcher alive).
	static std::shared_ptr<Octree> GetOctree(const std::shared_ptr<BatchBuilder> &self, uint32_t i) {
		svo_octree o;
		Check(svo_batcher_result(self->h_, i, nullptr, &o, nullptr));
		return Octree::FromView(o, self);
	}
	svo_build_info GetInfo(uint32_t i) const {
		svo_build_info info;
		Check(svo_batcher_result(h_, i, nullptr, nullptr, &info));
		return info;
	}

private:
	svo_batcher *h_ = nullptr;
};

// Resident octrees and continuous batching of trace / rebuild requests (svo_server).
class Server {
public:
	static std::shared_ptr<Server> Create(const svo_server_config &cfg = svo_server_config{}) {
		auto s = std::make_shared<Server>();
		Check(svo_server_create(&cfg, &s->h_));
		return s;
	}
	Server() = default;
	Server(const Server &) = delete;
	Server &operator=(const Server &) = delete;
	~Server() { svo_server_destroy(h_); }
	uint32_t BuildScene(const svo_triangle *tris_device, uint32_t n, uint32_t level) {
		uint32_t id;
		Check(svo_server_build_scene(h_, tris_device, n, level, &id));
		return id;
	}
	uint32_t AddOctree(const std::shared_ptr<Octree> &octree) {
		uint32_t id;
		Check(svo_server_add_octree(h_, &octree->Get(), &id));
		return id;
	}
	// Camera request: hits_host (page-locked for full overlap) receives 2 * n_primary hits.
	uint64_t SubmitCamera(uint32_t scene, const svo_camera &cam, uint32_t width, uint32_t height, uint32_t n_primary,
	                      uint64_t seed, svo_hit *hits_host) {
		svo_trace_request r{};
		r.scene = scene, r.mode = SVO_REQUEST_CAMERA, r.camera = cam;
		r.width = width, r.height = height, r.n_primary = n_primary, r.hits = hits_host, r.seed = seed;
		uint64_t t;
		Check(svo_server_submit_trace(h_, &r, &t));
		return t;
	}
	uint64_t SubmitRays(uint32_t scene, const svo_ray *rays_host, uint32_t n, svo_hit *hits_host) {
		svo_trace_request r{};
		r.scene = scene, r.mode = SVO_REQUEST_RAYS, r.rays = rays_host, r.n_rays = n, r.hits = hits_host;
		uint64_t t;
		Check(svo_server_submit_trace(h_, &r, &t));
		return t;
	}
	uint64_t SubmitRebuild(uint32_t scene, const svo_triangle *tris_device, uint32_t n, uint32_t level) {
		uint64_t t;
		Check(svo_server_submit_rebuild(h_, scene, tris_device, n, level, &t));
		return t;
	}
	svo_request_result Wait(uint64_t ticket, int timeout_ms = -1) {
		svo_request_result r{};
		Check(svo_server_wait(h_, ticket, timeout_ms, &r));
		return r;
	}
	svo_server_stats Stats() const {
		svo_server_stats st{};
		svo_server_get_stats(h_, &st);
		return st;
	}

private:
	svo_server *h_ = nullptr;
};

} // namespace svo
