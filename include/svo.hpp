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
	static std::shared_ptr<Octree> Create() { return std::make_shared<Octree>(); }
	void Update(const std::shared_ptr<OctreeBuilder> &builder) {
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
	svo_octree octree_{};
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
	void CmdTrace(const svo_ray *rays_device, uint32_t n, svo_hit *hits_device, void *stream = nullptr) const {
		Check(svo_raycast(&octree_->Get(), rays_device, n, hits_device, nullptr, stream));
	}
	uint32_t GetWidth() const { return width_; }
	uint32_t GetHeight() const { return height_; }

private:
	std::shared_ptr<Octree> octree_;
	svo_camera camera_{};
	uint32_t width_ = 0, height_ = 0;
};

} // namespace svo
