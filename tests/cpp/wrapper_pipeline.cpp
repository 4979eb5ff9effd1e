// Drives the C++ host classes (include/svo.hpp) through the whole path the way the reference's loader
// thread and tracer do (src/LoaderThread.cpp:52-75, src/Application.cpp:144-152):
//   Scene -> Voxelizer -> OctreeBuilder -> CmdBuild -> Octree::Update -> OctreeTracer::CmdDrawPipeline
// Usage: wrapper_pipeline <triangles.bin> <level> <camera.bin (16 floats)> <width> <height> <out prefix>
// Writes <out>.frags (uint64), <out>.pool (uint32, range words), <out>.hits (svo_hit) and <out>.beam
// (float beam image) and <out>.pt (2 path-traced samples, rgb floats), and checks in-process that a
// two-mesh BatchBuilder, a Server camera request and an octree file round trip agree with the
// single-mesh classes.
#include <cstdio>
#include <fstream>
#include <iterator>
#include <vector>

#include "svo.hpp"

template <typename T> static std::vector<T> read_file(const char *path) {
	std::ifstream f(path, std::ios::binary);
	std::vector<char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
	std::vector<T> out(bytes.size() / sizeof(T));
	std::memcpy(out.data(), bytes.data(), out.size() * sizeof(T));
	return out;
}

template <typename T> static void write_file(const std::string &path, const std::vector<T> &v) {
	std::ofstream f(path, std::ios::binary);
	f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

int main(int argc, char **argv) {
	if (argc != 7) {
		std::fprintf(stderr, "usage: %s tris level camera width height out\n", argv[0]);
		return 2;
	}
	try {
		const auto tris = read_file<svo_triangle>(argv[1]);
		const uint32_t level = (uint32_t)std::atoi(argv[2]);
		const auto camf = read_file<float>(argv[3]);
		svo_camera cam;
		std::memcpy(&cam, camf.data(), sizeof(cam));
		const uint32_t width = (uint32_t)std::atoi(argv[4]), height = (uint32_t)std::atoi(argv[5]);
		const std::string out = argv[6];

		auto scene = svo::Scene::Create(tris);
		auto voxelizer = svo::Voxelizer::Create(scene, level);
		auto builder = svo::OctreeBuilder::Create(voxelizer);
		builder->CmdBuild();
		auto octree = svo::Octree::Create();
		octree->Update(builder);
		voxelizer->CmdVoxelize(); // record both passes again: same results
		voxelizer->CheckEmission();
		builder->Reserve(); // pool shrunk to the exact range: the re-recorded build fits it
		builder->CmdBuild();
		octree->Update(builder);
		auto tracer = svo::OctreeTracer::Create(octree, cam, width, height);
		svo::DeviceBuffer hits(sizeof(svo_hit) * width * height, nullptr);
		tracer->CmdDrawPipeline((svo_hit *)hits.get());
		// the same frame read back into (pageable) host memory while it is traced
		svo::DeviceBuffer hits2(sizeof(svo_hit) * width * height, nullptr);
		std::vector<svo_hit> to_host(width * height);
		tracer->CmdDrawPipelineToHost((svo_hit *)hits2.get(), to_host.data());

		std::vector<uint64_t> frags(voxelizer->GetVoxelFragmentCount());
		svo::Check(svo_download(frags.data(), voxelizer->GetVoxelFragmentList(), frags.size() * 8, 0, nullptr));
		std::vector<uint32_t> pool(octree->GetRange() / 4);
		svo::Check(svo_download(pool.data(), octree->GetBuffer(), octree->GetRange(), 0, nullptr));
		std::vector<svo_hit> h(width * height);
		svo::Check(svo_download(h.data(), hits.get(), h.size() * sizeof(svo_hit), 1, nullptr));
		if (std::memcmp(h.data(), to_host.data(), h.size() * sizeof(svo_hit)) != 0) {
			std::fprintf(stderr, "CmdDrawPipelineToHost differs from CmdDrawPipeline + download\n");
			return 4;
		}
		write_file(out + ".frags", frags);
		write_file(out + ".pool", pool);
		write_file(out + ".hits", h);

		// beam pre-pass (the reference tracer's beam image)
		svo::DeviceBuffer beam(sizeof(float) * svo_beam_texels(width, height), nullptr);
		tracer->CmdBeamRenderPass((float *)beam.get());
		std::vector<float> bimg(svo_beam_texels(width, height));
		svo::Check(svo_download(bimg.data(), beam.get(), bimg.size() * 4, 1, nullptr));
		write_file(out + ".beam", bimg);

		// a two-mesh batch equals the single builds
		auto batch = svo::BatchBuilder::Create();
		batch->Build({{scene->GetTriangles(), scene->GetTriangleCount(), level},
		              {scene->GetTriangles(), scene->GetTriangleCount(), level - 1}});
		auto b0 = svo::BatchBuilder::GetOctree(batch, 0);
		std::vector<uint32_t> bpool(b0->GetRange() / 4);
		svo::Check(svo_download(bpool.data(), b0->GetBuffer(), b0->GetRange(), 1, nullptr));
		if (bpool != pool) {
			std::fprintf(stderr, "batch octree differs from the single build\n");
			return 3;
		}
		auto v1 = svo::Voxelizer::Create(scene, level - 1);
		auto ob1 = svo::OctreeBuilder::Create(v1);
		ob1->CmdBuild();
		if (ob1->GetOctreeRange() != svo::BatchBuilder::GetOctree(batch, 1)->GetRange()) {
			std::fprintf(stderr, "batch range differs from the single build\n");
			return 3;
		}

		// a served camera request equals the tracer's frame (primary hits)
		{
			auto server = svo::Server::Create();
			const uint32_t sid = server->AddOctree(octree);
			std::vector<svo_hit> sh(2 * (size_t)width * height);
			const uint64_t t = server->SubmitCamera(sid, cam, width, height, width * height, 7, sh.data());
			server->Wait(t);
			if (std::memcmp(sh.data(), h.data(), h.size() * sizeof(svo_hit)) != 0) {
				std::fprintf(stderr, "served hits differ from the tracer's\n");
				return 4;
			}
		}

		// path tracer (PathTracer::Reset + CmdRender x2, constant light, 3 path vertices), noise byte i = 37 i
		{
			auto env = svo::EnvironmentMap::Create();
			auto lighting = svo::Lighting::Create(env);
			lighting->m_sun_radiance[0] = 1.0f, lighting->m_sun_radiance[1] = 2.0f, lighting->m_sun_radiance[2] = 3.0f;
			auto pt = svo::PathTracer::Create(octree, cam, lighting);
			pt->m_width = width, pt->m_height = height, pt->m_bounce = 3;
			pt->Reset();
			std::vector<uint8_t> noise(256 * 256 * 2);
			for (size_t i = 0; i < noise.size(); ++i) noise[i] = (uint8_t)(i * 37u);
			svo::Check(svo_path_tracer_set_noise(pt->Get(), noise.data(), nullptr));
			pt->CmdRender(nullptr, 2);
			if (pt->GetSPP() != 2) {
				std::fprintf(stderr, "path tracer sample count\n");
				return 6;
			}
			write_file(out + ".pt", pt->ExtractColorImage());
		}

		// octree file round trip
		octree->Save(out + ".svo");
		auto loaded = svo::Octree::Load(out + ".svo");
		std::vector<uint32_t> lpool(loaded->GetRange() / 4);
		svo::Check(svo_download(lpool.data(), loaded->GetBuffer(), loaded->GetRange(), 1, nullptr));
		if (lpool != pool || loaded->GetLevel() != level) {
			std::fprintf(stderr, "loaded octree differs\n");
			return 5;
		}
		std::printf("fragments %u range %llu words levels", voxelizer->GetVoxelFragmentCount(),
		            (unsigned long long)pool.size());
		const svo_build_info &info = builder->GetInfo();
		for (uint32_t d = 0; d < level; ++d) std::printf(" %u", info.level_nodes[d]);
		std::printf("\n");
	} catch (const svo::Error &e) {
		std::fprintf(stderr, "%s\n", e.what());
		return 1;
	}
	return 0;
}
