// harness.cpp — drives the reference's own shader code (compiled through glsl_shim.hpp by
// oracle/build_ref.py) the way its host code dispatches it.  TEST INFRASTRUCTURE ONLY.
//
// Invocations run one at a time in invocation order, with subgroups of one invocation — a legal
// Vulkan execution of every shader here.  Under that order the alloc shader hands out child blocks in
// word order and the tag shader's CAS loop folds colours in fragment-list order.
#include "glsl_shim.hpp"

#include <algorithm>
#include <cstdio>
#include <vector>

uint *uOctree;
uvec2 *uFragmentList;
uint uCounter, uAllocBegin, uAllocNum, uNumGroupX, uNumGroupY, uNumGroupZ;
uint kVoxelResolution, kFragmentCount, kTextureNum = 1;
uint uCountOnly, uTextureId, uAlbedo;
vec4 uPosition, uLook, uSide, uUp;
sampler2D uTextures[1];
thread_local uvec3 gl_GlobalInvocationID;
thread_local vec4 gl_FragCoord, gl_Position;
thread_local gl_PerVertex gl_in[3];
thread_local vec2 vTexcoord[3], gTexcoord;
thread_local uint gAxis;
thread_local uvec4 gAABB;
thread_local uvec2 gDepthRange;

uint *uSobol;
uint uDimension;
sampler2D uEnvironmentMap, uNoise;
usampler2D uEnvMapAliasTable;
image2D uColor, uNormal;
uint uBounce, uLightType;
float uConstColor[3], uEnvMapRotation, uEnvMapMultiplier;
namespace ref_pt {
image2D uAlbedo; // path_tracer.comp's albedo target (the voxelizer's uAlbedo is its push constant)
}

static thread_local vec4 g_emitted[3];
static thread_local int g_emit_count;
void EmitVertex() {
	if (g_emit_count < 3) g_emitted[g_emit_count] = gl_Position;
	++g_emit_count;
}
void EndPrimitive() {}

#include "gen_octree_init_node_comp.hpp"
#include "gen_octree_tag_node_comp.hpp"
#include "gen_octree_alloc_node_comp.hpp"
#include "gen_octree_modify_arg_comp.hpp"
#include "gen_octree.hpp"
#include "gen_camera.hpp"
#include "gen_util.hpp"
namespace ref_diffuse {
using namespace ::ref_util;
}
#include "gen_diffuse.hpp"
#include "gen_voxelizer_geom.hpp"
#include "gen_voxelizer_conservative_geom.hpp"
#include "gen_voxelizer_frag.hpp"
#include "gen_sobol.hpp"
#include "gen_mis.hpp"
#include "gen_environment_map.hpp"
#include "gen_sobol_comp.hpp"
namespace ref_pt {
using namespace ::ref_octree;
using namespace ::ref_camera;
using namespace ::ref_util;
using namespace ::ref_diffuse;
using namespace ::ref_mis;
using namespace ::ref_envmap;
using namespace ::ref_sobol;
} // namespace ref_pt
#include "gen_path_tracer_comp.hpp"
#include "gen_envmap_cpp.hpp"

static uint group_x_64(uint x) { return (x >> 6u) + ((x & 0x3fu) ? 1u : 0u); }

template <typename F> static void dispatch(uint groups, F &&shader) {
	for (uint i = 0; i < groups * 64u; ++i) {
		gl_GlobalInvocationID = uvec3(i, 0u, 0u);
		shader();
	}
}

extern "C" {

// OctreeBuilder::CmdBuild (src/OctreeBuilder.cpp:142-210): build info {0, 8}, indirect {1,1,1},
// then per level init -> tag -> (alloc -> modify_arg).  Returns (counter + 1) * 8 words
// (GetOctreeRange, src/OctreeBuilder.cpp:212-214) or 0 if the pool would overflow `capacity`.
uint64_t ref_build(const uint64_t *frags, uint32_t count, uint32_t level, uint32_t *pool, uint64_t capacity) {
	uOctree = pool;
	uFragmentList = (uvec2 *)frags;
	kVoxelResolution = 1u << level;
	kFragmentCount = count;
	uCounter = 0;
	uAllocBegin = 0;
	uAllocNum = 8;
	uNumGroupX = 1, uNumGroupY = 1, uNumGroupZ = 1;
	for (uint i = 1; i <= level; ++i) {
		if ((uint64_t)uAllocBegin + uAllocNum > capacity) return 0;
		dispatch(uNumGroupX, ref_init::init_main);
		dispatch(group_x_64(count), ref_tag::tag_main);
		if (i != level) {
			dispatch(uNumGroupX, ref_alloc::alloc_main);
			ref_modify::modify_main();
		}
	}
	return ((uint64_t)uCounter + 1u) * 8u;
}

// Octree_RayMarchLeaf with the iteration count (shader/octree.glsl:179-340), or the 5-argument
// variant (shader/octree.glsl:342-502) when with_iter == 0.  Per ray: hit, o_pos, o_color, o_normal,
// o_iter.
void ref_raycast(const uint32_t *pool, uint32_t n, const float *o, const float *d, int with_iter, uint32_t *hit,
                 float *pos, float *color, float *normal, uint32_t *iter) {
	uOctree = (uint *)pool;
	for (uint32_t r = 0; r < n; ++r) {
		vec3 vo(o[3 * r], o[3 * r + 1], o[3 * r + 2]), vd(d[3 * r], d[3 * r + 1], d[3 * r + 2]);
		vec3 p, c, nn;
		uint it = 0;
		bool h = with_iter ? ref_octree::Octree_RayMarchLeaf(vo, vd, p, c, nn, it)
		                   : ref_octree::Octree_RayMarchLeaf(vo, vd, p, c, nn);
		hit[r] = h;
		for (int k = 0; k < 3; ++k) {
			pos[3 * r + k] = p[k];
			color[3 * r + k] = c[k];
			normal[3 * r + k] = nn[k];
		}
		iter[r] = it;
	}
}

// Octree_RayMarchOcclude (shader/octree.glsl:504-629).
void ref_occlude(const uint32_t *pool, uint32_t n, const float *o, const float *d, uint32_t *hit) {
	uOctree = (uint *)pool;
	for (uint32_t r = 0; r < n; ++r)
		hit[r] = ref_octree::Octree_RayMarchOcclude(vec3(o[3 * r], o[3 * r + 1], o[3 * r + 2]),
		                                            vec3(d[3 * r], d[3 * r + 1], d[3 * r + 2]));
}

// The beam pre-pass of shader/octree_tracer_beam.frag:12-30 as OctreeTracer::CmdBeamRenderPass runs it
// (src/OctreeTracer.cpp:183-211): one texel per (beam_size x beam_size) pixel tile corner, width / height
// texels (x + beam_size - 1) / beam_size + 1 (src/OctreeTracer.cpp:6), Octree_RayMarchCoarse from the
// shader source; the texel arithmetic of the fragment shader's main() is restated here line for line.
static float ray_tangent(vec3 x, vec3 y) {
	float c = dot(x, y);
	return sqrt(1.0f - c * c) / abs(c);
}

void ref_beam(const uint32_t *pool, const float *cam16, uint32_t width, uint32_t height, uint32_t beam_size,
              float origin_size, float *beam) {
	uOctree = (uint *)pool;
	uPosition = vec4(cam16[0], cam16[1], cam16[2], cam16[3]);
	uLook = vec4(cam16[4], cam16[5], cam16[6], cam16[7]);
	uSide = vec4(cam16[8], cam16[9], cam16[10], cam16[11]);
	uUp = vec4(cam16[12], cam16[13], cam16[14], cam16[15]);
	const uint32_t bw = (width + beam_size - 1) / beam_size + 1, bh = (height + beam_size - 1) / beam_size + 1;
	const vec2 size((float)width, (float)height);
	const float bs = (float)beam_size;
	for (uint32_t by = 0; by < bh; ++by)
		for (uint32_t bx = 0; bx < bw; ++bx) {
			const vec2 fc((float)(int)bx, (float)(int)by);
			auto gen = [&](float ox, float oy) {
				vec2 c = (fc + vec2(ox, oy)) / size;
				c = c * bs;
				return ref_camera::Camera_GenRay(c);
			};
			vec2 c0 = fc / size;
			c0 = c0 * bs;
			vec3 o = vec3(uPosition.x, uPosition.y, uPosition.z), d = ref_camera::Camera_GenRay(c0);
			float t0 = ray_tangent(d, gen(0.5f, 0.5f));
			float t1 = ray_tangent(d, gen(-0.5f, 0.5f));
			float t2 = ray_tangent(d, gen(0.5f, -0.5f));
			float t3 = ray_tangent(d, gen(-0.5f, -0.5f));
			float dir_sz = 2.0f * max(max(t0, t1), max(t2, t3)), t, sz;
			beam[(uint64_t)by * bw + bx] =
			    ref_octree::Octree_RayMarchCoarse(o, d, origin_size, dir_sz, t, sz) ? max(0.0f, t - sz) : 1e10f;
		}
}

// shader/octree_tracer.frag:24: d = Camera_GenRay(ivec2(gl_FragCoord.xy) / vec2(uWidth, uHeight)).
void ref_camera_rays(const float *cam16, uint32_t width, uint32_t height, float *dirs) {
	uPosition = vec4(cam16[0], cam16[1], cam16[2], cam16[3]);
	uLook = vec4(cam16[4], cam16[5], cam16[6], cam16[7]);
	uSide = vec4(cam16[8], cam16[9], cam16[10], cam16[11]);
	uUp = vec4(cam16[12], cam16[13], cam16[14], cam16[15]);
	for (uint32_t y = 0; y < height; ++y)
		for (uint32_t x = 0; x < width; ++x) {
			vec2 coord = vec2((float)(int)x, (float)(int)y) / vec2((float)width, (float)height);
			vec3 dd = ref_camera::Camera_GenRay(coord);
			uint64_t i = (uint64_t)y * width + x;
			dirs[3 * i] = dd.x, dirs[3 * i + 1] = dd.y, dirs[3 * i + 2] = dd.z;
		}
}

// Diffuse_Sample (shader/diffuse.glsl:7-14) for a normal and a sample pair.
void ref_diffuse_sample(const float *normal, float u1, float u2, float *dir) {
	float pdf;
	vec3 dd = ref_diffuse::Diffuse_Sample(vec3(normal[0], normal[1], normal[2]), vec2(u1, u2), pdf);
	dir[0] = dd.x, dir[1] = dd.y, dir[2] = dd.z;
}

// Voxelizer (src/Voxelizer.cpp): vertex (pass-through), geometry and fragment shaders of the
// reference for one triangle given in the reference's [-1,1] space.  The fixed-function raster in
// between is the harness's:
//   conservative_sw = 0: voxelizer.geom, then every pixel whose closed square meets the projected
//                        triangle (overestimating conservative raster, evaluated in double);
//   conservative_sw = 1: voxelizer_conservative.geom (half-pixel dilation), then every pixel whose
//                        centre lies in the emitted triangle (closed test, double).
// Depth at the pixel centre is interpolated from the emitted vertices in double and rounded to float.
// Fragments are appended to out (uint64: x | y << 32).  Returns the number written.
static const float *g_texel = nullptr; // a 1x1 texture for the textured form (null: untextured)

uint64_t ref_voxelize_triangle(const float *v9, uint32_t albedo, uint32_t level, int conservative_sw, uint64_t *out,
                               uint64_t cap) {
	const uint32_t R = 1u << level;
	kVoxelResolution = R;
	for (int k = 0; k < 3; ++k) gl_in[k].gl_Position = vec4(v9[3 * k], v9[3 * k + 1], v9[3 * k + 2], 1.0f);
	g_emit_count = 0;
	if (conservative_sw)
		ref_vgeom_cons::geom_main();
	else
		ref_vgeom::geom_main();
	if (g_emit_count != 3) return 0;
	double X[3], Y[3], Z[3];
	for (int k = 0; k < 3; ++k) {
		X[k] = ((double)g_emitted[k].x + 1.0) * 0.5 * R;
		Y[k] = ((double)g_emitted[k].y + 1.0) * 0.5 * R;
		Z[k] = g_emitted[k].z;
	}
	double area = (X[1] - X[0]) * (Y[2] - Y[0]) - (Y[1] - Y[0]) * (X[2] - X[0]);
	if (area == 0.0) return 0;
	double sgn = area > 0 ? 1.0 : -1.0;
	int x0 = (int)std::floor(std::min({X[0], X[1], X[2]})) - 1, x1 = (int)std::floor(std::max({X[0], X[1], X[2]})) + 1;
	int y0 = (int)std::floor(std::min({Y[0], Y[1], Y[2]})) - 1, y1 = (int)std::floor(std::max({Y[0], Y[1], Y[2]})) + 1;
	x0 = std::max(x0, 0), y0 = std::max(y0, 0), x1 = std::min(x1, (int)R - 1), y1 = std::min(y1, (int)R - 1);
	uFragmentList = nullptr;
	uCountOnly = 1;
	uTextureId = g_texel ? 0u : 0xffffffffu;
	uTextures[0] = sampler2D{g_texel, 1, 1};
	uAlbedo = albedo;
	uint64_t n = 0;
	for (int py = y0; py <= y1; ++py)
		for (int px = x0; px <= x1; ++px) {
			bool inside = true;
			for (int k = 0; k < 3 && inside; ++k) {
				int q = (k + 1) % 3;
				double ea = -(Y[q] - Y[k]) * sgn, eb = (X[q] - X[k]) * sgn;
				double cx = px + 0.5, cy = py + 0.5;
				if (!conservative_sw) { // maximum of the edge function over the pixel square
					cx += ea > 0 ? 0.5 : -0.5;
					cy += eb > 0 ? 0.5 : -0.5;
				}
				inside = ea * (cx - X[k]) + eb * (cy - Y[k]) >= 0.0;
			}
			if (!inside) continue;
			double cx = px + 0.5, cy = py + 0.5;
			double l0 = ((X[1] - cx) * (Y[2] - cy) - (Y[1] - cy) * (X[2] - cx)) / area;
			double l1 = ((X[2] - cx) * (Y[0] - cy) - (Y[2] - cy) * (X[0] - cx)) / area;
			double z = l0 * Z[0] + l1 * Z[1] + (1.0 - l0 - l1) * Z[2];
			gl_FragCoord = vec4((float)cx, (float)cy, (float)z, 1.0f);
			uint before = uCounter;
			uvec2 frag;
			uFragmentList = &frag;
			uCounter = 0;
			try {
				ref_vfrag::frag_main();
			} catch (const glsl_discard &) {
				uCounter = before;
				continue;
			}
			// frag_main wrote nothing in count-only mode; run it again in write mode into `frag`
			uCountOnly = 0;
			uCounter = 0;
			ref_vfrag::frag_main();
			uCountOnly = 1;
			uCounter = before;
			if (n < cap) out[n] = (uint64_t)frag.x | ((uint64_t)frag.y << 32);
			++n;
		}
	return n;
}

// voxelizer.frag with uTextureId = 0 bound to a 1x1 texture of linear rgba `texel` (the value every
// filtered sample of it has, whatever the coordinate and level of detail): Sample()'s alpha discard and
// packUnorm4x8 colour, on the same raster as ref_voxelize_triangle.
uint64_t ref_voxelize_triangle_texel(const float *v9, const float *texel, uint32_t level, int conservative_sw,
                                     uint64_t *out, uint64_t cap) {
	g_texel = texel;
	uint64_t n = 0;
	try {
		n = ref_voxelize_triangle(v9, 0u, level, conservative_sw, out, cap);
	} catch (...) {
		g_texel = nullptr;
		throw;
	}
	g_texel = nullptr;
	return n;
}

// ------------------------------------------------------------------------------------------ path tracer
// The direction numbers of shader/sobol.comp (kMatrices, 64 x 32), as the shader source defines them.
static uint g_ref_matrices[64][32];
static bool g_ref_matrices_saved = false;
static void save_ref_matrices() {
	if (!g_ref_matrices_saved) std::memcpy(g_ref_matrices, ref_sobolc::kMatrices, sizeof(g_ref_matrices));
	g_ref_matrices_saved = true;
}
void ref_sobol_matrices(uint32_t *out) {
	save_ref_matrices();
	std::memcpy(out, g_ref_matrices, sizeof(g_ref_matrices));
}
// Runs shader/sobol.comp with other direction numbers (null: the shader's own).
static void use_matrices(const uint32_t *m) {
	save_ref_matrices();
	std::memcpy(ref_sobolc::kMatrices, m ? (const void *)m : (const void *)g_ref_matrices, sizeof(g_ref_matrices));
}

// Sobol::CmdNext (src/Sobol.cpp:46-52): one group of 64 invocations of shader/sobol.comp.
void ref_sobol_next(uint32_t *sobol, uint32_t dim) {
	use_matrices(nullptr);
	uSobol = sobol;
	uDimension = dim;
	for (uint i = 0; i < 64u; ++i) {
		gl_GlobalInvocationID = uvec3(i, 0u, 0u);
		ref_sobolc::sobol_main();
	}
}

// EnvironmentMap::weigh_hdr_image + generate_alias_table on an rgba float image (alpha overwritten with
// the weights).  Returns 0 when the weight sum is not positive (the reference would divide by it).
int ref_envmap_build(float *rgba, uint32_t w, uint32_t h, uint32_t *alias) {
	EnvironmentMap::HdrImg img{w, h, rgba};
	std::vector<double> weights = EnvironmentMap::weigh_hdr_image(&img);
	double sum = 0.0;
	for (double x : weights) sum += x;
	if (!(sum > 0.0)) return 0;
	EnvironmentMap::generate_alias_table(&weights, (EnvironmentMap::AliasPair *)alias);
	return 1;
}

// PathTracer::CmdRender (src/PathTracer.cpp:205-227), `samples` times: shader/path_tracer.comp over
// group_8(width) x group_8(height) groups of 8 x 8, then Sobol::CmdNext over (bounce + 1) * 2 dimensions
// (PathTracer::Reset, src/PathTracer.cpp:201), with the shader's direction numbers or `matrices` (64 x 32)
// when given.  noise: 256 x 256 RG8 as the R8G8_UNORM texture reads it.
void ref_path_trace(const uint32_t *pool, const float *cam16, uint32_t width, uint32_t height, uint32_t bounce,
                    uint32_t light_type, const float *const_color, float rot, float mult, const float *env_texels,
                    const uint32_t *env_alias, uint32_t env_w, uint32_t env_h, uint32_t *sobol, const uint8_t *noise,
                    float *color, uint32_t *albedo, uint32_t *normal, uint32_t samples, const uint32_t *matrices) {
	uOctree = (uint *)pool;
	uPosition = vec4(cam16[0], cam16[1], cam16[2], cam16[3]);
	uLook = vec4(cam16[4], cam16[5], cam16[6], cam16[7]);
	uSide = vec4(cam16[8], cam16[9], cam16[10], cam16[11]);
	uUp = vec4(cam16[12], cam16[13], cam16[14], cam16[15]);
	uBounce = bounce;
	uLightType = light_type;
	for (int k = 0; k < 3; ++k) uConstColor[k] = const_color[k];
	uEnvMapRotation = rot;
	uEnvMapMultiplier = mult;
	uEnvironmentMap = sampler2D{env_texels, (int)env_w, (int)env_h};
	uEnvMapAliasTable = usampler2D{env_alias, (int)env_w, (int)env_h};
	std::vector<float> nz(256 * 256 * 4);
	for (int i = 0; i < 256 * 256; ++i) {
		nz[4 * i] = (float)noise[2 * i] / 255.0f;
		nz[4 * i + 1] = (float)noise[2 * i + 1] / 255.0f;
		nz[4 * i + 2] = 0.0f;
		nz[4 * i + 3] = 1.0f;
	}
	uNoise = sampler2D{nz.data(), 256, 256};
	uColor = image2D{color, (int)width, (int)height, 0};
	ref_pt::uAlbedo = image2D{albedo, (int)width, (int)height, 1};
	uNormal = image2D{normal, (int)width, (int)height, 2};
	uSobol = sobol;
	const uint gx = (width + 7u) / 8u * 8u, gy = (height + 7u) / 8u * 8u;
	for (uint32_t s = 0; s < samples; ++s) {
		uSobol = sobol;
		for (uint y = 0; y < gy; ++y)
			for (uint x = 0; x < gx; ++x) {
				gl_GlobalInvocationID = uvec3(x, y, 0u);
				ref_pt::pt_main();
			}
		use_matrices(matrices);
		uDimension = (bounce + 1u) * 2u;
		for (uint i = 0; i < 64u; ++i) {
			gl_GlobalInvocationID = uvec3(i, 0u, 0u);
			ref_sobolc::sobol_main();
		}
	}
	use_matrices(nullptr);
}

} // extern "C"
