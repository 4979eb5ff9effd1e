// pt.cu — host side of the path tracer (PathTracer, src/PathTracer.{hpp,cpp}): the environment-map
// tables (EnvironmentMap::weigh_hdr_image / generate_alias_table, src/EnvironmentMap.cpp:81-160), the
// Sobol state and direction numbers (Sobol, src/Sobol.cpp; shader/sobol.comp), the accumulation targets
// and the C ABI.  The per-pixel paths are march.cu's wavefront kernels (pt_primary_kernel,
// pt_bounce_refill_kernel, pt_accumulate_kernel).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "svo_internal.h"

struct svo_envmap {
	float4 *texels = nullptr; // device: radiance rgb, pdf weight in w
	uint2 *alias = nullptr;   // device: (prob, alias) per texel
	uint32_t width = 0, height = 0;
	std::vector<float> rgba;       // host copy of the texels
	std::vector<uint32_t> table;   // host copy of the alias table
};

struct svo_path_tracer {
	uint32_t width = 0, height = 0, bounce = 0, spp = 0;
	float4 *color = nullptr;
	uint32_t *albedo = nullptr, *normal = nullptr;
	uint32_t *sobol = nullptr;    // kSobolWords: dimension values, then the sample index
	uint32_t *matrices = nullptr; // kSobolDims x 32 direction numbers
	uint8_t *noise = nullptr;     // 256 x 256 x 2
	unsigned long long *scratch = nullptr; // [1]: status word
	svo::PathState *paths = nullptr;       // one per pixel
	uint32_t *queue = nullptr;             // two queues of width x height path indices
	unsigned long long *wave = nullptr;    // per-sample tickets and counts (kPtScratchBytes)
};

namespace svo {

int svo_fail(int code, const char *fmt, ...);

namespace {

constexpr uint32_t kSobolDims = 64;                 // kMaxDimension (src/Sobol.cpp:3)
constexpr uint32_t kSobolWords = kSobolDims + 1;    // (kMaxDimension + 1) words (src/Sobol.cpp:4)
constexpr uint32_t kNoiseSize = 256;                // the noise texture's edge (texelFetch(uNoise, pixel & 0xff))
constexpr uint32_t kMaxBounce = kSobolDims / 2 - 1; // 2 * (bounce + 1) Sobol dimensions
constexpr double kPiD = 3.14159265358979323846;

int cuda_err(cudaError_t e, const char *what) {
	return svo_fail(SVO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}
#define PT_CK(call, what)                                                                                    \
	do {                                                                                                     \
		cudaError_t e_ = (call);                                                                             \
		if (e_ != cudaSuccess) return cuda_err(e_, what);                                                    \
	} while (0)

uint64_t splitmix64(uint64_t &s) {
	uint64_t z = (s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

// Whether poly (degree deg, bit deg and bit 0 set) is primitive over GF(2): x has order 2^deg - 1.
bool primitive(uint32_t poly, uint32_t deg) {
	const uint32_t period = (1u << deg) - 1u;
	uint32_t r = 1;
	for (uint32_t i = 1; i <= period; ++i) {
		r <<= 1;
		if (r >> deg) r ^= poly;
		if (r == 1u) return i == period;
	}
	return false;
}

} // namespace

// Default Sobol direction numbers (kSobolDims x 32, row d = dimension d, entry k = v_{k+1} as a 32-bit
// fraction).  Dimension 0 is van der Corput; dimension d >= 1 uses the d-th primitive polynomial over
// GF(2) in order of degree and coefficients, initial numbers m_1..m_s odd with m_k < 2^k drawn from a
// fixed splitmix64 stream, and the Bratley-Fox recurrence
//   m_k = 2 a_1 m_{k-1} ^ 4 a_2 m_{k-2} ^ ... ^ 2^s m_{k-s} ^ m_{k-s}.
// (The reference's shader/sobol.comp embeds the Joe-Kuo numbers; a caller may load any table with
// svo_path_tracer_set_sobol_matrices.)
void sobol_default_matrices(uint32_t *m32) {
	for (uint32_t k = 0; k < 32; ++k) m32[k] = 0x80000000u >> k;
	uint64_t rng = 0x50B01D1CE5EEDull;
	uint32_t dim = 1;
	for (uint32_t deg = 1; dim < kSobolDims; ++deg)
		for (uint32_t poly = (1u << deg) | 1u; poly < (2u << deg) && dim < kSobolDims; poly += 2)
			if (primitive(poly, deg)) {
				uint64_t m[33];
				for (uint32_t k = 1; k <= deg && k <= 32; ++k) m[k] = (splitmix64(rng) & ((1ull << k) - 1ull)) | 1ull;
				for (uint32_t k = deg + 1; k <= 32; ++k) {
					uint64_t v = m[k - deg] ^ (m[k - deg] << deg);
					for (uint32_t i = 1; i < deg; ++i)
						if ((poly >> (deg - i)) & 1u) v ^= m[k - i] << i;
					m[k] = v;
				}
				for (uint32_t k = 1; k <= 32; ++k) m32[dim * 32 + (k - 1)] = (uint32_t)(m[k] << (32 - k));
				++dim;
			}
}

// EnvironmentMap::weigh_hdr_image (src/EnvironmentMap.cpp:83-104): weight = luminance (float, BT.709
// coefficients) x sin of the row centre's polar angle (double); weights are scaled to average 1 and the
// alpha channel takes each weight as a float.  Returns false for an image of zero total weight.
bool envmap_weigh(float *rgba, uint32_t w, uint32_t h, std::vector<double> &weights) {
	const size_t n = (size_t)w * h;
	weights.resize(n);
	double sum = 0.0;
	for (uint32_t j = 0; j < h; ++j) {
		const double st = std::sin(kPiD * ((double)j + 0.5) / (double)h);
		for (uint32_t i = 0; i < w; ++i) {
			const float *c = rgba + 4 * ((size_t)j * w + i);
			const float lum = 0.2126f * c[0] + 0.7152f * c[1] + 0.0722f * c[2];
			weights[(size_t)j * w + i] = (double)lum * st;
			sum += weights[(size_t)j * w + i];
		}
	}
	if (!(sum > 0.0) || !std::isfinite(sum)) return false;
	const double mul = (double)n / sum;
	for (size_t i = 0; i < n; ++i) {
		weights[i] *= mul;
		rgba[4 * i + 3] = (float)weights[i];
	}
	return true;
}

// EnvironmentMap::generate_alias_table (src/EnvironmentMap.cpp:106-160): texels below weight 1 go on a
// "small" stack, the others on a "large" one; the top small texel takes probability weight x 2^32
// (clamped) and the top large texel as alias, which gives up 1 - weight and moves to the small stack
// once below 1.  Texels left on either stack get (0xffffffff, 0xffffffff).
void envmap_alias(std::vector<double> weights, uint32_t *table) {
	const uint32_t n = (uint32_t)weights.size();
	std::vector<uint32_t> small, large;
	small.reserve(n);
	large.reserve(n);
	for (uint32_t i = 0; i < n; ++i) (weights[i] < 1.0 ? small : large).push_back(i);
	while (!small.empty() && !large.empty()) {
		const uint32_t s = small.back(), l = large.back();
		small.pop_back();
		const double p = weights[s] * 4294967296.0;
		table[2 * s] = (uint32_t)(p < 0.0 ? 0.0 : (p > 4294967295.0 ? 4294967295.0 : p));
		table[2 * s + 1] = l;
		weights[l] -= 1.0 - weights[s];
		if (weights[l] < 1.0) {
			large.pop_back();
			small.push_back(l);
		}
	}
	while (!large.empty()) {
		table[2 * large.back()] = table[2 * large.back() + 1] = 0xffffffffu;
		large.pop_back();
	}
	while (!small.empty()) {
		table[2 * small.back()] = table[2 * small.back() + 1] = 0xffffffffu;
		small.pop_back();
	}
}

} // namespace svo

using namespace svo;

extern "C" {

int svo_sobol_default_matrices(uint32_t *out) {
	if (!out) return svo_fail(SVO_ERR_INVALID, "null argument");
	sobol_default_matrices(out);
	return SVO_OK;
}

int svo_envmap_create(const float *rgba, uint32_t width, uint32_t height, svo_envmap **out) {
	if (!rgba || !out) return svo_fail(SVO_ERR_INVALID, "null argument");
	*out = nullptr;
	if (!width || !height || (uint64_t)width * height > 0xffffffffull / 16)
		return svo_fail(SVO_ERR_INVALID, "environment map size %ux%u", width, height);
	svo_envmap *e = new svo_envmap();
	e->width = width, e->height = height;
	const size_t n = (size_t)width * height;
	e->rgba.assign(rgba, rgba + 4 * n);
	std::vector<double> weights;
	if (!envmap_weigh(e->rgba.data(), width, height, weights)) {
		delete e;
		return svo_fail(SVO_ERR_INVALID, "environment map has no positive luminance");
	}
	e->table.resize(2 * n);
	envmap_alias(weights, e->table.data());
	cudaError_t err = counted_malloc(&e->texels, n * sizeof(float4));
	if (err == cudaSuccess) err = counted_malloc(&e->alias, n * sizeof(uint2));
	if (err == cudaSuccess) err = cudaMemcpy(e->texels, e->rgba.data(), n * sizeof(float4), cudaMemcpyHostToDevice);
	if (err == cudaSuccess) err = cudaMemcpy(e->alias, e->table.data(), n * sizeof(uint2), cudaMemcpyHostToDevice);
	if (err != cudaSuccess) {
		cudaFree(e->texels);
		cudaFree(e->alias);
		delete e;
		return cuda_err(err, "environment map upload");
	}
	*out = e;
	return SVO_OK;
}

int svo_envmap_tables(const svo_envmap *e, float *rgba, uint32_t *alias) {
	if (!e) return svo_fail(SVO_ERR_INVALID, "null environment map");
	if (rgba) std::memcpy(rgba, e->rgba.data(), e->rgba.size() * sizeof(float));
	if (alias) std::memcpy(alias, e->table.data(), e->table.size() * sizeof(uint32_t));
	return SVO_OK;
}

void svo_envmap_destroy(svo_envmap *e) {
	if (!e) return;
	cudaFree(e->texels);
	cudaFree(e->alias);
	delete e;
}

void svo_path_tracer_destroy(svo_path_tracer *pt) {
	if (!pt) return;
	cudaFree(pt->color);
	cudaFree(pt->albedo);
	cudaFree(pt->normal);
	cudaFree(pt->sobol);
	cudaFree(pt->matrices);
	cudaFree(pt->noise);
	cudaFree(pt->scratch);
	cudaFree(pt->paths);
	cudaFree(pt->queue);
	cudaFree(pt->wave);
	delete pt;
}

// PathTracer::Reset (src/PathTracer.cpp:189-203): targets (re)made for the size and cleared to zero,
// Sobol state cleared (Sobol::Reset, src/Sobol.cpp:54-62).
int svo_path_tracer_reset(svo_path_tracer *pt, uint32_t width, uint32_t height, uint32_t bounce, void *stream) {
	if (!pt) return svo_fail(SVO_ERR_INVALID, "null path tracer");
	if (!width || !height || (uint64_t)width * height > (1ull << 31))
		return svo_fail(SVO_ERR_INVALID, "image size %ux%u", width, height);
	if (bounce < 1 || bounce > kMaxBounce) return svo_fail(SVO_ERR_INVALID, "bounce %u outside [1, %u]", bounce, kMaxBounce);
	cudaStream_t s = (cudaStream_t)stream;
	const size_t n = (size_t)width * height;
	if (n != (size_t)pt->width * pt->height || !pt->color) {
		PT_CK(cudaStreamSynchronize(s), "path tracer reset");
		cudaFree(pt->color);
		cudaFree(pt->albedo);
		cudaFree(pt->normal);
		cudaFree(pt->paths);
		cudaFree(pt->queue);
		pt->color = nullptr, pt->albedo = pt->normal = nullptr, pt->paths = nullptr, pt->queue = nullptr;
		PT_CK(counted_malloc(&pt->color, n * sizeof(float4)), "path tracer targets");
		PT_CK(counted_malloc(&pt->albedo, n * sizeof(uint32_t)), "path tracer targets");
		PT_CK(counted_malloc(&pt->normal, n * sizeof(uint32_t)), "path tracer targets");
		PT_CK(counted_malloc(&pt->paths, n * sizeof(PathState)), "path state");
		PT_CK(counted_malloc(&pt->queue, 2 * n * sizeof(uint32_t)), "path queues");
	}
	pt->width = width, pt->height = height, pt->bounce = bounce, pt->spp = 0;
	PT_CK(cudaMemsetAsync(pt->color, 0, n * sizeof(float4), s), "path tracer clear");
	PT_CK(cudaMemsetAsync(pt->albedo, 0, n * sizeof(uint32_t), s), "path tracer clear");
	PT_CK(cudaMemsetAsync(pt->normal, 0, n * sizeof(uint32_t), s), "path tracer clear");
	PT_CK(cudaMemsetAsync(pt->sobol, 0, kSobolWords * sizeof(uint32_t), s), "path tracer clear");
	PT_CK(cudaMemsetAsync(pt->scratch, 0, 2 * sizeof(unsigned long long), s), "path tracer clear");
	return SVO_OK;
}

int svo_path_tracer_create(uint32_t width, uint32_t height, uint32_t bounce, svo_path_tracer **out) {
	if (!out) return svo_fail(SVO_ERR_INVALID, "null argument");
	*out = nullptr;
	if (!width || !height || (uint64_t)width * height > (1ull << 31))
		return svo_fail(SVO_ERR_INVALID, "image size %ux%u", width, height);
	if (bounce < 1 || bounce > kMaxBounce) return svo_fail(SVO_ERR_INVALID, "bounce %u outside [1, %u]", bounce, kMaxBounce);
	svo_path_tracer *pt = new svo_path_tracer();
	std::vector<uint32_t> m(kSobolDims * 32);
	sobol_default_matrices(m.data());
	// default noise: white noise from a fixed splitmix64 stream (the reference ships a blue-noise table,
	// src/Noise.inl, which a caller can load with svo_path_tracer_set_noise)
	std::vector<uint8_t> noise(kNoiseSize * kNoiseSize * 2);
	uint64_t rng = 0xB1E5EED0DDull;
	for (size_t i = 0; i < noise.size(); i += 8) {
		const uint64_t z = splitmix64(rng);
		for (size_t b = 0; b < 8; ++b) noise[i + b] = (uint8_t)(z >> (8 * b));
	}
	cudaError_t e = counted_malloc(&pt->sobol, kSobolWords * sizeof(uint32_t));
	if (e == cudaSuccess) e = counted_malloc(&pt->matrices, m.size() * sizeof(uint32_t));
	if (e == cudaSuccess) e = counted_malloc(&pt->noise, noise.size());
	if (e == cudaSuccess) e = counted_malloc(&pt->scratch, 2 * sizeof(unsigned long long));
	if (e == cudaSuccess) e = counted_malloc(&pt->wave, kPtScratchBytes);
	if (e == cudaSuccess) e = cudaMemcpy(pt->matrices, m.data(), m.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(pt->noise, noise.data(), noise.size(), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) {
		svo_path_tracer_destroy(pt);
		return cuda_err(e, "path tracer allocation");
	}
	int rc = svo_path_tracer_reset(pt, width, height, bounce, nullptr);
	if (rc == SVO_OK) rc = cudaStreamSynchronize(nullptr) == cudaSuccess ? SVO_OK : cuda_err(cudaGetLastError(), "path tracer reset");
	if (rc != SVO_OK) {
		svo_path_tracer_destroy(pt);
		return rc;
	}
	*out = pt;
	return SVO_OK;
}

int svo_path_tracer_set_noise(svo_path_tracer *pt, const uint8_t *rg, void *stream) {
	if (!pt || !rg) return svo_fail(SVO_ERR_INVALID, "null argument");
	PT_CK(cudaMemcpyAsync(pt->noise, rg, kNoiseSize * kNoiseSize * 2, cudaMemcpyDefault, (cudaStream_t)stream),
	      "noise upload");
	return SVO_OK;
}

int svo_path_tracer_set_sobol_matrices(svo_path_tracer *pt, const uint32_t *m, void *stream) {
	if (!pt || !m) return svo_fail(SVO_ERR_INVALID, "null argument");
	PT_CK(cudaMemcpyAsync(pt->matrices, m, kSobolDims * 32 * sizeof(uint32_t), cudaMemcpyDefault, (cudaStream_t)stream),
	      "Sobol matrix upload");
	return SVO_OK;
}

// PathTracer::CmdRender (src/PathTracer.cpp:205-227), `samples` times: one sample per pixel, then the
// Sobol step.  Lighting::GetFinalLightType: an environment-map request without a map renders with the
// constant colour.
int svo_path_tracer_render(svo_path_tracer *pt, const svo_octree *o, const svo_camera *cam, const svo_lighting *l,
                           uint32_t samples, void *stream) {
	if (!pt || !o || !o->words || !cam || !l) return svo_fail(SVO_ERR_INVALID, "null argument");
	if (o->level < SVO_LEVEL_MIN || o->level > SVO_LEVEL_MAX || o->range_words < 8 || o->range_words % 8)
		return svo_fail(SVO_ERR_INVALID, "malformed octree handle");
	if (l->type > 1) return svo_fail(SVO_ERR_INVALID, "light type %u", l->type);
	cudaStream_t s = (cudaStream_t)stream;
	PtArgs a;
	std::memset(&a, 0, sizeof(a));
	a.pool = o->words;
	a.range = o->range_words;
	a.level = o->level;
	a.cam = *cam;
	a.width = pt->width, a.height = pt->height, a.bounce = pt->bounce;
	a.light_type = (l->type == 1 && l->envmap) ? 1u : 0u;
	for (int k = 0; k < 3; ++k) a.const_color[k] = l->sun_radiance[k];
	a.env_rotation = l->envmap_rotation;
	a.env_multiplier = l->envmap_multiplier;
	if (a.light_type == 1) {
		a.env.texels = l->envmap->texels;
		a.env.alias = l->envmap->alias;
		a.env.width = l->envmap->width;
		a.env.height = l->envmap->height;
	}
	a.sobol = pt->sobol;
	a.noise = pt->noise;
	a.color = pt->color, a.albedo = pt->albedo, a.normal = pt->normal;
	a.paths = pt->paths;
	a.queue[0] = pt->queue;
	a.queue[1] = pt->queue + (size_t)pt->width * pt->height;
	a.tickets = pt->wave;
	a.counts = reinterpret_cast<uint32_t *>(pt->wave + kPtMaxVertices);
	a.status = reinterpret_cast<uint32_t *>(pt->scratch + 1);
	for (uint32_t i = 0; i < samples; ++i) {
		PT_CK(pt_render_launch(a, s), "path tracer render");
		PT_CK(sobol_next_launch(pt->sobol, pt->matrices, 2u * (pt->bounce + 1u), s), "Sobol step");
		++pt->spp;
	}
	return SVO_OK;
}

int svo_path_tracer_info(const svo_path_tracer *pt, uint32_t *spp, uint32_t *status) {
	if (!pt) return svo_fail(SVO_ERR_INVALID, "null path tracer");
	if (spp) *spp = pt->spp;
	if (status) {
		PT_CK(cudaMemcpy(status, pt->scratch + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost), "status readback");
	}
	return SVO_OK;
}

int svo_path_tracer_images(const svo_path_tracer *pt, void **color, void **albedo, void **normal, void **sobol) {
	if (!pt) return svo_fail(SVO_ERR_INVALID, "null path tracer");
	if (color) *color = pt->color;
	if (albedo) *albedo = pt->albedo;
	if (normal) *normal = pt->normal;
	if (sobol) *sobol = pt->sobol;
	return SVO_OK;
}

// PathTracer::ExtractColorImage / ExtractAlbedoImage / ExtractNormalImage (src/PathTracer.cpp:229-298):
// width x height x 3 floats; albedo and normal decoded from their 8-bit unorm / snorm words.
int svo_path_tracer_extract(const svo_path_tracer *pt, uint32_t image, float *rgb, void *stream) {
	if (!pt || !rgb) return svo_fail(SVO_ERR_INVALID, "null argument");
	if (image > 2) return svo_fail(SVO_ERR_INVALID, "image %u (0 colour, 1 albedo, 2 normal)", image);
	cudaStream_t s = (cudaStream_t)stream;
	const size_t n = (size_t)pt->width * pt->height;
	if (image == 0) {
		std::vector<float4> c(n);
		PT_CK(cudaMemcpyAsync(c.data(), pt->color, n * sizeof(float4), cudaMemcpyDeviceToHost, s), "extract");
		PT_CK(cudaStreamSynchronize(s), "extract");
		for (size_t i = 0; i < n; ++i) rgb[3 * i] = c[i].x, rgb[3 * i + 1] = c[i].y, rgb[3 * i + 2] = c[i].z;
		return SVO_OK;
	}
	std::vector<uint32_t> w(n);
	PT_CK(cudaMemcpyAsync(w.data(), image == 1 ? pt->albedo : pt->normal, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
	      "extract");
	PT_CK(cudaStreamSynchronize(s), "extract");
	for (size_t i = 0; i < n; ++i)
		for (int k = 0; k < 3; ++k) {
			const uint32_t b = (w[i] >> (8 * k)) & 0xffu;
			rgb[3 * i + k] = image == 1 ? (float)b / 255.0f : std::fmax((float)(int8_t)b / 127.0f, -1.0f);
		}
	return SVO_OK;
}

} // extern "C"
