// texture.cu — texture-sampled fragment colour (shader/voxelizer.frag:27-36): a textured triangle's
// fragment takes packUnorm4x8 of its texture sampled at the pixel centre's interpolated texture
// coordinate, and is discarded when the sampled alpha is below 0.5.
//
// Rule (shared with the oracle, oracle/oracle.c):
//   * textures are RGBA8 with sRGB-encoded colour and linear alpha (VK_FORMAT_R8G8B8A8_SRGB,
//     src/Scene.cpp:262-264), with a full mip chain (Image::QueryMipLevel) made on the host: level l+1
//     texel (i, j) is the bilinear sample, in linear space with clamp-to-edge, of level l at the texel's
//     centre mapped into level l (the linear-filter blit of CmdGenerateMipmap2D), re-encoded to sRGB
//     bytes (round to nearest);
//   * the texture coordinate is the vertex coordinates' barycentric blend at the pixel centre of the
//     dominant-axis projection (exact int64 edge functions on the snapped vertices, float blend);
//   * the level of detail is log2 of the larger screen-space footprint of a pixel (exact partial
//     derivatives of the affine mapping, x and y), the sampler VK_FILTER_LINEAR / REPEAT /
//     MIPMAP_MODE_LINEAR (src/Scene.cpp:409-411): bilinear in level 0 for lod <= 0, else the blend of
//     the two nearest levels;
//   * colour bytes round to nearest after clamping; alpha < 0.5 discards the fragment.
// Untextured triangles (texture id 0xffffffff or beyond the set, as src/Scene.cpp:311-341 remaps
// failed loads) keep their constant colour.  Candidate fragments come from the ordinary voxelizer;
// one look-back compaction keeps the survivors in order.
//
// This translation unit is compiled with -fmad=false and IEEE division / square root, like the march,
// so the float arithmetic is the oracle's operation for operation.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "svo_internal.h"

struct svo_texture_set {
	std::vector<svo::TexDesc> desc;            // per texture
	std::vector<std::vector<uint8_t>> levels;  // per texture: every level's RGBA8 bytes, level 0 first
	svo::TexDesc *desc_dev = nullptr;
	float4 *texels_dev = nullptr;              // linear texels of every level of every texture
	uint32_t count = 0;
};

namespace svo {

int svo_fail(int code, const char *fmt, ...);

namespace {

// ------------------------------------------------------------------------------------------ host
double srgb_decode(double c) { return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4); }
double srgb_encode(double x) { return x <= 0.0031308 ? 12.92 * x : 1.055 * std::pow(x, 1.0 / 2.4) - 0.055; }
uint8_t to_byte(double x) { return (uint8_t)std::floor(std::fmin(std::fmax(x, 0.0), 1.0) * 255.0 + 0.5); }

// Level l+1 from level l (w x h -> max(1, w/2) x max(1, h/2)).
std::vector<uint8_t> next_level(const std::vector<uint8_t> &src, uint32_t w, uint32_t h, uint32_t w2, uint32_t h2) {
	double lin[256];
	for (int c = 0; c < 256; ++c) lin[c] = srgb_decode(c / 255.0);
	std::vector<uint8_t> dst((size_t)w2 * h2 * 4);
	for (uint32_t j = 0; j < h2; ++j)
		for (uint32_t i = 0; i < w2; ++i) {
			const double x = ((double)i + 0.5) * (double)w / (double)w2 - 0.5;
			const double y = ((double)j + 0.5) * (double)h / (double)h2 - 0.5;
			const double fx = std::floor(x), fy = std::floor(y), a = x - fx, b = y - fy;
			const int64_t i0 = (int64_t)fx, j0 = (int64_t)fy;
			auto cl = [](int64_t v, uint32_t n) { return (size_t)(v < 0 ? 0 : (v >= (int64_t)n ? n - 1 : v)); };
			const size_t xs[2] = {cl(i0, w), cl(i0 + 1, w)}, ys[2] = {cl(j0, h), cl(j0 + 1, h)};
			const double wt[4] = {(1 - a) * (1 - b), a * (1 - b), (1 - a) * b, a * b};
			for (int ch = 0; ch < 4; ++ch) {
				double acc = 0.0;
				for (int q = 0; q < 4; ++q) {
					const uint8_t v = src[(ys[q >> 1] * w + xs[q & 1]) * 4 + ch];
					acc += wt[q] * (ch < 3 ? lin[v] : v / 255.0);
				}
				dst[((size_t)j * w2 + i) * 4 + ch] = to_byte(ch < 3 ? srgb_encode(acc) : acc);
			}
		}
	return dst;
}

} // namespace

void texture_mip_chain(const uint8_t *rgba, uint32_t w, uint32_t h, std::vector<std::vector<uint8_t>> &levels) {
	levels.clear();
	levels.emplace_back(rgba, rgba + (size_t)w * h * 4);
	while (w > 1 || h > 1) {
		const uint32_t w2 = w > 1 ? w / 2 : 1, h2 = h > 1 ? h / 2 : 1;
		levels.push_back(next_level(levels.back(), w, h, w2, h2));
		w = w2, h = h2;
	}
}

// ------------------------------------------------------------------------------------------ device
constexpr uint32_t kUntextured = 0xffffffffu;

SVO_DEV int64_t snap_tex(float p, float scale) {
	float q = p > 0.0f ? p : 0.0f;
	q = q < 1.0f ? q : 1.0f;
	return (int64_t)__float2int_rn(q * scale);
}

// log2 for the level of detail: exponent + 2 atanh((m-1)/(m+1)) / ln 2 with m in [sqrt(1/2), sqrt(2)).
SVO_DEV float log2_svo(float x) {
	if (!(x > 0.0f)) return -1e30f;
	uint32_t bits = __float_as_uint(x);
	int e = (int)((bits >> 23) & 255u) - 127;
	float m = __uint_as_float((bits & 0x7fffffu) | 0x3f800000u);
	if (m > 1.41421356237309505f) {
		m = m * 0.5f;
		e += 1;
	}
	const float s = (m - 1.0f) / (m + 1.0f), s2 = s * s;
	float p = 1.0f / 11.0f;
	p = p * s2 + 1.0f / 9.0f;
	p = p * s2 + 1.0f / 7.0f;
	p = p * s2 + 1.0f / 5.0f;
	p = p * s2 + 1.0f / 3.0f;
	p = p * s2 + 1.0f;
	return (float)e + (2.0f * (s * p)) * 1.44269504088896341f;
}

// Bilinear REPEAT sample of level l of texture t.
SVO_DEV float4 tex_bilinear(const TexDesc &t, const float4 *__restrict__ texels, uint32_t l, float u, float v) {
	const int64_t W = max(1u, t.width >> l), H = max(1u, t.height >> l);
	const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
	const float fx = floorf(x), fy = floorf(y);
	const float a = x - fx, b = y - fy;
	// texel indices of coordinates beyond +-4e18 (or NaN) are taken at the bound: defined everywhere
	const int64_t ix = (int64_t)fminf(fmaxf(fx, -4e18f), 4e18f), jy = (int64_t)fminf(fmaxf(fy, -4e18f), 4e18f);
	const int64_t i0 = ((ix % W) + W) % W, j0 = ((jy % H) + H) % H;
	const int64_t i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
	const float4 *L = texels + t.level_off[l];
	const float4 t00 = __ldg(L + j0 * W + i0), t10 = __ldg(L + j0 * W + i1);
	const float4 t01 = __ldg(L + j1 * W + i0), t11 = __ldg(L + j1 * W + i1);
	const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
	float4 r;
	r.x = ((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x;
	r.y = ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y;
	r.z = ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z;
	r.w = ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w;
	return r;
}

SVO_DEV uint32_t unorm8(float v) { return (uint32_t)floorf(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f + 0.5f); }

// The fragment's colour and whether it survives, for candidate fragment `frag` of triangle `tri`.
SVO_DEV bool tex_fragment(uint64_t &frag, const svo_triangle &tri, const svo_triangle_uv &uv, uint32_t level,
                          const TexDesc *__restrict__ desc, const float4 *__restrict__ texels, uint32_t ntex) {
	if (uv.texture == kUntextured || uv.texture >= ntex) return true;
	const float scale = (float)(256 << level);
	int64_t X[3], Y[3], Z[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		X[k] = snap_tex(tri.v[3 * k], scale);
		Y[k] = snap_tex(tri.v[3 * k + 1], scale);
		Z[k] = snap_tex(tri.v[3 * k + 2], scale);
	}
	const int64_t e1x = X[1] - X[0], e1y = Y[1] - Y[0], e1z = Z[1] - Z[0];
	const int64_t e2x = X[2] - X[0], e2y = Y[2] - Y[0], e2z = Z[2] - Z[0];
	const int64_t nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
	const int64_t ax = nx < 0 ? -nx : nx, ay = ny < 0 ? -ny : ny, az = nz < 0 ? -nz : nz;
	const int axis = (ax > ay && ax > az) ? 0 : (ay > az ? 1 : 2);
	int64_t A[3], B[3];
#pragma unroll
	for (int k = 0; k < 3; ++k) {
		A[k] = axis == 0 ? Y[k] : (axis == 1 ? Z[k] : X[k]);
		B[k] = axis == 0 ? Z[k] : (axis == 1 ? X[k] : Y[k]);
	}
	const uint32_t fx = (uint32_t)frag, fy = (uint32_t)(frag >> 32);
	const int64_t vx = fx & 0xfffu, vy = (fx >> 12) & 0xfffu, vz = (fx >> 24) | ((fy >> 28) << 8);
	const int64_t pi = axis == 0 ? vy : (axis == 1 ? vz : vx), pj = axis == 0 ? vz : (axis == 1 ? vx : vy);
	const int64_t px = 256 * pi + 128, py = 256 * pj + 128;
	const int64_t a0 = A[1] - A[0], a1 = B[1] - B[0], b0 = A[2] - A[0], b1 = B[2] - B[0];
	const int64_t area = a0 * b1 - a1 * b0;
	if (area == 0) return true; // not a triangle of the projection (no candidate fragment has one)
	const int64_t q0 = px - A[0], q1 = py - B[0];
	const float fa = (float)area;
	const float l1 = (float)(q0 * b1 - q1 * b0) / fa, l2 = (float)(a0 * q1 - a1 * q0) / fa;
	const float du1 = uv.uv[2] - uv.uv[0], dv1 = uv.uv[3] - uv.uv[1];
	const float du2 = uv.uv[4] - uv.uv[0], dv2 = uv.uv[5] - uv.uv[1];
	const float u = (uv.uv[0] + l1 * du1) + l2 * du2, v = (uv.uv[1] + l1 * dv1) + l2 * dv2;
	// per-pixel partial derivatives of the barycentrics along the projection's two axes
	const float g1i = (float)(256 * b1) / fa, g1j = (float)(-256 * b0) / fa;
	const float g2i = (float)(-256 * a1) / fa, g2j = (float)(256 * a0) / fa;
	const TexDesc t = desc[uv.texture];
	const float W = (float)t.width, H = (float)t.height;
	const float dux = (g1i * du1 + g2i * du2) * W, dvx = (g1i * dv1 + g2i * dv2) * H;
	const float duy = (g1j * du1 + g2j * du2) * W, dvy = (g1j * dv1 + g2j * dv2) * H;
	const float rho = fmaxf(sqrtf(dux * dux + dvx * dvx), sqrtf(duy * duy + dvy * dvy));
	const float lod = log2_svo(rho);
	float4 c;
	if (!(lod > 0.0f)) {
		c = tex_bilinear(t, texels, 0, u, v);
	} else {
		const float d = fminf(lod, (float)(t.levels - 1));
		const uint32_t lo = (uint32_t)floorf(d), hi = min(lo + 1, t.levels - 1);
		const float f = d - (float)lo;
		const float4 c0 = tex_bilinear(t, texels, lo, u, v), c1 = tex_bilinear(t, texels, hi, u, v);
		c.x = (1.0f - f) * c0.x + f * c1.x;
		c.y = (1.0f - f) * c0.y + f * c1.y;
		c.z = (1.0f - f) * c0.z + f * c1.z;
		c.w = (1.0f - f) * c0.w + f * c1.w;
	}
	if (c.w < 0.5f) return false;
	const uint32_t rgb = unorm8(c.x) | (unorm8(c.y) << 8) | (unorm8(c.z) << 16);
	frag = (frag & 0xF0000000FFFFFFFFull) | ((uint64_t)rgb << 32);
	return true;
}

// The triangle of candidate fragment f: small triangles' fragments first (offsets small_off), then the
// units of large triangles (offsets unit_frag, triangle unit_tri).
SVO_DEV uint32_t triangle_of(const VoxWorkspace &w, uint32_t n, uint64_t f) {
	const uint64_t small_total = w.small_off[n];
	if (f < small_total) {
		uint32_t lo = 0, hi = n; // small_off[lo] <= f < small_off[hi]
		while (hi - lo > 1) {
			const uint32_t mid = (lo + hi) >> 1;
			if (w.small_off[mid] <= f) lo = mid; else hi = mid;
		}
		return lo;
	}
	const uint64_t g = f - small_total;
	const uint32_t units = w.unit_off[n];
	uint32_t lo = 0, hi = units;
	while (hi - lo > 1) {
		const uint32_t mid = (lo + hi) >> 1;
		if (w.unit_frag[mid] <= g) lo = mid; else hi = mid;
	}
	return w.unit_tri[lo];
}

constexpr int kTexTPB = 256;
constexpr int kTexIPT = 4;
constexpr uint32_t kTexTile = kTexTPB * kTexIPT;

// Texture sampling + order-preserving compaction of the candidates into `out`; out_count[0] = survivors.
__global__ void __launch_bounds__(kTexTPB) vox_texture_compact(const uint64_t *__restrict__ cand, uint64_t n_cand,
                                                             const svo_triangle *__restrict__ tris,
                                                             const svo_triangle_uv *__restrict__ uvs, uint32_t n_tris,
                                                             uint32_t level, VoxWorkspace w, const TexDesc *desc,
                                                             const float4 *texels, uint32_t ntex, uint64_t *out,
                                                             unsigned long long *out_count, uint32_t *tile_ticket,
                                                             unsigned long long *descs, uint32_t *status) {
	griddep_wait(); // programmatic dependent launch: the predecessor's writes are visible after this
	__shared__ uint32_t s_tile;
	__shared__ uint32_t s_warp[kTexTPB / 32 + 1];
	__shared__ unsigned long long s_prefix;
	if (threadIdx.x == 0) s_tile = atomicAdd(tile_ticket, 1u);
	__syncthreads();
	const uint32_t tile = s_tile;
	const uint64_t ntiles = (n_cand + kTexTile - 1) / kTexTile;
	if (tile >= ntiles) return; // one tile per block: only an uncleared ticket goes past the grid
	const uint64_t base = (uint64_t)tile * kTexTile + threadIdx.x;
	uint64_t frag[kTexIPT];
	uint32_t keep = 0, count = 0;
#pragma unroll
	for (int k = 0; k < kTexIPT; ++k) {
		const uint64_t f = base + (uint64_t)k * kTexTPB;
		if (f < n_cand) {
			frag[k] = cand[f];
			const uint32_t t = triangle_of(w, n_tris, f);
			if (tex_fragment(frag[k], tris[t], uvs[t], level, desc, texels, ntex)) keep |= 1u << k, ++count;
		}
	}
	uint32_t total;
	uint32_t run = block_exclusive_sum<uint32_t, kTexTPB>(count, s_warp, total);
	if (threadIdx.x < 32) {
		const unsigned long long p = tile_lookback_warp(descs, tile, 1u, total, status);
		if (threadIdx.x == 0) s_prefix = p;
	}
	__syncthreads();
	// survivors keep the candidates' order: thread-major inside the tile would break it, so the tile's
	// items are ranked item-major (k, thread) with one block scan per item slot
	const unsigned long long prefix = s_prefix;
	uint32_t before = 0;
#pragma unroll
	for (int k = 0; k < kTexIPT; ++k) {
		const uint32_t mine = (keep >> k) & 1u;
		uint32_t slot_total;
		__syncthreads();
		const uint32_t r = block_exclusive_sum<uint32_t, kTexTPB>(mine, s_warp, slot_total);
		if (mine) out[prefix + before + r] = frag[k];
		before += slot_total;
	}
	(void)run;
	if ((uint64_t)tile == ntiles - 1 && threadIdx.x == 0) out_count[0] = prefix + total;
}

} // namespace svo

namespace svo {

cudaError_t vox_texture_launch(const uint64_t *cand, uint64_t n_cand, const svo_triangle *tris,
                               const svo_triangle_uv *uvs, uint32_t n_tris, uint32_t level, const VoxWorkspace &w,
                               const svo_texture_set *set, uint64_t *out, unsigned long long *scratch,
                               cudaStream_t stream) {
	// scratch: [0] survivors, [1] tile ticket + status, [2..] look-back descriptors
	const uint64_t ntiles = (n_cand + kTexTile - 1) / kTexTile;
	cudaError_t e = cudaMemsetAsync(scratch, 0, (2 + ntiles) * sizeof(unsigned long long), stream);
	if (e != cudaSuccess || n_cand == 0) return e;
	uint32_t *ticket = reinterpret_cast<uint32_t *>(scratch + 1);
	SVO_LAUNCH("vox_texture", stream,
	           ::svo::launch_k(vox_texture_compact, (uint32_t)ntiles, kTexTPB, 0, stream, cand, n_cand, tris, uvs, n_tris, level, w, set ? set->desc_dev : nullptr,
	               set ? set->texels_dev : nullptr, set ? set->count : 0u, out, scratch, ticket, scratch + 2,
	               ticket + 1););
	return cudaGetLastError();
}

size_t vox_texture_scratch_bytes(uint64_t n_cand) { return (2 + (n_cand + kTexTile - 1) / kTexTile) * 8; }

cudaError_t texture_set_wait_fault(uint32_t limit, uint32_t withheld) { return set_wait_fault_here(limit, withheld); }

} // namespace svo

using namespace svo;

extern "C" {

int svo_texture_set_create(const uint8_t *const *rgba, const uint32_t *width, const uint32_t *height, uint32_t count,
                           svo_texture_set **out) {
	if (!out || (count && (!rgba || !width || !height))) return svo_fail(SVO_ERR_INVALID, "null argument");
	*out = nullptr;
	svo_texture_set *s = new svo_texture_set();
	s->count = count;
	size_t texels = 0;
	for (uint32_t t = 0; t < count; ++t) {
		if (!rgba[t] || !width[t] || !height[t] || width[t] > 32768 || height[t] > 32768) {
			delete s;
			return svo_fail(SVO_ERR_INVALID, "texture %u: null or size %ux%u", t, width[t], height[t]);
		}
		TexDesc d{};
		d.width = width[t], d.height = height[t];
		std::vector<std::vector<uint8_t>> levels;
		texture_mip_chain(rgba[t], width[t], height[t], levels);
		d.levels = (uint32_t)levels.size();
		for (uint32_t l = 0; l < d.levels; ++l) {
			d.level_off[l] = texels;
			texels += levels[l].size() / 4;
		}
		s->desc.push_back(d);
		for (auto &lv : levels) s->levels.push_back(std::move(lv));
	}
	// linear float texels: colour through the sRGB decode, alpha as is
	float lin[256];
	for (int c = 0; c < 256; ++c) lin[c] = (float)srgb_decode(c / 255.0);
	std::vector<float4> host(texels);
	size_t k = 0;
	for (const auto &lv : s->levels)
		for (size_t i = 0; i < lv.size(); i += 4)
			host[k++] = make_float4(lin[lv[i]], lin[lv[i + 1]], lin[lv[i + 2]], (float)(lv[i + 3] / 255.0));
	cudaError_t e = cudaSuccess;
	if (count) {
		e = counted_malloc(&s->desc_dev, count * sizeof(TexDesc));
		if (e == cudaSuccess) e = counted_malloc(&s->texels_dev, texels * sizeof(float4));
		if (e == cudaSuccess) e = cudaMemcpy(s->desc_dev, s->desc.data(), count * sizeof(TexDesc), cudaMemcpyHostToDevice);
		if (e == cudaSuccess) e = cudaMemcpy(s->texels_dev, host.data(), texels * sizeof(float4), cudaMemcpyHostToDevice);
	}
	if (e != cudaSuccess) {
		cudaFree(s->desc_dev);
		cudaFree(s->texels_dev);
		delete s;
		return svo_fail(SVO_ERR_CUDA, "texture upload: %s", cudaGetErrorString(e));
	}
	*out = s;
	return SVO_OK;
}

int svo_texture_set_level(const svo_texture_set *s, uint32_t texture, uint32_t level, uint8_t *rgba, uint32_t *width,
                          uint32_t *height) {
	if (!s || texture >= s->count) return svo_fail(SVO_ERR_INVALID, "no texture %u", texture);
	const TexDesc &d = s->desc[texture];
	if (level >= d.levels) return svo_fail(SVO_ERR_INVALID, "texture %u has %u levels", texture, d.levels);
	uint32_t first = 0;
	for (uint32_t t = 0; t < texture; ++t) first += s->desc[t].levels;
	const std::vector<uint8_t> &lv = s->levels[first + level];
	if (width) *width = d.width >> level ? d.width >> level : 1;
	if (height) *height = d.height >> level ? d.height >> level : 1;
	if (rgba) std::memcpy(rgba, lv.data(), lv.size());
	return SVO_OK;
}

void svo_texture_set_destroy(svo_texture_set *s) {
	if (!s) return;
	cudaFree(s->desc_dev);
	cudaFree(s->texels_dev);
	delete s;
}

} // extern "C"
