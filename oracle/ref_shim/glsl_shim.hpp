// glsl_shim.hpp — just enough GLSL 4.50 for C++ to compile the reference's compute, march, camera,
// diffuse and voxelizer shader source unchanged in meaning.  TEST INFRASTRUCTURE ONLY: it lets
// oracle/build_ref.py build the reference's own shader code on the CPU so the oracle can be checked
// against it.  Float semantics: every operation is a separately rounded binary32 operation (compile
// with -ffp-contract=off); float->uint conversion saturates like GPU hardware.
#pragma once
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>

typedef uint32_t uint;

// ------------------------------------------------------------------------------------------ vectors
template <typename T> struct tv2;
template <typename T> struct tv3;
template <typename T> struct tv4;

// Swizzle proxy overlaid (in a union) on the K components of its owner.
template <typename T, int K, int N, int A, int B, int C = 0> struct swz {
	T e[K];
	using V = typename std::conditional<N == 2, tv2<T>, tv3<T>>::type;
	operator V() const;
	swz &operator*=(T s) {
		e[A] *= s;
		e[B] *= s;
		if (N == 3) e[C] *= s;
		return *this;
	}
	swz &operator/=(T s) {
		e[A] /= s;
		e[B] /= s;
		if (N == 3) e[C] /= s;
		return *this;
	}
};

template <typename T> struct tv2 {
	T x, y;
	tv2() : x(0), y(0) {}
	explicit tv2(T s) : x(s), y(s) {}
	tv2(T a, T b) : x(a), y(b) {}
	template <typename U> explicit tv2(const tv2<U> &o) : x(cvt<U>(o.x)), y(cvt<U>(o.y)) {}
	T &operator[](int i) { return (&x)[i]; }
	T operator[](int i) const { return (&x)[i]; }
	template <typename U> static T cvt(U v);
};

template <typename T> struct tv3 {
	union {
		struct {
			T x, y, z;
		};
		swz<T, 3, 2, 0, 1> xy;
		swz<T, 3, 3, 0, 1, 2> xyz;
		swz<T, 3, 3, 1, 2, 0> yzx;
		swz<T, 3, 3, 2, 0, 1> zxy;
	};
	tv3() : x(0), y(0), z(0) {}
	tv3(T s) : x(s), y(s), z(s) {}
	tv3(T a, T b, T c) : x(a), y(b), z(c) {}
	tv3(const tv2<T> &v, T c) : x(v.x), y(v.y), z(c) {}
	tv3(const tv3 &o) : x(o.x), y(o.y), z(o.z) {}
	tv3 &operator=(const tv3 &o) {
		x = o.x, y = o.y, z = o.z;
		return *this;
	}
	template <typename U> explicit tv3(const tv3<U> &o) : x(tv2<T>::template cvt<U>(o.x)), y(tv2<T>::template cvt<U>(o.y)), z(tv2<T>::template cvt<U>(o.z)) {}
	T &operator[](int i) { return (&x)[i]; }
	T operator[](int i) const { return (&x)[i]; }
	// rvalue swizzles (the build recipe rewrites v.yzx into v._yzx() wherever it is not assigned to)
	tv2<T> _xy() const { return tv2<T>(x, y); }
	tv3 _xyz() const { return tv3(x, y, z); }
	tv3 _yzx() const { return tv3(y, z, x); }
	tv3 _zxy() const { return tv3(z, x, y); }
};

template <typename T> struct tv4 {
	union {
		struct {
			T x, y, z, w;
		};
		struct {
			T r, g, b, a;
		};
		swz<T, 4, 2, 0, 1> xy;
		swz<T, 4, 2, 2, 3> zw;
		swz<T, 4, 3, 0, 1, 2> xyz;
	};
	tv4() : x(0), y(0), z(0), w(0) {}
	tv4(T s) : x(s), y(s), z(s), w(s) {}
	tv4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
	tv4(const tv3<T> &v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
	tv4(const tv2<T> &a, const tv2<T> &b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
	tv4(const tv2<T> &a, T c, T d) : x(a.x), y(a.y), z(c), w(d) {}
	tv4(const tv4 &o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
	tv4 &operator=(const tv4 &o) {
		x = o.x, y = o.y, z = o.z, w = o.w;
		return *this;
	}
	T &operator[](int i) { return (&x)[i]; }
	T operator[](int i) const { return (&x)[i]; }
	tv2<T> _xy() const { return tv2<T>(x, y); }
	tv2<T> _zw() const { return tv2<T>(z, w); }
	tv3<T> _xyz() const { return tv3<T>(x, y, z); }
};

template <typename T, int K, int N, int A, int B, int C> swz<T, K, N, A, B, C>::operator V() const {
	if constexpr (N == 2)
		return tv2<T>(e[A], e[B]);
	else
		return tv3<T>(e[A], e[B], e[C]);
}

// float -> uint saturates (GPU behaviour); everything else is a plain C++ conversion
template <typename T> template <typename U> T tv2<T>::cvt(U v) {
	if constexpr (std::is_same<T, uint32_t>::value && std::is_floating_point<U>::value) {
		if (!(v > 0)) return 0u;
		if (v >= 4294967295.0) return 0xffffffffu;
		return (uint32_t)v;
	} else
		return (T)v;
}

typedef tv2<float> vec2;
typedef tv3<float> vec3;
typedef tv4<float> vec4;
typedef tv2<uint> uvec2;
typedef tv3<uint> uvec3;
typedef tv4<uint> uvec4;
typedef tv2<int> ivec2;
typedef tv3<bool> bvec3;

// uvec3(bvec3)
inline uvec3 to_uvec3(const bvec3 &b) { return uvec3(b.x, b.y, b.z); }

#define SHIM_BINOP(V, OP)                                                                                   \
	inline V operator OP(const V &a, const V &b) {                                                      \
		V r;                                                                                        \
		for (int i = 0; i < (int)(sizeof(V) / sizeof(a.x)); ++i) r[i] = a[i] OP b[i];              \
		return r;                                                                                   \
	}
#define SHIM_VEC_OPS(V, S, N)                                                                               \
	inline V operator+(const V &a, const V &b) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] + b[i]; return r; } \
	inline V operator-(const V &a, const V &b) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] - b[i]; return r; } \
	inline V operator*(const V &a, const V &b) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] * b[i]; return r; } \
	inline V operator/(const V &a, const V &b) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] / b[i]; return r; } \
	inline V operator+(const V &a, S s) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] + s; return r; } \
	inline V operator-(const V &a, S s) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] - s; return r; } \
	inline V operator*(const V &a, S s) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] * s; return r; } \
	inline V operator/(const V &a, S s) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] / s; return r; } \
	inline V operator+(S s, const V &a) { V r; for (int i = 0; i < N; ++i) r[i] = s + a[i]; return r; } \
	inline V operator-(S s, const V &a) { V r; for (int i = 0; i < N; ++i) r[i] = s - a[i]; return r; } \
	inline V operator*(S s, const V &a) { V r; for (int i = 0; i < N; ++i) r[i] = s * a[i]; return r; } \
	inline V operator/(S s, const V &a) { V r; for (int i = 0; i < N; ++i) r[i] = s / a[i]; return r; } \
	inline V &operator+=(V &a, const V &b) { for (int i = 0; i < N; ++i) a[i] += b[i]; return a; }     \
	inline V &operator-=(V &a, const V &b) { for (int i = 0; i < N; ++i) a[i] -= b[i]; return a; }     \
	inline V &operator*=(V &a, S s) { for (int i = 0; i < N; ++i) a[i] *= s; return a; }                \
	inline V &operator/=(V &a, S s) { for (int i = 0; i < N; ++i) a[i] /= s; return a; }                \
	inline bool operator==(const V &a, const V &b) { for (int i = 0; i < N; ++i) if (a[i] != b[i]) return false; return true; } \
	inline bool operator!=(const V &a, const V &b) { return !(a == b); }                                \
	inline V min(const V &a, const V &b) { V r; for (int i = 0; i < N; ++i) r[i] = b[i] < a[i] ? b[i] : a[i]; return r; } \
	inline V max(const V &a, const V &b) { V r; for (int i = 0; i < N; ++i) r[i] = a[i] < b[i] ? b[i] : a[i]; return r; } \
	inline V clamp(const V &x, const V &lo, const V &hi) { return min(max(x, lo), hi); }

SHIM_VEC_OPS(vec2, float, 2)
SHIM_VEC_OPS(vec3, float, 3)
SHIM_VEC_OPS(vec4, float, 4)
SHIM_VEC_OPS(uvec2, uint, 2)
SHIM_VEC_OPS(uvec3, uint, 3)
SHIM_VEC_OPS(uvec4, uint, 4)

SHIM_VEC_OPS(ivec2, int, 2)

inline vec3 &operator*=(vec3 &a, const vec3 &b) {
	for (int i = 0; i < 3; ++i) a[i] *= b[i];
	return a;
}
inline ivec2 operator&(const ivec2 &a, int m) { return ivec2(a.x & m, a.y & m); }
inline vec3 operator-(const vec3 &a) { return vec3(-a.x, -a.y, -a.z); }
inline vec2 operator-(const vec2 &a) { return vec2(-a.x, -a.y); }
inline uvec3 operator*(const uvec3 &a, const bvec3 &b) { return a * to_uvec3(b); }

// ------------------------------------------------------------------------------------------ scalar / vector functions
inline float abs(float x) { return std::fabs(x); }
inline vec2 abs(const vec2 &v) { return vec2(std::fabs(v.x), std::fabs(v.y)); }
inline vec3 abs(const vec3 &v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline uint min(uint a, uint b) { return b < a ? b : a; }
inline uint max(uint a, uint b) { return a < b ? b : a; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline uint clamp(uint x, uint lo, uint hi) { return min(max(x, lo), hi); }
inline float dot(const vec2 &a, const vec2 &b) { return a.x * b.x + a.y * b.y; }
inline float dot(const vec3 &a, const vec3 &b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline vec3 cross(const vec3 &a, const vec3 &b) {
	return vec3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float length(const vec3 &v) { return std::sqrt(dot(v, v)); }
inline vec3 normalize(const vec3 &v) { return v / length(v); }
inline float sqrt(float x) { return std::sqrt(x); }
#ifdef SHIM_ENGINE_TRIG
// GLSL leaves the precision of its transcendental built-ins to the implementation; this build evaluates
// them with the engine's restatements (oracle/svo_trig.h) so a comparison isolates the shader logic.
#include "../svo_trig.h"
inline float cos(float x) { float s, c; svo_sincos(x, &s, &c); return c; }
inline float sin(float x) { float s, c; svo_sincos(x, &s, &c); return s; }
#else
inline float cos(float x) { return std::cos(x); }
inline float sin(float x) { return std::sin(x); }
#endif
inline bvec3 greaterThanEqual(const uvec3 &a, const uvec3 &b) { return bvec3(a.x >= b.x, a.y >= b.y, a.z >= b.z); }
inline uint floatBitsToUint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline int findMSB(uint v) { return v ? 31 - __builtin_clz(v) : -1; }
inline int findLSB(uint v) { return v ? __builtin_ctz(v) : -1; }
inline vec2 fract(const vec2 &v) { return vec2(v.x - std::floor(v.x), v.y - std::floor(v.y)); }
inline bool glsl_isnan(float x) { return std::isnan(x); }
#ifdef SHIM_ENGINE_TRIG
inline float atan(float y, float x) { return svo_atan2(y, x); }
inline float acos(float x) { return svo_acos(x); }
#else
inline float atan(float y, float x) { return std::atan2(y, x); }
inline float acos(float x) { return std::acos(x); }
#endif
inline void barrier() {}
inline uint packUnorm4x8(const vec4 &v) {
	uint r = 0;
	for (int i = 0; i < 4; ++i) r |= (uint)std::lrint(clamp(v[i], 0.0f, 1.0f) * 255.0f) << (8 * i);
	return r;
}
inline vec4 unpackUnorm4x8(uint p) {
	return vec4((float)(p & 0xffu) / 255.0f, (float)((p >> 8) & 0xffu) / 255.0f, (float)((p >> 16) & 0xffu) / 255.0f,
	            (float)(p >> 24) / 255.0f);
}

struct mat3x2 {
	vec2 c[3];
	mat3x2(const vec2 &a, const vec2 &b, const vec2 &d) { c[0] = a, c[1] = b, c[2] = d; }
};
inline vec2 operator*(const mat3x2 &m, const vec3 &v) { return (m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z; }

// ------------------------------------------------------------------------------------------ atomics and subgroups
inline uint atomicAdd(uint &mem, uint v) { return std::atomic_ref<uint>(mem).fetch_add(v); }
inline uint atomicCompSwap(uint &mem, uint cmp, uint v) {
	std::atomic_ref<uint>(mem).compare_exchange_strong(cmp, v);
	return cmp;
}
// Subgroups of one invocation (a legal Vulkan subgroup size): invocations run one at a time, in order.
inline uvec4 subgroupBallot(bool b) { return uvec4(b ? 1u : 0u, 0u, 0u, 0u); }
inline bool subgroupElect() { return true; }
inline uint subgroupBallotBitCount(const uvec4 &b) { return (uint)__builtin_popcount(b.x); }
inline uint subgroupBroadcastFirst(uint v) { return v; }
inline uint subgroupBallotExclusiveBitCount(const uvec4 &) { return 0u; }

// ------------------------------------------------------------------------------------------ stages
struct glsl_discard {};

// Images and samplers as plain arrays.  The format conversions are the Vulkan rules as the engine
// states them: unorm8 stores round(clamp(v, 0, 1) * 255) with ties up and loads c / 255; snorm8 stores
// round(clamp(v, -1, 1) * 127) with ties up and loads max(c / 127, -1).
struct image2D {
	void *data = nullptr;
	int w = 0, h = 0;
	int format = 0; // 0 rgba32f, 1 rgba8 unorm, 2 rgba8 snorm
};
inline ivec2 imageSize(const image2D &im) { return ivec2(im.w, im.h); }
inline vec4 imageLoad(const image2D &im, const ivec2 &p) {
	const size_t i = (size_t)p.y * im.w + p.x;
	if (im.format == 0) {
		const float *f = (const float *)im.data + 4 * i;
		return vec4(f[0], f[1], f[2], f[3]);
	}
	const uint w = ((const uint *)im.data)[i];
	vec4 r;
	for (int k = 0; k < 4; ++k) {
		const uint b = (w >> (8 * k)) & 0xffu;
		r[k] = im.format == 1 ? (float)b / 255.0f : std::fmax((float)(int8_t)b / 127.0f, -1.0f);
	}
	return r;
}
inline void imageStore(image2D &im, const ivec2 &p, const vec4 &v) {
	const size_t i = (size_t)p.y * im.w + p.x;
	if (im.format == 0) {
		float *f = (float *)im.data + 4 * i;
		for (int k = 0; k < 4; ++k) f[k] = v[k];
		return;
	}
	uint w = 0;
	for (int k = 0; k < 4; ++k) {
		const uint b = im.format == 1 ? (uint)std::floor(clamp(v[k], 0.0f, 1.0f) * 255.0f + 0.5f)
		                              : (uint)(int)std::floor(clamp(v[k], -1.0f, 1.0f) * 127.0f + 0.5f) & 0xffu;
		w |= b << (8 * k);
	}
	((uint *)im.data)[i] = w;
}

// A float texture (4 channels per texel).  texture() is VK_FILTER_LINEAR with repeat addressing: the 4
// texels around (u W - 1/2, v H - 1/2), integer coordinates wrapped.
struct sampler2D {
	const float *texels = nullptr;
	int w = 0, h = 0;
};
struct usampler2D {
	const uint *texels = nullptr; // 2 channels per texel
	int w = 0, h = 0;
};
inline ivec2 textureSize(const sampler2D &s, int) { return ivec2(s.w, s.h); }
inline vec4 texelFetch(const sampler2D &s, const ivec2 &p, int) {
	const float *t = s.texels + 4 * ((size_t)p.y * s.w + p.x);
	return vec4(t[0], t[1], t[2], t[3]);
}
inline uvec4 texelFetch(const usampler2D &s, const ivec2 &p, int) {
	const uint *t = s.texels + 2 * ((size_t)p.y * s.w + p.x);
	return uvec4(t[0], t[1], 0u, 1u);
}
inline vec4 texture(const sampler2D &s, const vec2 &uv) {
	if (!s.texels) throw std::runtime_error("texture sampling of an unbound sampler");
	const float x = uv.x * (float)s.w - 0.5f, y = uv.y * (float)s.h - 0.5f;
	const float fx = std::floor(x), fy = std::floor(y);
	const float a = x - fx, b = y - fy;
	const int64_t W = s.w, H = s.h;
	const int64_t i0 = (((int64_t)fx % W) + W) % W, j0 = (((int64_t)fy % H) + H) % H;
	const int64_t i1 = i0 + 1 == W ? 0 : i0 + 1, j1 = j0 + 1 == H ? 0 : j0 + 1;
	const float *t00 = s.texels + 4 * (j0 * W + i0), *t10 = s.texels + 4 * (j0 * W + i1);
	const float *t01 = s.texels + 4 * (j1 * W + i0), *t11 = s.texels + 4 * (j1 * W + i1);
	const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
	vec4 r;
	for (int k = 0; k < 4; ++k) r[k] = ((w00 * t00[k] + w10 * t10[k]) + w01 * t01[k]) + w11 * t11[k];
	return r;
}

struct gl_PerVertex {
	vec4 gl_Position;
};

// ------------------------------------------------------------------------------------------ bound resources
// The recipe deletes the shaders' buffer / uniform / push-constant / interface declarations; these
// globals take their place and the harness sets them before running a shader.
extern uint *uOctree;
extern uvec2 *uFragmentList;
extern uint uCounter, uAllocBegin, uAllocNum, uNumGroupX, uNumGroupY, uNumGroupZ;
extern uint kVoxelResolution, kFragmentCount, kTextureNum;
extern uint uCountOnly, uTextureId, uAlbedo;
extern vec4 uPosition, uLook, uSide, uUp;
extern sampler2D uTextures[1];
// path tracer (shader/path_tracer.comp, sobol.glsl / sobol.comp, environment_map.glsl); its uAlbedo image is
// declared in the harness's ref_pt namespace (the voxelizer's uAlbedo is a push constant)
extern uint *uSobol;
extern uint uDimension;
extern sampler2D uEnvironmentMap, uNoise;
extern usampler2D uEnvMapAliasTable;
extern image2D uColor, uNormal;
extern uint uBounce, uLightType;
extern float uConstColor[3], uEnvMapRotation, uEnvMapMultiplier;
extern thread_local uvec3 gl_GlobalInvocationID;
extern thread_local vec4 gl_FragCoord, gl_Position;
extern thread_local gl_PerVertex gl_in[3];
extern thread_local vec2 vTexcoord[3], gTexcoord;
extern thread_local uint gAxis;
extern thread_local uvec4 gAABB;
extern thread_local uvec2 gDepthRange;
void EmitVertex();
void EndPrimitive();
