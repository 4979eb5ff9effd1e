// io.cu — host-side scene and octree files: an OBJ loader with the reference's normalisation
// (Scene::load_meshes, src/Scene.cpp:36-147) and a raw octree file (node words with a small header).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <array>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "svo_internal.h"

namespace svo {

int svo_fail(int code, const char *fmt, ...);

namespace {

// ------------------------------------------------------------------------------------------ OBJ
struct ObjFile {
	std::vector<float> v;                          // x, y, z per vertex
	std::vector<int> tri;                          // 3 vertex indices per triangle
	std::vector<int> tri_mat;                      // material per triangle (-1: none)
	std::vector<std::string> mat_names;            // usemtl names in order of first use
	std::unordered_map<std::string, std::array<float, 3>> kd; // Kd per newmtl
	std::vector<std::string> mtl_order;            // newmtl names in file order
};

std::string dir_of(const std::string &path) {
	const size_t s = path.find_last_of("/\\");
	return s == std::string::npos ? std::string() : path.substr(0, s + 1);
}

// Reads a whole text file; false when it cannot be read.
bool read_text(const std::string &path, std::string &out) {
	FILE *f = fopen(path.c_str(), "rb");
	if (!f) return false;
	char buf[1 << 16];
	size_t n;
	out.clear();
	while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out.append(buf, n);
	fclose(f);
	return true;
}

void parse_mtl(const std::string &text, ObjFile &obj) {
	std::string cur;
	size_t pos = 0;
	while (pos < text.size()) {
		size_t end = text.find('\n', pos);
		if (end == std::string::npos) end = text.size();
		std::string line = text.substr(pos, end - pos);
		pos = end + 1;
		const char *p = line.c_str();
		while (*p == ' ' || *p == '\t') ++p;
		if (!strncmp(p, "newmtl", 6) && (p[6] == ' ' || p[6] == '\t')) {
			p += 6;
			while (*p == ' ' || *p == '\t') ++p;
			cur = p;
			while (!cur.empty() && (cur.back() == '\r' || cur.back() == ' ' || cur.back() == '\t')) cur.pop_back();
			if (!obj.kd.count(cur)) obj.mtl_order.push_back(cur);
			obj.kd[cur] = {0.0f, 0.0f, 0.0f};
		} else if (!strncmp(p, "Kd", 2) && (p[2] == ' ' || p[2] == '\t') && !cur.empty()) {
			float r = 0, g = 0, b = 0;
			if (sscanf(p + 2, "%f %f %f", &r, &g, &b) >= 1) {
				obj.kd[cur] = {r, g, b};
			}
		}
	}
}

// One face-vertex token "v", "v/t", "v//n" or "v/t/n" (1-based, negative = relative to the end).
bool face_index(const char *tok, int nv, int &out) {
	char *end = nullptr;
	const long i = strtol(tok, &end, 10);
	if (end == tok || i == 0) return false;
	const long idx = i > 0 ? i - 1 : nv + i;
	if (idx < 0 || idx >= nv) return false;
	out = (int)idx;
	return true;
}

int parse_obj(const std::string &path, ObjFile &obj) {
	std::string text;
	if (!read_text(path, text)) return svo_fail(SVO_ERR_INVALID, "cannot read %s: %s", path.c_str(), strerror(errno));
	std::unordered_map<std::string, int> mat_index;
	int mat = -1;
	size_t pos = 0, line_no = 0;
	std::vector<int> poly;
	while (pos < text.size()) {
		size_t end = text.find('\n', pos);
		if (end == std::string::npos) end = text.size();
		std::string line = text.substr(pos, end - pos);
		pos = end + 1;
		++line_no;
		const char *p = line.c_str();
		while (*p == ' ' || *p == '\t') ++p;
		if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
			float x, y, z;
			if (sscanf(p + 1, "%f %f %f", &x, &y, &z) != 3)
				return svo_fail(SVO_ERR_INVALID, "%s:%zu: malformed vertex", path.c_str(), line_no);
			obj.v.push_back(x), obj.v.push_back(y), obj.v.push_back(z);
		} else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
			poly.clear();
			const int nv = (int)(obj.v.size() / 3);
			char *q = const_cast<char *>(p + 1);
			for (;;) {
				while (*q == ' ' || *q == '\t' || *q == '\r') ++q;
				if (!*q) break;
				int idx;
				if (!face_index(q, nv, idx))
					return svo_fail(SVO_ERR_INVALID, "%s:%zu: bad face index", path.c_str(), line_no);
				poly.push_back(idx);
				while (*q && *q != ' ' && *q != '\t' && *q != '\r') ++q;
			}
			if (poly.size() < 3) return svo_fail(SVO_ERR_INVALID, "%s:%zu: face with fewer than 3 vertices", path.c_str(), line_no);
			for (size_t k = 1; k + 1 < poly.size(); ++k) { // fan, as the loader's triangulation does for convex faces
				obj.tri.push_back(poly[0]), obj.tri.push_back(poly[k]), obj.tri.push_back(poly[k + 1]);
				obj.tri_mat.push_back(mat);
			}
		} else if (!strncmp(p, "usemtl", 6) && (p[6] == ' ' || p[6] == '\t')) {
			std::string name = p + 7;
			while (!name.empty() && (name.back() == '\r' || name.back() == ' ' || name.back() == '\t')) name.pop_back();
			while (!name.empty() && (name.front() == ' ' || name.front() == '\t')) name.erase(name.begin());
			auto it = mat_index.find(name);
			if (it == mat_index.end()) {
				it = mat_index.emplace(name, (int)obj.mat_names.size()).first;
				obj.mat_names.push_back(name);
			}
			mat = it->second;
		} else if (!strncmp(p, "mtllib", 6) && (p[6] == ' ' || p[6] == '\t')) {
			std::string name = p + 7;
			while (!name.empty() && (name.back() == '\r' || name.back() == ' ' || name.back() == '\t')) name.pop_back();
			while (!name.empty() && (name.front() == ' ' || name.front() == '\t')) name.erase(name.begin());
			std::string mtl;
			if (read_text(dir_of(path) + name, mtl)) parse_mtl(mtl, obj);
		}
	}
	return SVO_OK;
}

// glm::packUnorm4x8 of one channel: round(clamp(x, 0, 1) * 255).
uint32_t unorm8(float x) {
	x = x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x);
	return (uint32_t)std::round(x * 255.0f);
}

// ------------------------------------------------------------------------------------------ octree file
struct OctreeFileHeader {
	char magic[8];         // "SVOOCT01"
	uint32_t level;
	uint32_t range_words;
	uint32_t header_bytes; // 32
	uint32_t reserved[3];
};
static_assert(sizeof(OctreeFileHeader) == 32, "header layout");

// Structure check of a node pool read from a file: every interior word points inside the range at a
// whole child block.  (The march checks pointers too; this rejects a damaged file before any upload.)
bool pool_is_well_formed(const uint32_t *w, uint32_t range) {
	for (uint32_t i = 0; i < range; ++i) {
		const uint32_t x = w[i];
		if ((x & 0x80000000u) && !(x & 0x40000000u)) {
			const uint32_t c = x & 0x3fffffffu;
			if (c % 8 || c < 8 || (uint64_t)c + 8 > range) return false;
		}
	}
	return true;
}

} // namespace
} // namespace svo

using namespace svo;

extern "C" {

void svo_free_host(void *p) { free(p); }

int svo_load_obj(const char *path, svo_triangle **tris_host, uint32_t *n_tris) {
	if (!path || !tris_host || !n_tris) return svo_fail(SVO_ERR_INVALID, "null argument");
	*tris_host = nullptr;
	*n_tris = 0;
	ObjFile obj;
	int rc = parse_obj(path, obj);
	if (rc) return rc;
	if (obj.kd.empty()) return svo_fail(SVO_ERR_INVALID, "%s: no material found", path); // src/Scene.cpp:47-50
	const size_t nt = obj.tri.size() / 3;
	if (nt == 0) return svo_fail(SVO_ERR_INVALID, "%s: empty mesh", path);
	if (nt > 0xffffffffull) return svo_fail(SVO_ERR_CAPACITY, "%s: too many triangles", path);
	// bounds of the vertices the faces use, then (p - center) / (max extent / 2) -> [-1, 1]
	// (src/Scene.cpp:63-99), and p = (p_ref + 1) / 2 -> [0, 1]
	float pmin[3] = {3.4e38f, 3.4e38f, 3.4e38f}, pmax[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
	for (int idx : obj.tri)
		for (int k = 0; k < 3; ++k) {
			const float x = obj.v[3 * (size_t)idx + k];
			pmin[k] = x < pmin[k] ? x : pmin[k];
			pmax[k] = x > pmax[k] ? x : pmax[k];
		}
	float ext3[3], center[3];
	for (int k = 0; k < 3; ++k) ext3[k] = pmax[k] - pmin[k];
	const float extent = (ext3[0] > (ext3[1] > ext3[2] ? ext3[1] : ext3[2]) ? ext3[0] : (ext3[1] > ext3[2] ? ext3[1] : ext3[2])) * 0.5f;
	if (!(extent > 0.0f)) return svo_fail(SVO_ERR_INVALID, "%s: degenerate bounds", path);
	const float inv_extent = 1.0f / extent;
	for (int k = 0; k < 3; ++k) center[k] = (pmax[k] + pmin[k]) * 0.5f;
	svo_triangle *out = (svo_triangle *)malloc(nt * sizeof(svo_triangle));
	if (!out) return svo_fail(SVO_ERR_OOM, "host allocation");
	for (size_t t = 0; t < nt; ++t) {
		svo_triangle &T = out[t];
		for (int c = 0; c < 3; ++c)
			for (int k = 0; k < 3; ++k) {
				const float pr = (obj.v[3 * (size_t)obj.tri[3 * t + c] + k] - center[k]) * inv_extent;
				float p = (pr + 1.0f) * 0.5f;
				T.v[3 * c + k] = p < 0.0f ? 0.0f : (p > 1.0f ? 1.0f : p);
			}
		// per-material albedo, packUnorm4x8(vec4(Kd, 0)) (src/Scene.cpp:109,164); faces before any usemtl, or
		// naming an undefined material, take the first material of the library
		auto it = obj.tri_mat[t] < 0 ? obj.kd.end() : obj.kd.find(obj.mat_names[obj.tri_mat[t]]);
		if (it == obj.kd.end()) it = obj.kd.find(obj.mtl_order[0]);
		const uint32_t rgb = unorm8(it->second[0]) | (unorm8(it->second[1]) << 8) | (unorm8(it->second[2]) << 16);
		T.rgb[0] = T.rgb[1] = T.rgb[2] = rgb;
	}
	*tris_host = out;
	*n_tris = (uint32_t)nt;
	return SVO_OK;
}

int svo_octree_write_host(const uint32_t *words, uint32_t range_words, uint32_t level, const char *path) {
	if (!words || !path) return svo_fail(SVO_ERR_INVALID, "null argument");
	if (level < SVO_LEVEL_MIN || level > SVO_LEVEL_MAX || range_words < 8 || range_words % 8)
		return svo_fail(SVO_ERR_INVALID, "malformed octree (level %u, range %u)", level, range_words);
	FILE *f = fopen(path, "wb");
	if (!f) return svo_fail(SVO_ERR_INVALID, "cannot write %s: %s", path, strerror(errno));
	OctreeFileHeader h;
	memset(&h, 0, sizeof(h));
	memcpy(h.magic, "SVOOCT01", 8);
	h.level = level;
	h.range_words = range_words;
	h.header_bytes = sizeof(h);
	const bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(words, 4, range_words, f) == range_words;
	if (fclose(f) != 0 || !ok) return svo_fail(SVO_ERR_INVALID, "write to %s failed", path);
	return SVO_OK;
}

int svo_octree_read_host(const char *path, uint32_t **words, uint32_t *range_words, uint32_t *level) {
	if (!path || !words || !range_words || !level) return svo_fail(SVO_ERR_INVALID, "null argument");
	*words = nullptr;
	FILE *f = fopen(path, "rb");
	if (!f) return svo_fail(SVO_ERR_INVALID, "cannot read %s: %s", path, strerror(errno));
	OctreeFileHeader h;
	if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, "SVOOCT01", 8) || h.header_bytes != sizeof(h) ||
	    h.level < SVO_LEVEL_MIN || h.level > SVO_LEVEL_MAX || h.range_words < 8 || h.range_words % 8 ||
	    h.range_words > SVO_MAX_POOL_WORDS) {
		fclose(f);
		return svo_fail(SVO_ERR_INVALID, "%s: not an octree file", path);
	}
	uint32_t *w = (uint32_t *)malloc((size_t)h.range_words * 4);
	if (!w) {
		fclose(f);
		return svo_fail(SVO_ERR_OOM, "host allocation");
	}
	const bool ok = fread(w, 4, h.range_words, f) == h.range_words;
	const bool extra = fgetc(f) != EOF;
	fclose(f);
	if (!ok || extra) {
		free(w);
		return svo_fail(SVO_ERR_INVALID, "%s: size does not match its header", path);
	}
	if (!pool_is_well_formed(w, h.range_words)) {
		free(w);
		return svo_fail(SVO_ERR_INVALID, "%s: a child pointer lies outside the octree", path);
	}
	*words = w;
	*range_words = h.range_words;
	*level = h.level;
	return SVO_OK;
}

int svo_octree_save(const svo_octree *o, const char *path, void *stream) {
	if (!o || !o->words) return svo_fail(SVO_ERR_INVALID, "null octree");
	std::vector<uint32_t> host(o->range_words);
	cudaError_t e = cudaMemcpyAsync(host.data(), o->words, (size_t)o->range_words * 4, cudaMemcpyDeviceToHost,
	                                (cudaStream_t)stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
	if (e != cudaSuccess) {
		cudaGetLastError();
		return svo_fail(SVO_ERR_CUDA, "octree download: %s", cudaGetErrorString(e));
	}
	return svo_octree_write_host(host.data(), o->range_words, o->level, path);
}

int svo_octree_load(const char *path, svo_octree *out, void *stream) {
	if (!out) return svo_fail(SVO_ERR_INVALID, "null output octree");
	uint32_t *w = nullptr, range = 0, level = 0;
	int rc = svo_octree_read_host(path, &w, &range, &level);
	if (rc) return rc;
	void *dev = nullptr;
	cudaError_t e = counted_malloc_async(&dev, (size_t)range * 4, (cudaStream_t)stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(dev, w, (size_t)range * 4, cudaMemcpyHostToDevice, (cudaStream_t)stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream); // the host copy is freed next
	free(w);
	if (e != cudaSuccess) {
		if (dev) cudaFreeAsync(dev, (cudaStream_t)stream);
		cudaGetLastError();
		return svo_fail(e == cudaErrorMemoryAllocation ? SVO_ERR_OOM : SVO_ERR_CUDA, "octree upload: %s",
		                cudaGetErrorString(e));
	}
	memset(out, 0, sizeof(*out));
	out->words = (uint32_t *)dev;
	out->capacity = range;
	out->range_words = range;
	out->level = level;
	out->owned = 1;
	return SVO_OK;
}

} // extern "C"
