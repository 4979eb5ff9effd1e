/*
 * oracle.h — CPU oracle for the sparse-voxel-octree hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's algorithm
 * (AdamYuan/SparseVoxelOctree) used to check the CUDA engine and to time the CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the engine
 * never calls it.
 *
 * Parity pinning: oracle/build_ref.py compiles the reference's own GLSL compute and march source
 * through a C++ shim into oracle/_ref/ and tests/test_oracle_pin.py checks this oracle against it;
 * tests/golden/ holds fixtures generated that way.
 */
#ifndef SVO_ORACLE_H
#define SVO_ORACLE_H

#include "../include/svo.h"
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Worker threads (0 = all hardware threads). */
void oracle_set_threads(int n);
int oracle_get_threads(void);

/* ---- voxelize: conservative raster restated in fixed point (see oracle.c) ---- */
/* Fragment count of every triangle (counts[t]); returns the total. */
uint64_t oracle_voxelize_count(const svo_triangle *tris, uint32_t n, uint32_t level, uint32_t *counts);
/* Writes fragments in canonical order (triangle, span, position).  `offsets` = exclusive prefix of counts
 * (n+1 entries). */
void oracle_voxelize_emit(const svo_triangle *tris, uint32_t n, uint32_t level, const uint64_t *offsets,
                          uint64_t *frags);

/* Per-triangle setup exposed for tests: axis, pixel AABB, depth range, span orientation. */
typedef struct oracle_tri_info {
	int32_t axis, i0, i1, j0, j1, z0, z1, cols, degenerate;
	uint32_t rgb;
} oracle_tri_info;
void oracle_triangle_info(const svo_triangle *tri, uint32_t level, oracle_tri_info *info);

/* ---- build ---- */
#define ORACLE_COLOR_DET 0 /* channel-wise integer mean (the engine's rule) */
#define ORACLE_COLOR_REF 1 /* the reference's CAS running mean, fragments applied in list order */
/* Builds the octree with the reference's level loop (shader/octree_{init,tag,alloc}_node.comp,
 * octree_modify_arg.comp driven as in src/OctreeBuilder.cpp:142-210), child blocks allocated in word
 * order.  Writes at most `capacity` words to pool; returns the range in words, or 0 with *status set
 * to SVO_ERR_CAPACITY if the pool is too small.  level_nodes (may be NULL) gets non-empty node counts
 * per depth 1..level. */
uint64_t oracle_build(const uint64_t *frags, uint64_t count, uint32_t level, int color_mode, uint32_t *pool,
                      uint64_t capacity, uint32_t *level_nodes, int *status);

/* Breadth-first renumbering of child blocks (children visited in word order); writes the canonical
 * pool to `out` (range words).  Returns 0 on success, -1 on a malformed pool. */
int oracle_canonicalize(const uint32_t *pool, uint64_t range, uint32_t *out);

/* ---- march ---- */
/* Octree_RayMarchLeaf (shader/octree.glsl:179-340) per ray.  fetches (may be NULL) gets per-ray node
 * loads. */
void oracle_raycast(const uint32_t *pool, uint64_t range, uint32_t level, const svo_ray *rays, uint64_t n,
                    svo_hit *hits, uint32_t *fetches);
/* Camera_GenRay (shader/camera.glsl:11-14) at ivec2(pixel)/size (shader/octree_tracer.frag:24). */
void oracle_camera_rays(const svo_camera *cam, uint32_t width, uint32_t height, svo_ray *rays);
/* Octree_RayMarchOcclude per ray: 1 when the ray hits a leaf. */
void oracle_occlude(const uint32_t *pool, uint64_t range, uint32_t level, const svo_ray *rays, uint64_t n,
                    uint32_t *occluded);
/* Beam pre-pass texels and the primary rays it advances. */
void oracle_beam(const uint32_t *pool, uint64_t range, uint32_t level, const svo_camera *cam, uint32_t width,
                 uint32_t height, uint32_t beam_size, float *beam);
void oracle_camera_rays_beam(const svo_camera *cam, uint32_t width, uint32_t height, const float *beam,
                             uint32_t beam_size, svo_ray *rays);
/* Diffuse_Sample for one normal and sample pair (shader/diffuse.glsl:7-14, shader/util.glsl:5-9). */
void oracle_diffuse_sample(const float nrm[3], float u1, float u2, float out[3]);
/* Cosine bounce rays for hits (shader/diffuse.glsl:7-14 + shader/util.glsl:5-9). */
void oracle_bounce_rays(const svo_hit *hits, uint64_t n, uint64_t seed, svo_ray *rays);

/* ---- path tracer ---- */
/* One sample per pixel of shader/path_tracer.comp (ConstColorPathTrace / EnvMapPathTrace and the running
 * means of main()), updating color (4 floats per pixel), albedo and normal (rgba8 unorm / snorm words)
 * in place.  sobol: the Sobol state (2 * (bounce + 1) values, then the sample index); noise: 256 x 256
 * RG8; env_texels / env_alias: the environment map tables (light_type 1). */
void oracle_pt_render(const uint32_t *pool, uint64_t range, uint32_t level, const svo_camera *cam, uint32_t width,
                      uint32_t height, uint32_t bounce, uint32_t light_type, const float *const_color, float rot,
                      float mult, const float *env_texels, const uint32_t *env_alias, uint32_t env_w, uint32_t env_h,
                      const uint32_t *sobol, const uint8_t *noise, float *color, uint32_t *albedo, uint32_t *normal);
/* Sobol::CmdNext (shader/sobol.comp:70-86) for `dim` dimensions of 32 direction numbers each. */
void oracle_sobol_next(uint32_t *sobol, const uint32_t *matrices, uint32_t dim);
/* EnvironmentMap::weigh_hdr_image + generate_alias_table (src/EnvironmentMap.cpp:83-160). */
int oracle_envmap_build(float *rgba, uint32_t w, uint32_t h, uint32_t *alias);
/* ---- textured voxelization ---- */
/* The mip chain of an RGBA8 texture (every level's bytes, level 0 first); returns the level count. */
uint32_t oracle_texture_mips(const uint8_t *rgba, uint32_t w, uint32_t h, uint8_t *out);
/* shader/voxelizer.frag:27-36 over the canonical fragments: textured triangles' fragments coloured by
 * their texture or dropped (alpha < 0.5).  Returns the count written to out. */
uint64_t oracle_voxelize_textured(const svo_triangle *tris, const svo_triangle_uv *uvs, uint32_t n, uint32_t level,
                                  const uint8_t *const *textures, const uint32_t *widths, const uint32_t *heights,
                                  uint32_t count, uint64_t *out);
/* sin x, cos x, atan2(y, x), acos x by the engine's restatements (oracle/svo_trig.h). */
void oracle_trig(float x, float y, float *out);

#ifdef __cplusplus
}
#endif

#endif
