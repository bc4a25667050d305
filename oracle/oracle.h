/*
 * oracle.h - CPU restatement of MiTrace's path-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300 kernels
 * and the timed CPU baseline; nothing in the product library links or calls
 * it.  Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline and the
 * --impl reference arm) load it.
 *
 * Parity status: the reference cannot be built here (its CMake fetches GLM,
 * nlohmann_json, spdlog, argparse and stb over the network and none of them is
 * installed), and it ships no unit tests, golden images or golden vectors.  The
 * restatement is therefore "parity unpinned" against reference outputs; it is
 * pinned instead against known-answer tests derived from the mathematics
 * (Moller-Trumbore hits, BRDF normalisation, ACES values, Philox4x32-10
 * published vectors) and against the reference's own test fixtures
 * (assets/tests/cornell_box_test) read as data.
 *
 * The scene description is the product's boundary format (mitrace_gpu.h);
 * the oracle only reads it.
 */
#ifndef MITRACE_ORACLE_H
#define MITRACE_ORACLE_H

#include "../include/mitrace_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

#define ORC_RNG_MT19937 0 /* std::mt19937 seeded per tile, as RenderBlock does  */
#define ORC_RNG_COUNTER 1 /* Philox4x32-10 keyed by (pixel, sample, bounce, slot) */

/* BVH build restated from src/Scene/BVH.cpp:117-282 with the depth handling of
 * src/Scene/Mesh.cpp:37-40.  Arrays are malloc'ed; release with orc_free. */
int orc_bvh_build(const float* positions, uint32_t num_triangles, uint32_t max_triangles,
                  uint32_t max_depth, mt_bvh_node** nodes, uint32_t* num_nodes,
                  uint32_t** indices, uint32_t* num_indices);
void orc_free(void* p);

int orc_scene_create(const mt_scene_desc* scene, const mt_config* cfg, orc_scene** out);
void orc_scene_destroy(orc_scene* s);
/* Number of BVH nodes / indices the oracle built (or was given) for a mesh. */
int orc_scene_mesh_bvh(const orc_scene* s, uint32_t mesh, const mt_bvh_node** nodes,
                       uint32_t* num_nodes, const uint32_t** indices, uint32_t* num_indices);

/* IntersectScene (src/Tracer/Intersect.cpp:201-219) for a batch of rays.
 * query: MT_QUERY_CLOSEST / MT_QUERY_CLOSEST_COUNT fill the hit record with the
 * winning instance's counters; MT_QUERY_ANY writes 1 into hit.instance when the
 * closest hit lies at world distance <= ray.tmax, else 0.
 * totals (optional, 3 x n): bvh tests (pops), inner-node expansions and
 * triangle tests summed over ALL instances the ray visited. */
int orc_trace_rays(const orc_scene* s, const mt_ray* rays, uint64_t n, mt_hit* hits, int query,
                   uint32_t* totals, int threads);

/* FP64 twin: for each ray whose hit names (instance, triangle), recompute the
 * world distance and barycentrics in double precision.  out: 3 doubles/ray
 * (NaN for misses). */
int orc_trace_f64(const orc_scene* s, const mt_ray* rays, const mt_hit* hits, uint64_t n,
                  double* out);

/* BRDF.hpp:52-97 on a batch. */
int orc_brdf_batch(const mt_brdf_query* q, uint64_t n, mt_brdf_result* out);
int orc_brdf_sample(const mt_brdf_sample_query* q, uint64_t n, mt_brdf_sample_result* out);

/* Camera::GenerateCameraRay (src/Tracer/Camera.cpp:17-50) for (u, v) pairs. */
int orc_camera_rays(const orc_scene* s, const float* uv, uint64_t n, mt_ray* out);

/* Philox4x32-10 on (counter, key); out gets 4 words. */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Tracer::RenderBlock over the tiles that intersect rows [row0, row1) with the
 * reference's tile queue and worker threads (threads <= 0: all cores).
 * rgb_out holds the full W*H*3 image; only the band's rows are written.
 * rays / samples get the reference's counters (Tracer.cpp:146,319,342). */
int orc_render(const orc_scene* s, int rng_mode, int threads, uint32_t row0, uint32_t row1,
               float* rgb_out, uint64_t* rays, uint64_t* samples);

/* Per-sample tonemapped outputs (before the firefly clamp) of the pixels in
 * rows [row0,row1), layout [sample][row-row0][x][3]; counter RNG only. */
int orc_render_samples(const orc_scene* s, int threads, uint32_t row0, uint32_t row1,
                       float* out);

/* Firefly clamp + average of one pixel's samples (Tracer.cpp:490-548, 593-601).
 * debug_mode MT_DEBUG_PIXEL_STANDARD_DEVIATION / MT_DEBUG_FIREFLY_ELIMINATION
 * return the clamp's sigma / dropped-sample count (before the heatmap). */
int orc_resolve_pixel(const float* samples_rgb, uint32_t n, int firefly_enable, float k,
                      int debug_mode, float out_rgb[3]);

/* Adjoint check: renders with the counter RNG, and adds dL/dparameters for
 * L = sum over pixels/channels of (image - target)^2, replaying each kept
 * sample's path with its decisions held fixed (same convention and gradient
 * layout as mt_render_grad). */
int orc_render_grad(const orc_scene* s, const float* target, float* image, float* loss, float* d_base,
                    float* d_rough, float* d_metal, float* d_light, float* d_texels, int threads);

/* ACES fit (Tracer.cpp:212-222). */
void orc_aces(const float in_rgb[3], float exposure_mul, float out_rgb[3]);

const char* orc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
