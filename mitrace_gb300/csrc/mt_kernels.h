// mt_kernels.h - buffers shared by the host orchestration and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "../../include/mitrace_gpu.h"

namespace mt {

struct DevScene;

// Per-path state of one wavefront batch, structure-of-arrays, indexed by the
// path's position in the batch.
struct PathState {
    float4* ro;        // ray origin
    float4* rd;        // ray direction
    float4* cur;       // currentEnergy of the shading walk (Tracer.cpp:236)
    float4* tot;       // totalEnergy of the path generation (Tracer.cpp:138)
    float4* prev;      // base colour of the previous vertex (Tracer.cpp:247)
    float4* emit;      // LightOutput::emittedLight
    float4* direct;    // LightOutput::directLight
    float4* indirect;  // LightOutput::indirectLight
    float4* sky;       // LightOutput::skyLight
    float4* hitA;      // world position xyz, world distance
    uint4* hitB;       // instance (MT_NO_HIT on miss), triangle, u bits, v bits
    // debug render modes only (null otherwise): first-hit value rgb and the
    // number of path steps (w); first-hit BVH / triangle tests (x has bit 31
    // set when the first step hit), summed BVH / triangle tests of all steps
    float4* dval = nullptr;
    uint4* dcnt = nullptr;
};

// Shadow rays queued by the shade stage.
struct ShadowQueue {
    float4* o;  // origin xyz, max distance |lightVec|
    float4* d;  // direction xyz, owning path index (bits)
    float4* c;  // contribution xyz, 1 = direct (first vertex) / 0 = indirect
};

struct WaveBuffers {
    uint32_t* q[2];                // ping-pong queues of live path indices
    uint32_t* counts;              // [0],[1] queue sizes, [2] / [5] shadow-queue size
                                   // of even / odd bounces, [3] extend / [4] shadow
                                   // ray fetch counters, [7] debug heatmap maximum
    unsigned long long* rays;      // [0] extension rays, [1] shadow rays traced
    float* sr;                     // per-sample tonemapped R, sample-major in a band
    float* sg;
    float* sb;
    // optional: a second stream and two events of the owner, with which a
    // bounce's shadow rays are traced beside the next bounce's extension rays
    cudaStream_t side = nullptr;
    cudaEvent_t ev_shaded = nullptr, ev_shadowed = nullptr;
};
// counts[] slot of the shadow-queue size of bounce b
__host__ __device__ inline int sq_slot(uint32_t b) { return (b & 1u) ? 5 : 2; }

// Per-vertex records written by a recording (path-replay) pass of the render
// stages; null pointers in ordinary renders.  Vertex record of path p, bounce b:
// vert[(p * bounces + b) * 5 + k]
//   k=0  shading normal N, material index (bits)
//   k=1  view direction V = -ray, flags (bits, MT_VREC_*)
//   k=2  sampled next direction, NL / pdf (energy = brdf * this)
//   k=3  light direction, NL * falloff / pick (NEE = cur * brdf * lightColor * this)
//   k=4  uv, chosen light index (bits), spot factor
// Path record: path[2p] = (total radiance before ACES, hit vertices),
//              path[2p+1] = (sky sample, bounce of the miss or -1).
struct RecordBuffers {
    float4* vert = nullptr;
    float4* path = nullptr;
    // radiance-cache training records (NrcShade::rec, 8 float4 per vertex): the
    // shadow stage writes an unoccluded NEE contribution into float4 7
    float4* nrc = nullptr;
};
#define MT_VREC_HIT 1u
#define MT_VREC_CHOSEN 2u
#define MT_VREC_VISIBLE 4u
#define MT_VREC_NEXT 8u

// Optional per-stage CUDA-event timing and traversal counters of a render.
struct Profiler {
    bool timing = false;
    bool counting = false;
    unsigned long long* d_counts = nullptr;  // [extend pops, inner, tris, shadow pops, inner, tris]
    std::vector<cudaEvent_t> pool;
    std::vector<std::pair<int, size_t>> marks;  // (stage, index of start event in pool)
    size_t used = 0;
    void begin(int stage, cudaStream_t st);
    void end(int stage, cudaStream_t st);
    cudaError_t collect(double* ms, uint64_t* launches);
    ~Profiler();
};

cudaError_t launch_trace(const DevScene& S, const mt_ray* rays, uint64_t n, mt_hit* hits, int query,
                         uint32_t* fetch, cudaStream_t st);
cudaError_t launch_brdf(const mt_brdf_query* q, uint64_t n, mt_brdf_result* out, cudaStream_t st);
cudaError_t launch_brdf_sample(const mt_brdf_sample_query* q, uint64_t n, mt_brdf_sample_result* out,
                               cudaStream_t st);
struct NrcShade;
// Optional batch settings beyond a plain band render.
struct BatchExtra {
    const NrcShade* nrc = nullptr;  // radiance-cache hooks of the shade stage
    uint32_t sample_base = 0;       // added to every path's sample index
    uint32_t scatter_mul = 0;       // nonzero: path p renders pixel (p * mul + add) mod W*H
    uint32_t scatter_add = 0;
    cudaEvent_t query_after = nullptr;  // cache queries wait for this event (the frame's training)
};

// Loads the render stages' kernels now (lazy module loading would load each at
// its first launch).
cudaError_t preload_render_kernels();

cudaError_t launch_batch(const DevScene& S, const PathState& P, const ShadowQueue& SQ,
                         const WaveBuffers& W, uint64_t g0, uint32_t n, uint32_t band_pix,
                         uint32_t pix_base, cudaStream_t st, uint64_t* launches, Profiler* prof,
                         const RecordBuffers* rec = nullptr, const BatchExtra* extra = nullptr);
cudaError_t launch_resolve(const DevScene& S, const WaveBuffers& W, uint32_t band_pix,
                           uint32_t pix_base, float* out, cudaStream_t st, Profiler* prof);
// k_resolve on caller planes (sample-major: plane[s * npix + j]) for the
// mt_resolve_batch test entry; writes npix RGB triples to out.
cudaError_t launch_resolve_planes(const float* sr, const float* sg, const float* sb, uint32_t npix, uint32_t spp,
                                  int enable, float k, int debug_mode, float* out, cudaStream_t st);
// SM count of the current device (cached per device).
int device_sm_count();

// True when S.debug_mode ends with WaitForRender's heatmap post-processing.
bool debug_needs_post(int mode);
// Heatmap post-processing of a whole W*H image (scratch: one device word).
cudaError_t launch_debug_post(float* img, uint64_t npix, int mode, uint32_t* scratch, cudaStream_t st);

// Host BVH builder (mt_bvh.cpp).
int build_bvh(const float* positions, uint32_t num_triangles, uint32_t max_triangles,
              uint32_t cfg_max_depth, std::vector<mt_bvh_node>& nodes,
              std::vector<uint32_t>& indices, std::string& err);

}  // namespace mt
