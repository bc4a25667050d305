/*
 * mitrace_gpu.h - C ABI of the GB300 (sm_103a) path tracer that stands in for
 * MiTrace's Tracer::Tracer render entry point.
 *
 * Everything crossing this boundary is plain C: POD structs, raw pointers and
 * sizes.  No exception, C++ type or torch type crosses it.  Every function
 * returns an mt_status (MT_OK on success); mt_last_error() gives a
 * human-readable message for the last failure on the calling thread.
 *
 * Reference interface that each group replaces (paths inside the MiTrace
 * project):
 *   mt_create / mt_destroy   Tracer::Tracer(shared_ptr<RenderBuffer>, const Scene&)
 *                            src/Tracer/Tracer.hpp:121, Tracer.cpp:633-640, plus the
 *                            Scene::Scene data it reads (src/Scene/Scene.hpp:30)
 *   mt_start                 Tracer::StartRender()     Tracer.hpp:124, Tracer.cpp:718-779
 *   mt_wait                  Tracer::WaitForRender()   Tracer.hpp:125, Tracer.cpp:781-799
 *   mt_kill                  Tracer::KillRender()      Tracer.hpp:126, Tracer.cpp:801-804
 *   mt_get_stats             Tracer::GetStats()        Tracer.hpp:127, Tracer.cpp:806-821
 *   mt_is_done               Tracer::IsDone()          Tracer.hpp:128, Tracer.cpp:823-828
 *   mt_trace_rays*           Tracer::IntersectScene()  src/Tracer/Intersect.hpp:10,
 *                            Intersect.cpp:201-219 (closest hit) and the shadow-ray
 *                            use of it at Tracer.cpp:317-322 (any hit)
 *   mt_brdf_batch            Tracer::BRDF::EvaluateBRDF/DiffusePdf/SpecularPdf
 *                            src/Tracer/BRDF.hpp:52-97
 *   mt_bvh_build             Scene::BVH::BVH(const Mesh&, ...) src/Scene/BVH.hpp:135,
 *                            BVH.cpp:274-282 (host builder, same topology)
 */
#ifndef MITRACE_GPU_H
#define MITRACE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MT_ABI_VERSION 1

typedef enum mt_status {
    MT_OK = 0,
    MT_ERR_CUDA = 1,     /* a CUDA runtime call failed */
    MT_ERR_OOM = 2,      /* device or host allocation failed */
    MT_ERR_INVALID = 3,  /* bad argument or malformed scene */
    MT_ERR_TIMEOUT = 4,  /* a bounded wait ran out */
    MT_ERR_KILLED = 5,   /* the render was cancelled with mt_kill */
    MT_ERR_STATE = 6     /* call not valid in the handle's current state */
} mt_status;

/* ------------------------------------------------------------------------ */
/* Scene description (host memory, borrowed for the duration of mt_create).  */
/* ------------------------------------------------------------------------ */

/* One flattened BVH node, 32 bytes, same meaning as Scene::BVHNode
 * (src/Scene/BVH.hpp:74-119): an AABB and either two child node indices
 * (inner node) or {first index | 0x80000000, count} into the index array. */
typedef struct mt_bvh_node {
    float lo[3];
    float hi[3];
    uint32_t a; /* child A, or leaf: first index | MT_BVH_LEAF_BIT */
    uint32_t b; /* child B, or leaf: triangle count                */
} mt_bvh_node;

#define MT_BVH_LEAF_BIT 0x80000000u

/* A de-indexed triangle mesh as Scene::Mesh holds it (src/Scene/Mesh.hpp:13-42,
 * Mesh.cpp:24-41): 3 vertices per triangle, in triangle order. */
typedef struct mt_mesh_desc {
    uint32_t num_triangles;
    const float* positions; /* 9 * num_triangles floats (required)          */
    const float* normals;   /* 9 * num_triangles floats (required)          */
    const float* uv0;       /* 6 * num_triangles floats, or NULL            */
    /* Optional prebuilt BVH in the reference layout.  When NULL the library
     * builds one on the host with mt_bvh_build semantics, if the mesh has more
     * than bvh_max_triangles triangles and BVHs are enabled (Mesh.cpp:37-40).
     * mt_create rejects (MT_ERR_INVALID) a prebuilt BVH whose inner nodes'
     * children are not adjacent (b == a + 1, as the reference's builder lays
     * them out), that has 2^31 nodes or more, a node or leaf range out of
     * bounds, or a depth beyond the traversal stack. */
    const mt_bvh_node* bvh_nodes;
    uint32_t num_bvh_nodes;
    const uint32_t* bvh_indices;
    uint32_t num_bvh_indices;
} mt_mesh_desc;

/* Texture: Scene::Texture + Scene::Image (src/Scene/Texture.hpp, Image.hpp).
 * Texels are RGB8 (alpha dropped, Image.cpp:93) or, for the float
 * environment-map extension, RGB32F.  Exactly one of rgb8 / rgb32f is set. */
typedef struct mt_texture_desc {
    uint32_t width;
    uint32_t height;
    const uint8_t* rgb8;
    const float* rgb32f;
    int32_t filter;    /* 0 nearest, 1 linear (Image::FilterMode)     */
    float offset[2];   /* KHR_texture_transform offset (Texture.cpp:12-15) */
    float scale[2];    /* KHR_texture_transform scale                 */
} mt_texture_desc;

#define MT_FILTER_NEAREST 0
#define MT_FILTER_LINEAR 1

/* Scene::Material (src/Scene/Material.hpp:11-136).  Texture slots are indices
 * into mt_scene_desc.textures or -1. */
typedef struct mt_material_desc {
    float base_color_factor[4];
    float emissive_factor[3];
    float normal_scale;
    float metallic_factor;
    float roughness_factor;
    float occlusion_strength;
    int32_t base_color_tex;
    int32_t metallic_roughness_tex;
    int32_t normal_tex;
    int32_t occlusion_tex;
    int32_t emissive_tex;
} mt_material_desc;

/* Scene::MeshInstance (src/Scene/Mesh.hpp:44-72): mesh, material and a
 * column-major model-to-world matrix (glm::mat4 layout). */
typedef struct mt_instance_desc {
    uint32_t mesh;
    uint32_t material;
    float transform[16];
} mt_instance_desc;

/* Scene::Light (src/Scene/Light.hpp:14-66) after its constructor ran:
 * color already multiplied by intensity, cone angles as cosines, direction
 * = rotation applied to (0,0,-1). */
typedef struct mt_light_desc {
    int32_t type; /* MT_LIGHT_* */
    float position[3];
    float color[3];
    float point_size;
    float spot_inner_cos;
    float spot_outer_cos;
    float direction[3];
} mt_light_desc;

#define MT_LIGHT_POINT 0
#define MT_LIGHT_DIRECTIONAL 1
#define MT_LIGHT_SPOT 2
#define MT_LIGHT_AREA 3

/* Scene::Camera (src/Scene/Camera.hpp:10-36). */
typedef struct mt_camera_desc {
    int32_t type; /* 0 perspective, 1 orthographic */
    float camera_to_world[16];
    float yfov;        /* radians */
    float aspect;      /* camera aspect ratio */
    float ortho_size[2];
} mt_camera_desc;

typedef struct mt_scene_desc {
    uint32_t num_meshes;
    const mt_mesh_desc* meshes;
    uint32_t num_instances;
    const mt_instance_desc* instances;
    uint32_t num_materials;
    const mt_material_desc* materials;
    uint32_t num_textures;
    const mt_texture_desc* textures;
    uint32_t num_lights;
    const mt_light_desc* lights;
    mt_camera_desc camera;
    int32_t env_texture; /* index into textures, or -1 (Scene::SampleSkybox) */
} mt_scene_desc;

/* The hot-path subset of Config::ConfigOptions (src/CLI/Config.hpp:43-80),
 * passed explicitly instead of through the global singleton. */
typedef struct mt_config {
    uint32_t width;
    uint32_t height;
    uint32_t samples;
    uint32_t bounces;
    float ev_exposure;
    float hdri_primary_intensity;
    float hdri_secondary_intensity;
    float emission_base_intensity;
    int32_t bvh_disable;
    uint32_t bvh_max_triangles;
    uint32_t bvh_max_depth;
    int32_t firefly_enable;
    float firefly_threshold;
    float terminate_energy;
    int32_t debug_mode; /* MT_DEBUG_* (Config::DebugMode), 0 = DebugNone */
    uint32_t reserved0;
    uint64_t seed;      /* seeds the counter-based RNG */
    uint32_t reserved[8];
} mt_config;

/* Debug render modes, the values of Config::DebugMode (src/CLI/Config.hpp:16-40).
 * A sample of a debug render is ProcessDebugRay's value (Tracer.cpp:366-488)
 * instead of the tonemapped radiance; samples are averaged (with the firefly
 * clamp when enabled) as usual, and the modes marked (h) end with
 * WaitForRender's heatmap post-processing over the whole image
 * (Tracer.cpp:695-716: intensity / maximum intensity, colour ramp or grey).
 * MT_DEBUG_COLOR_PER_MESH hashes the instance index (the reference hashes the
 * low bits of the MeshInstance's address).  PIXEL_STANDARD_DEVIATION and
 * FIREFLY_ELIMINATION render the normal samples; the firefly clamp then
 * replaces each pixel's samples with the sigma of their intensities or the
 * number of samples it dropped (Tracer.cpp:516-523, 537-544) before the
 * heatmap.  With firefly_enable 0 the clamp never runs and they heatmap the
 * plain image, as the reference does.  Debug modes work with mt_render_device and
 * mt_start/mt_wait; the adjoint, the radiance cache and the allocation-free
 * entry point reject them. */
#define MT_DEBUG_NONE 0
#define MT_DEBUG_PRIMARY_BVH_TESTS 1          /* (h) */
#define MT_DEBUG_TOTAL_BVH_TESTS 2            /* (h) */
#define MT_DEBUG_PRIMARY_TRIANGLE_TESTS 3     /* (h) */
#define MT_DEBUG_TOTAL_TRIANGLE_TESTS 4       /* (h) */
#define MT_DEBUG_ALBEDO 5
#define MT_DEBUG_METALLIC_ROUGHNESS 6
#define MT_DEBUG_GEOMETRIC_NORMAL 7
#define MT_DEBUG_SHADING_NORMAL 8
#define MT_DEBUG_DIRECT_ONLY 9
#define MT_DEBUG_INDIRECT_ONLY 10
#define MT_DEBUG_EMISSION 11
#define MT_DEBUG_COLOR_PER_MESH 12
#define MT_DEBUG_COLOR_PER_TRIANGLE 13
#define MT_DEBUG_COLOR_PER_BOUNDING_VOLUME 14
#define MT_DEBUG_BOUNCES 15                   /* (h) */
#define MT_DEBUG_DEPTH 16                     /* (h, grey) */
#define MT_DEBUG_FIRST_HIT_FRESNEL 17
#define MT_DEBUG_FIRST_HIT_BRDF 18            /* (h, grey) */
#define MT_DEBUG_FIRST_HIT_PDF 19
#define MT_DEBUG_REFLECTED_DIRECTION 20
#define MT_DEBUG_PIXEL_STANDARD_DEVIATION 21  /* (h, grey) */
#define MT_DEBUG_FIREFLY_ELIMINATION 22       /* (h) */
#define MT_DEBUG_COUNT 23

/* Fills *cfg with the reference defaults (Config.hpp:50-70). */
void mt_config_defaults(mt_config* cfg);

/* ------------------------------------------------------------------------ */
/* Handle lifecycle and the Tracer-equivalent render API.                   */
/* ------------------------------------------------------------------------ */

typedef struct mt_handle mt_handle;

typedef struct mt_stats {
    float progress;                 /* 0..1                              */
    float time_elapsed;             /* seconds since mt_start            */
    float estimated_time_remaining; /* seconds                           */
    float reserved;
    uint64_t rays;                  /* path + shadow rays (Tracer.cpp:146,319), counted
                                       as the reference counts them: a shadow ray
                                       whose contribution is exactly zero counts,
                                       although it is not traced (its visibility
                                       cannot change the image) */
    uint64_t samples;               /* camera samples (Tracer.cpp:342)   */
} mt_stats;

/* Uploads the scene to the current CUDA device, builds missing BVHs on the
 * host, and allocates the render state.  *out is NULL on failure. */
mt_status mt_create(const mt_scene_desc* scene, const mt_config* cfg, mt_handle** out);
void mt_destroy(mt_handle* h);

/* Device memory a destroyed handle used stays cached by the library for the
 * next handle on the same device (at most MT_DEVICE_CACHE_BYTES per device,
 * default an eighth of its memory; 0 turns the cache off), so that a new
 * handle does not pay for allocating its render state again.  This call gives
 * every cached block back to the driver.  No counterpart in the reference. */
void mt_release_cached_memory(void);

/* Starts an asynchronous render on the handle's own stream and returns.
 * Calling it while a render is running returns MT_ERR_STATE. */
mt_status mt_start(mt_handle* h);
/* Blocks until the render ends; copies the W*H*3 float RGB image (row-major,
 * y*W+x, tonemapped, as RenderBuffer holds it) into rgb_out when it is not
 * NULL.  Returns MT_ERR_KILLED if mt_kill stopped the render. */
mt_status mt_wait(mt_handle* h, float* rgb_out);
/* Cooperative cancel, callable from any thread (Tracer.cpp:801-804). */
mt_status mt_kill(mt_handle* h);
/* Thread-safe progress/counters, callable while a render runs. */
mt_status mt_get_stats(const mt_handle* h, mt_stats* out);
/* 1 when a render was started and has finished, else 0. */
int mt_is_done(const mt_handle* h);

/* Seed of the counter-based RNG for the handle's later renders (the value
 * mt_config.seed gave at mt_create).  The reference reseeds every tile of every
 * render from std::random_device (Tracer.cpp:564); here a render's random
 * numbers are a function of (seed, pixel, sample, bounce), so a caller that
 * wants independent images changes the seed between them.  Not while an
 * asynchronous render runs. */
mt_status mt_set_seed(mt_handle* h, uint64_t seed);

/* Render into a caller-owned DEVICE buffer (W*H*3 floats) enqueued on the
 * given CUDA stream (0 = the legacy default stream).  Returns when the work is
 * enqueued; mt_get_stats reports its rays once the stream has finished it.
 * Part of the work (each bounce's shadow rays) runs on a second stream of the
 * handle, forked from and joined back into the given stream by events, so the
 * render completes on that stream as one unit (also under stream capture). */
mt_status mt_render_device(mt_handle* h, float* d_rgb_out, void* cuda_stream);

/* Render of image rows [row0, row1) into a caller-owned DEVICE buffer holding
 * the whole W*H*3 image (only those rows are written), enqueued on
 * cuda_stream: Tracer::RenderBlock (Tracer.cpp:550-616) over the blocks of
 * those rows.  A pixel's samples and random numbers do not depend on the band,
 * so bands of one image rendered on several GPUs (one handle each) assemble
 * the image mt_render_device renders.  Heatmap debug modes, which normalise
 * over the whole image, need row0 = 0 and row1 = height. */
mt_status mt_render_rows_device(mt_handle* h, uint32_t row0, uint32_t row1, float* d_rgb_out, void* cuda_stream);

/* Allocation-free render of rows [row0, row1) into a caller-owned DEVICE
 * buffer holding the whole W*H*3 image (only those rows are written), enqueued
 * on cuda_stream (0 = the legacy default stream).  No counterpart in the
 * reference: it exists for callers that must not allocate GPU memory while
 * they render (a fixed memory budget reserved up front, a frame loop or host
 * callback that must not block in the allocator, an allocator hooked by
 * another library).  All scratch lives in one static device array of
 * MT_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * exit; one call renders at most MT_NOALLOC_MAX_PATHS paths
 * ((row1 - row0) * width * samples), larger requests return MT_ERR_INVALID.
 * Calls share that array: work of two calls that overlaps on the GPU races, so
 * serialise them.  The first call on a device looks up the array's address;
 * make it before any stream capture.  Same kernels and results as
 * mt_render_device for those rows.  mt_get_stats counts the call's samples
 * but not its rays (their counters stay in the shared array). */
#define MT_NOALLOC_MAX_PATHS 65536u
#define MT_NOALLOC_SCRATCH_BYTES (16u << 20)
mt_status mt_render_rows_noalloc(mt_handle* h, uint32_t row0, uint32_t row1, float* d_rgb_out,
                                 void* cuda_stream);

/* ------------------------------------------------------------------------ */
/* Path-replay adjoint (no reference counterpart: gradient of an image loss). */
/* ------------------------------------------------------------------------ */

/* Device buffers of mt_render_grad.  Gradients are ADDED to d_* (zero them
 * first).  d_texels covers the texels of every RGB32F texture that some
 * material uses as its base-colour texture, W*H*3 floats each, concatenated in
 * texture-index order; pass NULL to skip texel gradients.  With d_image set,
 * the gradient that flows into the image is d_image itself (any loss of the
 * caller's); target may then be NULL and loss is not written. */
typedef struct mt_grad_buffers {
    const float* target; /* W*H*3 target image                                  */
    float* image;        /* W*H*3 out: the rendered image                       */
    float* loss;         /* 1 float out: sum over pixels/channels of (image-target)^2 */
    float* d_base;       /* num_materials*3: dL/d base_color_factor rgb          */
    float* d_roughness;  /* num_materials: dL/d roughness_factor                 */
    float* d_metallic;   /* num_materials: dL/d metallic_factor                  */
    float* d_light;      /* num_lights: dL/d s, light colour scaled by s at s=1  */
    float* d_texels;     /* see above, or NULL                                   */
    const float* d_image; /* W*H*3 dL/d(image), or NULL for the L2 loss above   */
} mt_grad_buffers;

#define MT_GRAD_MAX_BOUNCES 16

/* Parameter updates between renders of an inverse-rendering loop, without
 * re-uploading the scene (blocking; not while mt_start runs).  The counts, the
 * materials' texture slots and the lights' types must stay as uploaded. */
mt_status mt_update_materials(mt_handle* h, const mt_material_desc* materials, uint32_t n);
mt_status mt_update_lights(mt_handle* h, const mt_light_desc* lights, uint32_t n);
/* Replaces all texels of texture index (same size and format as uploaded:
 * W*H*3 bytes for RGB8, W*H*3 floats for RGB32F), host memory. */
mt_status mt_update_texture(mt_handle* h, uint32_t index, const void* texels);

/* Renders the image (same estimator and counter RNG as mt_render_device) and
 * accumulates dL/dparameters by replaying every path from its seed.  Sampling
 * decisions and pdfs, light-pick probabilities, the energy cut-off and the
 * firefly mask are held constant.  Needs bounces <= MT_GRAD_MAX_BOUNCES.
 * Enqueued on cuda_stream (0 = the legacy default stream). */
mt_status mt_render_grad(mt_handle* h, const mt_grad_buffers* g, void* cuda_stream);

/* ------------------------------------------------------------------------ */
/* Neural radiance cache (no reference counterpart).                        */
/* ------------------------------------------------------------------------ */

/* The cache is an MLP, MT_NRC_INPUTS -> 4 hidden layers of MT_NRC_WIDTH (ReLU)
 * -> RGB, without bias terms (the constant-1 input lanes act as biases), BF16
 * weights and activations with FP32 accumulation.  Its input is the encoding
 * of a 20-float feature record (five float4):
 *   f0 = (position normalised to the scene's world box, roughness)
 *   f1 = (outgoing direction wo = -ray direction,
 *         bounce budget left (bounces - 1 - k) / (bounces - 1) at bounce k)
 *   f2 = (shading normal,
 *         cut-off headroom clamp(log2(|totalEnergy| / terminate_energy) / 16, 0, 1))
 *   f3 = (diffuse albedo base*(1-metallic), unused)
 *   f4 = (specular albedo mix(0.04, base, metallic), unused)
 * Encoding (80 lanes): 12 triangle-wave octaves per position axis (36),
 * real spherical harmonics through band 3 of wo (16) and of the normal (16),
 * roughness (1), diffuse (3) and specular (3) albedo, the bounce budget and
 * the cut-off headroom (2), three constant 1s.  The two path-state lanes let
 * one network serve vertices whose remaining paths the bounce limit and the
 * energy cut-off truncate differently.
 * Parameters, FP32 master copy: W0 (64 x 80), W1, W2, W3 (64 x 64), W4 (3 x
 * 64), each row-major [out][in] like a torch Linear weight, concatenated. */
#define MT_NRC_INPUTS 80u
#define MT_NRC_WIDTH 64u
#define MT_NRC_FEATURES 20u
#define MT_NRC_PARAMS (80u * 64u + 3u * 64u * 64u + 64u * 3u) /* 17,600 */

typedef struct mt_nrc_config {
    uint32_t train_paths;  /* full-length training paths traced per frame (65,536) */
    uint32_t train_batch;  /* training samples (path vertices) per Adam step (16,384) */
    uint32_t train_steps;  /* Adam steps per frame (128; replayed as one CUDA graph) */
    uint32_t spp;          /* cached-render samples per pixel per frame (4) */
    float learning_rate;   /* Adam step size (1e-2) */
    float beta1, beta2;    /* Adam moment decays (0.9, 0.99) */
    float epsilon;         /* Adam denominator guard (1e-15) */
    float rough_min;       /* a vertex with roughness >= this is diffuse-ish (0.3) */
    uint32_t seed;         /* weight initialisation and training-path seed */
    float ema_decay;       /* the renderer queries an exponential moving average
                              of the trained weights (bias-corrected) with this
                              decay; 0 queries the trained weights themselves (0.9) */
    uint32_t end_at;       /* where a cached path ends (MT_NRC_END_*) */
    float target_cap;      /* upper bound, per channel, on the radiance times
                              2^-ev_exposure that the rest of a training path
                              adds to its vertex's target; <= 0: none (0.5).
                              The reference tonemaps every sample (ACES, which
                              saturates: 0.62 at 0.5, 0.92 at 2, 1.03 at
                              infinity) and its firefly rule drops rare
                              outliers, so the plain estimate hardly contains
                              rare very bright suffixes (a sun reached after a
                              diffuse bounce); uncapped, the cache learns their
                              mean and the cached image turns brighter the
                              longer it trains */
    uint32_t reserved[3];
} mt_nrc_config;

/* mt_nrc_config::end_at.
 * AFTER_DIFFUSE: the path ends at the first vertex after a diffuse-ish one
 *   (bounce >= 1) and the cache stands for that vertex's whole outgoing
 *   radiance, its next-event estimate included.
 * AT_DIFFUSE: the path ends at its first diffuse-ish vertex (the primary one
 *   included) after that vertex's next-event estimate, and the cache stands
 *   for the radiance the vertex reflects from the rest of its path (the
 *   estimate excluded).  The cache is trained for the mode it serves. */
#define MT_NRC_END_AFTER_DIFFUSE 0u
#define MT_NRC_END_AT_DIFFUSE 1u

/* Counters of the cache (mt_nrc_get_stats synchronizes the device). */
typedef struct mt_nrc_stats {
    uint64_t frames;        /* mt_nrc_frame calls since mt_nrc_enable */
    uint64_t adam_steps;    /* optimizer steps since enable / set_params */
    uint32_t train_samples; /* vertices recorded by the last frame's training paths */
    uint32_t queries;       /* cache queries of the last frame's render */
    float train_loss;       /* mean relative L2 loss of the last frame's steps */
    float reserved[3];
} mt_nrc_stats;

void mt_nrc_config_defaults(mt_nrc_config* c);
/* Allocates the cache on the handle and initialises its weights (Xavier
 * uniform from seed) and Adam state.  Calling it again re-initialises. */
mt_status mt_nrc_enable(mt_handle* h, const mt_nrc_config* c);
/* One frame of the cached renderer, enqueued on cuda_stream:
 *  1. trace train_paths full-length plain paths from random pixels, record
 *     every vertex's features and the radiance the rest of its path carried
 *     back ((path total - total before the vertex's NEE) / throughput; with
 *     MT_NRC_END_AT_DIFFUSE the vertex's own NEE is subtracted as well; the
 *     numerator capped at target_cap * 2^ev_exposure per channel);
 *  2. take train_steps Adam steps on batches of those vertices (relative L2
 *     loss |y - t|^2 / (y^2 + 0.01), y held constant in the denominator);
 *  3. if d_accum is not NULL, render spp samples per pixel in which a path
 *     ends where end_at says and adds throughput * max(cache(vertex), 0)
 *     instead of tracing on; resolve them
 *     like mt_render_device (per-sample ACES, firefly clamp over the frame's
 *     spp) and fold the frame into d_accum (W*H*3) as a running mean:
 *     accum += (frame - accum) / (accum_index + 1).
 * Frames draw distinct random numbers (sample indices continue across frames).
 * Steps 1 and 2 run on a stream of the cache beside step 3, whose cache
 * queries wait for them; the frame completes on cuda_stream. */
mt_status mt_nrc_frame(mt_handle* h, float* d_accum, uint32_t accum_index, void* cuda_stream);
mt_status mt_nrc_get_stats(mt_handle* h, mt_nrc_stats* out);
/* Copies the FP32 master parameters out / in (MT_NRC_PARAMS floats, host).
 * Setting them resets the Adam moments, the step count and the moving average. */
mt_status mt_nrc_get_params(mt_handle* h, float* params);
mt_status mt_nrc_set_params(mt_handle* h, const float* params);
/* Cache outputs for n feature records (device buffers: n*20 floats in, n*3
 * out; the records 16-byte aligned), from the weights the renderer queries
 * (see ema_decay). */
mt_status mt_nrc_infer(mt_handle* h, const float* d_features, uint32_t n, float* d_rgb, void* cuda_stream);
/* One Adam step on n samples (device buffers: n*20 feature floats, n*3 target
 * floats).  d_loss (1 float, may be NULL) receives the batch's mean relative
 * L2 loss before the step; d_grad (MT_NRC_PARAMS floats, may be NULL) the
 * gradient the step used.  n <= 4 * train_batch. */
mt_status mt_nrc_train_step(mt_handle* h, const float* d_features, const float* d_targets, uint32_t n,
                            float* d_loss, float* d_grad, void* cuda_stream);
/* The FP32 input encoding of n feature records (n*20 floats in, n*80 out); no
 * handle needed. */
mt_status mt_nrc_encode(const float* d_features, uint32_t n, float* d_encoded, void* cuda_stream);

/* ------------------------------------------------------------------------ */
/* Ray queries (test and microbench entry points).                          */
/* ------------------------------------------------------------------------ */

/* 32-byte ray.  tmax is only read by any-hit queries: the ray counts as
 * occluded when the closest-hit semantics of IntersectScene would report a
 * hit at world distance <= tmax (Tracer.cpp:322). */
typedef struct mt_ray {
    float origin[3];
    float tmax;
    float direction[3];
    float pad;
} mt_ray;

/* 32-byte hit record of the closest hit (RayHit, src/Tracer/Ray.hpp:24-43).
 * instance == MT_NO_HIT on a miss.  bvh_tests / tri_tests are the counters of
 * the winning instance only, as RayHit carries them (Intersect.cpp:186-187);
 * they are filled only by the counting query variant. */
typedef struct mt_hit {
    float distance; /* world-space distance (Intersect.cpp:182)          */
    float u;        /* barycentric weight of vertex 1                     */
    float v;        /* barycentric weight of vertex 2                     */
    uint32_t instance;
    uint32_t triangle;
    uint32_t bv_index;
    uint32_t bvh_tests;
    uint32_t tri_tests;
} mt_hit;

#define MT_NO_HIT 0xFFFFFFFFu

#define MT_QUERY_CLOSEST 0
#define MT_QUERY_ANY 1          /* writes occluded (1) / visible (0) into hit.instance */
#define MT_QUERY_CLOSEST_COUNT 2 /* closest hit plus bvh/triangle test counters */
/* Closest hit; bv_index / bvh_tests / tri_tests then hold the inner-node
 * expansions, BVH pops and triangle tests summed over ALL instances the ray
 * visited (the work the traversal did, not only the winner's counters). */
#define MT_QUERY_CLOSEST_TOTALS 3

/* Host buffers: copies rays in, runs the query, copies hits out (blocking). */
mt_status mt_trace_rays(mt_handle* h, const mt_ray* rays, uint64_t n, mt_hit* hits, int query);
/* Device buffers on a caller stream (0 = the legacy default stream); does not block. */
mt_status mt_trace_rays_device(mt_handle* h, const mt_ray* d_rays, uint64_t n, mt_hit* d_hits,
                               int query, void* cuda_stream);

/* ------------------------------------------------------------------------ */
/* BRDF batch (test entry point).                                           */
/* ------------------------------------------------------------------------ */

/* One BRDF query: L, V, N unit-ish vectors plus material scalars. */
typedef struct mt_brdf_query {
    float L[3];
    float V[3];
    float N[3];
    float base_color[3];
    float roughness;
    float metallic;
} mt_brdf_query;

/* Output per query: EvaluateBRDF rgb, DiffusePdf, SpecularPdf. */
typedef struct mt_brdf_result {
    float f[3];
    float diffuse_pdf;
    float specular_pdf;
} mt_brdf_result;

/* Host buffers; needs no scene (h may be NULL). */
mt_status mt_brdf_batch(const mt_brdf_query* q, uint64_t n, mt_brdf_result* out);

/* One bounce sample of GeneratePath (Tracer.cpp:177-203, SampleGGXDirection
 * 49-72, cosine sampling 26-47) with its uniforms given: u[0] picks the lobe
 * (GGX when below the specular probability), u[1], u[2] draw the direction,
 * u[3], u[4] the cosine fallback of a GGX reflection below the surface. */
typedef struct mt_brdf_sample_query {
    float V[3];
    float N[3];
    float base_color[3];
    float roughness;
    float metallic;
    float u[5];
} mt_brdf_sample_query;

/* Sampled direction L, the mixture pdf (1-ps) DiffusePdf + ps SpecularPdf,
 * the specular probability ps, and the lobe: 0 cosine, 1 GGX, 2 GGX fell back
 * to cosine. */
typedef struct mt_brdf_sample_result {
    float L[3];
    float pdf;
    float specular_probability;
    int32_t lobe;
} mt_brdf_sample_result;

mt_status mt_brdf_sample_batch(const mt_brdf_sample_query* q, uint64_t n, mt_brdf_sample_result* out);

/* CleanupFireflies + averaging of RenderBlock (Tracer.cpp:490-548, 593-600)
 * on given samples (test entry point; the render's own resolve kernel):
 * samples_rgb holds npix pixels x spp samples x RGB, pixel-major, host memory;
 * rgb_out gets npix RGB means.  debug_mode MT_DEBUG_PIXEL_STANDARD_DEVIATION /
 * MT_DEBUG_FIREFLY_ELIMINATION give the clamp's sigma / dropped-sample count
 * per pixel (before WaitForRender's heatmap), as those modes do.  Needs no scene. */
mt_status mt_resolve_batch(const float* samples_rgb, uint32_t npix, uint32_t spp, int firefly_enable, float k,
                           int debug_mode, float* rgb_out);

/* ------------------------------------------------------------------------ */
/* Host BVH builder.                                                        */
/* ------------------------------------------------------------------------ */

/* Builds the BVH of one de-indexed mesh with the reference's split rule
 * (centroid mean, straddlers duplicated, child box = clipped parent) and its
 * flattening order.  max_depth is Config::bvhMaxDepth (the builder applies the
 * two "-1" steps of Mesh.cpp:40 and BVH.cpp:211 itself).  The arrays are
 * allocated by the library; free them with mt_bvh_free. */
mt_status mt_bvh_build(const float* positions, uint32_t num_triangles, uint32_t max_triangles,
                       uint32_t max_depth, mt_bvh_node** nodes, uint32_t* num_nodes,
                       uint32_t** indices, uint32_t* num_indices);
void mt_bvh_free(mt_bvh_node* nodes, uint32_t* indices);

/* ------------------------------------------------------------------------ */
/* Image output (RenderBuffer::GetPixelsRGB8 / SaveToFile*,                  */
/* src/Tracer/RenderBuffer.cpp:37-84).                                      */
/* ------------------------------------------------------------------------ */

/* Device: W*H*3 floats -> W*H*3 bytes, clamp(v * 255, 0, 255) truncated, as
 * FloatToU8 does (RenderBuffer.cpp:37-40).  Enqueued on cuda_stream. */
mt_status mt_image_rgb8(const float* d_rgb, uint32_t width, uint32_t height, uint8_t* d_rgb8,
                        void* cuda_stream);
/* Host: an 8-bit RGB PNG of rgb8 (rows top to bottom, as the RenderBuffer). */
mt_status mt_write_png(const char* path, const uint8_t* rgb8, uint32_t width, uint32_t height);
/* Host: a Radiance .hdr (RGBE) of the float image, as SaveToFileHDR writes the
 * RenderBuffer's (tonemapped) floats. */
mt_status mt_write_hdr(const char* path, const float* rgb, uint32_t width, uint32_t height);

/* ------------------------------------------------------------------------ */
/* Diagnostics.                                                             */
/* ------------------------------------------------------------------------ */

/* Per-stage profile of the wavefront render.  Stages are MT_STAGE_*. */
typedef struct mt_stage_profile {
    uint64_t launches;
    double milliseconds; /* summed CUDA-event time of the stage's launches   */
    uint64_t rays;       /* rays the stage traced (extend / shadow)          */
    uint64_t node_pops;  /* BVH stack pops, all instances (bvhTests)         */
    uint64_t inner_pops; /* pops that expanded an inner node (2 child boxes) */
    uint64_t tri_tests;  /* triangle tests, all instances (triangleTests)    */
} mt_stage_profile;

#define MT_STAGE_RAYGEN 0
#define MT_STAGE_EXTEND 1
#define MT_STAGE_SHADE 2
#define MT_STAGE_SHADOW 3
#define MT_STAGE_FINALIZE 4
#define MT_STAGE_RESOLVE 5
#define MT_NUM_STAGES 6

typedef struct mt_profile {
    mt_stage_profile stage[MT_NUM_STAGES];
} mt_profile;

/* timing: record CUDA events around every stage launch of later renders.
 * counting: later renders use traversal kernels that also tally node pops,
 * inner pops and triangle tests (slower; meant for an untimed pass). */
mt_status mt_profile_enable(mt_handle* h, int timing, int counting);
/* Synchronizes the handle's render and returns the accumulated profile. */
mt_status mt_profile_read(mt_handle* h, mt_profile* out);
mt_status mt_profile_reset(mt_handle* h);

const char* mt_last_error(void);
int mt_abi_version(void);
/* Number of kernel launches this handle issued since creation. */
uint64_t mt_kernel_launches(const mt_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* MITRACE_GPU_H */
