// mt_nrc.h - neural radiance cache: network buffers, the render-stage hooks and
// the launchers of its BF16 tensor-core kernels (mt_nrc.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mt_kernels.h"

namespace mt {

// Network dimensions.  The output layer is padded to 8 rows in the weight
// blob (16 in the kernels' shared-memory operands); rows 3.. stay zero.
constexpr int kNrcIn = 80;
constexpr int kNrcW = 64;
constexpr int kNrcOutPad = 8;
constexpr int kNrcParams = 80 * 64 + 3 * 64 * 64 + 64 * 3;
// BF16 weight blob: byte for byte the shared-memory operands of the tensor-core
// kernels (W_l as N = out rows x K = in, canonical K-major core matrices of 8
// rows x 16 bytes; the output layer padded to 16 rows, rows 3.. zero), so a
// kernel takes it with one bulk copy.  The backward pass reads the same bytes
// transposed.
constexpr int kNrcFwdElems = 64 * 80 + 3 * 64 * 64 + 16 * 64;  // 18,432 (36,864 bytes)

// Render-stage hooks of one wavefront batch.
#define MT_NRC_OFF 0
#define MT_NRC_QUERY 1  // end paths where NrcShade::end_at says, queue a cache query
#define MT_NRC_TRAIN 2  // record every vertex of full-length training paths
struct NrcShade {
    int mode = MT_NRC_OFF;
    uint32_t end_at = MT_NRC_END_AFTER_DIFFUSE;  // mt_nrc_config::end_at
    float rough_min = 0.3f;
    float lo[3] = {0, 0, 0};       // world box lower corner
    float inv_ext[3] = {1, 1, 1};  // 1 / world box extent
    // QUERY: query records, 6 float4 each: the 5 feature float4 of the header
    //        and (throughput rgb, path index bits).
    // TRAIN: vertex records of path p, bounce k at rec[(p * bounces + k) * 8]:
    //        the 6 float4 of a query record, (radiance collected before the
    //        vertex's NEE, 1 = recorded) and the vertex's NEE contribution when
    //        its shadow ray was unoccluded (written by the shadow stage, else 0).
    float4* rec = nullptr;
    uint32_t* count = nullptr;  // QUERY: queries appended
    // QUERY: bf16 forward weight blob; queries are also added to *total.
    const void* net = nullptr;
    uint32_t* total = nullptr;
    int* err = nullptr;  // device error word (MT_ERRBIT_TIMEOUT)
    // TRAIN: training samples (5 feature float4 + target float4 each).
    float4* samples = nullptr;
    uint32_t* sample_count = nullptr;
    uint32_t sample_cap = 0;
    // TRAIN: upper bound on the radiance a vertex's suffix adds to its path
    // (per channel, before the division by throughput); 0 = none.
    float target_cap = 0.0f;
};

// Cache queries of a batch: adds throughput * max(cache, 0) to P.indirect.
cudaError_t launch_nrc_query(const void* net, const PathState& P, const float4* rec, const uint32_t* count,
                             uint32_t capacity, uint32_t* total, int* err, cudaStream_t st);
// Training targets of a batch of training paths -> samples, placed in path
// order (scratch: n uint32 for the per-path counts and offsets).
cudaError_t launch_nrc_targets(const PathState& P, const NrcShade& N, uint32_t n, uint32_t bounces,
                               uint32_t* scratch, cudaStream_t st);
// Plain inference into out (n x 3).
cudaError_t launch_nrc_infer(const void* net, const float* features, uint32_t n, float* out, int* err,
                             cudaStream_t st);
cudaError_t launch_nrc_encode(const float* features, uint32_t n, float* out, cudaStream_t st);

// One training step.  Rows r < rows read sample fmix32(step * rows + r) mod
// *count of the (features, targets) arrays when count is not null (random
// draws with replacement, step = the device step counter; an empty set trains
// on nothing), else sample r.  The step number lives on the device so that a
// frame's steps can be replayed as one CUDA graph.  feat: the 5 feature float4 of sample
// i start at feat[i * fstride]; targets: tstride floats per sample (rgb first).
struct NrcTrainArgs {
    const float4* feat;
    uint32_t fstride;  // float4 per sample in feat
    const float* targets;
    uint32_t tstride;
    const uint32_t* count;
    uint32_t count_cap;  // samples the arrays hold (*count may run past it)
    uint32_t rows;
};
struct NrcOptimizer {
    float* master;      // kNrcParams fp32 weights
    float* m;           // Adam first moments
    float* v;           // Adam second moments
    float* partial;     // splits x kNrcParams weight-gradient partial sums (one per training CTA)
    void* fwd;          // bf16 blob of the trained weights
    void* infer;        // bf16 blob the renderer queries (moving average)
    float* ema;         // fp32 moving average (zero-started, bias-corrected on use)
    float ema_decay;    // 0: infer = trained weights
    uint32_t max_rows;  // rows of a step at most
    uint32_t max_splits;  // training CTAs (gradient partials) at most
    float lr, beta1, beta2, eps;
    uint64_t step;      // Adam steps taken (host copy)
    uint32_t* d_step;   // Adam steps taken (device; the kernels' bias corrections and sample draws)
    uint32_t* d_done;   // Adam blocks finished with the current step (the last one advances d_step)
    int* err;           // device error word (MT_ERRBIT_TIMEOUT)
};
cudaError_t launch_nrc_train_step(NrcOptimizer& O, const NrcTrainArgs& a, float* loss, float* grad_out,
                                  cudaStream_t st);
// Sets the kernels' shared-memory limits (before any stream capture).
cudaError_t nrc_prepare();
// Writes the bf16 blobs from the fp32 master weights (and restarts the average).
cudaError_t launch_nrc_publish(const NrcOptimizer& O, cudaStream_t st);
// running mean: accum += (frame - accum) / (index + 1)
cudaError_t launch_nrc_blend(float* accum, const float* frame, uint64_t n, uint32_t index, cudaStream_t st);

}  // namespace mt
