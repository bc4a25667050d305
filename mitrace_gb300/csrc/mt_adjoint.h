// mt_adjoint.h - buffers and launchers of the path-replay adjoint.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mt_kernels.h"

#define MT_GRAD_MAX_BOUNCES 16

namespace mt {

struct GradParams {
    const float* target;       // W*H*3, or nullptr when d_image is given
    const float* d_image;      // W*H*3 dL/d(image), or nullptr for the L2 loss
    float* loss;               // 1
    float* d_base;             // materials * 3
    float* d_rough;            // materials
    float* d_metal;            // materials
    float* d_light;            // lights
    float* d_texels;           // RGB32F base-colour textures, or nullptr
    const long long* texel_off;  // per texture: float offset into d_texels, or -1
    float4* pix;               // per band pixel: (mean, threshold, 2 / kept, -), (residual rgb, -)
    uint32_t smem_materials;   // materials reduced in shared memory (0: global atomics)
    uint32_t smem_lights;
    uint32_t* order;           // per replayed path of a batch: path indices grouped by vertex count
    uint32_t* bins;            // kAdjointBins counts, then kAdjointBins cursors
};
// paths of a batch are processed grouped by vertex count (0..MT_GRAD_MAX_BOUNCES)
// so that a warp's threads walk equally long paths; the last bin holds the
// paths without a gradient (firefly-rejected samples)
constexpr uint32_t kAdjointBins = MT_GRAD_MAX_BOUNCES + 2;

cudaError_t launch_grad_pixel(const DevScene& S, const WaveBuffers& W, uint32_t band_pix, uint32_t pix_base,
                              const float* image, const GradParams& G, cudaStream_t st);
cudaError_t launch_adjoint(const DevScene& S, const GradParams& G, const RecordBuffers& R, const WaveBuffers& W,
                           uint64_t g0, uint32_t n, uint32_t band_pix, cudaStream_t st);

}  // namespace mt
