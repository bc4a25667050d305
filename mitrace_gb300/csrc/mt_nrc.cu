// mt_nrc.cu - neural radiance cache kernels.
//
// The cache maps a surface vertex (position, outgoing direction, normal,
// roughness, albedos) to the radiance the rest of its path would carry back.
// Network: 80 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU, no biases; BF16 weights and
// activations on the tensor cores with FP32 accumulation.
//
//   k_nrc_infer_tc fused encoding + 5 layers on tcgen05 (TMEM accumulators,
//                  operands in shared memory), 128-row tiles per warpgroup.
//   k_nrc_train_tc one training step's forward pass, relative-L2 loss
//                  gradient, backward pass and weight gradient on tcgen05:
//                  a CTA per 128-row tile, every product an M = 128 MMA into
//                  TMEM, the backward and weight-gradient operands read as
//                  transposed (MN-major) views of the forward ones; one
//                  gradient partial per CTA.
//   k_nrc_adam     sums the partials in a fixed order, Adam, and rewrites the
//                  BF16 weight blobs (the kernels' shared-memory operand image).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>

#include "mt_device.cuh"
#include "mt_nrc.h"

namespace mt {
namespace {

using bf16 = __nv_bfloat16;

// ---------------------------------------------------------------------------
// Layouts
// ---------------------------------------------------------------------------
// element offset of W_l in the blob, and of its (o, i) entry: core matrix
// (o / 8, i / 8) of the K-major operand, 8 x 8 elements each
__host__ __device__ constexpr int blob_off(int l) { return l == 0 ? 0 : 64 * 80 + (l - 1) * 64 * 64; }
__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? 80 : 64; }
__host__ __device__ constexpr int blob_index(int l, int o, int i)
{
    return blob_off(l) + ((o >> 3) * (layer_in(l) >> 3) + (i >> 3)) * 64 + (o & 7) * 8 + (i & 7);
}
__host__ __device__ constexpr int master_off(int l) { return l == 0 ? 0 : 5120 + (l - 1) * 4096; }
__host__ __device__ constexpr int layer_out(int l) { return l == 4 ? 3 : 64; }
static_assert(blob_off(4) + 16 * 64 == kNrcFwdElems, "forward blob size");
static_assert(master_off(4) + 3 * 64 == kNrcParams, "parameter count");

__device__ __forceinline__ void param_coords(int q, int& l, int& o, int& i)
{
    if (q < 5120) {
        l = 0;
        o = q / 80;
        i = q - o * 80;
    } else if (q < 17408) {
        const int r = q - 5120;
        l = 1 + r / 4096;
        const int s = r - (l - 1) * 4096;
        o = s >> 6;
        i = s & 63;
    } else {
        l = 4;
        const int r = q - 17408;
        o = r >> 6;
        i = r & 63;
    }
}

// ---------------------------------------------------------------------------
// Input encoding
// ---------------------------------------------------------------------------
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// Triangle wave of period 1 with values in [-1, 1].
__device__ __forceinline__ float tri_wave(float s)
{
    const float f = s - floorf(s);
    return fabsf(4.0f * f - 2.0f) - 1.0f;
}

// Lanes [0,36) (12 octaves per position axis), [68,75) and [77,80).
template <class Out>
__device__ __forceinline__ void encode_part0(float4 f0, float4 f3, float4 f4, Out out)
{
    const float p[3] = {clamp01(f0.x), clamp01(f0.y), clamp01(f0.z)};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float s = p[d];
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            out(d * 12 + j, tri_wave(s));
            s *= 2.0f;
        }
    }
    out(68, f0.w);
    out(69, f3.x);
    out(70, f3.y);
    out(71, f3.z);
    out(72, f4.x);
    out(73, f4.y);
    out(74, f4.z);
#pragma unroll
    for (int k = 77; k < 80; ++k) out(k, 1.0f);
}

// Real spherical harmonics of bands 0..3 of a unit vector (16 lanes from base).
template <class Out>
__device__ __forceinline__ void sh16(float x, float y, float z, int base, Out out)
{
    const float xx = x * x, yy = y * y, zz = z * z;
    out(base + 0, 0.28209479177387814f);
    out(base + 1, -0.48860251190291987f * y);
    out(base + 2, 0.48860251190291987f * z);
    out(base + 3, -0.48860251190291987f * x);
    out(base + 4, 1.0925484305920792f * x * y);
    out(base + 5, -1.0925484305920792f * y * z);
    out(base + 6, 0.94617469575756f * zz - 0.31539156525252f);
    out(base + 7, -1.0925484305920792f * x * z);
    out(base + 8, 0.54627421529603959f * (xx - yy));
    out(base + 9, 0.59004358992664352f * y * (yy - 3.0f * xx));
    out(base + 10, 2.8906114426405538f * x * y * z);
    out(base + 11, 0.45704579946446572f * y * (1.0f - 5.0f * zz));
    out(base + 12, 0.3731763325901154f * z * (5.0f * zz - 3.0f));
    out(base + 13, 0.45704579946446572f * x * (1.0f - 5.0f * zz));
    out(base + 14, 1.4453057213202769f * z * (xx - yy));
    out(base + 15, 0.59004358992664352f * x * (3.0f * yy - xx));
}

// Lanes [36,68): harmonics of wo and of the normal; 75, 76: the bounce budget
// left and the cut-off headroom.
template <class Out>
__device__ __forceinline__ void encode_part1(float4 f1, float4 f2, Out out)
{
    sh16(f1.x, f1.y, f1.z, 36, out);
    sh16(f2.x, f2.y, f2.z, 52, out);
    out(75, f1.w);
    out(76, f2.w);
}

// BF16 pair packing (round to nearest even), low half first.
__device__ __forceinline__ uint32_t pack2(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05, accumulators in TMEM)
// ---------------------------------------------------------------------------
// A CTA runs two warpgroups; each owns tiles of 128 rows (thread r of the
// warpgroup owns row r and TMEM lane r) with its own operand buffer, mbarrier
// and 64 TMEM columns, so one warpgroup's MMAs overlap the other's epilogue.
// Per layer: the layer input sits in shared memory as a K-major BF16 operand in
// the canonical no-swizzle layout (8-row x 16-byte core matrices); one thread
// issues the layer's tcgen05.mma (M = 128, N = 64, or 16 for the padded output
// layer; K in steps of 16) into the warpgroup's TMEM accumulator and commits to
// its mbarrier; the warpgroup waits (bounded), reads its rows back with
// tcgen05.ld, applies ReLU, rounds to BF16 and writes the next operand.  The
// weights are staged once per CTA in the same layout.
constexpr int kTcRows = 128;
constexpr int kTcGroups = 2;
constexpr int kTcW0 = 0;                          // 64 x 80: 8 n-groups x 10 k-chunks x 128 B
constexpr int kTcW1 = kTcW0 + 64 * 80 * 2;        // 64 x 64 each
constexpr int kTcW4 = kTcW1 + 3 * 64 * 64 * 2;    // 16 x 64 (rows 3..15 zero)
constexpr int kTcA = kTcW4 + 16 * 64 * 2;         // per warpgroup: 128 x 80 operand tile
constexpr int kTcABytes = kTcRows * 80 * 2;
constexpr int kTcRec = kTcA + kTcGroups * kTcABytes;  // per warpgroup: the tile's feature records
constexpr int kTcRecBytes = kTcRows * 6 * 16;          // 128 records of up to 6 float4
constexpr int kTcBar = kTcRec + kTcGroups * kTcRecBytes;  // per warpgroup: MMA mbarrier (8 B)
constexpr int kTcRecBar = kTcBar + 8 * kTcGroups;     // per warpgroup: record-copy mbarrier (8 B)
constexpr int kTcWBar = kTcRecBar + 8 * kTcGroups;    // weight-copy mbarrier (8 B)
constexpr int kTcTmem = kTcWBar + 8;                  // TMEM base address (4 B)
constexpr int kTcFlag = kTcTmem + 4;                  // per warpgroup: timeout flag (4 B)
constexpr int kTcSmem = kTcFlag + 4 * kTcGroups;
static_assert(kTcRec % 16 == 0 && kTcRecBytes % 16 == 0, "bulk-copy alignment");
constexpr uint32_t kTcWBytes = kNrcFwdElems * 2;       // the weight blob = the operands at kTcW0..
static_assert(kTcA == kTcW0 + static_cast<int>(kTcWBytes) && kTcWBytes % 16 == 0, "weight image");
constexpr uint32_t kTcCols = 64 * kTcGroups;          // TMEM columns per CTA
constexpr uint32_t kTcWaitLimit = 1u << 24;           // mbarrier polls before giving up

// Element (row, k) of a K-major operand with kc 8-element k-chunks per row, in
// bytes from the operand's start.
__device__ __forceinline__ uint32_t canon_off(uint32_t row, uint32_t k, uint32_t kc)
{
    return (((row >> 3) * kc + (k >> 3)) * 64 + (row & 7) * 8 + (k & 7)) * 2;
}

// tcgen05 shared-memory matrix descriptor: start, leading-dimension byte offset
// (next core matrix along K), stride byte offset (next 8-row group), version 1,
// no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(lbo >> 4) << 16) |
           (static_cast<uint64_t>(sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, dense, M = 128.
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

// Waits for phase `parity` of the mbarrier, polling at most `limit` times;
// false when the bound ran out.
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred q;\nmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\nselp.b32 %0, 1, 0, q;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
// Ties the registers of a TMEM load to the point after tcgen05.wait::ld: the
// empty statement is ordered after the wait (both volatile) and every later use
// reads its outputs, so no use can be scheduled before the data has arrived.
__device__ __forceinline__ void tc_touch16(float (&v)[16])
{
    asm volatile(""
                 : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6]), "+f"(v[7]),
                   "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]), "+f"(v[12]), "+f"(v[13]), "+f"(v[14]),
                   "+f"(v[15]));
}
// 16 columns, waited for
__device__ __forceinline__ void tc_load16(uint32_t taddr, float (&v)[16])
{
    tc_ld16(taddr, v);
    tc_wait_ld();
    tc_touch16(v);
}
// 64 consecutive columns: four loads in flight, one wait
__device__ __forceinline__ void tc_load64(uint32_t taddr, float (&v)[4][16])
{
#pragma unroll
    for (int q = 0; q < 4; ++q) tc_ld16(taddr + 16 * q, v[q]);
    tc_wait_ld();
#pragma unroll
    for (int q = 0; q < 4; ++q) tc_touch16(v[q]);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// barrier of one warpgroup (named barrier 1 + group, 128 threads)
__device__ __forceinline__ void group_sync(uint32_t group)
{
    asm volatile("bar.sync %0, 128;\n" ::"r"(1u + group) : "memory");
}

// Programmatic dependent launch: the next kernel of the stream (launched with
// programmatic serialization) may start its CTAs now; and this thread waits
// until the kernel before it has completed and its writes are visible.
__device__ __forceinline__ void pdl_allow_next() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_wait_prev() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// Issues one layer: D[128 x n] = A[128 x 8*kc] * W^T, W given as n x 8*kc.
__device__ __forceinline__ void tc_layer(uint32_t tmem, uint32_t a_base, uint32_t w_base, uint32_t kc, uint32_t n,
                                         uint32_t bar)
{
    const uint32_t idesc = tc_idesc(n);
    for (uint32_t j = 0; j < kc / 2; ++j) {
        const uint64_t a = smem_desc(a_base + j * 256, 128, kc * 128);
        const uint64_t b = smem_desc(w_base + j * 256, 128, kc * 128);
        tc_mma(tmem, a, b, idesc, j > 0 ? 1u : 0u);
    }
    tc_commit(bar);
}

// The weight blob is the operand image at kTcW0: one bulk copy (TMA) into
// shared memory completing on the mbarrier wbar (initialised, count 1, by the
// calling thread, which alone issues it).
__device__ __forceinline__ void fetch_weights(const bf16* __restrict__ blob, uint32_t smem_w, uint32_t wbar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(wbar), "r"(kTcWBytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_w),
                 "l"(blob), "r"(kTcWBytes), "r"(wbar)
                 : "memory");
}

template <bool PATHS>
__global__ void __launch_bounds__(kTcRows * kTcGroups) k_nrc_infer_tc(const bf16* __restrict__ blob,
                                                                      const float4* __restrict__ feat, uint32_t n_host,
                                                                      const uint32_t* __restrict__ count,
                                                                      float* __restrict__ out, PathState P,
                                                                      uint32_t* total, int* err,
                                                                      uint32_t wait_limit)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* smem = tc_smem;
    const uint32_t s0 = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t group = tid >> 7, row = tid & 127;
    const uint32_t bar = s0 + kTcBar + 8 * group;
    const uint32_t rbar = s0 + kTcRecBar + 8 * group;
    const uint32_t wbar = s0 + kTcWBar;
    volatile int* flag = reinterpret_cast<volatile int*>(smem + kTcFlag) + group;
    if (row == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(rbar));
        if (tid == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(wbar));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        *flag = 0;
        if (tid == 0) fetch_weights(blob, s0 + kTcW0, wbar);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s0 + kTcTmem),
                     "r"(kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<const uint32_t*>(smem + kTcTmem) + 64u * group;
    const uint32_t lane_addr = tmem + (((warp & 3u) * 32u) << 16);
    unsigned char* A = smem + kTcA + group * kTcABytes;
    const uint32_t a_s = s0 + kTcA + group * kTcABytes;

    const uint32_t n = PATHS ? *count : n_host;
    if (total && blockIdx.x == 0 && tid == 0) atomicAdd(total, n);
    const uint32_t tiles = (n + kTcRows - 1) / kTcRows;
    constexpr uint32_t kStride = PATHS ? 6 : 5;  // float4 per record
    const float4* rec = reinterpret_cast<const float4*>(smem + kTcRec + group * kTcRecBytes);
    const uint32_t rec_s = s0 + kTcRec + group * kTcRecBytes;
    // the records of a tile arrive as one bulk copy (TMA) completing on rbar,
    // issued by row 0 one tile ahead (while the current tile's MMAs run)
    auto fetch_records = [&](uint32_t t) {
        if (row != 0 || t >= tiles) return;
        const uint32_t rows = min(static_cast<uint32_t>(kTcRows), n - t * kTcRows);
        const uint32_t bytes = rows * kStride * 16u;
        const float4* src = feat + static_cast<uint64_t>(t) * kTcRows * kStride;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(rbar), "r"(bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(rec_s),
            "l"(src), "r"(bytes), "r"(rbar)
            : "memory");
    };
    uint32_t phase = 0, rphase = 0;
    bool copy_pending = false;  // a record copy was issued and not yet waited for
    const uint32_t first_tile = blockIdx.x * kTcGroups + group;
    fetch_records(first_tile);
    copy_pending = first_tile < tiles;
    // the MMA issuer of each warpgroup waits for the weights once
    bool w_ready = true;
    if (row == 0 && !tc_wait(wbar, 0, wait_limit)) {
        w_ready = false;
        *flag = 1;  // seen after the first group_sync below
    }
    for (uint32_t tile = first_tile; tile < tiles; tile += gridDim.x * kTcGroups) {
        const uint32_t r = tile * kTcRows + row;
        if (tc_wait(rbar, rphase, wait_limit)) {
            rphase ^= 1;
            copy_pending = false;
        } else {
            *flag = 1;  // the copy stays pending; the exit path waits for it (parity rphase)
        }
        group_sync(group);
        if (*flag) {
            if (row == 0) atomicOr(err, MT_ERRBIT_TIMEOUT);
            break;
        }
        float4 thr = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // PATHS: throughput, path index
        // layer-0 operand: this thread's row, encoded
        {
            float e[80];
            if (r < n) {
                const float4* f = rec + row * kStride;
                auto put = [&](int k, float v) { e[k] = v; };
                encode_part0(f[0], f[3], f[4], put);
                encode_part1(f[1], f[2], put);
                if (PATHS) thr = f[5];
            } else {
#pragma unroll
                for (int k = 0; k < 80; ++k) e[k] = 0.0f;
            }
#pragma unroll
            for (int c = 0; c < 10; ++c) {
                const uint4 v = make_uint4(pack2(e[8 * c], e[8 * c + 1]), pack2(e[8 * c + 2], e[8 * c + 3]),
                                           pack2(e[8 * c + 4], e[8 * c + 5]), pack2(e[8 * c + 6], e[8 * c + 7]));
                *reinterpret_cast<uint4*>(A + canon_off(row, 8 * c, 10)) = v;
            }
        }
        bool timed_out = false;
        float y[16];
#pragma unroll 1
        for (uint32_t l = 0; l < 5; ++l) {
            fence_async_smem();
            tc_fence_before();
            group_sync(group);
            tc_fence_after();
            if (row == 0) {
                const uint32_t w = l == 0 ? kTcW0 : (l == 4 ? kTcW4 : kTcW1 + (l - 1) * 64 * 64 * 2);
                tc_layer(tmem, a_s, s0 + w, l == 0 ? 10 : 8, l == 4 ? 16 : 64, bar);
            }
            if (l == 0) {
                // every row of the group has read its record: the buffer takes the next tile's
                fetch_records(tile + gridDim.x * kTcGroups);
                copy_pending = tile + gridDim.x * kTcGroups < tiles;
            }
            if (!tc_wait(bar, phase, wait_limit)) *flag = 1;
            phase ^= 1;
            group_sync(group);
            if (*flag) {
                timed_out = true;
                break;
            }
            tc_fence_after();
            if (l < 4) {
                float vq[4][16];
                tc_load64(lane_addr, vq);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float* v = vq[q];
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const float* x = v + 8 * c;
                        const uint4 o = make_uint4(pack2(fmaxf(x[0], 0.0f), fmaxf(x[1], 0.0f)),
                                                   pack2(fmaxf(x[2], 0.0f), fmaxf(x[3], 0.0f)),
                                                   pack2(fmaxf(x[4], 0.0f), fmaxf(x[5], 0.0f)),
                                                   pack2(fmaxf(x[6], 0.0f), fmaxf(x[7], 0.0f)));
                        *reinterpret_cast<uint4*>(A + canon_off(row, 16 * q + 8 * c, 8)) = o;
                    }
                }
            } else {
                tc_load16(lane_addr, y);
            }
        }
        if (timed_out) {
            if (row == 0) atomicOr(err, MT_ERRBIT_TIMEOUT);
            break;
        }
        if (r < n) {
            if (PATHS) {
                const float4 q = thr;
                const uint32_t p = __float_as_uint(q.w);
                const float4 a = P.indirect[p];
                P.indirect[p] = make_float4(a.x + q.x * fmaxf(y[0], 0.0f), a.y + q.y * fmaxf(y[1], 0.0f),
                                            a.z + q.z * fmaxf(y[2], 0.0f), a.w);
            } else {
                out[3ull * r + 0] = y[0];
                out[3ull * r + 1] = y[1];
                out[3ull * r + 2] = y[2];
            }
        }
    }
    // release TMEM only when no MMA of this CTA can still be in flight: after a
    // timeout, wait (bounded) for the warpgroup's last commit first; and do not
    // leave while a record copy still writes this CTA's shared memory
    if (*flag && row == 0) (void)tc_wait(bar, phase ^ 1, kTcWaitLimit);
    if (copy_pending && row == 0) (void)tc_wait(rbar, rphase, kTcWaitLimit);
    if (!w_ready) (void)tc_wait(wbar, 0, kTcWaitLimit);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem - 64u * group),
                     "r"(kTcCols));
    }
}

__global__ void k_nrc_encode(const float4* __restrict__ feat, uint32_t n, float* __restrict__ out)
{
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const float4* f = feat + 5ull * r;
        float* o = out + 80ull * r;
        auto put = [&](int k, float v) { o[k] = v; };
        encode_part0(f[0], f[3], f[4], put);
        encode_part1(f[1], f[2], put);
    }
}

// 32-bit integer finaliser (MurmurHash3 fmix32): row -> pseudo-random sample.
__device__ __forceinline__ uint32_t mix32(uint32_t h)
{
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

// ---------------------------------------------------------------------------
// Training on the 5th-generation tensor cores (tcgen05): forward, loss,
// backward and weight gradient of a training step in one kernel
// ---------------------------------------------------------------------------
// One warpgroup per CTA, one 128-row tile at a time (thread r <-> row r <->
// TMEM lane r).  Every activation is written once, by the thread that owns
// its row, in the canonical K-major no-swizzle layout (8-row x 16-byte core
// matrices) that the next forward MMA reads as its A operand: the input X
// (128 x 80), the hidden outputs H0..H3 (128 x 64) and the loss gradient of
// the layer being differentiated, dY (128 x 64, or 128 x 16 at the output).
// The backward and weight-gradient products read the same bytes transposed:
//   backward   dX_l = dY_l W_l        A = dY_l (K-major, K = out_l),
//                                     B = W_l read MN-major (N = in_l, K = out_l)
//   gradient   dW_l^T = X_l^T dY_l    A = X_l read MN-major (M = in_l, padded to
//                                     128; lanes >= in_l are not read back),
//                                     B = dY_l read MN-major (N = out_l, K = rows)
// so no transposed copy is ever written.  In every descriptor the leading
// byte offset (LBO) is the stride between core matrices along K and the stride
// byte offset (SBO) the stride along M/N: for a K-major operand LBO = 128 B
// (the next 8 K elements) and SBO = one 8-row group; for an MN-major view of
// the same bytes LBO = one 8-row group (now 8 K values) and SBO = 128 B.  TMEM columns: [0,64) forward accumulator, [64,128) backward
// accumulator, 128 + 64 l the gradient of layer l (accumulated over the CTA's
// tiles).  The CTA's weight-gradient sums are written to its partial row, which
// k_nrc_adam adds up in CTA order.  Waits on the mbarrier are bounded as in
// the inference kernel.
constexpr int kTrRows = 128;
constexpr int kTrX = kTcW4 + 16 * 64 * 2;        // X: 128 x 80
constexpr int kTrH = kTrX + kTrRows * 80 * 2;    // H0..H3: 128 x 64 each
constexpr int kTrDY = kTrH + 4 * kTrRows * 64 * 2;  // dY: 128 x 64 (128 x 16 at the output layer)
// 8 KB after dY: whichever way a descriptor's two strides are read, no
// operand read reaches past the allocation (checked below)
constexpr int kTrPad = kTrDY + kTrRows * 64 * 2;
constexpr int kTrBar = kTrPad + 8192;
constexpr int kTrWBar = kTrBar + 8;  // weight-copy mbarrier
constexpr int kTrTmem = kTrWBar + 8;
constexpr int kTrFlag = kTrTmem + 4;
constexpr int kTrSmem = kTrFlag + 12;
constexpr uint32_t kTrCols = 512;
static_assert(kTrX % 1024 == 0 && kTrH % 1024 == 0 && kTrDY % 1024 == 0, "operand alignment");
// The transposed reads of X and H3 as 128-row A operands run up to 1 KB past
// their buffers (into H0 and dY).  Bounds that hold for either reading of the
// two strides (all groups at the larger stride): X, H3 and dY as MN-major
// operands, W4 as the backward B operand.
static_assert(kTrX + 30 * 1280 + 128 <= kTrSmem, "X read bound");
static_assert(kTrH + 3 * kTrRows * 128 + 30 * 1024 + 128 <= kTrSmem, "H3 read bound");
static_assert(kTrDY + 22 * 1024 + 128 <= kTrBar, "dY read bound");
static_assert(kTcW4 + 8 * 1024 + 128 <= kTrSmem, "W4 read bound");

__device__ __forceinline__ uint32_t tr_act(int l) { return l == 0 ? kTrX : kTrH + (l - 1) * kTrRows * 128; }
__device__ __forceinline__ uint32_t tr_w(int l) { return l == 0 ? kTcW0 : (l == 4 ? kTcW4 : kTcW1 + (l - 1) * 64 * 64 * 2); }

// D (+)= A B over ksteps K-steps of 16, descriptor starts advancing by a_step /
// b_step bytes per step.
__device__ __forceinline__ void tc_gemm(uint32_t d, uint32_t a, uint32_t a_lbo, uint32_t a_sbo, uint32_t a_step,
                                        uint32_t b, uint32_t b_lbo, uint32_t b_sbo, uint32_t b_step, uint32_t ksteps,
                                        uint32_t idesc, bool accumulate)
{
    for (uint32_t j = 0; j < ksteps; ++j)
        tc_mma(d, smem_desc(a + j * a_step, a_lbo, a_sbo), smem_desc(b + j * b_step, b_lbo, b_sbo), idesc,
               (accumulate || j > 0) ? 1u : 0u);
}

__global__ void __launch_bounds__(kTrRows) k_nrc_train_tc(const bf16* __restrict__ fwd, NrcTrainArgs a,
                                                         uint32_t tiles, float* __restrict__ partial, float* loss,
                                                         const uint32_t* __restrict__ step, int* err,
                                                         uint32_t wait_limit)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    unsigned char* smem = tc_smem;
    const uint32_t s0 = static_cast<uint32_t>(__cvta_generic_to_shared(smem));
    const uint32_t tid = threadIdx.x, warp = tid >> 5, row = tid;
    const uint32_t bar = s0 + kTrBar, wbar = s0 + kTrWBar;
    volatile int* flag = reinterpret_cast<volatile int*>(smem + kTrFlag);
    // launched with programmatic serialization after the previous step's Adam:
    // the set-up below overlaps that kernel's tail; everything it writes (the
    // weights, the step counter, the partial rows it reads) is touched only
    // after pdl_wait_prev
    pdl_allow_next();
    bool w_wait = tid == 0;  // the MMA issuer still has to see the weights arrive
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(wbar));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        *flag = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(s0 + kTrTmem),
                     "r"(kTrCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<const uint32_t*>(smem + kTrTmem);
    const uint32_t lane_addr = tmem + ((warp * 32u) << 16);
    pdl_wait_prev();
    // forward weights (canonical K-major, N = out rows, K = in) by one bulk
    // copy, in flight while the rows are gathered and encoded
    if (tid == 0) fetch_weights(fwd, s0 + kTcW0, wbar);

    const uint32_t cnt = a.count ? min(*a.count, a.count_cap) : a.rows;
    const uint32_t base = *step * a.rows;
    const uint32_t n = cnt ? a.rows : 0;  // valid rows (none when there is nothing to train on)
    const float scale = n ? 1.0f / (3.0f * static_cast<float>(n)) : 0.0f;
    float lsum = 0.0f;
    uint32_t phase = 0;
    bool first = true, timed_out = false;

    // every thread of the warpgroup waits for the last commit; false on timeout
    auto wait_mma = [&]() -> bool {
        if (!tc_wait(bar, phase, wait_limit)) *flag = 1;
        phase ^= 1;
        __syncthreads();
        if (*flag) return false;
        tc_fence_after();
        return true;
    };
    // generic-proxy shared-memory writes -> visible to the next MMA
    auto publish = [&]() {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    };

    for (uint32_t tile = blockIdx.x; tile < tiles && !timed_out; tile += gridDim.x) {
        const uint32_t r = tile * kTrRows + row;
        const bool valid = r < n;
        const uint32_t sample = a.count ? (n ? mix32(base + r) % cnt : 0u) : r;
        float target[3] = {0.0f, 0.0f, 0.0f};  // loaded with the record, used after the forward pass
        if (valid) {
#pragma unroll
            for (int c = 0; c < 3; ++c) target[c] = a.targets[static_cast<uint64_t>(sample) * a.tstride + c];
        }
        {  // encoded input row
            float e[80];
            if (valid) {
                const float4* f = a.feat + static_cast<uint64_t>(sample) * a.fstride;
                auto put = [&](int k, float v) { e[k] = v; };
                encode_part0(f[0], f[3], f[4], put);
                encode_part1(f[1], f[2], put);
            } else {
#pragma unroll
                for (int k = 0; k < 80; ++k) e[k] = 0.0f;
            }
#pragma unroll
            for (int c = 0; c < 10; ++c)
                *reinterpret_cast<uint4*>(smem + kTrX + canon_off(row, 8 * c, 10)) =
                    make_uint4(pack2(e[8 * c], e[8 * c + 1]), pack2(e[8 * c + 2], e[8 * c + 3]),
                               pack2(e[8 * c + 4], e[8 * c + 5]), pack2(e[8 * c + 6], e[8 * c + 7]));
        }
        if (w_wait) {
            if (tc_wait(wbar, 0, wait_limit))
                w_wait = false;
            else
                *flag = 1;
        }
        publish();
        if (*flag) {
            timed_out = true;
            break;
        }
        // forward
        uint32_t mask[4][2];
#pragma unroll 1
        for (int l = 0; l < 5 && !timed_out; ++l) {
            const uint32_t kc = l == 0 ? 10 : 8;
            if (tid == 0) {
                tc_gemm(tmem, s0 + tr_act(l), 128, kc * 128, 256, s0 + tr_w(l), 128, kc * 128, 256, kc / 2,
                        tc_idesc(l == 4 ? 16 : 64), false);
                tc_commit(bar);
            }
            if (!wait_mma()) {
                timed_out = true;
                break;
            }
            if (l < 4) {
                uint32_t m0 = 0, m1 = 0;
                unsigned char* H = smem + tr_act(l + 1);
                float vq[4][16];
                tc_load64(lane_addr, vq);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float* v = vq[q];
                    uint32_t bits = 0;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        if (v[j] > 0.0f) bits |= 1u << j;
                        v[j] = fmaxf(v[j], 0.0f);
                    }
                    if (q < 2) m0 |= bits << (16 * q); else m1 |= bits << (16 * (q - 2));
#pragma unroll
                    for (int c = 0; c < 2; ++c) {
                        const float* x = v + 8 * c;
                        *reinterpret_cast<uint4*>(H + canon_off(row, 16 * q + 8 * c, 8)) =
                            make_uint4(pack2(x[0], x[1]), pack2(x[2], x[3]), pack2(x[4], x[5]), pack2(x[6], x[7]));
                    }
                }
                mask[l][0] = m0;
                mask[l][1] = m1;
            } else {
                float y[16];
                tc_load16(lane_addr, y);
                // relative L2 loss |y - t|^2 / (y^2 + 0.01), y constant in the denominator
                float dy[3] = {0.0f, 0.0f, 0.0f};
                if (valid) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float diff = y[c] - target[c];
                        const float den = y[c] * y[c] + 0.01f;
                        lsum += diff * diff / den;
                        dy[c] = 2.0f * diff / den * scale;
                    }
                }
                *reinterpret_cast<uint4*>(smem + kTrDY + canon_off(row, 0, 2)) =
                    make_uint4(pack2(dy[0], dy[1]), pack2(dy[2], 0.0f), 0u, 0u);
                *reinterpret_cast<uint4*>(smem + kTrDY + canon_off(row, 8, 2)) = make_uint4(0u, 0u, 0u, 0u);
            }
            publish();
        }
        // backward: layers 4..1 (input gradient and weight gradient), then the
        // first layer's weight gradient
#pragma unroll 1
        for (int l = 4; l >= 0 && !timed_out; --l) {
            const uint32_t kcy = l == 4 ? 2 : 8;            // k-chunks of dY_l (out_l / 8)
            const uint32_t kin = l == 0 ? 10 : 8;           // k-chunks of the layer input (in_l / 8)
            if (tid == 0) {
                if (l > 0)  // dH = dY_l W_l -> TMEM [64, 128); W_l read MN-major
                    tc_gemm(tmem + 64, s0 + kTrDY, 128, kcy * 128, 256, s0 + tr_w(l), kin * 128, 128,
                            2 * kin * 128, kcy / 2, tc_idesc(64) | (1u << 16), false);
                // dW_l^T += X_l^T dY_l -> TMEM [128 + 64 l, ...); both operands MN-major
                tc_gemm(tmem + 128 + 64 * l, s0 + tr_act(l), kin * 128, 128, 2 * kin * 128, s0 + kTrDY, kcy * 128,
                        128, 2 * kcy * 128, kTrRows / 16, tc_idesc(l == 4 ? 16 : 64) | (1u << 15) | (1u << 16),
                        !first);
                tc_commit(bar);
            }
            if (!wait_mma()) {
                timed_out = true;
                break;
            }
            if (l == 0) break;
            // dY_{l-1} = dH masked by the ReLU of H_{l-1}
            float vq[4][16];
            tc_load64(lane_addr + 64, vq);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float* v = vq[q];
                const uint32_t bits = (q < 2 ? mask[l - 1][0] >> (16 * q) : mask[l - 1][1] >> (16 * (q - 2)));
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (!((bits >> j) & 1u)) v[j] = 0.0f;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const float* x = v + 8 * c;
                    *reinterpret_cast<uint4*>(smem + kTrDY + canon_off(row, 16 * q + 8 * c, 8)) =
                        make_uint4(pack2(x[0], x[1]), pack2(x[2], x[3]), pack2(x[4], x[5]), pack2(x[6], x[7]));
                }
            }
            publish();
        }
        first = false;
    }
    // this CTA's weight-gradient sums (TMEM lane i = input i of the layer)
    float* out = partial + static_cast<uint64_t>(blockIdx.x) * kNrcParams;
    if (!timed_out) {
#pragma unroll 1
        for (int l = 0; l < 5; ++l) {
            const int in = layer_in(l), outs = layer_out(l);
            const int nq = l == 4 ? 1 : 4;
            for (int q = 0; q < nq; ++q) {
                float v[16];
                tc_load16(lane_addr + 128 + 64 * l + 16 * q, v);
                if (static_cast<int>(row) < in) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int o = 16 * q + j;
                        if (o < outs) out[master_off(l) + o * in + row] = v[j];
                    }
                }
            }
        }
    } else {
        // a timed-out CTA contributes nothing to this step's gradient
        for (int q = tid; q < kNrcParams; q += blockDim.x) out[q] = 0.0f;
        if (tid == 0) atomicOr(err, MT_ERRBIT_TIMEOUT);
    }
    if (loss) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
        if ((tid & 31) == 0) atomicAdd(loss, lsum * scale);
    }
    // release TMEM only when no MMA of this CTA can still be in flight: after a
    // timeout, wait (bounded) for the last commit first
    if (*flag && tid == 0) (void)tc_wait(bar, phase ^ 1, kTcWaitLimit);
    if (w_wait) (void)tc_wait(wbar, 0, kTcWaitLimit);  // the weight copy still writes shared memory
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTrCols));
    }
}

// ---------------------------------------------------------------------------
// Adam and weight publication
// ---------------------------------------------------------------------------
__device__ __forceinline__ void publish_param(bf16* fwd, bf16* infer, int q, float w, float wi)
{
    int l, o, i;
    param_coords(q, l, o, i);
    fwd[blob_index(l, o, i)] = __float2bfloat16_rn(w);
    infer[blob_index(l, o, i)] = __float2bfloat16_rn(wi);
}

// Bias corrections 1 - beta^t of the moments and of the zero-started weight
// average, t = the device step counter + 1 (the step being taken).  Every
// block reads the counter before it signals `done`; the last block to finish
// advances the counter, so the next step's kernels see it incremented.
// A block owns 32 consecutive parameters (lane = parameter, so every load of
// a partial row is one coalesced 128-byte line); warp w loads partials w,
// w + kAdamWarps, ..., w + 7 kAdamWarps at once and adds them pairwise, and
// warp 0 adds the warps' sums in order, so the gradient is the same on every
// run.
constexpr int kAdamWarps = 16;

__global__ void __launch_bounds__(kAdamWarps * 32) k_nrc_adam(float* __restrict__ master, float* __restrict__ m,
                                                              float* __restrict__ v, const float* __restrict__ partial,
                                                              uint32_t splits, float lr, float b1, float b2, float eps,
                                                              bf16* fwd, float* grad_out, bf16* infer,
                                                              float* __restrict__ ema, float decay,
                                                              uint32_t* __restrict__ step, uint32_t* __restrict__ done)
{
    __shared__ float red[kAdamWarps][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q = blockIdx.x * 32 + lane;
    pdl_wait_prev();   // the partial rows of this step are complete
    pdl_allow_next();  // the next step's training CTAs may set up meanwhile
    const float t = static_cast<float>(*step + 1u);
    float part = 0.0f;
    if (q < kNrcParams) {
        float acc[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t s = warp + k * kAdamWarps;
            acc[k] = s < splits ? partial[static_cast<uint64_t>(s) * kNrcParams + q] : 0.0f;
        }
        part = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
        for (uint32_t s = warp + 8 * kAdamWarps; s < splits; s += kAdamWarps)
            part += partial[static_cast<uint64_t>(s) * kNrcParams + q];
    }
    red[warp][lane] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(done, 1u) == gridDim.x - 1) {
            *done = 0u;
            atomicAdd(step, 1u);
        }
    }
    if (warp != 0 || q >= kNrcParams) return;
    float gsum = 0.0f;
#pragma unroll
    for (int w = 0; w < kAdamWarps; ++w) gsum += red[w][lane];
    const float bc1 = 1.0f - powf(b1, t), bc2 = 1.0f - powf(b2, t), ema_bc = 1.0f - powf(decay, t);
    if (grad_out) grad_out[q] = gsum;
    const float mm = b1 * m[q] + (1.0f - b1) * gsum;
    const float vv = b2 * v[q] + (1.0f - b2) * gsum * gsum;
    m[q] = mm;
    v[q] = vv;
    const float w = master[q] - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    master[q] = w;
    float wi = w;
    if (decay > 0.0f) {
        const float e = decay * ema[q] + (1.0f - decay) * w;
        ema[q] = e;
        wi = e / ema_bc;
    }
    publish_param(fwd, infer, q, w, wi);
}

__global__ void k_nrc_publish(const float* __restrict__ master, bf16* fwd, bf16* infer, float* __restrict__ ema)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= kNrcParams) return;
    ema[q] = 0.0f;
    publish_param(fwd, infer, q, master[q], master[q]);
}

__global__ void k_nrc_blend(float* __restrict__ accum, const float* __restrict__ frame, uint64_t n, float w)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        accum[i] += (frame[i] - accum[i]) * w;
}

// ---------------------------------------------------------------------------
// Training targets from recorded training paths
// ---------------------------------------------------------------------------
// Training samples of path p, in bounce order: calls keep(k, record, target)
// for every recorded vertex whose target is usable and mark(record) for every
// recorded vertex.
template <class Keep, class Mark>
__device__ __forceinline__ void path_targets(const PathState& P, const NrcShade& N, uint32_t p, uint32_t bounces,
                                             Keep keep, Mark mark)
{
    const float4 e = P.emit[p], d = P.direct[p], ind = P.indirect[p], s = P.sky[p];
    const float tot[3] = {((e.x + d.x) + ind.x) + s.x, ((e.y + d.y) + ind.y) + s.y, ((e.z + d.z) + ind.z) + s.z};
    for (uint32_t k = 0; k < bounces; ++k) {
        float4* r = N.rec + (static_cast<uint64_t>(p) * bounces + k) * 8;
        const float4 pre = r[6];
        if (pre.w != 1.0f) break;  // vertices are recorded in bounce order
        mark(r);
        const float cur[3] = {r[5].x, r[5].y, r[5].z};
        // AT_DIFFUSE: the cache stands for what the vertex reflects from the
        // rest of its path, so its own NEE is part of the prefix
        const float4 nee = N.end_at == MT_NRC_END_AT_DIFFUSE ? r[7] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float prv[3] = {pre.x + nee.x, pre.y + nee.y, pre.z + nee.z};
        float tg[3];
        bool ok = true;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ok = ok && cur[c] > 1e-6f;
            float sfx = fmaxf(tot[c] - prv[c], 0.0f);
            if (N.target_cap > 0.0f) sfx = fminf(sfx, N.target_cap);
            tg[c] = sfx / cur[c];
            ok = ok && isfinite(tg[c]);
        }
        if (ok) keep(r, tg);
    }
}

// Pass 1: usable samples per path.
__global__ void k_nrc_target_count(PathState P, NrcShade N, uint32_t n, uint32_t bounces, uint32_t* counts)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        uint32_t c = 0;
        path_targets(P, N, p, bounces, [&](const float4*, const float*) { ++c; }, [](float4*) {});
        counts[p] = c;
    }
}

// Exclusive prefix of the per-path counts, continuing after the samples
// already in the buffer (*N.sample_count), which then counts these as well:
// one block of 1024 threads, 16 consecutive paths per thread per tile.
__global__ void __launch_bounds__(1024) k_nrc_target_scan(NrcShade N, uint32_t n, uint32_t* counts)
{
    __shared__ uint32_t warp_sum[32];
    __shared__ uint32_t carry;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = *N.sample_count;
    __syncthreads();
    constexpr uint32_t kPer = 16, kTile = 1024 * kPer;
    for (uint32_t t0 = 0; t0 < n; t0 += kTile) {
        const uint32_t first = t0 + tid * kPer;
        uint32_t v[kPer], sum = 0;
#pragma unroll
        for (uint32_t i = 0; i < kPer; ++i) {
            v[i] = first + i < n ? counts[first + i] : 0u;
            sum += v[i];
        }
        uint32_t incl = sum;  // inclusive scan of the threads' sums
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += x;
        }
        if (lane == 31) warp_sum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sum[lane], wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t x = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= static_cast<uint32_t>(o)) wi += x;
            }
            warp_sum[lane] = wi - w;  // exclusive over warps
        }
        __syncthreads();
        uint32_t run = carry + warp_sum[warp] + (incl - sum);
#pragma unroll
        for (uint32_t i = 0; i < kPer; ++i) {
            if (first + i < n) counts[first + i] = run;
            run += v[i];
        }
        __syncthreads();
        if (tid == 1023) carry = run;
        __syncthreads();
    }
    if (tid == 0) *N.sample_count = carry;
}

// Pass 2: the samples at their places (training vertices in path order, so
// a frame's sample buffer is the same on every run).
__global__ void k_nrc_targets(PathState P, NrcShade N, uint32_t n, uint32_t bounces, const uint32_t* offsets)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        uint32_t slot = offsets[p];
        path_targets(
            P, N, p, bounces,
            [&](const float4* r, const float* tg) {
                if (slot < N.sample_cap) {
                    float4* o = N.samples + static_cast<uint64_t>(slot) * 6;
#pragma unroll
                    for (int i = 0; i < 5; ++i) o[i] = r[i];
                    o[5] = make_float4(tg[0], tg[1], tg[2], 0.0f);
                }
                ++slot;
            },
            [](float4* r) { r[6].w = 0.0f; });
    }
}

int sms() { return device_sm_count(); }

// The shared-memory limit of a kernel is an attribute per device: raised once
// per device (the flags are indexed by the current device).
constexpr int kMaxDevices = 64;
template <class K>
cudaError_t allow_smem(K kernel, size_t bytes, bool (&done)[kMaxDevices])
{
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) dev = 0;
    if (done[dev]) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(bytes));
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

// Polls of the inference kernel's in-loop mbarrier waits.  MT_NRC_WAIT_LIMIT
// lowers it for tests (0: every wait gives up at once, as if the tensor cores
// never answered); the wait before TMEM is released always keeps the full bound.
uint32_t infer_wait_limit()
{
    const char* v = std::getenv("MT_NRC_WAIT_LIMIT");
    if (!v || !*v) return kTcWaitLimit;
    return static_cast<uint32_t>(std::strtoul(v, nullptr, 10));
}

template <bool PATHS>
cudaError_t infer(const void* net, const float4* feat, uint32_t n_host, const uint32_t* count, uint32_t capacity,
                  float* out, const PathState& P, uint32_t* total, int* err, cudaStream_t st)
{
    static bool ok[kMaxDevices] = {};
    cudaError_t e = allow_smem(k_nrc_infer_tc<PATHS>, kTcSmem, ok);
    if (e != cudaSuccess) return e;
    uint64_t blocks = (static_cast<uint64_t>(capacity) + kTcRows * kTcGroups - 1) / (kTcRows * kTcGroups);
    const uint64_t cap = static_cast<uint64_t>(sms()) * 2;  // 2 x 77 KB of shared memory per SM
    if (blocks > cap) blocks = cap;
    if (blocks == 0) blocks = 1;
    k_nrc_infer_tc<PATHS><<<static_cast<unsigned>(blocks), kTcRows * kTcGroups, kTcSmem, st>>>(
        static_cast<const bf16*>(net), feat, n_host, count, out, P, total, err, infer_wait_limit());
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_nrc_query(const void* net, const PathState& P, const float4* rec, const uint32_t* count,
                             uint32_t capacity, uint32_t* total, int* err, cudaStream_t st)
{
    return infer<true>(net, rec, 0, count, capacity, nullptr, P, total, err, st);
}

cudaError_t launch_nrc_infer(const void* net, const float* features, uint32_t n, float* out, int* err,
                             cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    return infer<false>(net, reinterpret_cast<const float4*>(features), n, nullptr, n, out, PathState{}, nullptr,
                        err, st);
}

cudaError_t launch_nrc_encode(const float* features, uint32_t n, float* out, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((n + 127) / 128, 1024));
    k_nrc_encode<<<blocks, 128, 0, st>>>(reinterpret_cast<const float4*>(features), n, out);
    return cudaGetLastError();
}

cudaError_t launch_nrc_targets(const PathState& P, const NrcShade& N, uint32_t n, uint32_t bounces,
                               uint32_t* scratch, cudaStream_t st)
{
    const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((n + 255) / 256, 4096));
    k_nrc_target_count<<<blocks ? blocks : 1, 256, 0, st>>>(P, N, n, bounces, scratch);
    k_nrc_target_scan<<<1, 1024, 0, st>>>(N, n, scratch);
    k_nrc_targets<<<blocks ? blocks : 1, 256, 0, st>>>(P, N, n, bounces, scratch);
    return cudaGetLastError();
}

cudaError_t launch_nrc_train_step(NrcOptimizer& O, const NrcTrainArgs& a, float* loss, float* grad_out,
                                  cudaStream_t st)
{
    if (a.rows == 0 || a.rows > O.max_rows) return cudaErrorInvalidValue;
    // shared-memory limits were raised by nrc_prepare (no attribute call here:
    // this function is also recorded into a CUDA graph).  One CTA per 128-row
    // tile up to max_splits CTAs (each then loops over tiles); one gradient
    // partial per CTA.
    const uint32_t tiles = (a.rows + kTrRows - 1) / kTrRows;
    const uint32_t splits = std::min<uint32_t>(tiles, O.max_splits);
    // both kernels with programmatic serialization: each may start while the
    // one before it drains, and waits (griddepcontrol.wait) before it reads
    // that kernel's output
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(splits);
    lc.blockDim = dim3(kTrRows);
    lc.dynamicSmemBytes = kTrSmem;
    lc.stream = st;
    lc.attrs = attr;
    lc.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&lc, k_nrc_train_tc, static_cast<const bf16*>(O.fwd), a, tiles, O.partial,
                                       loss, static_cast<const uint32_t*>(O.d_step), O.err, infer_wait_limit());
    if (e != cudaSuccess) return e;
    O.step += 1;
    lc.gridDim = dim3((kNrcParams + 31) / 32);
    lc.blockDim = dim3(kAdamWarps * 32);
    lc.dynamicSmemBytes = 0;
    return cudaLaunchKernelEx(&lc, k_nrc_adam, O.master, O.m, O.v, static_cast<const float*>(O.partial), splits,
                              O.lr, O.beta1, O.beta2, O.eps, static_cast<bf16*>(O.fwd), grad_out,
                              static_cast<bf16*>(O.infer), O.ema, O.ema_decay, O.d_step, O.d_done);
}

cudaError_t nrc_prepare()
{
    static bool ok_t[kMaxDevices] = {}, ok_i0[kMaxDevices] = {}, ok_i1[kMaxDevices] = {};
    cudaError_t e = allow_smem(k_nrc_train_tc, kTrSmem, ok_t);
    if (e == cudaSuccess) e = allow_smem(k_nrc_infer_tc<false>, kTcSmem, ok_i0);
    if (e == cudaSuccess) e = allow_smem(k_nrc_infer_tc<true>, kTcSmem, ok_i1);
    // with lazy module loading a kernel is loaded at its first launch, which
    // can hold up the other stream of a frame; the cache's kernels and the
    // render's hook variant are loaded here instead
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_nrc_adam);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_nrc_targets);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_nrc_target_count);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_nrc_target_scan);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_nrc_blend);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_nrc_publish);
    if (e == cudaSuccess) e = preload_render_kernels();
    return e;
}

cudaError_t launch_nrc_publish(const NrcOptimizer& O, cudaStream_t st)
{
    k_nrc_publish<<<(kNrcParams + 255) / 256, 256, 0, st>>>(O.master, static_cast<bf16*>(O.fwd),
                                                           static_cast<bf16*>(O.infer), O.ema);
    return cudaGetLastError();
}

cudaError_t launch_nrc_blend(float* accum, const float* frame, uint64_t n, uint32_t index, cudaStream_t st)
{
    const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((n + 255) / 256, 8192));
    k_nrc_blend<<<blocks ? blocks : 1, 256, 0, st>>>(accum, frame, n, 1.0f / static_cast<float>(index + 1));
    return cudaGetLastError();
}

}  // namespace mt
