// mt_kernels.cu - sm_103a kernels of the wavefront path tracer.
//
// The reference walks one path at a time per CPU thread (Tracer::RenderBlock ->
// ProcessRayForward -> GeneratePath, src/Tracer/Tracer.cpp:134-348, 550-616).
// Here a batch of paths (pixels x samples of one image band) moves through
// bounce-synchronous stages; between stages the live paths are compacted into
// queues with warp-aggregated atomics:
//   raygen   camera rays + jitter              (Tracer.cpp:578-586, Camera.cpp:17-50)
//   extend   closest hit of live paths         (Tracer.cpp:145, Intersect.cpp:201-219)
//   shade    miss/sky, emission, light pick, shadow-ray setup, lobe sampling,
//            energy cut-off                    (Tracer.cpp:147-208, 243-339)
//   shadow   occlusion of the NEE rays          (Tracer.cpp:317-336)
//   finalize per-sample total + ACES            (Tracer.cpp:344-346, 212-222)
//   resolve  per-pixel firefly clamp + mean     (Tracer.cpp:490-548, 593-601)
#include <cuda_runtime.h>

#include <mutex>

#include "mt_device.cuh"
#include "mt_kernels.h"
#include "mt_nrc.h"

// Occupancy hint of the traversal kernels: blocks of 128 threads per SM that
// the register allocation must allow (7 -> at most 72 registers per thread).
// Measured on the material grid render (Mrays/s): 6 blocks 1041, 7 blocks
// 1049, 8 blocks 1034; on the 6.1 M-triangle incoherent batch the any-hit
// query gains from 8 blocks (63.6 against 61.6 Mrays/s; closest hit the same),
// so the any-hit test kernel takes MT_TRACE_ANY_MIN_BLOCKS.
#ifndef MT_TRAVERSE_MIN_BLOCKS
#define MT_TRAVERSE_MIN_BLOCKS 7
#endif
#ifndef MT_TRACE_ANY_MIN_BLOCKS
#define MT_TRACE_ANY_MIN_BLOCKS 8
#endif

namespace mt {

__device__ __forceinline__ uint32_t warp_append(uint32_t* counter)
{
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, static_cast<uint32_t>(__popc(mask)));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// ---------------------------------------------------------------------------
// Ray queries
// ---------------------------------------------------------------------------
// Ray-query work for trace_persistent: rays in, mt_hit records out.
template <int QUERY>
struct QueryWork {
    const mt_ray* rays;
    mt_hit* hits;
    uint32_t n;
    uint32_t idx;
    __device__ bool fetch(uint32_t i, f3& o, f3& d, float& tmax)
    {
        if (i >= n) return false;
        idx = i;
        const float4 a = __ldg(reinterpret_cast<const float4*>(rays + i));
        const float4 b = __ldg(reinterpret_cast<const float4*>(rays + i) + 1);
        o = xyz(a);
        d = xyz(b);
        tmax = a.w;
        return true;
    }
    __device__ void finish(const SceneHit& sh)
    {
        mt_hit h;
        if (QUERY == MT_QUERY_ANY) {
            h.distance = h.u = h.v = 0.0f;
            h.instance = sh.hit ? 1u : 0u;
            h.triangle = h.bv_index = h.bvh_tests = h.tri_tests = 0;
        } else if (sh.hit) {
            h.distance = sh.dist;
            h.u = sh.u;
            h.v = sh.v;
            h.instance = sh.inst;
            h.triangle = sh.tri;
            h.bv_index = sh.bv;
            h.bvh_tests = sh.bvh_tests;
            h.tri_tests = sh.tri_tests;
        } else {
            h.distance = h.u = h.v = 0.0f;
            h.instance = MT_NO_HIT;
            h.triangle = h.bv_index = h.bvh_tests = h.tri_tests = 0;
        }
        if (QUERY == MT_QUERY_CLOSEST_TOTALS) {
            h.bv_index = sh.tot_inner;
            h.bvh_tests = sh.tot_pops;
            h.tri_tests = sh.tot_tris;
        }
        float4* dst = reinterpret_cast<float4*>(hits + idx);
        dst[0] = make_float4(h.distance, h.u, h.v, __uint_as_float(h.instance));
        dst[1] = make_float4(__uint_as_float(h.triangle), __uint_as_float(h.bv_index),
                             __uint_as_float(h.bvh_tests), __uint_as_float(h.tri_tests));
    }
};

template <int QUERY>
__global__ void __launch_bounds__(128, QUERY == MT_QUERY_ANY ? MT_TRACE_ANY_MIN_BLOCKS : MT_TRAVERSE_MIN_BLOCKS) k_trace(DevScene S, const mt_ray* __restrict__ rays, uint32_t n,
                                               mt_hit* __restrict__ hits, uint32_t* fetch)
{
    QueryWork<QUERY> W{rays, hits, n, 0};
    constexpr bool kCount = QUERY == MT_QUERY_CLOSEST_COUNT || QUERY == MT_QUERY_CLOSEST_TOTALS;
    // IntersectScene as is (every met instance opened); leaf pairs for the
    // closest-hit query
    trace_persistent<kCount, QUERY == MT_QUERY_ANY, false, 32, QUERY == MT_QUERY_CLOSEST>(S, W, fetch);
}

__global__ void k_brdf(const mt_brdf_query* __restrict__ q, uint64_t n, mt_brdf_result* __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const mt_brdf_query x = q[i];
        const f3 L = ld3(x.L), V = ld3(x.V), N = ld3(x.N), B = ld3(x.base_color);
        const f3 f = eval_brdf(L, V, N, B, x.roughness, x.metallic);
        mt_brdf_result r;
        r.f[0] = f.x;
        r.f[1] = f.y;
        r.f[2] = f.z;
        r.diffuse_pdf = diffuse_pdf(L, N);
        r.specular_pdf = specular_pdf(L, V, N, x.roughness);
        out[i] = r;
    }
}

// The bounce sampling of GeneratePath (Tracer.cpp:177-203) with its uniforms
// given: lobe choice, direction, and the mixture pdf.
__global__ void k_brdf_sample(const mt_brdf_sample_query* __restrict__ q, uint64_t n,
                              mt_brdf_sample_result* __restrict__ out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const mt_brdf_sample_query x = q[i];
        const f3 V = ld3(x.V), N = ld3(x.N), B = ld3(x.base_color);
        const f3 rd = -V;
        const float ps = specular_probability(V, N, B, x.metallic);
        f3 nd;
        int lobe = 0;
        if (x.u[0] < ps) {
            lobe = 1;
            if (!ggx_reflection(rd, N, x.roughness, x.u[1], x.u[2], nd)) {
                lobe = 2;
                nd = cosine_hemisphere(x.u[3], x.u[4], N);
            }
        } else {
            nd = cosine_hemisphere(x.u[1], x.u[2], N);
        }
        const float dp = diffuse_pdf(nd, N);
        const float sp = specular_pdf(nd, V, N, x.roughness);
        mt_brdf_sample_result r;
        r.L[0] = nd.x;
        r.L[1] = nd.y;
        r.L[2] = nd.z;
        r.pdf = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, ps), dp), __fmul_rn(ps, sp));
        r.specular_probability = ps;
        r.lobe = lobe;
        out[i] = r;
    }
}

// ---------------------------------------------------------------------------
// Wavefront render stages
// ---------------------------------------------------------------------------
struct BatchInfo {
    uint64_t g0;        // first path (sample-major index inside the band)
    uint32_t n;         // paths in this batch
    uint32_t band_pix;  // pixels in the band
    uint32_t pix_base;  // first pixel (y*W+x) of the band
    uint32_t sample_base;  // added to the sample index of every path
    uint32_t scatter_mul;  // nonzero: path p is pixel (p * mul + add) mod W*H, sample sample_base
    uint32_t scatter_add;
    uint32_t tiled;     // nonzero: a sample's paths visit the band in pixel tiles (tile_pixel)
};

// Pixel tiles of MT_PIXEL_TILE_W x (32 / MT_PIXEL_TILE_W): with `tiled`, the 32
// consecutive paths of a warp cover one tile instead of 32 pixels of a row, so
// their camera rays (and the origins of the next bounces) lie close together
// and the warp's lanes walk the same nodes and leaves.  The order only decides
// which path computes which (pixel, sample); every path's result, which the
// counter-based draws key by pixel and sample, is unchanged.
#ifndef MT_PIXEL_TILE_W
#define MT_PIXEL_TILE_W 4
#endif
static_assert(MT_PIXEL_TILE_W >= 1 && MT_PIXEL_TILE_W <= 32 && 32 % MT_PIXEL_TILE_W == 0, "tile width");

// Row-major offset inside a band of width W and band_pix pixels of the k-th
// pixel in tile order: whole tiles first (row of tiles by row of tiles), then
// the columns right of the last whole tile in those rows, then the rows below
// the last whole row of tiles, both row-major.  A bijection of [0, band_pix).
__device__ __forceinline__ uint32_t tile_pixel(uint32_t k, uint32_t W, uint32_t band_pix)
{
    constexpr uint32_t TW = MT_PIXEL_TILE_W, TH = 32 / MT_PIXEL_TILE_W;
    const uint32_t rows = band_pix / W;
    const uint32_t rfull = rows - rows % TH;
    const uint32_t wfull = W - W % TW;
    if (k < rfull * wfull) {
        const uint32_t t = k >> 5, w = k & 31u;
        const uint32_t per_row = wfull / TW;
        const uint32_t tr = t / per_row, tc = t - tr * per_row;
        return (tr * TH + w / TW) * W + tc * TW + w % TW;
    }
    if (k < rfull * W) {
        const uint32_t m = k - rfull * wfull, mw = W - wfull;
        const uint32_t y = m / mw;
        return y * W + wfull + (m - y * mw);
    }
    return k;
}

__device__ __forceinline__ void path_coords(const DevScene& S, const BatchInfo& B, uint32_t p,
                                            uint32_t& pixel, uint32_t& sample)
{
    if (B.scatter_mul) {
        const uint64_t npix = static_cast<uint64_t>(S.width) * S.height;
        pixel = static_cast<uint32_t>((static_cast<uint64_t>(p) * B.scatter_mul + B.scatter_add) % npix);
        sample = B.sample_base;
        return;
    }
    const uint64_t g = B.g0 + p;
    uint32_t k;
    if (g >> 32) {
        sample = static_cast<uint32_t>(g / B.band_pix);
        k = static_cast<uint32_t>(g - static_cast<uint64_t>(sample) * B.band_pix);
    } else {  // 32-bit division for the common case
        const uint32_t g32 = static_cast<uint32_t>(g);
        sample = g32 / B.band_pix;
        k = g32 - sample * B.band_pix;
    }
    pixel = B.pix_base + (B.tiled ? tile_pixel(k, S.width, B.band_pix) : k);
    sample += B.sample_base;
}

__global__ void __launch_bounds__(256) k_raygen(DevScene S, PathState P, BatchInfo B,
                                                uint32_t* __restrict__ q0, uint32_t* counts,
                                                RecordBuffers R)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counts[0] = B.n;
        counts[3] = 0;  // ray fetch counter of the first extend
    }
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < B.n; p += gridDim.x * blockDim.x) {
        uint32_t pixel, sample;
        path_coords(S, B, p, pixel, sample);
        const uint32_t x = pixel % S.width, y = pixel / S.width;
        const uint4 r = draw(S, pixel, sample, 0, SLOT_JITTER);
        const float u = __fadd_rn(__fmul_rn(static_cast<float>(x), S.px_w), urange(r.x, 0.0f, S.px_w));
        const float v = __fadd_rn(__fmul_rn(static_cast<float>(y), S.px_h), urange(r.y, 0.0f, S.px_h));
        f3 o, d;
        camera_ray(S, u, v, o, d);
        P.ro[p] = make_float4(o.x, o.y, o.z, 0.0f);
        P.rd[p] = make_float4(d.x, d.y, d.z, 0.0f);
        const float4 one = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        P.cur[p] = one;
        P.tot[p] = one;
        P.prev[p] = zero;
        P.emit[p] = zero;
        P.direct[p] = zero;
        P.indirect[p] = zero;
        P.sky[p] = zero;
        q0[p] = p;
        if (P.dval) {
            P.dval[p] = zero;
            P.dcnt[p] = make_uint4(0u, 0u, 0u, 0u);
        }
        if (R.path) {
            R.path[2 * p] = zero;
            R.path[2 * p + 1] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        }
    }
}

// Adds this thread's traversal totals to cnt[0..2] (pops, inner pops, tri tests)
// with one atomic per warp.
__device__ __forceinline__ void flush_counts(unsigned long long* cnt, uint32_t pops, uint32_t inner,
                                             uint32_t tris)
{
    unsigned long long a = pops, b = inner, c = tris;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
        c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if ((threadIdx.x & 31) == 0 && cnt) {
        atomicAdd(cnt + 0, a);
        atomicAdd(cnt + 1, b);
        atomicAdd(cnt + 2, c);
    }
}

// Extension rays of the live paths (queue q) -> hit records per path.
template <bool COUNT, bool DBG>
struct ExtendWork {
    PathState P;
    const uint32_t* q;
    uint32_t n;
    uint32_t p;
    uint32_t pops, inner, tris;
    int debug_mode;
    __device__ bool fetch(uint32_t i, f3& o, f3& d, float& tmax)
    {
        if (i >= n) return false;
        p = q[i];
        o = xyz(P.ro[p]);
        d = xyz(P.rd[p]);
        tmax = 0.0f;
        return true;
    }
    __device__ void finish(const SceneHit& h)
    {
        if (COUNT) {
            pops += h.tot_pops;
            inner += h.tot_inner;
            tris += h.tot_tris;
        }
        if (h.hit) {
            P.hitA[p] = make_float4(h.world_pos.x, h.world_pos.y, h.world_pos.z, h.dist);
            P.hitB[p] = make_uint4(h.inst, h.tri, __float_as_uint(h.u), __float_as_uint(h.v));
        } else {
            P.hitB[p] = make_uint4(MT_NO_HIT, 0u, 0u, 0u);
        }
        if (DBG && P.dcnt) {
            // PathStep debug counters (Tracer.cpp:171-175); they are the winning
            // instance's (COUNT traversals only), a miss step adds nothing
            float4 v = P.dval[p];
            uint4 c = P.dcnt[p];
            if (h.hit) {
                if (v.w == 0.0f) {
                    c.x = h.bvh_tests | 0x80000000u;
                    c.y = h.tri_tests;
                    if (debug_mode == MT_DEBUG_COLOR_PER_BOUNDING_VOLUME) {
                        const f3 col = random_color_u16(h.bv);
                        v.x = col.x;
                        v.y = col.y;
                        v.z = col.z;
                    }
                }
                c.z += h.bvh_tests;
                c.w += h.tri_tests;
                P.dcnt[p] = c;
            }
            v.w += 1.0f;
            P.dval[p] = v;
        }
    }
};

// CHUNK: instances per world-box pass (64 for the plain render of a scene with
// more than 32 instances; the counting and debug forms keep 32, which visits
// the same nodes in the same order).
template <bool COUNT, bool DBG, int CHUNK = 32>
__global__ void __launch_bounds__(128, MT_TRAVERSE_MIN_BLOCKS) k_extend(DevScene S, PathState P,
                                                const uint32_t* __restrict__ q,
                                                uint32_t* counts, int cur, int sqi,
                                                unsigned long long* rays,
                                                unsigned long long* cnt)
{
    const uint32_t n = counts[cur];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // the next queue and this bounce's shadow queue start empty; the
        // previous bounce's shadow stage, which may still run beside this
        // kernel, counts in the other shadow-queue slot
        counts[cur ^ 1] = 0;
        counts[sqi] = 0;
        atomicAdd(rays, static_cast<unsigned long long>(n));
    }
    ExtendWork<COUNT, DBG> W{P, q, n, 0, 0, 0, 0, S.debug_mode};
    trace_persistent<COUNT, false, !DBG, CHUNK, false, true>(S, W, &counts[3]);  // debug counts visit every instance
    if (COUNT) flush_counts(cnt, W.pops, W.inner, W.tris);
}

__device__ __forceinline__ f3 ld4(const float4* p, uint32_t i)
{
    const float4 v = p[i];
    return {v.x, v.y, v.z};
}
__device__ __forceinline__ void st4(float4* p, uint32_t i, f3 v, float w = 0.0f)
{
    p[i] = make_float4(v.x, v.y, v.z, w);
}

// HOOKS: the radiance-cache and debug-mode code paths; REC: the adjoint's
// vertex and path records.  The plain render runs the variant without either
// (a smaller body: the shading stage waits on instruction fetch).
// Occupancy hint of the shade kernel (blocks of 128 threads per SM): 8 caps it
// at 64 registers with a few bytes of spills; the kernel waits on scattered
// path-state and material loads, so more resident warps pay (measured on the
// material grid render, shade ms: 80 registers 135, 78 registers 140, 72 registers 145,
// 64 registers 117, 48 registers 121).
#ifndef MT_SHADE_MIN_BLOCKS
#define MT_SHADE_MIN_BLOCKS 8
#endif
template <bool HOOKS, bool REC>
__global__ void __launch_bounds__(128, MT_SHADE_MIN_BLOCKS) k_shade(DevScene S, PathState P, ShadowQueue SQ,
                                               BatchInfo B, uint32_t bounce,
                                               const uint32_t* __restrict__ q,
                                               uint32_t* __restrict__ nq, uint32_t* counts,
                                               int cur, int sqi, RecordBuffers R, NrcShade NC,
                                               unsigned long long* shadow_rays)
{
    const uint32_t n = counts[cur];
    // this bounce's extension is done and the previous bounce's shadow stage
    // has finished: the ray fetch counters of the next extension and of this
    // bounce's shadow stage start at zero
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        counts[3] = 0;
        counts[4] = 0;
    }
    uint32_t untraced = 0;  // zero-contribution shadow rays counted, not queued
    // one path that hit: the shading body (Tracer.cpp:150-233, 255-336)
    auto shade_hit = [&](const uint32_t p) {
        const uint4 hb = P.hitB[p];
        const f3 rd = ld4(P.rd, p);
        const f3 cur_e = ld4(P.cur, p);
            uint32_t pixel, sample;
            path_coords(S, B, p, pixel, sample);
            const float4 ha = P.hitA[p];
            const f3 hit_pos = xyz(ha);
            const float hit_dist = ha.w;
            const float bu = __uint_as_float(hb.z), bv = __uint_as_float(hb.w);
            const DevInstance& I = S.instances[hb.x];
            const DevMesh m = S.meshes[__ldg(&I.mesh)];
            // RayHitGeometryInfo (Ray.cpp:7-48)
            const uint32_t tri = m.attr_off + hb.y;
            const float w = __fsub_rn(__fsub_rn(1.0f, bu), bv);
            const float* nr = S.normals + 9ull * tri;
            f3 ni = {__fadd_rn(__fadd_rn(__fmul_rn(w, __ldg(nr + 0)), __fmul_rn(bu, __ldg(nr + 3))), __fmul_rn(bv, __ldg(nr + 6))),
                     __fadd_rn(__fadd_rn(__fmul_rn(w, __ldg(nr + 1)), __fmul_rn(bu, __ldg(nr + 4))), __fmul_rn(bv, __ldg(nr + 7))),
                     __fadd_rn(__fadd_rn(__fmul_rn(w, __ldg(nr + 2)), __fmul_rn(bu, __ldg(nr + 5))), __fmul_rn(bv, __ldg(nr + 8)))};
            ni = normalize(ni);
            float model[16];
    #pragma unroll
            for (int k = 0; k < 16; ++k) model[k] = __ldg(&I.model[k]);
            // normalize(model * vec4(n, 0)) with the vec4 pairwise dot
            const float nx = mrow(model, 0, ni.x, ni.y, ni.z, 0.0f);
            const float ny = mrow(model, 1, ni.x, ni.y, ni.z, 0.0f);
            const float nz = mrow(model, 2, ni.x, ni.y, ni.z, 0.0f);
            const float nw = mrow(model, 3, ni.x, ni.y, ni.z, 0.0f);
            const float ns = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)),
                                                                  __fadd_rn(__fmul_rn(nz, nz), __fmul_rn(nw, nw)))));
            const f3 geom_n = {__fmul_rn(nx, ns), __fmul_rn(ny, ns), __fmul_rn(nz, ns)};
            float tu = 0.0f, tv = 0.0f;
            if (m.has_uv) {
                const float* uv = S.uvs + 6ull * tri;
                tu = __fadd_rn(__fadd_rn(__fmul_rn(w, __ldg(uv + 0)), __fmul_rn(bu, __ldg(uv + 2))), __fmul_rn(bv, __ldg(uv + 4)));
                tv = __fadd_rn(__fadd_rn(__fmul_rn(w, __ldg(uv + 1)), __fmul_rn(bu, __ldg(uv + 3))), __fmul_rn(bv, __ldg(uv + 5)));
            }
            const MatPoint mp = sample_material(S, __ldg(&I.material), tu, tv);
            const f3 base = {__fadd_rn(__fmul_rn(mp.base.x, 0.96f), 0.04f),
                             __fadd_rn(__fmul_rn(mp.base.y, 0.96f), 0.04f),
                             __fadd_rn(__fmul_rn(mp.base.z, 0.96f), 0.04f)};
            const f3 N = compute_normal(geom_n, mp.normal);
            const f3 view = -rd;

            // Emission (Tracer.cpp:255)
            const f3 emit_now = ld4(P.emit, p) + (cur_e * S.emission_base) * mp.emission;
            st4(P.emit, p, emit_now);
            float seen_diffuse = 0.0f;
            bool end_here = false;  // AT_DIFFUSE query: the path ends after this vertex's NEE
            if (HOOKS && NC.mode != MT_NRC_OFF) {
                // Radiance-cache feature record of this vertex (mt_nrc.h)
                seen_diffuse = P.prev[p].w;
                const bool query =
                    NC.mode == MT_NRC_QUERY && (NC.end_at == MT_NRC_END_AT_DIFFUSE
                                                    ? mp.roughness >= NC.rough_min
                                                    : bounce >= 1 && seen_diffuse != 0.0f);
                float4* fr = nullptr;
                if (query)
                    fr = NC.rec + 6ull * warp_append(NC.count);
                else if (NC.mode == MT_NRC_TRAIN)
                    fr = NC.rec + (static_cast<uint64_t>(p) * S.bounces + bounce) * 8;
                if (fr) {
                    const f3 pn = {(hit_pos.x - NC.lo[0]) * NC.inv_ext[0], (hit_pos.y - NC.lo[1]) * NC.inv_ext[1],
                                   (hit_pos.z - NC.lo[2]) * NC.inv_ext[2]};
                    const float m = mp.metallic;
                    // what the rest of the path may still collect: the bounce budget
                    // left and the headroom above the energy cut-off
                    const float remaining = S.bounces > 1 ? static_cast<float>(S.bounces - 1 - bounce) /
                                                                static_cast<float>(S.bounces - 1)
                                                          : 0.0f;
                    float headroom = 1.0f;
                    if (S.terminate_energy > 0.0f) {
                        const float te = length(ld4(P.tot, p));
                        headroom = fminf(fmaxf(log2f(fmaxf(te, 1e-30f) / S.terminate_energy) * 0.0625f, 0.0f), 1.0f);
                    }
                    fr[0] = make_float4(pn.x, pn.y, pn.z, mp.roughness);
                    fr[1] = make_float4(view.x, view.y, view.z, remaining);
                    fr[2] = make_float4(N.x, N.y, N.z, headroom);
                    fr[3] = make_float4(base.x * (1.0f - m), base.y * (1.0f - m), base.z * (1.0f - m), 0.0f);
                    fr[4] = make_float4(0.04f * (1.0f - m) + base.x * m, 0.04f * (1.0f - m) + base.y * m,
                                        0.04f * (1.0f - m) + base.z * m, 0.0f);
                    fr[5] = make_float4(cur_e.x, cur_e.y, cur_e.z, __uint_as_float(p));
                    if (!query) {
                        const f3 pre = ((emit_now + ld4(P.direct, p)) + ld4(P.indirect, p)) + ld4(P.sky, p);
                        fr[6] = make_float4(pre.x, pre.y, pre.z, 1.0f);
                        fr[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // NEE, set by the shadow stage
                    }
                }
                if (query) {
                    if (NC.end_at != MT_NRC_END_AT_DIFFUSE) return;  // the cache stands in for the rest
                    end_here = true;
                }
                if (mp.roughness >= NC.rough_min) seen_diffuse = 1.0f;
            }
            float4* vr = REC && R.vert ? R.vert + (static_cast<uint64_t>(p) * S.bounces + bounce) * 5 : nullptr;
            if (vr) {
                vr[0] = make_float4(N.x, N.y, N.z, __uint_as_float(__ldg(&I.material)));
                vr[1] = make_float4(view.x, view.y, view.z, __uint_as_float(MT_VREC_HIT));
                vr[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                vr[3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                vr[4] = make_float4(tu, tv, __uint_as_float(0u), 0.0f);
                R.path[2 * p].w = static_cast<float>(bounce + 1);
            }

            // Weighted reservoir light pick (Tracer.cpp:257-279)
            int chosen = -1;
            float pick = 0.0f, total = 0.0f;
            uint4 rp = make_uint4(0, 0, 0, 0);
            for (uint32_t li = 0; li < S.num_lights; ++li) {
                if ((li & 3) == 0) rp = draw(S, pixel, sample, bounce, SLOT_LIGHT_PICK + (li >> 2));
                const DevLight& L = S.lights[li];
                const f3 lp = f3{__ldg(&L.pos[0]), __ldg(&L.pos[1]), __ldg(&L.pos[2])} - hit_pos;
                const float score = __fdiv_rn(__ldg(&L.simple), __fadd_rn(dot(lp, lp), 1.0f));
                total = __fadd_rn(total, score);
                const uint32_t word = (li & 3) == 0 ? rp.x : ((li & 3) == 1 ? rp.y : ((li & 3) == 2 ? rp.z : rp.w));
                if (__fmul_rn(urange(word, 0.0f, 1.0f), total) < score) {
                    chosen = static_cast<int>(li);
                    pick = score;
                }
            }
            pick = __fdiv_rn(pick, total);
            if (chosen >= 0) {
                const DevLight& L = S.lights[chosen];
                const int type = __ldg(&L.type);
                const f3 lpos0 = {__ldg(&L.pos[0]), __ldg(&L.pos[1]), __ldg(&L.pos[2])};
                f3 lpos = lpos0;
                if (type == MT_LIGHT_POINT || type == MT_LIGHT_SPOT) {
                    const uint4 rj = draw(S, pixel, sample, bounce, SLOT_LIGHT_JITTER);
                    const float a = urange(rj.x, 0.0f, __fmul_rn(2.0f, kPi));
                    const float b = urange(rj.y, -kPi / 2.0f, kPi / 2.0f);
                    float sa, ca, sb, cb;
                    sincosf(a, &sa, &ca);  // one argument reduction for both
                    sincosf(b, &sb, &cb);
                    const f3 dir = normalize(f3{__fmul_rn(ca, cb), sb, __fmul_rn(sa, cb)});
                    lpos = lpos0 + dir * __ldg(&L.point_size);
                }
                const f3 lvec = lpos - hit_pos;
                const float llen = length(lvec);
                const f3 ldir = lvec * __fdiv_rn(1.0f, llen);  // normalize(lvec), its length formed once
                f3 lcol = {__ldg(&L.color[0]), __ldg(&L.color[1]), __ldg(&L.color[2])};
                float spot = 1.0f;
                if (type == MT_LIGHT_SPOT) {
                    const f3 sd = {__ldg(&L.dir[0]), __ldg(&L.dir[1]), __ldg(&L.dir[2])};
                    const float dd = dot(-ldir, sd);
                    const float inten = __fdiv_rn(__fsub_rn(dd, __ldg(&L.outer_cos)),
                                                  __fsub_rn(__ldg(&L.inner_cos), __ldg(&L.outer_cos)));
                    spot = gclamp(inten, 0.0f, 1.0f);
                    lcol = lcol * spot;
                }
                const f3 brdf = eval_brdf(ldir, view, N, base, mp.roughness, mp.metallic);
                const float nl = gmax(dot(N, ldir), 0.0f);
                const float fall = __fdiv_rn(1.0f, __fadd_rn(__fmul_rn(llen, llen), 1.0f));
                const f3 le = brdf * nl * fall;
                const f3 contrib = ((cur_e * le) * lcol) / pick;
                // A shadow ray whose contribution is exactly zero (the light
                // below the surface: nl = 0) cannot change the image whatever
                // it meets (nor a cache training record, whose NEE term stays
                // zero); unless adjoint records or debug counts need its
                // visit it is counted, as the reference counts it
                // (Tracer.cpp:319), but not traced.
                const bool trace = vr || P.dval || !(contrib.x == 0.0f && contrib.y == 0.0f && contrib.z == 0.0f);
                if (trace) {
                    const uint32_t slot = warp_append(&counts[sqi]);
                    const f3 so = hit_pos + lvec * 0.0001f;
                    SQ.o[slot] = make_float4(so.x, so.y, so.z, llen);
                    SQ.d[slot] = make_float4(ldir.x, ldir.y, ldir.z, __uint_as_float(p));
                    SQ.c[slot] = make_float4(contrib.x, contrib.y, contrib.z, static_cast<float>(bounce));
                } else {
                    ++untraced;
                }
                if (vr) {
                    vr[1].w = __uint_as_float(MT_VREC_HIT | MT_VREC_CHOSEN);
                    vr[3] = make_float4(ldir.x, ldir.y, ldir.z, nl * fall / pick);
                    vr[4].z = __uint_as_float(static_cast<uint32_t>(chosen));
                    vr[4].w = spot;
                }
            }

            // First-hit debug values (ProcessDebugRay, Tracer.cpp:411-482)
            const bool dbg0 = HOOKS && P.dval && bounce == 0;
            if (dbg0) {
                f3 dv = splat(0.0f);
                bool set = true;
                switch (S.debug_mode) {
                    case MT_DEBUG_ALBEDO: dv = base; break;
                    case MT_DEBUG_METALLIC_ROUGHNESS: dv = f3{0.0f, mp.metallic, mp.roughness}; break;
                    case MT_DEBUG_GEOMETRIC_NORMAL: dv = geom_n * 0.5f + splat(0.5f); break;
                    case MT_DEBUG_SHADING_NORMAL: dv = N * 0.5f + splat(0.5f); break;
                    case MT_DEBUG_COLOR_PER_MESH: dv = random_color_u16(hb.x); break;
                    case MT_DEBUG_COLOR_PER_TRIANGLE: dv = random_color_u16(hb.y); break;
                    case MT_DEBUG_DEPTH: dv = splat(length(hit_pos - ld4(P.ro, p))); break;
                    case MT_DEBUG_FIRST_HIT_FRESNEL:
                        dv = fresnel_schlick(gmax(dot(N, -rd), 0.0f), base_reflectivity(base, mp.metallic));
                        break;
                    default: set = false; break;
                }
                if (set) {
                    const float4 o = P.dval[p];
                    P.dval[p] = make_float4(dv.x, dv.y, dv.z, o.w);
                }
            }

            if (HOOKS && end_here) return;  // the cache stands in for the reflected rest

            // Bounce sampling (Tracer.cpp:177-208); the last vertex never extends
            // (the debug modes that show the first vertex's sample draw it anyway).
            const bool last = bounce + 1 >= S.bounces;
            if (last && !(dbg0 && (S.debug_mode == MT_DEBUG_FIRST_HIT_BRDF || S.debug_mode == MT_DEBUG_FIRST_HIT_PDF)))
                return;
            const float ps = specular_probability(view, N, base, mp.metallic);
            const uint4 rl = draw(S, pixel, sample, bounce, SLOT_LOBE);
            f3 nd;
            // the diffuse lobe and the GGX fallback share one cosine sample
            // (one copy of its code), with the uniforms of their draw
            uint32_t cu1 = rl.y, cu2 = rl.z;
            bool cosine = true;
            if (urange(rl.x, 0.0f, 1.0f) < ps) {
                cosine = !ggx_reflection(rd, N, mp.roughness, urange(rl.y, 0.0f, 1.0f), urange(rl.z, 0.0f, 1.0f), nd);
                if (cosine) {
                    const uint4 rf = draw(S, pixel, sample, bounce, SLOT_FALLBACK);
                    cu1 = rf.x;
                    cu2 = rf.y;
                }
            }
            if (cosine) nd = cosine_hemisphere(urange(cu1, 0.0f, 1.0f), urange(cu2, 0.0f, 1.0f), N);
            const float dp = diffuse_pdf(nd, N);
            const float sp = specular_pdf(nd, view, N, mp.roughness);
            const float pdf = __fadd_rn(__fmul_rn(__fsub_rn(1.0f, ps), dp), __fmul_rn(ps, sp));
            const f3 brdf = eval_brdf(nd, view, N, base, mp.roughness, mp.metallic);
            const float nl = gmax(dot(N, nd), 0.0f);
            const f3 energy = pdf > 0.0f ? brdf * __fdiv_rn(nl, pdf) : splat(0.0f);
            if (dbg0 && (S.debug_mode == MT_DEBUG_FIRST_HIT_BRDF || S.debug_mode == MT_DEBUG_FIRST_HIT_PDF)) {
                const float4 o = P.dval[p];
                const float dv = S.debug_mode == MT_DEBUG_FIRST_HIT_PDF ? pdf : __fadd_rn(__fadd_rn(brdf.x, brdf.y), brdf.z);
                P.dval[p] = make_float4(dv, dv, dv, o.w);
            }
            if (last) return;
            if (chosen >= 0) st4(P.cur, p, cur_e * energy);  // Tracer.cpp:339
            if (vr) {
                vr[1].w = __uint_as_float(__float_as_uint(vr[1].w) | MT_VREC_NEXT);
                vr[2] = make_float4(nd.x, nd.y, nd.z, pdf > 0.0f ? nl / pdf : 0.0f);
            }
            const f3 tot = ld4(P.tot, p) * energy;
            st4(P.tot, p, tot);
            if (length(tot) < S.terminate_energy) return;  // Tracer.cpp:207-208
            if (dbg0 && S.debug_mode == MT_DEBUG_REFLECTED_DIRECTION) {
                // path[1].ray.direction * 0.5 + 0.5: the path has a second step
                const float4 o = P.dval[p];
                const f3 dv = nd * 0.5f + splat(0.5f);
                P.dval[p] = make_float4(dv.x, dv.y, dv.z, o.w);
            }
            const f3 ro = xyz(P.ro[p]);
            const f3 no = (ro + rd * hit_dist) + N * 0.0001f;
            st4(P.ro, p, no);
            st4(P.rd, p, nd);
            st4(P.prev, p, base, seen_diffuse);
            nq[warp_append(&counts[cur ^ 1])] = p;
    };
    // A miss costs a sky lookup, a hit the whole body above: misses are
    // handled as a warp reads the queue, hits are collected per warp in shared
    // memory and shaded 32 at a time, so a warp's lanes run the long body
    // together instead of beside lanes that have finished (blocks of 128
    // threads: four warps, each holding fewer than 64 hits at a time)
    __shared__ uint32_t s_hits[4][64];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    uint32_t next = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32u;
    uint32_t held = 0;
    while (true) {
        if (held < 32 && next < n) {
            const uint32_t i = next + lane;
            next += nwarps * 32u;
            bool hit = false;
            uint32_t p = 0;
            if (i < n) {
                p = q[i];
                if (P.hitB[p].x == MT_NO_HIT) {
                    // Tracer.cpp:244-252: previous vertex's base colour times energy times sky.
                    const f3 rd = ld4(P.rd, p);
                    const f3 cur_e = ld4(P.cur, p);
                    const f3 color = bounce > 0 ? ld4(P.prev, p) : splat(1.0f);
                    const f3 sky = sample_sky(S, rd, bounce == 0);
                    st4(P.sky, p, ld4(P.sky, p) + (color * cur_e) * sky);
                    if (REC && R.path) R.path[2 * p + 1] = make_float4(sky.x, sky.y, sky.z, static_cast<float>(bounce));
                } else {
                    hit = true;
                }
            }
            const uint32_t m = __ballot_sync(MT_FULL, hit);
            if (hit) s_hits[wib][held + __popc(m & ((1u << lane) - 1u))] = p;
            held += __popc(m);
            __syncwarp();
            continue;
        }
        if (held == 0) break;
        const uint32_t take = held < 32 ? held : 32;
        held -= take;
        const bool active = lane < take;
        const uint32_t p = active ? s_hits[wib][held + lane] : 0u;
        __syncwarp();
        if (active) shade_hit(p);
    }
    uint32_t u = untraced;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) u += __shfl_down_sync(MT_FULL, u, o);
    if (lane == 0 && u) atomicAdd(shadow_rays, static_cast<unsigned long long>(u));
}

// Shadow rays queued by k_shade: an unoccluded ray adds its contribution to
// the owning path's direct (first vertex) or indirect light (Tracer.cpp:322-336).
template <bool COUNT>
struct ShadowWork {
    PathState P;
    ShadowQueue SQ;
    RecordBuffers R;
    uint32_t bounces;
    uint32_t n;
    uint32_t i;
    uint32_t pops, inner, tris;
    __device__ bool fetch(uint32_t k, f3& o, f3& d, float& tmax)
    {
        if (k >= n) return false;
        i = k;
        const float4 a = SQ.o[k], b = SQ.d[k];
        o = xyz(a);
        d = xyz(b);
        tmax = a.w;
        return true;
    }
    __device__ void finish(const SceneHit& h)
    {
        if (COUNT) {
            pops += h.tot_pops;
            inner += h.tot_inner;
            tris += h.tot_tris;
        }
        if (h.hit) return;
        const float4 c = SQ.c[i];
        const uint32_t p = __float_as_uint(SQ.d[i].w);
        if (R.vert) {
            float4* vr = R.vert + (static_cast<uint64_t>(p) * bounces + static_cast<uint32_t>(c.w)) * 5;
            vr[1].w = __uint_as_float(__float_as_uint(vr[1].w) | MT_VREC_VISIBLE);
        }
        if (R.nrc)  // radiance-cache training record: this vertex's NEE contribution
            R.nrc[(static_cast<uint64_t>(p) * bounces + static_cast<uint32_t>(c.w)) * 8 + 7] =
                make_float4(c.x, c.y, c.z, 0.0f);
        float4* acc = c.w == 0.0f ? P.direct : P.indirect;
        const float4 a = acc[p];
        acc[p] = make_float4(__fadd_rn(a.x, c.x), __fadd_rn(a.y, c.y), __fadd_rn(a.z, c.z), 0.0f);
    }
};

template <bool COUNT, int CHUNK = 32>
__global__ void __launch_bounds__(128, MT_TRAVERSE_MIN_BLOCKS) k_shadow(DevScene S, PathState P, ShadowQueue SQ,
                                                uint32_t* counts, int sqi,
                                                unsigned long long* rays,
                                                unsigned long long* cnt,
                                                RecordBuffers R)
{
    const uint32_t n = counts[sqi];
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(rays, static_cast<unsigned long long>(n));
    ShadowWork<COUNT> W{P, SQ, R, S.bounces, n, 0, 0, 0, 0};
    trace_persistent<COUNT, true, true, CHUNK, false, true>(S, W, &counts[4]);
    if (COUNT) flush_counts(cnt, W.pops, W.inner, W.tris);
}

// The per-sample value of a debug render mode (ProcessDebugRay,
// Tracer.cpp:366-488) from the path's debug planes and light accumulators.
__device__ __forceinline__ f3 debug_sample(const DevScene& S, const PathState& P, uint32_t p, f3 total_aces)
{
    const float4 v = P.dval[p];
    const uint4 c = P.dcnt[p];
    const bool hit = (c.x & 0x80000000u) != 0;
    const f3 black = splat(0.0f);
    switch (S.debug_mode) {
        case MT_DEBUG_PRIMARY_BVH_TESTS: return hit ? splat(static_cast<float>(c.x & 0x7fffffffu)) : black;
        case MT_DEBUG_TOTAL_BVH_TESTS: return hit ? splat(static_cast<float>(c.z)) : black;
        case MT_DEBUG_PRIMARY_TRIANGLE_TESTS: return hit ? splat(static_cast<float>(c.y)) : black;
        case MT_DEBUG_TOTAL_TRIANGLE_TESTS: return hit ? splat(static_cast<float>(c.w)) : black;
        case MT_DEBUG_BOUNCES: return hit ? splat(v.w) : black;
        case MT_DEBUG_DIRECT_ONLY: return aces(ld4(P.direct, p), S.exposure);
        case MT_DEBUG_INDIRECT_ONLY: return aces(ld4(P.indirect, p) + ld4(P.sky, p), S.exposure);
        case MT_DEBUG_EMISSION: return aces(ld4(P.emit, p), S.exposure);
        case MT_DEBUG_ALBEDO:
        case MT_DEBUG_METALLIC_ROUGHNESS:
        case MT_DEBUG_GEOMETRIC_NORMAL:
        case MT_DEBUG_SHADING_NORMAL:
        case MT_DEBUG_COLOR_PER_MESH:
        case MT_DEBUG_COLOR_PER_TRIANGLE:
        case MT_DEBUG_DEPTH:
        case MT_DEBUG_FIRST_HIT_FRESNEL:
        case MT_DEBUG_FIRST_HIT_BRDF:
        case MT_DEBUG_FIRST_HIT_PDF:
        case MT_DEBUG_REFLECTED_DIRECTION: return xyz(v);
        case MT_DEBUG_COLOR_PER_BOUNDING_VOLUME: return xyz(v);
        default: return total_aces;
    }
}

__global__ void __launch_bounds__(256) k_finalize(DevScene S, PathState P, BatchInfo B,
                                                  float* __restrict__ sr, float* __restrict__ sg,
                                                  float* __restrict__ sb, RecordBuffers R)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < B.n; p += gridDim.x * blockDim.x) {
        const f3 total = ((ld4(P.emit, p) + ld4(P.direct, p)) + ld4(P.indirect, p)) + ld4(P.sky, p);
        if (R.path) {
            R.path[2 * p].x = total.x;
            R.path[2 * p].y = total.y;
            R.path[2 * p].z = total.z;
        }
        f3 c = aces(total, S.exposure);
        if (P.dval) c = debug_sample(S, P, p, c);
        // plane slot of the path's (pixel, sample): sample-major, row-major pixels
        uint64_t g = B.g0 + p;
        if (B.tiled) {
            uint32_t pixel, sample;
            path_coords(S, B, p, pixel, sample);
            g = static_cast<uint64_t>(sample - B.sample_base) * B.band_pix + (pixel - B.pix_base);
        }
        sr[g] = c.x;
        sg[g] = c.y;
        sb[g] = c.z;
    }
}

// CleanupFireflies + average (Tracer.cpp:490-548, 593-600): population
// mean/variance of the sample intensities in sample order, reject
// |I - mean| > k*sigma, mean of the rest.  DebugPixelStandardDeviation turns
// every sample into sigma (taken before any sample is dropped) and
// DebugFireflyElimination into the number of dropped samples; both then
// divide the sum by spp, as CleanupFireflies returns buffer.size() for them.
// Without the clamp neither mode touches the samples.
__global__ void __launch_bounds__(256) k_resolve(const float* __restrict__ sr, const float* __restrict__ sg,
                                                 const float* __restrict__ sb, uint32_t band_pix,
                                                 uint32_t spp, uint32_t pix_base, int enable, float k,
                                                 int debug_mode, float* __restrict__ out)
{
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < band_pix; j += gridDim.x * blockDim.x) {
        f3 acc = splat(0.0f);
        uint32_t kept = spp;
        if (enable) {
            float sum = 0.0f;
            for (uint32_t s = 0; s < spp; ++s) {
                const uint64_t g = static_cast<uint64_t>(s) * band_pix + j;
                sum = __fadd_rn(sum, __fdiv_rn(__fadd_rn(__fadd_rn(sr[g], sg[g]), sb[g]), 3.0f));
            }
            const float mean = __fdiv_rn(sum, static_cast<float>(spp));
            float var = 0.0f;
            for (uint32_t s = 0; s < spp; ++s) {
                const uint64_t g = static_cast<uint64_t>(s) * band_pix + j;
                const float df = __fsub_rn(__fdiv_rn(__fadd_rn(__fadd_rn(sr[g], sg[g]), sb[g]), 3.0f), mean);
                var = __fadd_rn(var, __fmul_rn(df, df));
            }
            var = __fdiv_rn(var, static_cast<float>(spp));
            const float sigma = __fsqrt_rn(var);
            if (debug_mode == MT_DEBUG_PIXEL_STANDARD_DEVIATION) {
                for (uint32_t s = 0; s < spp; ++s) acc = acc + splat(sigma);
            } else {
                const float thr = __fmul_rn(k, sigma);
                for (uint32_t s = 0; s < spp; ++s) {
                    const uint64_t g = static_cast<uint64_t>(s) * band_pix + j;
                    const f3 c = {sr[g], sg[g], sb[g]};
                    const float in = __fdiv_rn(__fadd_rn(__fadd_rn(c.x, c.y), c.z), 3.0f);
                    if (fabsf(__fsub_rn(in, mean)) > thr)
                        --kept;
                    else
                        acc = acc + c;
                }
                if (debug_mode == MT_DEBUG_FIREFLY_ELIMINATION) {
                    const float dropped = static_cast<float>(spp - kept);
                    acc = splat(0.0f);
                    for (uint32_t s = 0; s < spp; ++s) acc = acc + splat(dropped);
                    kept = spp;
                }
            }
            if (kept == 0) kept = 1;
        } else {
            for (uint32_t s = 0; s < spp; ++s) {
                const uint64_t g = static_cast<uint64_t>(s) * band_pix + j;
                acc = acc + f3{sr[g], sg[g], sb[g]};
            }
        }
        const f3 r = acc / static_cast<float>(kept);
        float* o = out + 3ull * (pix_base + j);
        o[0] = r.x;
        o[1] = r.y;
        o[2] = r.z;
    }
}

// ApplyHeatMapPostProcessing (Tracer.cpp:672-693): the maximum of the pixel
// intensities (r+g+b)/3 (non-negative floats compare like their bit patterns),
// then every pixel mapped to the ramp of Heatmap (Tracer.cpp:650-670) or grey.
__global__ void k_debug_max(const float* __restrict__ img, uint64_t npix, uint32_t* max_bits)
{
    float m = 0.0f;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < npix;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const float in = __fdiv_rn(__fadd_rn(__fadd_rn(img[3 * i], img[3 * i + 1]), img[3 * i + 2]), 3.0f);
        m = fmaxf(m, in);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(max_bits, __float_as_uint(m));
}

__global__ void k_debug_heatmap(float* __restrict__ img, uint64_t npix, const uint32_t* max_bits, int colorful)
{
    const float maxI = __uint_as_float(*max_bits);
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < npix;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const float in = __fdiv_rn(__fadd_rn(__fadd_rn(img[3 * i], img[3 * i + 1]), img[3 * i + 2]), 3.0f);
        const float t = maxI > 0.0f ? __fdiv_rn(in, maxI) : 0.0f;
        f3 c = splat(t);
        if (colorful) c = heatmap(t);
        img[3 * i] = c.x;
        img[3 * i + 1] = c.y;
        img[3 * i + 2] = c.z;
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
// Launch geometry per device: the SM count and the resident-wave grid of every
// persistent kernel, computed once per device under a lock (devices may differ
// in SM count, and several host threads may launch at once).
struct DeviceGrids {
    int sms = 1;
    unsigned ext[4] = {}, sh[3] = {}, trace[4] = {};
};

template <class K>
static unsigned persistent_grid(K kernel, int block, int sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return static_cast<unsigned>(per_sm * sms);
}

static const DeviceGrids& device_grids()
{
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static DeviceGrids grids[kMaxDevices];
    static bool ready[kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) dev = 0;
    std::lock_guard<std::mutex> lk(mu);
    DeviceGrids& g = grids[dev];
    if (!ready[dev]) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        g.sms = sms > 0 ? sms : 1;
        g.ext[0] = persistent_grid(k_extend<false, false>, 128, g.sms);
        g.ext[1] = persistent_grid(k_extend<true, false>, 128, g.sms);
        g.ext[2] = persistent_grid(k_extend<true, true>, 128, g.sms);
        g.ext[3] = persistent_grid(k_extend<false, false, 64>, 128, g.sms);
        g.sh[0] = persistent_grid(k_shadow<false>, 128, g.sms);
        g.sh[1] = persistent_grid(k_shadow<true>, 128, g.sms);
        g.sh[2] = persistent_grid(k_shadow<false, 64>, 128, g.sms);
        g.trace[MT_QUERY_CLOSEST] = persistent_grid(k_trace<MT_QUERY_CLOSEST>, 128, g.sms);
        g.trace[MT_QUERY_ANY] = persistent_grid(k_trace<MT_QUERY_ANY>, 128, g.sms);
        g.trace[MT_QUERY_CLOSEST_COUNT] = persistent_grid(k_trace<MT_QUERY_CLOSEST_COUNT>, 128, g.sms);
        g.trace[MT_QUERY_CLOSEST_TOTALS] = persistent_grid(k_trace<MT_QUERY_CLOSEST_TOTALS>, 128, g.sms);
        ready[dev] = true;
    }
    return g;
}

cudaError_t preload_render_kernels()
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k_raygen);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_shade<true, true>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_shade<false, true>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_shade<false, false>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_finalize);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_resolve);
    if (e == cudaSuccess) (void)device_grids();  // the traversal kernels (occupancy queries)
    return e;
}

int device_sm_count() { return device_grids().sms; }

static unsigned grid_for(uint64_t n, unsigned block, unsigned per_sm)
{
    const uint64_t need = (n + block - 1) / block;
    const uint64_t cap = static_cast<uint64_t>(device_sm_count()) * per_sm;
    return static_cast<unsigned>(need < cap ? (need ? need : 1) : cap);
}

template <int Q>
static cudaError_t trace_chunks(const DevScene& S, const mt_ray* rays, uint64_t n, mt_hit* hits,
                                uint32_t* fetch, cudaStream_t st)
{
    const unsigned grid = device_grids().trace[Q];
    const uint64_t chunk = 1ull << 30;
    for (uint64_t b = 0; b < n; b += chunk) {
        const uint32_t m = static_cast<uint32_t>(n - b < chunk ? n - b : chunk);
        cudaError_t e = cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
        k_trace<Q><<<grid, 128, 0, st>>>(S, rays + b, m, hits + b, fetch);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_trace(const DevScene& S, const mt_ray* rays, uint64_t n, mt_hit* hits, int query,
                         uint32_t* fetch, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    switch (query) {
        case MT_QUERY_ANY: return trace_chunks<MT_QUERY_ANY>(S, rays, n, hits, fetch, st);
        case MT_QUERY_CLOSEST_COUNT: return trace_chunks<MT_QUERY_CLOSEST_COUNT>(S, rays, n, hits, fetch, st);
        case MT_QUERY_CLOSEST_TOTALS: return trace_chunks<MT_QUERY_CLOSEST_TOTALS>(S, rays, n, hits, fetch, st);
        default: return trace_chunks<MT_QUERY_CLOSEST>(S, rays, n, hits, fetch, st);
    }
}

cudaError_t launch_brdf(const mt_brdf_query* q, uint64_t n, mt_brdf_result* out, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_brdf<<<grid_for(n, 128, 32), 128, 0, st>>>(q, n, out);
    return cudaGetLastError();
}

cudaError_t launch_brdf_sample(const mt_brdf_sample_query* q, uint64_t n, mt_brdf_sample_result* out,
                               cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_brdf_sample<<<grid_for(n, 128, 32), 128, 0, st>>>(q, n, out);
    return cudaGetLastError();
}

void Profiler::begin(int stage, cudaStream_t st)
{
    if (!timing) return;
    if (used + 2 > pool.size()) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        pool.push_back(a);
        pool.push_back(b);
    }
    cudaEventRecord(pool[used], st);
    marks.push_back({stage, used});
    used += 2;
}

void Profiler::end(int stage, cudaStream_t st)
{
    (void)stage;
    if (!timing) return;
    cudaEventRecord(pool[marks.back().second + 1], st);
}

cudaError_t Profiler::collect(double* ms, uint64_t* launches)
{
    for (const auto& m : marks) {
        cudaError_t e = cudaEventSynchronize(pool[m.second + 1]);
        if (e != cudaSuccess) return e;
        float t = 0.0f;
        e = cudaEventElapsedTime(&t, pool[m.second], pool[m.second + 1]);
        if (e != cudaSuccess) return e;
        ms[m.first] += t;
        launches[m.first] += 1;
    }
    marks.clear();
    used = 0;
    return cudaSuccess;
}

Profiler::~Profiler()
{
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
}

cudaError_t launch_batch(const DevScene& S, const PathState& P, const ShadowQueue& SQ,
                         const WaveBuffers& W, uint64_t g0, uint32_t n, uint32_t band_pix,
                         uint32_t pix_base, cudaStream_t st, uint64_t* launches, Profiler* prof,
                         const RecordBuffers* rec, const BatchExtra* extra)
{
    RecordBuffers R = rec ? *rec : RecordBuffers{};
    const BatchExtra X = extra ? *extra : BatchExtra{};
    const NrcShade NC = X.nrc ? *X.nrc : NrcShade{};
    if (NC.mode == MT_NRC_TRAIN) R.nrc = NC.rec;
    // tile order for image batches; the adjoint's record batches keep the
    // row-major order that its replay indexes paths by
    const uint32_t tiled = !rec && !X.scatter_mul && S.width && band_pix % S.width == 0;
    BatchInfo B{g0, n, band_pix, pix_base, X.sample_base, X.scatter_mul, X.scatter_add, tiled};
    const unsigned gw = grid_for(n, 128, 16);
    const DeviceGrids& G = device_grids();
    const unsigned* g_ext = G.ext;
    const unsigned* g_sh = G.sh;
    const bool wide = S.num_instances > 32;
    const bool count = prof && prof->counting;
    unsigned long long* cnt = prof ? prof->d_counts : nullptr;
    auto begin = [&](int s) { if (prof) prof->begin(s, st); };
    auto end = [&](int s) { if (prof) prof->end(s, st); };
    begin(MT_STAGE_RAYGEN);
    k_raygen<<<grid_for(n, 256, 8), 256, 0, st>>>(S, P, B, W.q[0], W.counts, R);
    end(MT_STAGE_RAYGEN);
    uint64_t l = 1;
    int cur = 0;
    // A bounce's shadow rays and the next bounce's extension rays are
    // independent (both come from the bounce's shading), so with a side stream
    // the shadow stage runs there, beside the next extension, and fills that
    // kernel's tail; the next shading waits for both.  Profiled renders keep
    // one stream, so that each stage's events time that stage alone.
    const bool overlap = W.side && !prof;
    cudaError_t e = cudaSuccess;
    for (uint32_t b = 0; b < S.bounces; ++b) {
        const int sqi = sq_slot(b);
        begin(MT_STAGE_EXTEND);
        if (P.dval)  // debug modes: counting traversal plus the per-path debug planes
            k_extend<true, true><<<g_ext[2], 128, 0, st>>>(S, P, W.q[cur], W.counts, cur, sqi, W.rays, cnt);
        else if (count)
            k_extend<true, false><<<g_ext[1], 128, 0, st>>>(S, P, W.q[cur], W.counts, cur, sqi, W.rays, cnt);
        else if (wide)
            k_extend<false, false, 64><<<g_ext[3], 128, 0, st>>>(S, P, W.q[cur], W.counts, cur, sqi, W.rays, cnt);
        else
            k_extend<false, false><<<g_ext[0], 128, 0, st>>>(S, P, W.q[cur], W.counts, cur, sqi, W.rays, cnt);
        end(MT_STAGE_EXTEND);
        if (overlap && b > 0 && e == cudaSuccess) e = cudaStreamWaitEvent(st, W.ev_shadowed, 0);
        begin(MT_STAGE_SHADE);
        if (NC.mode != MT_NRC_OFF || P.dval)
            k_shade<true, true><<<gw, 128, 0, st>>>(S, P, SQ, B, b, W.q[cur], W.q[cur ^ 1], W.counts, cur, sqi, R,
                                                    NC, W.rays + 1);
        else if (R.vert || R.path)
            k_shade<false, true><<<gw, 128, 0, st>>>(S, P, SQ, B, b, W.q[cur], W.q[cur ^ 1], W.counts, cur, sqi, R,
                                                     NC, W.rays + 1);
        else
            k_shade<false, false><<<gw, 128, 0, st>>>(S, P, SQ, B, b, W.q[cur], W.q[cur ^ 1], W.counts, cur, sqi,
                                                      R, NC, W.rays + 1);
        end(MT_STAGE_SHADE);
        cudaStream_t ss = st;
        if (overlap && e == cudaSuccess) {
            e = cudaEventRecord(W.ev_shaded, st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(W.side, W.ev_shaded, 0);
            ss = W.side;
        }
        begin(MT_STAGE_SHADOW);
        if (prof && prof->counting)
            k_shadow<true><<<g_sh[1], 128, 0, ss>>>(S, P, SQ, W.counts, sqi, W.rays + 1, cnt ? cnt + 3 : nullptr, R);
        else if (wide)
            k_shadow<false, 64><<<g_sh[2], 128, 0, ss>>>(S, P, SQ, W.counts, sqi, W.rays + 1, nullptr, R);
        else
            k_shadow<false><<<g_sh[0], 128, 0, ss>>>(S, P, SQ, W.counts, sqi, W.rays + 1, nullptr, R);
        end(MT_STAGE_SHADOW);
        if (overlap && e == cudaSuccess) e = cudaEventRecord(W.ev_shadowed, W.side);
        l += 3;
        cur ^= 1;
    }
    if (overlap && S.bounces > 0 && e == cudaSuccess) e = cudaStreamWaitEvent(st, W.ev_shadowed, 0);
    if (e != cudaSuccess) return e;
    if (NC.mode == MT_NRC_TRAIN) {
        // training paths feed the cache only; no image samples
        e = launch_nrc_targets(P, NC, n, S.bounces, W.q[0], st);  // the queues are free after the bounces
        if (e != cudaSuccess) return e;
        if (launches) *launches += l + 3;
        return cudaSuccess;
    }
    if (NC.mode == MT_NRC_QUERY) {
        if (X.query_after) e = cudaStreamWaitEvent(st, X.query_after, 0);
        if (e == cudaSuccess) e = launch_nrc_query(NC.net, P, NC.rec, NC.count, n, NC.total, NC.err, st);
        if (e != cudaSuccess) return e;
        ++l;
    }
    begin(MT_STAGE_FINALIZE);
    k_finalize<<<grid_for(n, 256, 8), 256, 0, st>>>(S, P, B, W.sr, W.sg, W.sb, R);
    end(MT_STAGE_FINALIZE);
    ++l;
    if (launches) *launches += l;
    return cudaGetLastError();
}

bool debug_needs_post(int mode)
{
    switch (mode) {
        case MT_DEBUG_PRIMARY_BVH_TESTS: case MT_DEBUG_TOTAL_BVH_TESTS: case MT_DEBUG_PRIMARY_TRIANGLE_TESTS:
        case MT_DEBUG_TOTAL_TRIANGLE_TESTS: case MT_DEBUG_BOUNCES: case MT_DEBUG_FIREFLY_ELIMINATION:
        case MT_DEBUG_DEPTH: case MT_DEBUG_FIRST_HIT_BRDF: case MT_DEBUG_PIXEL_STANDARD_DEVIATION: return true;
        default: return false;
    }
}

cudaError_t launch_debug_post(float* img, uint64_t npix, int mode, uint32_t* scratch, cudaStream_t st)
{
    if (!debug_needs_post(mode) || npix == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const unsigned grid = grid_for(npix, 256, 8);
    k_debug_max<<<grid, 256, 0, st>>>(img, npix, scratch);
    const bool colorful = !(mode == MT_DEBUG_DEPTH || mode == MT_DEBUG_FIRST_HIT_BRDF ||
                            mode == MT_DEBUG_PIXEL_STANDARD_DEVIATION);
    k_debug_heatmap<<<grid, 256, 0, st>>>(img, npix, scratch, colorful ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_resolve(const DevScene& S, const WaveBuffers& W, uint32_t band_pix, uint32_t pix_base,
                           float* out, cudaStream_t st, Profiler* prof)
{
    if (prof) prof->begin(MT_STAGE_RESOLVE, st);
    k_resolve<<<grid_for(band_pix, 256, 8), 256, 0, st>>>(W.sr, W.sg, W.sb, band_pix, S.spp, pix_base,
                                                          S.firefly_enable, S.firefly_k, S.debug_mode, out);
    if (prof) prof->end(MT_STAGE_RESOLVE, st);
    return cudaGetLastError();
}

cudaError_t launch_resolve_planes(const float* sr, const float* sg, const float* sb, uint32_t npix, uint32_t spp,
                                  int enable, float k, int debug_mode, float* out, cudaStream_t st)
{
    if (npix == 0) return cudaSuccess;
    k_resolve<<<grid_for(npix, 256, 8), 256, 0, st>>>(sr, sg, sb, npix, spp, 0, enable, k, debug_mode, out);
    return cudaGetLastError();
}

}  // namespace mt
