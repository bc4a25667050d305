// mt_adjoint.cu - path-replay adjoint of the render (no reference counterpart).
//
// Gradient of L = sum over pixels and channels of (image - target)^2 with
// respect to every material's base colour factor, roughness factor and
// metallic factor, every light's intensity (a scale on its colour), and the
// texels of RGB32F base-colour textures.  The render is the reference estimator
// (Tracer.cpp:134-348) with the counter RNG: a batch of paths is replayed from
// its seeds by the forward stages with recording on (per-vertex records, O(batch)
// memory), then k_adjoint walks each path forward to rebuild the throughput and
// backward to push dL/d(sample) into the parameters.  Sampling decisions and
// pdfs, the light-pick probabilities, the energy cut-off and the firefly mask
// are held constant (the path-replay convention), so each sample's gradient is
// that of its BRDF, light and sky factors along the fixed path.
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mt_adjoint.h"
#include "mt_device.cuh"
#include "mt_kernels.h"

namespace mt {
namespace {

// ---------------------------------------------------------------------------
// Forward-mode duals over (base r, base g, base b, roughness, metallic)
// ---------------------------------------------------------------------------
struct D5 {
    float v;
    float g[5];
};
__device__ __forceinline__ D5 dconst(float v)
{
    D5 r;
    r.v = v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.g[k] = 0.0f;
    return r;
}
__device__ __forceinline__ D5 dvar(float v, int k)
{
    D5 r = dconst(v);
    r.g[k] = 1.0f;
    return r;
}
__device__ __forceinline__ D5 operator+(D5 a, D5 b)
{
    D5 r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.g[k] = a.g[k] + b.g[k];
    return r;
}
__device__ __forceinline__ D5 operator-(D5 a, D5 b)
{
    D5 r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.g[k] = a.g[k] - b.g[k];
    return r;
}
__device__ __forceinline__ D5 operator*(D5 a, D5 b)
{
    D5 r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.g[k] = a.g[k] * b.v + a.v * b.g[k];
    return r;
}
__device__ __forceinline__ D5 operator/(D5 a, D5 b)
{
    D5 r;
    r.v = a.v / b.v;
    const float ib2 = 1.0f / (b.v * b.v);
#pragma unroll
    for (int k = 0; k < 5; ++k) r.g[k] = (a.g[k] * b.v - a.v * b.g[k]) * ib2;
    return r;
}
__device__ __forceinline__ D5 operator*(D5 a, float s)
{
    D5 r;
    r.v = a.v * s;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.g[k] = a.g[k] * s;
    return r;
}
__device__ __forceinline__ D5 operator+(D5 a, float s)
{
    a.v += s;
    return a;
}
__device__ __forceinline__ D5 rsub(float s, D5 a)  // s - a
{
    D5 r;
    r.v = s - a.v;
#pragma unroll
    for (int k = 0; k < 5; ++k) r.g[k] = -a.g[k];
    return r;
}
__device__ __forceinline__ D5 dmax(D5 a, float lo) { return (a.v < lo) ? dconst(lo) : a; }
__device__ __forceinline__ D5 dclamp01(D5 a)
{
    if (a.v < 0.0f) return dconst(0.0f);
    if (a.v > 1.0f) return dconst(1.0f);
    return a;
}

// EvaluateBRDF (BRDF.hpp:52-77) with derivatives with respect to base colour,
// roughness and metallic; adj is dL/d(brdf rgb).  Adds the vector-Jacobian
// product into grad[5].
__device__ void brdf_vjp(f3 L, f3 V, f3 N, f3 base, float rough, float metal, f3 adj, float* grad)
{
    const float nl = fmaxf(L.x * N.x + L.y * N.y + L.z * N.z, 0.0f);
    const float nv = fmaxf(V.x * N.x + V.y * N.y + V.z * N.z, 0.0f);
    if (nl <= 0.0f || nv <= 0.0f) return;
    f3 h = {V.x + L.x, V.y + L.y, V.z + L.z};
    const float hl = rsqrtf(h.x * h.x + h.y * h.y + h.z * h.z);
    h = {h.x * hl, h.y * hl, h.z * hl};
    const float nh = fminf(fmaxf(N.x * h.x + N.y * h.y + N.z * h.z, 0.0f), 1.0f);
    const float hv = fminf(fmaxf(h.x * V.x + h.y * V.y + h.z * V.z, 0.0f), 1.0f);
    const D5 r = dmax(dvar(rough, 3), 0.05f);
    const D5 m = dvar(metal, 4);
    const D5 mc = dclamp01(m);
    const float p5 = pow5(1.0f - hv);
    // D (GGX) and G (Smith-Schlick), functions of roughness only
    const D5 a = r * r;
    const D5 a2 = a * a;
    D5 den = (a2 + (-1.0f)) * (nh * nh) + 1.0f;
    den = den * den * kPi;
    const D5 Dg = a2 / den;
    const D5 rr = r + 1.0f;
    const D5 k = rr * rr * 0.125f;
    const D5 g1 = dconst(nv) / (rsub(1.0f, k) * nv + k);
    const D5 g2 = dconst(nl) / (rsub(1.0f, k) * nl + k);
    const D5 DG = Dg * (g1 * g2);
    const float sden = fmaxf(4.0f * nv * nl, 0.001f);
    const float bc[3] = {base.x, base.y, base.z};
    const float ad[3] = {adj.x, adj.y, adj.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const D5 b = dvar(bc[c], c);
        const D5 f0 = rsub(1.0f, mc) * 0.04f + b * mc;
        const D5 F = f0 + rsub(1.0f, f0) * p5;
        const D5 kd = rsub(1.0f, F) * rsub(1.0f, m);
        const D5 f = kd * b * (1.0f / kPi) + DG * F * (1.0f / sden);
        if (f.v < 0.0f) continue;  // clamped at zero (BRDF.hpp:76)
#pragma unroll
        for (int q = 0; q < 5; ++q) grad[q] += ad[c] * f.g[q];
    }
}

__device__ __forceinline__ float aces_d(float x)
{
    const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
    const float n = x * (a * x + b), dn = x * (c * x + d) + e;
    return ((2.0f * a * x + b) * dn - n * (2.0f * c * x + d)) / (dn * dn);
}

// Texel taps of Image::Sample for a texture lookup at uv (weights of the
// nearest / quirky-linear filter, Image.cpp:17-61).
__device__ int texel_taps(const DevTexture& t, float uvx, float uvy, long long* idx, float* w)
{
    const float u = __fsub_rn(uvx, floorf(uvx));
    const float v = __fsub_rn(uvy, floorf(uvy));
    const int W = static_cast<int>(t.w), H = static_cast<int>(t.h);
    const long long maxIdx = static_cast<long long>(t.w) * t.h - 1;
    auto at = [&](int x, int y) {
        long long i = static_cast<long long>(y) * t.w + x;
        return i < 0 ? 0 : (i > maxIdx ? maxIdx : i);
    };
    if (t.filter == MT_FILTER_LINEAR) {
        const int x0 = static_cast<int>(floorf(__fmul_rn(u, static_cast<float>(W))));
        const int x1 = min(x0 + 1, W - 1);
        const int y0 = static_cast<int>(floorf(__fmul_rn(v, static_cast<float>(H))));
        const int y1 = min(y0 + 1, H - 1);
        const float sx = __fsub_rn(u, __fdiv_rn(static_cast<float>(x0), static_cast<float>(W)));
        const float sy = __fsub_rn(v, __fdiv_rn(static_cast<float>(y0), static_cast<float>(H)));
        idx[0] = at(x0, y0);
        w[0] = (1.0f - sx) * (1.0f - sy);
        idx[1] = at(x1, y0);
        w[1] = sx * (1.0f - sy);
        idx[2] = at(x0, y1);
        w[2] = (1.0f - sx) * sy;
        idx[3] = at(x1, y1);
        w[3] = sx * sy;
        return 4;
    }
    int ix = static_cast<int>(__fmul_rn(u, static_cast<float>(W))) % W;
    int iy = static_cast<int>(__fmul_rn(v, static_cast<float>(H))) % H;
    if (ix < 0) ix += W;
    if (iy < 0) iy += H;
    idx[0] = at(ix, iy);
    w[0] = 1.0f;
    return 1;
}

// Adds (x, y, z) to the RGB texel gradient at p, aggregated over the warp: the
// lanes that reach this call with the same texel (adjacent pixels of a sample
// often land on one texel) sum their values first and one of them issues the
// three atomics.
__device__ __forceinline__ void texel_add(float* p, float x, float y, float z)
{
    namespace cg = cooperative_groups;
    const cg::coalesced_group active = cg::coalesced_threads();
    const cg::coalesced_group same =
        cg::labeled_partition(active, static_cast<unsigned long long>(reinterpret_cast<uintptr_t>(p)));
    if (same.size() > 1) {
        x = cg::reduce(same, x, cg::plus<float>());
        y = cg::reduce(same, y, cg::plus<float>());
        z = cg::reduce(same, z, cg::plus<float>());
    }
    if (same.thread_rank() == 0) {
        atomicAdd(p, x);
        atomicAdd(p + 1, y);
        atomicAdd(p + 2, z);
    }
}

struct VertexMat {
    f3 base;       // remapped base colour 0.96 c + 0.04 (Tracer.cpp:159)
    float rough, metal;
    f3 emission;
    f3 tex_base;   // base-colour texel value (1 without a texture)
    float tex_r, tex_m;  // metallic-roughness texel g / b (1 without a texture)
};

__device__ VertexMat vertex_material(const DevScene& S, uint32_t mi, float u, float v)
{
    const MatPoint mp = sample_material(S, mi, u, v);
    const DevMaterial M = S.materials[mi];
    VertexMat r;
    r.base = {__fadd_rn(__fmul_rn(mp.base.x, 0.96f), 0.04f), __fadd_rn(__fmul_rn(mp.base.y, 0.96f), 0.04f),
              __fadd_rn(__fmul_rn(mp.base.z, 0.96f), 0.04f)};
    r.rough = mp.roughness;
    r.metal = mp.metallic;
    r.emission = mp.emission;
    r.tex_base = splat(1.0f);
    if (M.base_tex >= 0) {
        const f4 t = tex_sample(S, M.base_tex, u, v);
        r.tex_base = {t.x, t.y, t.z};
    }
    r.tex_r = r.tex_m = 1.0f;
    if (M.mr_tex >= 0) {
        const f4 t = tex_sample(S, M.mr_tex, u, v);
        r.tex_r = t.y;
        r.tex_m = t.z;
    }
    return r;
}

}  // namespace

// Per pixel of a band: firefly statistics (as k_resolve computes them), the
// residual image - target and the loss.
__global__ void k_grad_pixel(const float* __restrict__ sr, const float* __restrict__ sg,
                             const float* __restrict__ sb, uint32_t band_pix, uint32_t spp, uint32_t pix_base,
                             int enable, float kf, const float* __restrict__ image,
                             const float* __restrict__ target, const float* __restrict__ dimg,
                             float4* __restrict__ pix, float* loss)
{
    float local = 0.0f;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < band_pix; j += gridDim.x * blockDim.x) {
        float mean = 0.0f, thr = FLT_MAX;
        uint32_t kept = spp;
        if (enable) {
            float sum = 0.0f;
            for (uint32_t s = 0; s < spp; ++s) {
                const uint64_t g = static_cast<uint64_t>(s) * band_pix + j;
                sum = __fadd_rn(sum, __fdiv_rn(__fadd_rn(__fadd_rn(sr[g], sg[g]), sb[g]), 3.0f));
            }
            mean = __fdiv_rn(sum, static_cast<float>(spp));
            float var = 0.0f;
            for (uint32_t s = 0; s < spp; ++s) {
                const uint64_t g = static_cast<uint64_t>(s) * band_pix + j;
                const float df = __fsub_rn(__fdiv_rn(__fadd_rn(__fadd_rn(sr[g], sg[g]), sb[g]), 3.0f), mean);
                var = __fadd_rn(var, __fmul_rn(df, df));
            }
            var = __fdiv_rn(var, static_cast<float>(spp));
            thr = __fmul_rn(kf, __fsqrt_rn(var));
            for (uint32_t s = 0; s < spp; ++s) {
                const uint64_t g = static_cast<uint64_t>(s) * band_pix + j;
                const float in = __fdiv_rn(__fadd_rn(__fadd_rn(sr[g], sg[g]), sb[g]), 3.0f);
                if (fabsf(__fsub_rn(in, mean)) > thr) --kept;
            }
            if (kept == 0) kept = 1;
        }
        const uint64_t px = pix_base + j;
        float rx, ry, rz;  // half of dL/d(image)
        if (dimg) {
            rx = 0.5f * dimg[3 * px];
            ry = 0.5f * dimg[3 * px + 1];
            rz = 0.5f * dimg[3 * px + 2];
        } else {
            rx = image[3 * px] - target[3 * px];
            ry = image[3 * px + 1] - target[3 * px + 1];
            rz = image[3 * px + 2] - target[3 * px + 2];
            local += rx * rx + ry * ry + rz * rz;
        }
        pix[2 * j] = make_float4(mean, thr, 2.0f / static_cast<float>(kept), 0.0f);
        pix[2 * j + 1] = make_float4(rx, ry, rz, 0.0f);
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, local);
}

// The bin of path p of a batch: its vertex count, or the last bin when its
// sample is rejected by the firefly clamp (no gradient flows through it).
__device__ __forceinline__ uint32_t adjoint_bin(const DevScene& S, const GradParams& G, const RecordBuffers& R,
                                                const float* __restrict__ sr, const float* __restrict__ sg,
                                                const float* __restrict__ sb, uint64_t g0, uint32_t p,
                                                uint32_t band_pix)
{
    const uint64_t g = g0 + p;
    const uint32_t s = static_cast<uint32_t>(g / band_pix);
    const uint32_t j = static_cast<uint32_t>(g - static_cast<uint64_t>(s) * band_pix);
    if (S.firefly_enable) {
        const float4 px = G.pix[2 * j];
        const float in = __fdiv_rn(__fadd_rn(__fadd_rn(sr[g], sg[g]), sb[g]), 3.0f);
        if (fabsf(__fsub_rn(in, px.x)) > px.y) return kAdjointBins - 1;
    }
    const int nv = static_cast<int>(R.path[2 * p].w);
    return nv >= 0 && nv <= MT_GRAD_MAX_BOUNCES ? static_cast<uint32_t>(nv) : kAdjointBins - 1;
}

// Counting pass (first) and placement pass of the grouping by vertex count:
// lanes with the same bin reserve their slots with one atomic per warp.
template <bool PLACE>
__global__ void k_adjoint_order(DevScene S, GradParams G, RecordBuffers R, const float* __restrict__ sr,
                                const float* __restrict__ sg, const float* __restrict__ sb, uint64_t g0, uint32_t n,
                                uint32_t band_pix)
{
    const uint32_t lane = threadIdx.x & 31;
    uint32_t first[kAdjointBins];
    if (PLACE) {  // longest paths first: the short ones fill the launch's tail
        uint32_t acc = 0;
        for (int b = kAdjointBins - 2; b >= 0; --b) {
            first[b] = acc;
            acc += G.bins[b];
        }
        first[kAdjointBins - 1] = acc;
    }
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        const bool in = p < n;
        const uint32_t b = in ? adjoint_bin(S, G, R, sr, sg, sb, g0, p, band_pix) : 0xffffffffu;
        const uint32_t same = __match_any_sync(0xffffffffu, b);
        const uint32_t leader = __ffs(same) - 1;
        uint32_t slot = 0;
        if (in && lane == leader) slot = atomicAdd(&G.bins[(PLACE ? kAdjointBins : 0) + b], __popc(same));
        slot = __shfl_sync(0xffffffffu, slot, leader) + __popc(same & ((1u << lane) - 1u));
        if (PLACE && in && b < kAdjointBins - 1) G.order[first[b] + slot] = p;
    }
}

// One thread per path of a recorded batch, in the order k_adjoint_order
// gave (the rejected samples left out).
__global__ void __launch_bounds__(128) k_adjoint(DevScene S, GradParams G, RecordBuffers R, uint64_t g0,
                                                 uint32_t band_pix)
{
    extern __shared__ float sh[];  // per block: materials x 5, then lights
    const uint32_t nm = G.smem_materials, nlg = G.smem_lights;
    for (uint32_t i = threadIdx.x; i < nm * 5 + nlg; i += blockDim.x) sh[i] = 0.0f;
    uint32_t kept = 0;
    for (uint32_t b = 0; b + 1 < kAdjointBins; ++b) kept += G.bins[b];
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < kept; i += gridDim.x * blockDim.x) {
        const uint32_t p = G.order[i];
        const uint64_t g = g0 + p;
        const uint32_t s = static_cast<uint32_t>(g / band_pix);
        const uint32_t j = static_cast<uint32_t>(g - static_cast<uint64_t>(s) * band_pix);
        const float4 px = G.pix[2 * j];
        const float4 res = G.pix[2 * j + 1];
        const float4 pr0 = R.path[2 * p], pr1 = R.path[2 * p + 1];
        const float e = S.exposure;
        // dL/d(total) per channel: 2 r / kept * ACES'(total * exposure) * exposure
        const f3 gv = {res.x * px.z * aces_d(pr0.x * e) * e, res.y * px.z * aces_d(pr0.y * e) * e,
                       res.z * px.z * aces_d(pr0.z * e) * e};
        const int nv = static_cast<int>(pr0.w);
        const int miss = static_cast<int>(pr1.w);
        // forward: throughput before each vertex
        f3 cur[MT_GRAD_MAX_BOUNCES + 1];
        cur[0] = splat(1.0f);
        for (int i = 0; i < nv; ++i) {
            const float4* vr = R.vert + (static_cast<uint64_t>(p) * S.bounces + i) * 5;
            const uint32_t fl = __float_as_uint(vr[1].w);
            cur[i + 1] = cur[i];
            if ((fl & MT_VREC_CHOSEN) && (fl & MT_VREC_NEXT)) {
                const VertexMat vm = vertex_material(S, __float_as_uint(vr[0].w), vr[4].x, vr[4].y);
                const f3 fb = eval_brdf(xyz(vr[2]), xyz(vr[1]), xyz(vr[0]), vm.base, vm.rough, vm.metal);
                cur[i + 1] = cur[i] * (fb * vr[2].w);
            }
        }
        // backward
        f3 adj = splat(0.0f);
        f3 adj_base_sky = splat(0.0f);
        if (miss >= 0 && miss == nv) {
            const f3 sky = xyz(pr1);
            if (nv > 0) {
                const float4* vr = R.vert + (static_cast<uint64_t>(p) * S.bounces + (nv - 1)) * 5;
                const VertexMat vm = vertex_material(S, __float_as_uint(vr[0].w), vr[4].x, vr[4].y);
                adj = gv * vm.base * sky;
                adj_base_sky = gv * cur[nv] * sky;
            }
        }
        for (int i = nv - 1; i >= 0; --i) {
            const float4* vr = R.vert + (static_cast<uint64_t>(p) * S.bounces + i) * 5;
            const uint32_t fl = __float_as_uint(vr[1].w);
            const uint32_t mi = __float_as_uint(vr[0].w);
            const VertexMat vm = vertex_material(S, mi, vr[4].x, vr[4].y);
            const f3 N = xyz(vr[0]), V = xyz(vr[1]);
            float gr[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            if (i == nv - 1) {
                gr[0] += adj_base_sky.x;
                gr[1] += adj_base_sky.y;
                gr[2] += adj_base_sky.z;
            }
            const f3 adj_next = adj;
            if ((fl & MT_VREC_CHOSEN) && (fl & MT_VREC_NEXT)) {
                const f3 fb = eval_brdf(xyz(vr[2]), V, N, vm.base, vm.rough, vm.metal);
                adj = adj_next * (fb * vr[2].w);
                brdf_vjp(xyz(vr[2]), V, N, vm.base, vm.rough, vm.metal, (adj_next * cur[i]) * vr[2].w, gr);
            }
            adj = adj + (gv * S.emission_base) * vm.emission;
            if ((fl & MT_VREC_CHOSEN) && (fl & MT_VREC_VISIBLE)) {
                const uint32_t li = __float_as_uint(vr[4].z);
                const DevLight& L = S.lights[li];
                const f3 lc = f3{__ldg(&L.color[0]), __ldg(&L.color[1]), __ldg(&L.color[2])} * (vr[4].w * vr[3].w);
                const f3 fl_ = eval_brdf(xyz(vr[3]), V, N, vm.base, vm.rough, vm.metal);
                adj = adj + gv * fl_ * lc;
                brdf_vjp(xyz(vr[3]), V, N, vm.base, vm.rough, vm.metal, gv * cur[i] * lc, gr);
                const f3 c = cur[i] * fl_ * lc;
                const float dli = gv.x * c.x + gv.y * c.y + gv.z * c.z;
                if (li < nlg)
                    atomicAdd(&sh[nm * 5 + li], dli);
                else
                    atomicAdd(&G.d_light[li], dli);
            }
            // chain to the material factors (base = 0.96 tex * factor + 0.04)
            const f3 db = {gr[0] * 0.96f, gr[1] * 0.96f, gr[2] * 0.96f};
            const float dfac[5] = {db.x * vm.tex_base.x, db.y * vm.tex_base.y, db.z * vm.tex_base.z,
                                   gr[3] * vm.tex_r, gr[4] * vm.tex_m};
            if (mi < nm) {
#pragma unroll
                for (int q = 0; q < 5; ++q)
                    if (dfac[q] != 0.0f) atomicAdd(&sh[mi * 5 + q], dfac[q]);
            } else {
                atomicAdd(&G.d_base[3 * mi], dfac[0]);
                atomicAdd(&G.d_base[3 * mi + 1], dfac[1]);
                atomicAdd(&G.d_base[3 * mi + 2], dfac[2]);
                atomicAdd(&G.d_rough[mi], dfac[3]);
                atomicAdd(&G.d_metal[mi], dfac[4]);
            }
            // base-colour texels of RGB32F textures
            const DevMaterial M = S.materials[mi];
            if (G.d_texels && M.base_tex >= 0 && G.texel_off[M.base_tex] >= 0) {
                const DevTexture t = S.textures[M.base_tex];
                long long idx[4];
                float w[4];
                const int nt = texel_taps(t, __fadd_rn(__fmul_rn(vr[4].x, t.sclx), t.offx),
                                          __fadd_rn(__fmul_rn(vr[4].y, t.scly), t.offy), idx, w);
                float* dt = G.d_texels + G.texel_off[M.base_tex];
                for (int q = 0; q < nt; ++q) {
                    if (w[q] == 0.0f) continue;
                    texel_add(dt + 3 * idx[q], db.x * M.base[0] * w[q], db.y * M.base[1] * w[q],
                              db.z * M.base[2] * w[q]);
                }
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nm * 5; i += blockDim.x) {
        const float v = sh[i];
        if (v == 0.0f) continue;
        const uint32_t m = i / 5, q = i % 5;
        if (q < 3)
            atomicAdd(&G.d_base[3 * m + q], v);
        else if (q == 3)
            atomicAdd(&G.d_rough[m], v);
        else
            atomicAdd(&G.d_metal[m], v);
    }
    for (uint32_t i = threadIdx.x; i < nlg; i += blockDim.x)
        if (sh[nm * 5 + i] != 0.0f) atomicAdd(&G.d_light[i], sh[nm * 5 + i]);
}

cudaError_t launch_grad_pixel(const DevScene& S, const WaveBuffers& W, uint32_t band_pix, uint32_t pix_base,
                              const float* image, const GradParams& G, cudaStream_t st)
{
    const unsigned grid = static_cast<unsigned>((band_pix + 255) / 256 < 4096 ? (band_pix + 255) / 256 : 4096);
    k_grad_pixel<<<grid ? grid : 1, 256, 0, st>>>(W.sr, W.sg, W.sb, band_pix, S.spp, pix_base, S.firefly_enable,
                                                   S.firefly_k, image, G.target, G.d_image, G.pix,
                                                   G.d_image ? nullptr : G.loss);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(const DevScene& S, const GradParams& G, const RecordBuffers& R, const WaveBuffers& W,
                           uint64_t g0, uint32_t n, uint32_t band_pix, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(G.bins, 0, 2 * kAdjointBins * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    const unsigned og = static_cast<unsigned>((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    k_adjoint_order<false><<<og ? og : 1, 256, 0, st>>>(S, G, R, W.sr, W.sg, W.sb, g0, n, band_pix);
    k_adjoint_order<true><<<og ? og : 1, 256, 0, st>>>(S, G, R, W.sr, W.sg, W.sb, g0, n, band_pix);
    const size_t smem = (static_cast<size_t>(G.smem_materials) * 5 + G.smem_lights) * sizeof(float);
    const unsigned grid = static_cast<unsigned>((n + 127) / 128 < 8192 ? (n + 127) / 128 : 8192);
    k_adjoint<<<grid ? grid : 1, 128, smem, st>>>(S, G, R, g0, band_pix);
    return cudaGetLastError();
}

}  // namespace mt
