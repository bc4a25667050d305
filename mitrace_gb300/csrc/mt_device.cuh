// mt_device.cuh - device-side data layout and functions of the GB300 path tracer.
//
// Arithmetic that decides WHICH triangle a ray hits (slab test, Moller-Trumbore,
// ray-to-local transform, world distance) and the camera-ray construction use
// explicit round-to-nearest intrinsics (__fadd_rn/__fmul_rn/__fdiv_rn/
// __fsqrt_rn) so the compiler cannot contract them into FMAs; with the same
// association order as the reference's GLM calls this gives bit-identical
// results to the reference traversal run with IEEE single precision
// (src/Tracer/Intersect.cpp:9-219).  Shading uses the same exact operations;
// only the transcendental calls (sinf, cosf, acosf, atan2f, powf) can differ by
// an ulp from the host C library.
#pragma once
#include <type_traits>

#include <cfloat>
#include <cstdint>

#include "../../include/mitrace_gpu.h"

namespace mt {

// ---------------------------------------------------------------------------
// Exact-rounding vector math (GLM association order, see header comment).
// ---------------------------------------------------------------------------
struct f3 {
    float x, y, z;
};

__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 splat(float s) { return f3{s, s, s}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b)
{
    return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 operator-(f3 a, f3 b)
{
    return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b)
{
    return {__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 operator*(f3 a, float s)
{
    return {__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
__device__ __forceinline__ f3 operator*(float s, f3 a) { return a * s; }
__device__ __forceinline__ f3 operator/(f3 a, float s)
{
    return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)};
}
__device__ __forceinline__ f3 operator/(f3 a, f3 b)
{
    return {__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y), __fdiv_rn(a.z, b.z)};
}
__device__ __forceinline__ f3 operator+(f3 a, float s)
{
    return {__fadd_rn(a.x, s), __fadd_rn(a.y, s), __fadd_rn(a.z, s)};
}
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi)
{
    return gmin(gmax(x, lo), hi);
}
__device__ __forceinline__ f3 vmin(f3 a, f3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
__device__ __forceinline__ f3 vmax(f3 a, f3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
__device__ __forceinline__ float dot(f3 a, f3 b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ f3 cross(f3 a, f3 b)
{
    return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(b.y, a.z)),
            __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(b.z, a.x)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(b.x, a.y))};
}
__device__ __forceinline__ float length(f3 v) { return __fsqrt_rn(dot(v, v)); }
__device__ __forceinline__ f3 normalize(f3 v) { return v * __fdiv_rn(1.0f, __fsqrt_rn(dot(v, v))); }
__device__ __forceinline__ f3 reflect(f3 i, f3 n) { return i - n * dot(n, i) * 2.0f; }
__device__ __forceinline__ f3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ f3 xyz(float4 v) { return {v.x, v.y, v.z}; }

// Column-major 4x4 times (x, y, z, w): (c0*x + c1*y) + (c2*z + c3*w).
__device__ __forceinline__ float mrow(const float* m, int r, float x, float y, float z, float w)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(m[r], x), __fmul_rn(m[4 + r], y)),
                     __fadd_rn(__fmul_rn(m[8 + r], z), __fmul_rn(m[12 + r], w)));
}
__device__ __forceinline__ f3 xform_point(const float* m, f3 p)
{
    return {mrow(m, 0, p.x, p.y, p.z, 1.0f), mrow(m, 1, p.x, p.y, p.z, 1.0f),
            mrow(m, 2, p.x, p.y, p.z, 1.0f)};
}
__device__ __forceinline__ f3 xform_dir(const float* m, f3 d)
{
    return {mrow(m, 0, d.x, d.y, d.z, 0.0f), mrow(m, 1, d.x, d.y, d.z, 0.0f),
            mrow(m, 2, d.x, d.y, d.z, 0.0f)};
}

constexpr float kPi = 3.14159265358979323846f;

// ---------------------------------------------------------------------------
// Device scene layout.
// ---------------------------------------------------------------------------
// BVH node: two float4, (lo.xyz, a) and (hi.xyz, b) with a/b as raw bits, the
// reference's 32-byte node (src/Scene/BVH.hpp:74-119).  Node indices are the
// reference's, so the siblings of a pair sit at (a, a+1).
// Triangle slot: three float4 (v0.xyz | original triangle id, e1.xyz, e2.xyz);
// for BVH meshes the slots follow the BVH index array, so a leaf's triangles
// are contiguous; e1 = v1 - v0 and e2 = v2 - v0 are the same IEEE differences
// the Moller-Trumbore test forms.
struct DevMesh {
    uint32_t node_off;   // first node in DevScene::nodes (in nodes, not float4s)
    uint32_t slot_off;   // first triangle slot
    uint32_t num_slots;  // slots of this mesh (triangles, or BVH indices)
    uint32_t has_bvh;
    uint32_t attr_off;   // first triangle of this mesh in normals/uvs arrays
    uint32_t has_uv;
    uint32_t num_tris;
    uint32_t pad;
};

struct DevInstance {
    float model[16];
    float inv[16];
    float wlo[3];
    uint32_t mesh;
    float whi[3];
    uint32_t material;
};

struct DevMaterial {
    float base[4];
    float emissive[3];
    float normal_scale;
    float metallic;
    float roughness;
    int32_t base_tex, mr_tex, nrm_tex, em_tex;
};

struct DevTexture {
    const uint8_t* rgb8;
    const float* rgbf;
    uint32_t w, h;
    int32_t filter;
    float offx, offy, sclx, scly;
    uint32_t pad;
};

struct DevLight {
    int32_t type;
    float pos[3];
    float color[3];
    float dir[3];
    float point_size, inner_cos, outer_cos, simple;
};

struct DevScene {
    const float4* nodes;
    const float4* slots;
    const float* normals;  // 9 floats per triangle
    const float* uvs;      // 6 floats per triangle
    const DevMesh* meshes;
    const DevInstance* instances;
    const DevMaterial* materials;
    const DevTexture* textures;
    const DevLight* lights;
    uint32_t num_instances;
    uint32_t num_lights;
    int32_t env;
    float hdri_prim, hdri_sec, emission_base;
    // camera
    int32_t cam_type;
    float c2w[16];
    float fov_scale, cam_aspect, ortho_x, ortho_y;
    // render settings
    uint32_t width, height, bounces, spp;
    float terminate_energy, exposure, px_w, px_h, render_aspect;
    uint32_t key0, key1;
    int32_t firefly_enable;
    float firefly_k;
    int* error_flag;
    int32_t debug_mode;  // Config::DebugMode (MT_DEBUG_*), 0 = DebugNone
    int32_t trav_pops;      // node pops per lane between two leaf passes (>= 1)
    int32_t trav_prefetch;  // 1: prefetch a reached leaf's slots into L2
    int32_t trav_switch;    // lanes that wait before an instance switch runs (>= 1)
};

#define MT_STACK_SIZE 64
// Traversal settings chosen per scene at upload (DevScene::trav_pops /
// trav_prefetch): a scene whose nodes and triangle slots fit in a fraction of
// L2 pops up to MT_TRAVERSE_POPS_RESIDENT nodes per lane between two leaf
// passes of the warp and prefetches nothing; a larger scene pops one node per
// pass and has each leaf's triangle slots (the first 32) brought into L2 the
// moment a lane reaches the leaf, so that the leaf's warp pass finds them there
// (measured: +2% Mrays/s on an 11 MB scene, +10% on a 1.5 GB one).  Pops
// per pass on the material grid with batched instance switches, Mrays/s:
// 3 -> 1058, 4 -> 1049, 5 -> 1052.
#ifndef MT_TRAVERSE_POPS_RESIDENT
#define MT_TRAVERSE_POPS_RESIDENT 3
#endif
#ifndef MT_TRAVERSE_RESIDENT_L2_FRACTION
#define MT_TRAVERSE_RESIDENT_L2_FRACTION 0.5
#endif

// Requesting lanes served by one world-box pass on a one-chunk scene (1, 2, 4
// or 8).  A pass is a short dependent chain (shuffle, slab test, ballot), so
// two independent chains per pass hide each other's latency; more spill
// (material grid Mrays/s: 1 -> 1396, 2 -> 1449, 4 -> 1363, 8 -> 1273).
#ifndef MT_MASK_GROUP
#define MT_MASK_GROUP 2
#endif
// Instance switches (close an instance, open the next, finish a ray and fetch
// the next) of a scene whose switches are frequent run once at least
// DevScene::trav_switch lanes wait for one, or when no lane has a node or a
// leaf left; each switch is a long stretch of lane-divergent code (two 4x4
// matrices, exact divisions and square roots), so running it for several
// lanes at once costs little more than for one (measured on the 50-instance
// material grid: 1 lane 1035, 8 lanes 1046, 12 lanes 1050, 16 lanes 1050,
// 24 lanes 1035 Mrays/s; re-measured with the current world-box phase,
// batches and stack: 8 lanes 1442, 12 lanes 1467, 16 lanes 1480).
#ifndef MT_TRAVERSE_SWITCH_RESIDENT
#define MT_TRAVERSE_SWITCH_RESIDENT 16
#endif

// Bulk prefetch of [p, p + bytes) into L2 (no registers, no completion to wait
// for); p 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
#define MT_ERRBIT_STACK 1
#define MT_ERRBIT_TIMEOUT 2  // a bounded wait on the tensor cores ran out

// ---------------------------------------------------------------------------
// Intersection (restates src/Tracer/Intersect.cpp)
// ---------------------------------------------------------------------------
// IntersectRayAABB, Intersect.cpp:9-18, with 1/d hoisted (same values).
__device__ __forceinline__ float slab(f3 o, f3 inv, f3 lo, f3 hi)
{
    const f3 t1 = (lo - o) * inv;
    const f3 t2 = (hi - o) * inv;
    const f3 tmin = vmin(t1, t2);
    const f3 tmax = vmax(t1, t2);
    const float enter = gmax(gmax(tmin.x, tmin.y), tmin.z);
    const float exit = gmin(gmin(tmax.x, tmax.y), tmax.z);
    return enter <= exit ? exit : -1.0f;
}
// Moller-Trumbore (1997), two-sided with |det| > FLT_EPSILON, edge-inclusive.
// The det<0 branch is folded onto the det>0 one by negating u, v and det, which
// is exact, so the accept/reject decisions equal the two-branch form.
// On accept returns the raw numerators; t = dot(e2,q)/det, (u,v)/det.
__device__ __forceinline__ bool tri_test(f3 o, f3 d, f3 v0, f3 e1, f3 e2, float& t, float& u,
                                         float& v, float& det)
{
    const f3 p = cross(d, e2);
    det = dot(e1, p);
    if (!(fabsf(det) > FLT_EPSILON)) return false;
    const float sg = det > 0.0f ? 1.0f : -1.0f;
    const float adet = fabsf(det);
    const f3 s = o - v0;
    u = dot(s, p);
    const float us = u * sg;
    if (us < 0.0f || us > adet) return false;
    const f3 q = cross(s, e1);
    v = dot(d, q);
    const float vs = v * sg;
    if (vs < 0.0f || __fadd_rn(us, vs) > adet) return false;
    const float inv = __fdiv_rn(1.0f, det);
    t = __fmul_rn(dot(e2, q), inv);
    return true;
}

// tri_test in stages, so that a warp can vote between them: begin() applies
// the determinant and u rejections, second() the v rejection, ahead() the
// sign of t (known from dot(e2, q) and det before the division), finish()
// forms t and applies 0 < t < dist (each called on every lane, with the
// lane's result so far where it matters).  The same operations, values and
// decisions as tri_test followed by that range check.
struct TriStage {
    f3 e1, e2, sv, q;
    float det, sg, adet, us, u, v, tn, t, inv;
    __device__ __forceinline__ bool begin(f3 o, f3 d, float4 v0, float4 e1w, float4 e2w)
    {
        e1 = xyz(e1w);
        e2 = xyz(e2w);
        const f3 p = cross(d, e2);
        det = dot(e1, p);
        sg = det > 0.0f ? 1.0f : -1.0f;
        adet = fabsf(det);
        sv = o - xyz(v0);
        u = dot(sv, p);
        us = u * sg;
        return adet > FLT_EPSILON && !(us < 0.0f || us > adet);
    }
    __device__ __forceinline__ bool second(f3 d)
    {
        q = cross(sv, e1);
        v = dot(d, q);
        const float vs = v * sg;
        return !(vs < 0.0f || __fadd_rn(us, vs) > adet);
    }
    // the sign of t = tn * (1/det) before the division: a candidate whose t
    // cannot be positive drops out
    __device__ __forceinline__ bool ahead(bool ok)
    {
        tn = dot(e2, q);
        return ok && (det > 0.0f ? tn > 0.0f : tn < 0.0f);
    }
    // t is formed (one division, 1/det, which also scales u and v of the
    // winner) only on a lane that is still a candidate
    __device__ __forceinline__ bool finish(bool ok, float dist)
    {
        t = FLT_MAX;
        inv = 0.0f;
        if (ok) {
            inv = __fdiv_rn(1.0f, det);
            t = __fmul_rn(tn, inv);
        }
        return ok && t > 0.0f && t < dist;
    }
};

struct LocalHit {
    float t, u, v;
    uint32_t slot;     // winning slot (triangle id is in its v0.w)
    uint32_t bv;       // leaf node index (reference node numbering)
    uint32_t bvh_tests, tri_tests, inner;
};

__device__ __forceinline__ uint32_t f2u(float f) { return __float_as_uint(f); }

struct SceneHit {
    bool hit;
    uint32_t inst, tri, bv, bvh_tests, tri_tests;
    uint32_t tot_pops, tot_inner, tot_tris;  // summed over all visited instances (COUNT only)
    float u, v, dist;
    f3 world_pos;
};

// ---------------------------------------------------------------------------
// Scene traversal: IntersectScene / IntersectMeshInstance / IntersectTrianglesBVH
// (Intersect.cpp:20-219), warp-cooperative
// ---------------------------------------------------------------------------
// Every lane owns one ray and pops its own BVH nodes, but all lanes run one
// loop whatever instance they are in, and a leaf reached by any lane is tested
// by the whole warp: lane j tests triangle first + j (coalesced 48-byte slots)
// and a (t, index) arg-min picks the winner.  The reference tests a leaf's
// triangles in order, accepting t > 0 && t < dist with dist shrinking as it
// goes (Intersect.cpp:84-105); the survivor of that scan is the triangle with
// the smallest valid t, the first one on ties, which is exactly the
// lexicographic minimum, so the result (and every counter) is unchanged.
// Meshes without a BVH are one leaf holding all their triangles
// (IntersectTrianglesLinear, Intersect.cpp:20-45).
// Must be called by all 32 lanes of a warp together; inactive lanes help.
#define MT_FULL 0xffffffffu

// Persistent form: the warp keeps running until the work source is empty.  A
// lane whose ray is finished takes the next one (one atomic per warp), so no
// lane idles while its neighbours finish long rays.  The instance boxes a new
// ray meets are tested 32 at a time by the whole warp (one box per lane, then
// a ballot), the same test IntersectMeshInstance starts with.
//
// Work must provide, per lane:
//   bool fetch(uint32_t index, f3& o, f3& d, float& tmax)  (false: index past the end)
//   void finish(const SceneHit& h)
// True when the instance's world box starts farther along the ray than lim, by
// more than a margin for rounding (1e-4 of the distances and coordinates
// involved): no hit in it can then be accepted, since a closest hit must come
// in strictly below the best world distance and an occluder at or below the
// light distance.  The world box bounds the transformed triangles (the xyz of
// model * p is affine in p, and the box is the hull of the transformed local
// box corners).  A ray that starts inside the box never skips it.
__device__ __forceinline__ bool instance_beyond(const DevInstance& I, f3 o, f3 inv, float lim)
{
    const f3 wlo = {__ldg(&I.wlo[0]), __ldg(&I.wlo[1]), __ldg(&I.wlo[2])};
    const f3 whi = {__ldg(&I.whi[0]), __ldg(&I.whi[1]), __ldg(&I.whi[2])};
    const f3 t1 = (wlo - o) * inv;
    const f3 t2 = (whi - o) * inv;
    const f3 tmin = vmin(t1, t2);
    const float enter = gmax(gmax(tmin.x, tmin.y), tmin.z);
    const float mag = fmaxf(fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z)),
                            fmaxf(fmaxf(fmaxf(fabsf(wlo.x), fabsf(wlo.y)), fabsf(wlo.z)),
                                  fmaxf(fmaxf(fabsf(whi.x), fabsf(whi.y)), fabsf(whi.z))));
    return enter > lim + 1e-4f * (lim + mag);
}

// One world-box pass for G requesting lanes (the G lowest bits of nm) of a
// scene whose instances fit in one chunk: lane k holds the boxes of instances
// k and k + 32 (blo, bhi) and tests them against each of the G rays.
template <int G, int CHUNK, class M>
__device__ __forceinline__ void mask_group(uint32_t& nm, const DevScene& S, const f3* blo, const f3* bhi, f3 o,
                                           f3 winv, M& mask, bool& need_mask, uint32_t lane)
{
    uint32_t Ls[G];
    f3 bo[G], bi[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
        Ls[g] = __ffs(nm) - 1;
        nm &= nm - 1;
        bo[g] = {__shfl_sync(MT_FULL, o.x, Ls[g]), __shfl_sync(MT_FULL, o.y, Ls[g]), __shfl_sync(MT_FULL, o.z, Ls[g])};
        bi[g] = {__shfl_sync(MT_FULL, winv.x, Ls[g]), __shfl_sync(MT_FULL, winv.y, Ls[g]),
                 __shfl_sync(MT_FULL, winv.z, Ls[g])};
    }
    M m[G];
#pragma unroll
    for (int g = 0; g < G; ++g) m[g] = 0;
#pragma unroll
    for (int q = 0; q < CHUNK / 32; ++q) {
        const bool in = 32u * q + lane < S.num_instances;
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const bool meets = in && slab(bo[g], bi[g], blo[q], bhi[q]) >= 0.0f;
            m[g] |= static_cast<M>(__ballot_sync(MT_FULL, meets)) << (32 * q);
        }
    }
#pragma unroll
    for (int g = 0; g < G; ++g)
        if (lane == Ls[g]) {
            mask = m[g];
            need_mask = false;
        }
}

__device__ __forceinline__ uint32_t lowest_bit(uint32_t m) { return __ffs(static_cast<int>(m)) - 1; }
__device__ __forceinline__ uint32_t lowest_bit(unsigned long long m)
{
    return __ffsll(static_cast<long long>(m)) - 1;
}

// SKIP: instances whose world box lies beyond the current best hit (closest)
// or the light (any) are not opened.  The result, including the winner's
// counters, is unchanged; only the work summed over all instances (the totals
// query, the debug modes' traversal counts) needs every instance visited.
// CHUNK (32 or 64) instances are tested per warp pass of the world-box test;
// with 64 every lane tests two boxes and a ray's mask of met instances is 64
// bits wide (one pass instead of two per ray on a 33-64 instance scene).
// LEAF_PAIR: a warp pass tests two pending leaves at once; more registers and
// spills, which pays for long incoherent rays (closest-hit queries on the
// 6.1 M-triangle scene: 47.3 against 44.6 Mrays/s) but not for the render's
// short ones (material grid: 1416 against 1446 Mrays/s) nor for any-hit
// queries (60.2 against 63.9).
// STACK_TOP: the top entry of the traversal stack lives in registers (the near
// child pushed last is the next pop), the rest in local memory; it pays for
// the render's short rays (material grid: 1469 against 1447 Mrays/s) but not
// for long incoherent ones (46.3 against 47.2 Mrays/s closest hit).
template <bool COUNT, bool ANY, bool SKIP = true, int CHUNK = 32, bool LEAF_PAIR = false, bool STACK_TOP = false,
          class Work>
__device__ __forceinline__ void trace_persistent(const DevScene& S, Work& W, uint32_t* fetch_counter)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lane_lt = (1u << lane) - 1u;
    bool has_ray = false, exhausted = false;
    f3 o = splat(0.0f), d = splat(0.0f), winv = splat(0.0f);
    float tmax = 0.0f;
    SceneHit best;
    bool stopped = false;
    typedef typename std::conditional<CHUNK == 64, unsigned long long, uint32_t>::type imask_t;
    uint32_t chunk = 0;
    imask_t mask = 0;
    bool need_mask = false;
    bool in_inst = false;
    uint32_t ii = 0;
    f3 lo = splat(0.0f), ld = splat(0.0f), linv = splat(0.0f);
    const float4* nodes = S.nodes;
    uint32_t slot_base = 0;
    LocalHit h;
    int sp = 0;
    bool top = false;  // STACK_TOP: the stack's top entry is (top_node, top_dist)
    uint32_t top_node = 0;
    float top_dist = 0.0f;
    bool pending = false;
    uint32_t pfirst = 0, pcount = 0, pnode = 0;
    // Stack entries (and top_node): an inner node as its a word, the index of
    // its first child (siblings sit at (a, a + 1), 64 contiguous bytes), a leaf
    // as its own index | MT_BVH_LEAF_BIT.  A child's a word comes with its box,
    // so popping an inner node loads its children's boxes without first
    // loading the node itself.
    uint32_t stk_node[MT_STACK_SIZE];
    float stk_dist[MT_STACK_SIZE];

    while (true) {
        // A. lanes without a ray take the next ones
        const bool want = !has_ray && !exhausted;
        const uint32_t wm = __ballot_sync(MT_FULL, want);
        if (wm) {
            const uint32_t leader = __ffs(wm) - 1;
            uint32_t first = 0;
            if (lane == leader) first = atomicAdd(fetch_counter, static_cast<uint32_t>(__popc(wm)));
            first = __shfl_sync(MT_FULL, first, leader);
            if (want) {
                if (W.fetch(first + __popc(wm & lane_lt), o, d, tmax)) {
                    has_ray = true;
                    winv = {__fdiv_rn(1.0f, d.x), __fdiv_rn(1.0f, d.y), __fdiv_rn(1.0f, d.z)};
                    best.hit = false;
                    best.dist = FLT_MAX;
                    best.bvh_tests = best.tri_tests = 0;
                    best.tot_pops = best.tot_inner = best.tot_tris = 0;
                    best.inst = best.tri = best.bv = 0;
                    best.u = best.v = 0.0f;
                    best.world_pos = splat(0.0f);
                    stopped = false;
                    chunk = 0;
                    mask = 0;
                    need_mask = S.num_instances > 0;
                    in_inst = false;
                    sp = 0;
                    top = false;
                    pending = false;
                } else {
                    exhausted = true;
                }
            }
        }
        if (!__any_sync(MT_FULL, has_ray)) break;

        // B. instance boxes of the current chunk, one warp pass per requesting
        // lane.  When every instance fits in one chunk (the chunk is then 0
        // for every lane) each lane loads its boxes once for all the passes.
        uint32_t nm = __ballot_sync(MT_FULL, need_mask);
        if (nm) {
            const bool one_chunk = S.num_instances <= CHUNK;  // warp-uniform
            f3 blo[CHUNK / 32], bhi[CHUNK / 32];
#pragma unroll
            for (int q = 0; q < CHUNK / 32; ++q) {
                blo[q] = bhi[q] = splat(0.0f);
                const uint32_t k = 32u * q + lane;
                if (one_chunk && k < S.num_instances) {
                    const DevInstance& I = S.instances[k];
                    blo[q] = {__ldg(&I.wlo[0]), __ldg(&I.wlo[1]), __ldg(&I.wlo[2])};
                    bhi[q] = {__ldg(&I.whi[0]), __ldg(&I.whi[1]), __ldg(&I.whi[2])};
                }
            }
            // groups of requesting lanes share a pass: independent slab chains
            // overlap their latencies
            if (one_chunk) {
                if (MT_MASK_GROUP >= 8)
                    while (__popc(nm) >= 8) mask_group<8, CHUNK>(nm, S, blo, bhi, o, winv, mask, need_mask, lane);
                if (MT_MASK_GROUP >= 4)
                    while (__popc(nm) >= 4) mask_group<4, CHUNK>(nm, S, blo, bhi, o, winv, mask, need_mask, lane);
                if (MT_MASK_GROUP >= 2)
                    while (__popc(nm) >= 2) mask_group<2, CHUNK>(nm, S, blo, bhi, o, winv, mask, need_mask, lane);
            }
            while (nm) {
                const uint32_t L = __ffs(nm) - 1;
                nm &= nm - 1;
                const f3 bo = {__shfl_sync(MT_FULL, o.x, L), __shfl_sync(MT_FULL, o.y, L),
                               __shfl_sync(MT_FULL, o.z, L)};
                const f3 bi = {__shfl_sync(MT_FULL, winv.x, L), __shfl_sync(MT_FULL, winv.y, L),
                               __shfl_sync(MT_FULL, winv.z, L)};
                const uint32_t c0 = one_chunk ? 0u : __shfl_sync(MT_FULL, chunk, L);
                imask_t m = 0;
#pragma unroll
                for (int q = 0; q < CHUNK / 32; ++q) {  // lane tests instances c0 + lane (+ 32)
                    const uint32_t k = c0 + 32u * q + lane;
                    bool meets = false;
                    if (k < S.num_instances) {
                        f3 wlo = blo[q], whi = bhi[q];
                        if (!one_chunk) {
                            const DevInstance& I = S.instances[k];
                            wlo = {__ldg(&I.wlo[0]), __ldg(&I.wlo[1]), __ldg(&I.wlo[2])};
                            whi = {__ldg(&I.whi[0]), __ldg(&I.whi[1]), __ldg(&I.whi[2])};
                        }
                        meets = slab(bo, bi, wlo, whi) >= 0.0f;
                    }
                    m |= static_cast<imask_t>(__ballot_sync(MT_FULL, meets)) << (32 * q);
                }
                if (lane == L) {
                    mask = m;
                    need_mask = false;
                }
            }
        }

        // C. close the instance whose stack ran dry; open the next; finish the ray
        const bool want_switch = has_ray && !need_mask && !pending && sp == 0 && !top;
        bool run_switch = true;
        if (S.trav_switch > 1) {
            const uint32_t sw = __ballot_sync(MT_FULL, want_switch);
            if (sw && __popc(sw) < S.trav_switch)
                run_switch = __ballot_sync(MT_FULL, has_ray && (pending || sp > 0 || top)) == 0;
        }
        if (want_switch && run_switch) {
            if (in_inst) {
                if (COUNT) {
                    best.tot_pops += h.bvh_tests;
                    best.tot_inner += h.inner;
                    best.tot_tris += h.tri_tests;
                }
                if (!ANY && h.t < FLT_MAX) {
                    const DevInstance& I = S.instances[ii];
                    float model[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) model[q] = __ldg(&I.model[q]);
                    const f3 wp = xform_point(model, lo + h.t * ld);
                    const float wd = length(wp - o);
                    if (wd < best.dist) {
                        best.hit = true;
                        best.dist = wd;
                        best.world_pos = wp;
                        best.inst = ii;
                        best.tri = f2u(__ldg(&S.slots[3ull * (slot_base + h.slot)].w));
                        best.bv = h.bv;
                        best.u = h.u;
                        best.v = h.v;
                        best.bvh_tests = h.bvh_tests;
                        best.tri_tests = h.tri_tests;
                    }
                }
                in_inst = false;
            }
            if (mask == 0 && !stopped && chunk + CHUNK < S.num_instances) {
                chunk += CHUNK;
                need_mask = true;
            } else if (mask == 0 || stopped) {
                W.finish(best);
                has_ray = false;
            } else {
                uint32_t k = lowest_bit(mask);
                mask &= mask - 1;
                if (SKIP) {
                    const float lim = ANY ? tmax : best.dist;
                    while (instance_beyond(S.instances[chunk + k], o, winv, lim)) {
                        k = 0xffffffffu;
                        if (!mask) break;
                        k = lowest_bit(mask);
                        mask &= mask - 1;
                    }
                }
                if (k != 0xffffffffu) {
                    ii = chunk + k;
                    const DevInstance& I = S.instances[ii];
                    float inv[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) inv[q] = __ldg(&I.inv[q]);
                    lo = xform_point(inv, o);
                    ld = normalize(xform_dir(inv, d));
                    linv = {__fdiv_rn(1.0f, ld.x), __fdiv_rn(1.0f, ld.y), __fdiv_rn(1.0f, ld.z)};
                    const DevMesh m = S.meshes[__ldg(&I.mesh)];
                    nodes = S.nodes + 2ull * m.node_off;
                    slot_base = m.slot_off;
                    h.t = FLT_MAX;
                    h.u = h.v = 0.0f;
                    h.slot = h.bv = 0;
                    h.bvh_tests = h.tri_tests = h.inner = 0;
                    in_inst = true;
                    if (m.has_bvh) {
                        const float4 a = __ldg(nodes + 0), b = __ldg(nodes + 1);
                        const uint32_t root = (f2u(a.w) & MT_BVH_LEAF_BIT) ? MT_BVH_LEAF_BIT : f2u(a.w);
                        if (STACK_TOP) {
                            top_node = root;
                            top_dist = slab(lo, linv, xyz(a), xyz(b));
                            top = true;
                            sp = 0;
                        } else {
                            stk_node[0] = root;
                            stk_dist[0] = slab(lo, linv, xyz(a), xyz(b));
                            sp = 1;
                        }
                    } else {
                        pending = true;
                        pfirst = 0;
                        pcount = m.num_slots;
                        pnode = 0;
                    }
                }
            }
        }

        // D. node pops (IntersectTrianglesBVH's loop body): up to
        // S.trav_pops per pass, a lane stopping at its first leaf, so every
        // lane still visits its nodes in the reference's order and each leaf is
        // tested (phase E) before that lane's next pop
        const int pops = S.trav_pops > 1 ? S.trav_pops : 1;  // at least one pop per pass
#pragma unroll 1
        for (int pass = 0; pass < pops; ++pass) {
            const bool act = in_inst && !pending && (sp > 0 || top);
            if (pass > 0 && !__any_sync(MT_FULL, act)) break;
            if (act) {
                uint32_t ni;
                float nd;
                if (STACK_TOP && top) {
                    ni = top_node;
                    nd = top_dist;
                    top = false;
                } else {
                    --sp;
                    ni = stk_node[sp];
                    nd = stk_dist[sp];
                }
                if (COUNT) ++h.bvh_tests;
                if (!(nd < 0.0f) && !(nd > __fadd_rn(h.t, 0.1f))) {
                    if (ni & MT_BVH_LEAF_BIT) {
                        const uint32_t leaf = ni & ~MT_BVH_LEAF_BIT;
                        pending = true;
                        pfirst = f2u(__ldg(&nodes[2 * leaf].w)) & ~MT_BVH_LEAF_BIT;
                        pcount = f2u(__ldg(&nodes[2 * leaf + 1].w)) & ~MT_BVH_LEAF_BIT;
                        pnode = leaf;
                        if (S.trav_prefetch && pcount)
                            prefetch_l2(S.slots + 3ull * (slot_base + pfirst), 48u * (pcount < 32u ? pcount : 32u));
                    } else {
                        if (COUNT) ++h.inner;
                        // the children (na, na + 1) are the 64 bytes at node na
                        const uint32_t na = ni, nb = ni + 1;
                        const float4 a0 = __ldg(nodes + 2 * na), a1 = __ldg(nodes + 2 * na + 1);
                        const float4 b0 = __ldg(nodes + 2 * nb), b1 = __ldg(nodes + 2 * nb + 1);
                        const float da = slab(lo, linv, xyz(a0), xyz(a1));
                        const float db = slab(lo, linv, xyz(b0), xyz(b1));
                        const uint32_t ea = (f2u(a0.w) & MT_BVH_LEAF_BIT) ? (na | MT_BVH_LEAF_BIT) : f2u(a0.w);
                        const uint32_t eb = (f2u(b0.w) & MT_BVH_LEAF_BIT) ? (nb | MT_BVH_LEAF_BIT) : f2u(b0.w);
                        const float lim = __fadd_rn(h.t, 0.1f);
                        const bool pa = da >= 0.0f && da <= lim;
                        const bool pb = db >= 0.0f && db <= lim;
                        if (sp + 2 > MT_STACK_SIZE) {
                            atomicOr(S.error_flag, MT_ERRBIT_STACK);
                            sp = 0;
                            top = false;
                        } else if (STACK_TOP) {
                            // far child to memory, near child (popped next) to the top
                            if (pa && pb) {
                                const bool a_near = da < db;
                                stk_node[sp] = a_near ? eb : ea;
                                stk_dist[sp] = a_near ? db : da;
                                ++sp;
                                top_node = a_near ? ea : eb;
                                top_dist = a_near ? da : db;
                                top = true;
                            } else if (pa || pb) {
                                top_node = pa ? ea : eb;
                                top_dist = pa ? da : db;
                                top = true;
                            }
                        } else if (pa && pb) {
                            if (da < db) {
                                stk_node[sp] = eb; stk_dist[sp] = db; ++sp;
                                stk_node[sp] = ea; stk_dist[sp] = da; ++sp;
                            } else {
                                stk_node[sp] = ea; stk_dist[sp] = da; ++sp;
                                stk_node[sp] = eb; stk_dist[sp] = db; ++sp;
                            }
                        } else if (pa) {
                            stk_node[sp] = ea; stk_dist[sp] = da; ++sp;
                        } else if (pb) {
                            stk_node[sp] = eb; stk_dist[sp] = db; ++sp;
                        }
                    }
                }
            }
        }

        // E. the warp tests every pending leaf together
        // (the lane that reached the leaf takes the result: IntersectTrianglesBVH's
        // accept step, and for the any-hit query the stop at a blocking hit)
        auto leaf_done = [&](uint32_t count, uint32_t bidx, float bt, float bu, float bv) {
            if (COUNT) h.tri_tests += count;
            pending = false;
            if (bidx != 0xffffffffu) {
                h.t = bt;
                h.u = bu;
                h.v = bv;
                h.slot = pfirst + bidx;
                h.bv = pnode;
                if (ANY) {
                    const DevInstance& I = S.instances[ii];
                    float model[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) model[q] = __ldg(&I.model[q]);
                    const f3 wp = xform_point(model, lo + bt * ld);
                    if (!(length(wp - o) > tmax)) {
                        stopped = true;
                        best.hit = true;
                        best.inst = ii;
                        if (COUNT) {
                            best.tot_pops += h.bvh_tests;
                            best.tot_inner += h.inner;
                            best.tot_tris += h.tri_tests;
                        }
                        sp = 0;
                        top = false;
                        mask = 0;
                        in_inst = false;
                    }
                }
            }
        };
        // the (t, index) minimum of one chunk of 32 triangles: valid t are > 0,
        // whose IEEE bit patterns order like the values, so one unsigned min
        // finds the smallest t and the lowest lane holding it is the first such
        // triangle of the chunk
        auto chunk_min = [&](bool ok, float t, float u, float v, float inv, uint32_t c, float& bt, float& bu,
                             float& bv, uint32_t& bidx) {
            const uint32_t key = ok ? __float_as_uint(t) : 0xffffffffu;
            const uint32_t kmin = __reduce_min_sync(MT_FULL, key);
            if (kmin != 0xffffffffu && __uint_as_float(kmin) < bt) {
                const uint32_t w = __ffs(__ballot_sync(MT_FULL, key == kmin)) - 1;
                float uu = 0.0f, vv = 0.0f;
                if (lane == w) {
                    uu = __fmul_rn(u, inv);
                    vv = __fmul_rn(v, inv);
                }
                bt = __uint_as_float(kmin);
                bidx = c + w;
                bu = __shfl_sync(MT_FULL, uu, w);
                bv = __shfl_sync(MT_FULL, vv, w);
            }
        };
        uint32_t pm = __ballot_sync(MT_FULL, pending);
        // LEAF_PAIR: two pending leaves per pass, independent load/test/reduce
        // chains
        while (LEAF_PAIR && (pm & (pm - 1))) {
            const uint32_t La = __ffs(pm) - 1;
            pm &= pm - 1;
            const uint32_t Lb = __ffs(pm) - 1;
            pm &= pm - 1;
            const f3 roa = {__shfl_sync(MT_FULL, lo.x, La), __shfl_sync(MT_FULL, lo.y, La),
                            __shfl_sync(MT_FULL, lo.z, La)};
            const f3 rda = {__shfl_sync(MT_FULL, ld.x, La), __shfl_sync(MT_FULL, ld.y, La),
                            __shfl_sync(MT_FULL, ld.z, La)};
            const f3 rob = {__shfl_sync(MT_FULL, lo.x, Lb), __shfl_sync(MT_FULL, lo.y, Lb),
                            __shfl_sync(MT_FULL, lo.z, Lb)};
            const f3 rdb = {__shfl_sync(MT_FULL, ld.x, Lb), __shfl_sync(MT_FULL, ld.y, Lb),
                            __shfl_sync(MT_FULL, ld.z, Lb)};
            const float dista = __shfl_sync(MT_FULL, h.t, La), distb = __shfl_sync(MT_FULL, h.t, Lb);
            const uint32_t basea = __shfl_sync(MT_FULL, slot_base + pfirst, La);
            const uint32_t baseb = __shfl_sync(MT_FULL, slot_base + pfirst, Lb);
            const uint32_t ca = __shfl_sync(MT_FULL, pcount, La), cb = __shfl_sync(MT_FULL, pcount, Lb);
            float bta = FLT_MAX, bua = 0.0f, bva = 0.0f, btb = FLT_MAX, bub = 0.0f, bvb = 0.0f;
            uint32_t bia = 0xffffffffu, bib = 0xffffffffu;
            const uint32_t cmax = ca > cb ? ca : cb;
            for (uint32_t c = 0; c < cmax; c += 32) {
                const uint32_t i = c + lane;
                const bool ina = i < ca, inb = i < cb;
                float4 A0 = make_float4(0.f, 0.f, 0.f, 0.f), A1 = A0, A2 = A0, B0 = A0, B1 = A0, B2 = A0;
                if (ina) {
                    const float4* sl = S.slots + 3ull * (basea + i);
                    A0 = __ldg(sl); A1 = __ldg(sl + 1); A2 = __ldg(sl + 2);
                }
                if (inb) {
                    const float4* sl = S.slots + 3ull * (baseb + i);
                    B0 = __ldg(sl); B1 = __ldg(sl + 1); B2 = __ldg(sl + 2);
                }
                TriStage sa, sb;
                bool oka = sa.begin(roa, rda, A0, A1, A2) && ina;  // every lane runs each stage
                bool okb = sb.begin(rob, rdb, B0, B1, B2) && inb;
                if (__any_sync(MT_FULL, oka || okb)) {
                    oka = sa.second(rda) && oka;
                    okb = sb.second(rdb) && okb;
                    oka = sa.ahead(oka);
                    okb = sb.ahead(okb);
                    if (__any_sync(MT_FULL, oka || okb)) {
                        oka = sa.finish(oka, dista);
                        okb = sb.finish(okb, distb);
                        chunk_min(oka, sa.t, sa.u, sa.v, sa.inv, c, bta, bua, bva, bia);
                        chunk_min(okb, sb.t, sb.u, sb.v, sb.inv, c, btb, bub, bvb, bib);
                    }
                }
            }
            if (lane == La) leaf_done(ca, bia, bta, bua, bva);
            if (lane == Lb) leaf_done(cb, bib, btb, bub, bvb);
        }
        while (pm) {
            const uint32_t L = __ffs(pm) - 1;
            pm &= pm - 1;
            const f3 ro = {__shfl_sync(MT_FULL, lo.x, L), __shfl_sync(MT_FULL, lo.y, L),
                           __shfl_sync(MT_FULL, lo.z, L)};
            const f3 rd = {__shfl_sync(MT_FULL, ld.x, L), __shfl_sync(MT_FULL, ld.y, L),
                           __shfl_sync(MT_FULL, ld.z, L)};
            const float dist = __shfl_sync(MT_FULL, h.t, L);
            const uint32_t base = __shfl_sync(MT_FULL, slot_base + pfirst, L);
            const uint32_t count = __shfl_sync(MT_FULL, pcount, L);
            float bt = FLT_MAX, bu = 0.0f, bv = 0.0f;
            uint32_t bidx = 0xffffffffu;
            for (uint32_t c = 0; c < count; c += 32) {
                const uint32_t i = c + lane;
                // the staged test with a warp vote after each stage: the rest
                // runs only while some lane still has a candidate (per leaf visit,
                // ~28% of the material grid's chunks lose every lane at the u
                // bound and ~70% at the v bound)
                float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, C = A;
                if (i < count) {
                    const float4* sl = S.slots + 3ull * (base + i);
                    A = __ldg(sl);
                    B = __ldg(sl + 1);
                    C = __ldg(sl + 2);
                }
                // TriStage's operations written out (the form that measured
                // fastest here); every lane runs each stage
                const f3 e1 = xyz(B), e2 = xyz(C);
                const f3 pv = cross(rd, e2);
                const float det = dot(e1, pv);
                const float sg = det > 0.0f ? 1.0f : -1.0f;
                const float adet = fabsf(det);
                const f3 sv = ro - xyz(A);
                const float u = dot(sv, pv);
                const float us = u * sg;
                bool ok = i < count && adet > FLT_EPSILON && !(us < 0.0f || us > adet);
                if (__any_sync(MT_FULL, ok)) {
                    const f3 q = cross(sv, e1);
                    const float v = dot(rd, q);
                    const float vs = v * sg;
                    ok = ok && !(vs < 0.0f || __fadd_rn(us, vs) > adet);
                    if (__any_sync(MT_FULL, ok)) {
                        // t = tn * (1/det) is positive only when tn and det
                        // have the same sign: a candidate behind the origin
                        // (the triangle a secondary ray leaves, most often)
                        // drops out before the division, and a chunk left
                        // with none skips it
                        const float tn = dot(e2, q);
                        ok = ok && (det > 0.0f ? tn > 0.0f : tn < 0.0f);
                        if (__any_sync(MT_FULL, ok)) {
                            float t = FLT_MAX, inv = 0.0f;
                            if (ok) {
                                inv = __fdiv_rn(1.0f, det);
                                t = __fmul_rn(tn, inv);
                            }
                            ok = ok && t > 0.0f && t < dist;
                            chunk_min(ok, t, u, v, inv, c, bt, bu, bv, bidx);
                        }
                    }
                }
            }
            if (lane == L) leaf_done(count, bidx, bt, bu, bv);
        }
    }
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the draw slots shared with the
// CPU oracle's counter mode.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

__device__ __forceinline__ float u01(uint32_t x)
{
    return __fmul_rn(static_cast<float>(x >> 8), 1.0f / 16777216.0f);
}
// a + (b - a) * u, in the libstdc++ uniform_real_distribution order u*(b-a)+a.
__device__ __forceinline__ float urange(uint32_t x, float a, float b)
{
    return __fadd_rn(__fmul_rn(u01(x), __fsub_rn(b, a)), a);
}

enum : uint32_t { SLOT_JITTER = 0, SLOT_LOBE = 1, SLOT_FALLBACK = 2, SLOT_LIGHT_JITTER = 3, SLOT_LIGHT_PICK = 4 };

__device__ __forceinline__ uint4 draw(const DevScene& S, uint32_t pixel, uint32_t sample,
                                      uint32_t bounce, uint32_t slot)
{
    return philox(make_uint4(pixel, sample, (bounce << 8) | slot, 0u), S.key0, S.key1);
}

// ---------------------------------------------------------------------------
// Camera (src/Tracer/Camera.cpp:17-50)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void camera_ray(const DevScene& S, float u, float v, f3& o, f3& d)
{
    if (S.cam_type == 0) {
        const float px = __fmul_rn(__fmul_rn(__fsub_rn(__fmul_rn(2.0f, u), 1.0f), S.fov_scale),
                                   S.render_aspect);
        const float py = __fmul_rn(__fsub_rn(__fmul_rn(2.0f, v), 1.0f), S.fov_scale);
        // normalize(vec4(px, -py, -1, 0)): vec4 dot pairs (x+y) + (z+w)
        const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(px, px), __fmul_rn(-py, -py)),
                                   __fadd_rn(1.0f, 0.0f));
        const float s = __fdiv_rn(1.0f, __fsqrt_rn(l2));
        const float cx = __fmul_rn(px, s), cy = __fmul_rn(-py, s), cz = __fmul_rn(-1.0f, s),
                    cw = __fmul_rn(0.0f, s);
        o = {mrow(S.c2w, 0, 0, 0, 0, 1), mrow(S.c2w, 1, 0, 0, 0, 1), mrow(S.c2w, 2, 0, 0, 0, 1)};
        d = normalize(f3{mrow(S.c2w, 0, cx, cy, cz, cw), mrow(S.c2w, 1, cx, cy, cz, cw),
                         mrow(S.c2w, 2, cx, cy, cz, cw)});
    } else {
        const float px = __fdiv_rn(
            __fmul_rn(__fmul_rn(__fsub_rn(__fmul_rn(2.0f, u), 1.0f), S.ortho_x), S.render_aspect),
            S.cam_aspect);
        const float py = __fmul_rn(__fsub_rn(__fmul_rn(2.0f, v), 1.0f), S.ortho_y);
        o = {mrow(S.c2w, 0, px, -py, 0, 1), mrow(S.c2w, 1, px, -py, 0, 1),
             mrow(S.c2w, 2, px, -py, 0, 1)};
        d = normalize(f3{mrow(S.c2w, 0, 0, 0, -1, 0), mrow(S.c2w, 1, 0, 0, -1, 0),
                         mrow(S.c2w, 2, 0, 0, -1, 0)});
    }
}

// ---------------------------------------------------------------------------
// BRDF (src/Tracer/BRDF.hpp:9-97)
// ---------------------------------------------------------------------------
// x^5 for x in [0, 1] (the Schlick factor's pow(1 - cos, 5)) by compensated
// products: Dekker's TwoProduct, with an FMA giving each product's rounding
// error exactly (Ogita, Rump and Oishi, "Accurate sum and dot product", 2005).
// x^2 = p2 + e2 and p2^2 = p4 + e4 exactly, so x^4 = p4 + (e4 + 2 p2 e2)
// up to e2^2 (2^-48 relative); p4 x = p5 + e5 exactly, so
// x^5 = p5 + (e5 + (e4 + 2 p2 e2) x), and the one rounding of that sum leaves
// the result within 2^-45 relative of x^5 before it: the correctly rounded
// value except when x^5 lies that close to a rounding tie.  The reference's
// powf is within 1 ulp; a general power function is much more code.
__device__ __forceinline__ float pow5(float x)
{
    const float p2 = __fmul_rn(x, x);
    const float e2 = __fmaf_rn(x, x, -p2);
    const float p4 = __fmul_rn(p2, p2);
    const float t4 = __fmaf_rn(__fmul_rn(2.0f, p2), e2, __fmaf_rn(p2, p2, -p4));
    const float p5 = __fmul_rn(p4, x);
    const float e5 = __fmaf_rn(p4, x, -p5);
    return __fadd_rn(p5, __fmaf_rn(t4, x, e5));
}
__device__ __forceinline__ f3 fresnel_schlick(float c, f3 f0)
{
    c = gclamp(c, 0.0f, 1.0f);
    const float p = pow5(__fsub_rn(1.0f, c));
    return f0 + (splat(1.0f) - f0) * splat(p);
}
__device__ __forceinline__ f3 base_reflectivity(f3 base, float metallic)
{
    metallic = gclamp(metallic, 0.0f, 1.0f);
    return splat(0.04f) * __fsub_rn(1.0f, metallic) + base * metallic;
}
__device__ __forceinline__ float distribution_ggx(float nh, float r)
{
    nh = gclamp(nh, 0.0f, 1.0f);
    const float a = __fmul_rn(r, r);
    const float a2 = __fmul_rn(a, a);
    const float nh2 = __fmul_rn(nh, nh);
    float den = __fadd_rn(__fmul_rn(nh2, __fsub_rn(a2, 1.0f)), 1.0f);
    den = __fmul_rn(__fmul_rn(kPi, den), den);
    return __fdiv_rn(a2, den);
}
__device__ __forceinline__ float geometry_schlick_ggx(float nv, float r)
{
    nv = gclamp(nv, 0.0f, 1.0f);
    const float rr = __fadd_rn(r, 1.0f);
    const float k = __fmul_rn(__fmul_rn(rr, rr), 0.125f);  // the same rounded value as x / 8
    const float den = __fadd_rn(__fmul_rn(nv, __fsub_rn(1.0f, k)), k);
    return __fdiv_rn(nv, den);
}
__device__ __forceinline__ f3 eval_brdf(f3 L, f3 V, f3 N, f3 base, float roughness, float metallic)
{
    roughness = gmax(roughness, 0.05f);
    const float nl = gmax(dot(N, L), 0.0f);
    const float nv = gmax(dot(N, V), 0.0f);
    if (nl <= 0.0f || nv <= 0.0f) return splat(0.0f);
    const f3 h = normalize(V + L);
    const float nh = gmax(dot(N, h), 0.0f);
    const float hv = gmax(dot(h, V), 0.0f);
    const f3 f0 = base_reflectivity(base, metallic);
    const f3 f = fresnel_schlick(hv, f0);
    const float dd = distribution_ggx(nh, roughness);
    const float g = __fmul_rn(geometry_schlick_ggx(nv, roughness), geometry_schlick_ggx(nl, roughness));
    const f3 kd = (splat(1.0f) - f) * __fsub_rn(1.0f, metallic);
    const f3 diffuse = (kd * base) / kPi;
    const f3 spec = (f * __fmul_rn(dd, g)) /
                    gmax(__fmul_rn(__fmul_rn(4.0f, nv), nl), 0.001f);
    return vmax(diffuse + spec, splat(0.0f));
}
__device__ __forceinline__ float diffuse_pdf(f3 L, f3 N) { return __fdiv_rn(gmax(dot(N, L), 0.0f), kPi); }
__device__ __forceinline__ float specular_pdf(f3 L, f3 V, f3 N, float roughness)
{
    const float nl = gmax(dot(N, L), 0.0f);
    const float nv = gmax(dot(N, V), 0.0f);
    if (nl <= 0.0f || nv <= 0.0f) return 0.0f;
    const f3 h = normalize(V + L);
    const float nh = gmax(dot(N, h), 0.0f);
    const float vh = gmax(dot(V, h), 0.0f);
    if (vh <= 0.0f) return 0.0f;
    return __fdiv_rn(__fmul_rn(distribution_ggx(nh, gmax(roughness, 0.05f)), nh), __fmul_rn(4.0f, vh));
}

// ---------------------------------------------------------------------------
// Sampling helpers (src/Tracer/Tracer.cpp:26-121)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void build_tbn(f3 n, f3& t, f3& b)
{
    const f3 up = (fabsf(n.z) < 0.999f) ? f3{0, 0, 1} : f3{1, 0, 0};
    t = normalize(cross(up, n));
    b = cross(n, t);
}
__device__ __forceinline__ f3 cosine_hemisphere(float u1, float u2, f3 n)
{
    const float r = __fsqrt_rn(u1);
    const float phi = __fmul_rn(__fmul_rn(2.0f, kPi), u2);
    f3 t, b;
    build_tbn(n, t, b);
    float sp, cp;
    sincosf(phi, &sp, &cp);  // one argument reduction for both
    const float lx = __fmul_rn(r, cp), ly = __fmul_rn(r, sp);
    const float lz = __fsqrt_rn(gmax(0.0f, __fsub_rn(1.0f, u1)));
    return normalize(t * lx + b * ly + n * lz);
}
__device__ __forceinline__ float specular_probability(f3 view, f3 n, f3 base, float metallic)
{
    const f3 f0 = base_reflectivity(base, metallic);
    const f3 f = fresnel_schlick(gmax(dot(n, view), 0.0f), f0);
    const float p = __fdiv_rn(__fadd_rn(__fadd_rn(f.x, f.y), f.z), 3.0f);
    return gclamp(p, 0.05f, 0.95f);
}

// SampleGGXDirection (Tracer.cpp:49-72) with its two uniforms given: the half
// vector of the GGX lobe, flipped toward the viewer, and the reflection of the
// incident direction rd about it.  False when the reflection points below the
// surface (the caller then draws a cosine sample instead).
__device__ __forceinline__ bool ggx_reflection(f3 rd, f3 N, float roughness, float u1, float u2, f3& out)
{
    const float alpha = gmax(__fmul_rn(roughness, roughness), 0.0025f);
    const float alpha2 = __fmul_rn(alpha, alpha);
    const float phi = __fmul_rn(__fmul_rn(2.0f, kPi), u2);
    const float tan2 = __fdiv_rn(__fmul_rn(alpha2, u1), gmax(__fsub_rn(1.0f, u1), 0.0001f));
    const float cosT = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(1.0f, tan2)));
    const float sinT = __fsqrt_rn(gmax(0.0f, __fsub_rn(1.0f, __fmul_rn(cosT, cosT))));
    f3 t, b;
    build_tbn(N, t, b);
    float sp, cp;
    sincosf(phi, &sp, &cp);  // one argument reduction for both
    f3 h = normalize(t * __fmul_rn(sinT, cp) + b * __fmul_rn(sinT, sp) + N * cosT);
    if (dot(h, -rd) < 0.0f) h = -h;
    const f3 r = reflect(rd, h);
    if (!(dot(r, N) > 0.0f)) return false;
    out = normalize(r);
    return true;
}
__device__ __forceinline__ f3 compute_normal(f3 surf, f3 tex)
{
    const f3 n = normalize(surf);
    const f3 up = (fabsf(n.y) < 0.9f) ? f3{0, 1, 0} : f3{1, 0, 0};
    const f3 t = normalize(cross(n, up));
    const f3 b = normalize(cross(t, n));
    const f3 r = {__fadd_rn(__fadd_rn(__fmul_rn(t.x, tex.x), __fmul_rn(b.x, tex.y)), __fmul_rn(n.x, tex.z)),
                  __fadd_rn(__fadd_rn(__fmul_rn(t.y, tex.x), __fmul_rn(b.y, tex.y)), __fmul_rn(n.y, tex.z)),
                  __fadd_rn(__fadd_rn(__fmul_rn(t.z, tex.x), __fmul_rn(b.z, tex.y)), __fmul_rn(n.z, tex.z))};
    return normalize(r);
}
__device__ __forceinline__ f3 aces(f3 c, float expo)
{
    const f3 col = c * expo;
    return (col * (col * 2.51f + 0.03f)) / (col * (col * 2.43f + 0.59f) + 0.14f);
}

// ---------------------------------------------------------------------------
// Textures and materials (Image.cpp:11-75, Texture.cpp:12-61, Material.hpp:82-135)
// ---------------------------------------------------------------------------
struct f4 {
    float x, y, z, w;
};
__device__ __forceinline__ f4 texel(const DevTexture& t, int x, int y)
{
    long long idx = (static_cast<long long>(y) * t.w + x) * 3;
    const long long maxIdx = static_cast<long long>(t.w) * t.h * 3 - 3;
    idx = idx < 0 ? 0 : (idx > maxIdx ? maxIdx : idx);
    if (t.rgbf) return {__ldg(t.rgbf + idx), __ldg(t.rgbf + idx + 1), __ldg(t.rgbf + idx + 2), 1.0f};
    return {__fdiv_rn(static_cast<float>(__ldg(t.rgb8 + idx)), 255.0f),
            __fdiv_rn(static_cast<float>(__ldg(t.rgb8 + idx + 1)), 255.0f),
            __fdiv_rn(static_cast<float>(__ldg(t.rgb8 + idx + 2)), 255.0f), 1.0f};
}
__device__ __forceinline__ f4 mix4(f4 a, f4 b, float s)
{
    const float r = __fsub_rn(1.0f, s);
    return {__fadd_rn(__fmul_rn(a.x, r), __fmul_rn(b.x, s)), __fadd_rn(__fmul_rn(a.y, r), __fmul_rn(b.y, s)),
            __fadd_rn(__fmul_rn(a.z, r), __fmul_rn(b.z, s)), __fadd_rn(__fmul_rn(a.w, r), __fmul_rn(b.w, s))};
}
__device__ __forceinline__ f4 image_sample(const DevTexture& t, float uvx, float uvy)
{
    const float u = __fsub_rn(uvx, floorf(uvx));
    const float v = __fsub_rn(uvy, floorf(uvy));
    const int W = static_cast<int>(t.w), H = static_cast<int>(t.h);
    if (t.filter == MT_FILTER_LINEAR) {
        const int x0 = static_cast<int>(floorf(__fmul_rn(u, static_cast<float>(W))));
        const int x1 = min(x0 + 1, W - 1);
        const int y0 = static_cast<int>(floorf(__fmul_rn(v, static_cast<float>(H))));
        const int y1 = min(y0 + 1, H - 1);
        const float sx = __fsub_rn(u, __fdiv_rn(static_cast<float>(x0), static_cast<float>(W)));
        const float sy = __fsub_rn(v, __fdiv_rn(static_cast<float>(y0), static_cast<float>(H)));
        return mix4(mix4(texel(t, x0, y0), texel(t, x1, y0), sx),
                    mix4(texel(t, x0, y1), texel(t, x1, y1), sx), sy);
    }
    int ix = static_cast<int>(__fmul_rn(u, static_cast<float>(W))) % W;
    int iy = static_cast<int>(__fmul_rn(v, static_cast<float>(H))) % H;
    if (ix < 0) ix += W;
    if (iy < 0) iy += H;
    return texel(t, ix, iy);
}
__device__ __forceinline__ f4 tex_sample(const DevScene& S, int ti, float u, float v)
{
    const DevTexture t = S.textures[ti];
    return image_sample(t, __fadd_rn(__fmul_rn(u, t.sclx), t.offx), __fadd_rn(__fmul_rn(v, t.scly), t.offy));
}

struct MatPoint {
    f4 base;
    float metallic, roughness;
    f3 normal, emission;
};

__device__ __forceinline__ MatPoint sample_material(const DevScene& S, uint32_t mi, float u, float v)
{
    const DevMaterial M = S.materials[mi];
    MatPoint p;
    if (M.base_tex >= 0) {
        const f4 t = tex_sample(S, M.base_tex, u, v);
        p.base = {__fmul_rn(t.x, M.base[0]), __fmul_rn(t.y, M.base[1]), __fmul_rn(t.z, M.base[2]),
                  __fmul_rn(t.w, M.base[3])};
    } else {
        p.base = {M.base[0], M.base[1], M.base[2], M.base[3]};
    }
    if (M.mr_tex >= 0) {
        const f4 t = tex_sample(S, M.mr_tex, u, v);
        p.metallic = __fmul_rn(t.z, M.metallic);
        p.roughness = __fmul_rn(t.y, M.roughness);
    } else {
        p.metallic = M.metallic;
        p.roughness = M.roughness;
    }
    if (M.nrm_tex >= 0) {
        const f4 t = tex_sample(S, M.nrm_tex, u, v);
        p.normal = normalize((f3{t.x, t.y, t.z} * M.normal_scale * 2.0f) + (-1.0f));
    } else {
        p.normal = f3{0.0f, 0.0f, 1.0f};
    }
    if (M.em_tex >= 0) {
        const f4 t = tex_sample(S, M.em_tex, u, v);
        p.emission = f3{t.x, t.y, t.z} * f3{M.emissive[0], M.emissive[1], M.emissive[2]};
    } else {
        p.emission = f3{M.emissive[0], M.emissive[1], M.emissive[2]};
    }
    return p;
}

// Scene::SampleSkybox (Scene.cpp:61-73), Image::SampleEquirectangular (Image.cpp:63-75)
__device__ __forceinline__ f3 sample_sky(const DevScene& S, f3 d, bool primary)
{
    if (S.env < 0) return splat(0.0f);
    const float mult = primary ? S.hdri_prim : S.hdri_sec;
    const float theta = atan2f(d.z, d.x);
    const float phi = acosf(__fdiv_rn(d.y, length(d)));
    const float u = __fdiv_rn(__fadd_rn(theta, kPi), __fmul_rn(2.0f, kPi));
    const float v = __fdiv_rn(phi, kPi);
    const DevTexture t = S.textures[S.env];
    const f4 c = image_sample(t, u, v);
    return f3{__fmul_rn(c.x, mult), __fmul_rn(c.y, mult), __fmul_rn(c.z, mult)};
}

// RandomColorFromU16 (Tracer.cpp:350-364): an integer hash of the low 16 bits,
// 3 bits per channel.
__device__ __forceinline__ f3 random_color_u16(uint32_t value)
{
    uint32_t x = value & 0xffffu;
    x ^= x >> 7;
    x *= 0x2C1B3C6Du;
    x ^= x >> 12;
    x *= 0x297A2D39u;
    x ^= x >> 15;
    const uint32_t v = x & 0xffffu;
    return {__fdiv_rn(static_cast<float>((v & 0x01C0u) >> 6), 7.0f), __fdiv_rn(static_cast<float>((v & 0x0038u) >> 3), 7.0f),
            __fdiv_rn(static_cast<float>(v & 0x0007u), 7.0f)};
}

// Heatmap (Tracer.cpp:650-670): blue, cyan, green, yellow, red; glm::mix(a, b, f)
// = a * (1 - f) + b * f.
__device__ __forceinline__ f3 heatmap(float t)
{
    t = fminf(fmaxf(t, 0.0f), 1.0f);
    const float x = __fmul_rn(t, 4.0f);
    const int i = min(static_cast<int>(x), 3);
    const float fr = __fsub_rn(x, static_cast<float>(i));
    const float r = __fsub_rn(1.0f, fr);
    const float R[5] = {0, 0, 0, 1, 1}, G[5] = {0, 1, 1, 1, 0}, B[5] = {1, 1, 0, 0, 0};
    return {__fadd_rn(__fmul_rn(R[i], r), __fmul_rn(R[i + 1], fr)), __fadd_rn(__fmul_rn(G[i], r), __fmul_rn(G[i + 1], fr)),
            __fadd_rn(__fmul_rn(B[i], r), __fmul_rn(B[i + 1], fr))};
}

}  // namespace mt
