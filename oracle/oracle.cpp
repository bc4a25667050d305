// oracle.cpp - CPU restatement of MiTrace's path-tracing hot path.
//
// TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
// product library never links or calls this file.  Parity against the
// reference's own outputs is UNPINNED: the reference cannot be built here
// (network-fetched GLM/nlohmann_json/spdlog/argparse/stb) and ships no tests or
// golden vectors.  Each function cites the reference file:line it restates.
//
// Two builds (oracle/Makefile):
//   liboracle.so       -O2 -ffp-contract=off   bit-exact checker
//   liboracle_fast.so  -Ofast -DORC_FAITHFUL_COST   timed CPU baseline with the
//                      reference's release flags (without -march=native so the
//                      same file builds on x86-64 and aarch64) and the
//                      reference's per-ray 4x4 inverse.
//
// Arithmetic conventions restated from GLM 1.0.3 (third-party, not present in
// the reference tree; the reference calls it at the cited lines):
//   dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z  (vec3);  vec4 pairs (x+y) + (z+w)
//   cross(a,b) = (a.y*b.z - b.y*a.z, a.z*b.x - b.z*a.x, a.x*b.y - b.x*a.y)
//   normalize(v) = v * (1 / sqrt(dot(v,v))),  length(v) = sqrt(dot(v,v))
//   min(x,y) = (y < x) ? y : x,  max(x,y) = (x < y) ? y : x
//   mat4 * vec4 = (c0*x + c1*y) + (c2*z + c3*w)   (columns c_i)
//   mat3 * vec3 = (c0*x + c1*y) + c2*z  per row
//   mix(a,b,t) = a*(1-t) + b*t,  reflect(I,N) = I - N*dot(N,I)*2
//   intersectRayTriangle: Moller & Trumbore (1997), two-sided with
//   |det| > FLT_EPSILON and edge-inclusive bounds; u,v weight vertices 1,2.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <random>
#include <string>
#include <thread>
#ifdef __linux__
#include <pthread.h>
#include <sched.h>
#endif
#include <vector>

namespace {

thread_local std::string g_err;

int fail(const std::string& msg, int code = MT_ERR_INVALID)
{
    g_err = msg;
    return code;
}

// ----------------------------------------------------------------------------
// GLM-convention vector math
// ----------------------------------------------------------------------------
struct V2 {
    float x, y;
};
struct V3 {
    float x, y, z;
};
struct V4 {
    float x, y, z, w;
};

inline V3 v3(float s) { return {s, s, s}; }
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
inline V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }

inline float gmin(float x, float y) { return (y < x) ? y : x; }
inline float gmax(float x, float y) { return (x < y) ? y : x; }
inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
inline V3 vmin(V3 a, V3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b)
{
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
inline float length(V3 v) { return std::sqrt(dot(v, v)); }
inline V3 normalize(V3 v)
{
    const float s = 1.0f / std::sqrt(dot(v, v));
    return v * s;
}
inline V3 reflect(V3 i, V3 n) { return i - n * dot(n, i) * 2.0f; }

// Column-major 4x4, m[c*4 + r] (glm::mat4 memory layout).
struct M4 {
    float m[16];
};

inline V4 mul(const M4& M, V4 v)
{
    const float* c0 = M.m;
    const float* c1 = M.m + 4;
    const float* c2 = M.m + 8;
    const float* c3 = M.m + 12;
    V4 r;
    r.x = (c0[0] * v.x + c1[0] * v.y) + (c2[0] * v.z + c3[0] * v.w);
    r.y = (c0[1] * v.x + c1[1] * v.y) + (c2[1] * v.z + c3[1] * v.w);
    r.z = (c0[2] * v.x + c1[2] * v.y) + (c2[2] * v.z + c3[2] * v.w);
    r.w = (c0[3] * v.x + c1[3] * v.y) + (c2[3] * v.z + c3[3] * v.w);
    return r;
}
inline V3 xyz(V4 v) { return {v.x, v.y, v.z}; }
// glm::normalize on a vec4: the vec4 dot product pairs terms, (x*x + y*y) + (z*z + w*w).
inline V4 normalize4(V4 v)
{
    const float s = 1.0f / std::sqrt((v.x * v.x + v.y * v.y) + (v.z * v.z + v.w * v.w));
    return {v.x * s, v.y * s, v.z * s, v.w * s};
}

// Inverse by cofactor expansion (the reference calls glm::inverse per ray per
// instance, Intersect.cpp:151-152; the value does not depend on the ray, so
// the checker computes it once per instance; the timed build recomputes it per
// ray to keep the reference's cost).
M4 inverse4(const M4& A)
{
    const float* a = A.m;
    float inv[16];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] +
             a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] -
             a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] +
             a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] -
              a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] -
             a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] +
             a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] -
             a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] +
              a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] +
             a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] -
             a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] +
              a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] -
              a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] -
             a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] +
             a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] -
              a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] +
              a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    const float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    M4 r;
    const float s = 1.0f / det;
    for (int i = 0; i < 16; ++i) r.m[i] = inv[i] * s;
    return r;
}

// ----------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), counter-based RNG.
// ----------------------------------------------------------------------------
inline uint32_t mulhi32(uint32_t a, uint32_t b)
{
    return static_cast<uint32_t>((static_cast<uint64_t>(a) * b) >> 32);
}

void philox4x32_10(const uint32_t in[4], const uint32_t key_in[2], uint32_t out[4])
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += W0;
            k1 += W1;
        }
        const uint32_t hi0 = mulhi32(M0, c0), lo0 = M0 * c0;
        const uint32_t hi1 = mulhi32(M1, c2), lo1 = M1 * c2;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

inline float u01(uint32_t x) { return static_cast<float>(x >> 8) * (1.0f / 16777216.0f); }

// Random-draw slots of the counter RNG.  The reference draws from one
// sequential mt19937 stream (Tracer.hpp:71-72); the GPU and the counter mode
// of this checker key each draw by (pixel, sample, bounce, slot, component).
enum : uint32_t {
    SLOT_JITTER = 0,       // camera jitter x, y           (Tracer.cpp:584-585)
    SLOT_LOBE = 1,         // lobe choice, direction u1 u2 (Tracer.cpp:181, 36-37, 52-53)
    SLOT_FALLBACK = 2,     // GGX fallback cosine u1 u2    (Tracer.cpp:71)
    SLOT_LIGHT_JITTER = 3, // point-light jitter phi theta (Tracer.cpp:89-90)
    SLOT_LIGHT_PICK = 4    // + light/4: reservoir draws   (Tracer.cpp:270)
};

struct Rng {
    int mode = ORC_RNG_MT19937;
    std::mt19937 gen;
    uint32_t key[2] = {0, 0};
    uint32_t pixel = 0, sample = 0;

    float uniform(float a, float b, uint32_t bounce, uint32_t slot, uint32_t comp)
    {
        if (mode == ORC_RNG_MT19937) {
            std::uniform_real_distribution<float> d(a, b);
            return d(gen);
        }
        const uint32_t ctr[4] = {pixel, sample, (bounce << 8) | slot, 0u};
        uint32_t o[4];
        philox4x32_10(ctr, key, o);
        return u01(o[comp & 3]) * (b - a) + a;
    }
};

constexpr float kPi = 3.14159265358979323846f;

// ----------------------------------------------------------------------------
// BVH build, restated from src/Scene/BVH.cpp
// ----------------------------------------------------------------------------
struct TreeNode {
    std::vector<uint32_t> tris;
    V3 lo, hi;
    std::unique_ptr<TreeNode> a, b;
    bool leaf = true;
};

struct BuildCtx {
    const V3* pos;
};

// BVHTreeNode::ComputeAABB, BVH.cpp:29-50
void compute_aabb(const BuildCtx& c, TreeNode& n)
{
    V3 mn = v3(std::numeric_limits<float>::max());
    V3 mx = v3(std::numeric_limits<float>::lowest());
    for (uint32_t t : n.tris) {
        const V3 v0 = c.pos[t * 3 + 0], v1 = c.pos[t * 3 + 1], v2 = c.pos[t * 3 + 2];
        mn = vmin(mn, vmin(v0, vmin(v1, v2)));
        mx = vmax(mx, vmax(v0, vmax(v1, v2)));
    }
    n.lo = mn;
    n.hi = mx;
}

// FindCenterOfMass, BVH.cpp:52-63
V3 center_of_mass(const BuildCtx& c, const TreeNode& n)
{
    V3 sum = v3(0.0f);
    for (uint32_t t : n.tris) {
        const V3 v0 = c.pos[t * 3 + 0], v1 = c.pos[t * 3 + 1], v2 = c.pos[t * 3 + 2];
        sum = sum + ((v0 + v1) + v2);
    }
    return sum / static_cast<float>(n.tris.size() * 3);
}

inline float comp(V3 v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }
inline void set_comp(V3& v, int axis, float s)
{
    if (axis == 0)
        v.x = s;
    else if (axis == 1)
        v.y = s;
    else
        v.z = s;
}

// SplitTriangles, BVH.cpp:65-102: straddlers go to both sides.
void split(const BuildCtx& c, const TreeNode& n, int axis, float pos, std::vector<uint32_t>& L,
           std::vector<uint32_t>& R)
{
    for (uint32_t t : n.tris) {
        const V3 v0 = c.pos[t * 3 + 0], v1 = c.pos[t * 3 + 1], v2 = c.pos[t * 3 + 2];
        const V3 bmin = vmin(v0, vmin(v1, v2));
        const V3 bmax = vmax(v0, vmax(v1, v2));
        if (comp(bmin, axis) < pos) L.push_back(t);
        if (comp(bmax, axis) >= pos) R.push_back(t);
    }
}

// ComputeSplitScore, BVH.cpp:105-115
float split_score(size_t total, size_t l, size_t r)
{
    if (l == total || r == total) return std::numeric_limits<float>::max();
    return static_cast<float>(l + r) / static_cast<float>(total);
}

// Subdivide, BVH.cpp:117-195.  maxDepth is unsigned and recursion stops
// creating grandchildren once it reaches 0 (the children made at that level
// stay leaves whatever their size).
void subdivide(const BuildCtx& c, TreeNode& n, unsigned maxTri, unsigned maxDepth)
{
    if (n.tris.size() <= static_cast<size_t>(maxTri)) return;
    const V3 com = center_of_mass(c, n);
    std::vector<uint32_t> L[3], R[3];
    float score[3];
    for (int ax = 0; ax < 3; ++ax) {
        split(c, n, ax, comp(com, ax), L[ax], R[ax]);
        score[ax] = split_score(n.tris.size(), L[ax].size(), R[ax].size());
    }
    const float big = std::numeric_limits<float>::max();
    if (score[0] == big && score[1] == big && score[2] == big) return;
    int ax;
    if (score[0] < score[1] && score[0] < score[2])
        ax = 0;
    else if (score[1] < score[2])
        ax = 1;
    else
        ax = 2;
    n.a = std::make_unique<TreeNode>();
    n.b = std::make_unique<TreeNode>();
    n.a->tris = std::move(L[ax]);
    n.b->tris = std::move(R[ax]);
    n.a->lo = n.lo;
    n.a->hi = n.hi;
    set_comp(n.a->hi, ax, comp(com, ax));
    n.b->lo = n.lo;
    n.b->hi = n.hi;
    set_comp(n.b->lo, ax, comp(com, ax));
    n.leaf = false;
    if (maxDepth > 0) {
        subdivide(c, *n.a, maxTri, maxDepth - 1);
        subdivide(c, *n.b, maxTri, maxDepth - 1);
    }
}

struct FlatBVH {
    std::vector<mt_bvh_node> nodes;
    std::vector<uint32_t> indices;
};

void set_box(mt_bvh_node& d, const TreeNode& n)
{
    d.lo[0] = n.lo.x;
    d.lo[1] = n.lo.y;
    d.lo[2] = n.lo.z;
    d.hi[0] = n.hi.x;
    d.hi[1] = n.hi.y;
    d.hi[2] = n.hi.z;
}

// FlattenRecursive, BVH.cpp:223-259: siblings adjacent, A's subtree first.
void flatten_pair(FlatBVH& f, const TreeNode& A, const TreeNode& B, uint32_t& ia, uint32_t& ib)
{
    ia = static_cast<uint32_t>(f.nodes.size());
    ib = ia + 1;
    f.nodes.push_back(mt_bvh_node{});
    f.nodes.push_back(mt_bvh_node{});
    set_box(f.nodes[ia], A);
    set_box(f.nodes[ib], B);
    const TreeNode* kids[2] = {&A, &B};
    const uint32_t slots[2] = {ia, ib};
    for (int k = 0; k < 2; ++k) {
        const TreeNode& n = *kids[k];
        if (n.leaf) {
            const uint32_t first = static_cast<uint32_t>(f.indices.size());
            f.indices.insert(f.indices.end(), n.tris.begin(), n.tris.end());
            f.nodes[slots[k]].a = first | MT_BVH_LEAF_BIT;
            f.nodes[slots[k]].b = static_cast<uint32_t>(n.tris.size());
        } else {
            uint32_t ca, cb;
            flatten_pair(f, *n.a, *n.b, ca, cb);
            f.nodes[slots[k]].a = ca;
            f.nodes[slots[k]].b = cb;
        }
    }
}

// BVH::BVH + BVHTree + Flatten, BVH.cpp:204-212, 261-282; depth per Mesh.cpp:40.
int build_bvh(const V3* pos, uint32_t T, uint32_t maxTri, uint32_t cfgMaxDepth, FlatBVH& out)
{
    if (T == 0) return fail("Cannot compute AABB for a BVH node with no triangles.");
    BuildCtx c{pos};
    TreeNode root;
    root.tris.resize(T);
    for (uint32_t i = 0; i < T; ++i) root.tris[i] = i;
    compute_aabb(c, root);
    const unsigned meshDepth = cfgMaxDepth - 1u;  // Mesh.cpp:40
    const unsigned treeDepth = meshDepth - 1u;    // BVH.cpp:211
    subdivide(c, root, maxTri, treeDepth);
    if (root.leaf)
        return fail("BVH root could not be split; the reference flattens null children here "
                    "(BVH.cpp:264-265)");
    out.nodes.clear();
    out.indices.clear();
    out.nodes.push_back(mt_bvh_node{});
    out.nodes.push_back(mt_bvh_node{});  // slot 1 is never used (BVH.cpp:265-266)
    uint32_t ca, cb;
    flatten_pair(out, *root.a, *root.b, ca, cb);
    set_box(out.nodes[0], root);
    out.nodes[0].a = ca;
    out.nodes[0].b = cb;
    return MT_OK;
}

// ----------------------------------------------------------------------------
// Scene
// ----------------------------------------------------------------------------
struct Mesh {
    std::vector<V3> pos, nrm;
    std::vector<V2> uv0;
    bool hasBVH = false;
    FlatBVH bvh;
    V3 lo, hi;  // Mesh::CalculateAABB, Mesh.cpp:43-54
};

struct Texture {
    uint32_t w = 0, h = 0;
    std::vector<uint8_t> rgb8;
    std::vector<float> rgbf;
    int filter = MT_FILTER_NEAREST;
    V2 offset{0, 0}, scale{1, 1};
    bool valid() const { return w > 0 && h > 0; }
};

struct Material {
    V4 baseFactor;
    V3 emissive;
    float normalScale, metallic, roughness;
    int baseTex, mrTex, nrmTex, emTex;
};

struct Instance {
    uint32_t mesh, material;
    M4 model, inv;
    V3 wlo, whi;
};

struct Light {
    int type;
    V3 pos, color, dir;
    float pointSize, innerCos, outerCos;
    float simpleIntensity;  // PrepareLights, Tracer.cpp:123-132
};

struct Camera {
    int type;
    M4 c2w;
    float fov, aspect;
    V2 ortho;
};

}  // namespace

struct orc_scene {
    std::vector<Mesh> meshes;
    std::vector<Texture> textures;
    std::vector<Material> materials;
    std::vector<Instance> instances;
    std::vector<Light> lights;
    Camera cam;
    int env = -1;
    mt_config cfg;
};

namespace {

// ----------------------------------------------------------------------------
// Intersection, restated from src/Tracer/Intersect.cpp
// ----------------------------------------------------------------------------
// IntersectRayAABB, Intersect.cpp:9-18: exit distance, or -1.
inline float ray_aabb(V3 o, V3 d, V3 lo, V3 hi)
{
    const V3 inv = V3{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    const V3 t1 = (lo - o) * inv;
    const V3 t2 = (hi - o) * inv;
    const V3 tmin = vmin(t1, t2);
    const V3 tmax = vmax(t1, t2);
    const float enter = gmax(gmax(tmin.x, tmin.y), tmin.z);
    const float exit = gmin(gmin(tmax.x, tmax.y), tmax.z);
    return enter <= exit ? exit : -1.0f;
}

// Moller-Trumbore, two-sided, edge-inclusive (glm::intersectRayTriangle as
// called at Intersect.cpp:34-35, 94-95).
inline bool ray_tri(V3 o, V3 d, V3 v0, V3 v1, V3 v2, float& bu, float& bv, float& t)
{
    const V3 e1 = v1 - v0;
    const V3 e2 = v2 - v0;
    const V3 p = cross(d, e2);
    const float det = dot(e1, p);
    V3 q;
    float u, v;
    if (det > FLT_EPSILON) {
        const V3 s = o - v0;
        u = dot(s, p);
        if (u < 0.0f || u > det) return false;
        q = cross(s, e1);
        v = dot(d, q);
        if (v < 0.0f || u + v > det) return false;
    } else if (det < -FLT_EPSILON) {
        const V3 s = o - v0;
        u = dot(s, p);
        if (u > 0.0f || u < det) return false;
        q = cross(s, e1);
        v = dot(d, q);
        if (v > 0.0f || u + v < det) return false;
    } else {
        return false;
    }
    const float inv = 1.0f / det;
    t = dot(e2, q) * inv;
    bu = u * inv;
    bv = v * inv;
    return true;
}

struct Hit {
    bool hit = false;
    uint32_t inst = 0, tri = 0, bv = 0, bvhTests = 0, triTests = 0;
    float u = 0, v = 0, dist = 0;
    V3 worldPos{0, 0, 0};
};

struct StackEntry {
    uint32_t node;
    float dist;
};

// IntersectTrianglesLinear, Intersect.cpp:20-45
void tris_linear(const Mesh& m, V3 o, V3 d, float& dist, float& bu, float& bv, uint32_t& tri,
                 uint32_t& triTests)
{
    const uint32_t T = static_cast<uint32_t>(m.pos.size() / 3);
    for (uint32_t i = 0; i < T; ++i) {
        float u, v, t;
        ++triTests;
        if (ray_tri(o, d, m.pos[i * 3], m.pos[i * 3 + 1], m.pos[i * 3 + 2], u, v, t)) {
            if (t > 0.0f && t < dist) {
                dist = t;
                bu = u;
                bv = v;
                tri = i;
            }
        }
    }
}

// IntersectTrianglesBVH, Intersect.cpp:47-141.  Stack DFS keyed on the box
// EXIT distance with 0.1 slack; the nearer child is pushed last.
void tris_bvh(const Mesh& m, V3 o, V3 d, float& dist, float& bu, float& bv, uint32_t& bvIdx,
              uint32_t& tri, uint32_t& bvhTests, uint32_t& triTests, uint32_t& innerPops,
              std::vector<StackEntry>& stack)
{
    const float minDelta = 0.1f;
    const mt_bvh_node* nodes = m.bvh.nodes.data();
    const uint32_t* idx = m.bvh.indices.data();
    auto box = [&](const mt_bvh_node& n) {
        return ray_aabb(o, d, V3{n.lo[0], n.lo[1], n.lo[2]}, V3{n.hi[0], n.hi[1], n.hi[2]});
    };
    stack.clear();
    stack.push_back({0, box(nodes[0])});
    while (!stack.empty()) {
        const StackEntry e = stack.back();
        stack.pop_back();
        ++bvhTests;
        const mt_bvh_node& n = nodes[e.node];
        if (e.dist < 0.0f) continue;
        if (e.dist > dist + minDelta) continue;
        if (n.a & MT_BVH_LEAF_BIT) {
            const uint32_t first = n.a & ~MT_BVH_LEAF_BIT;
            const uint32_t count = n.b & ~MT_BVH_LEAF_BIT;
            for (uint32_t i = first; i < first + count; ++i) {
                const uint32_t t = idx[i];
                float u, v, tt;
                ++triTests;
                if (ray_tri(o, d, m.pos[t * 3], m.pos[t * 3 + 1], m.pos[t * 3 + 2], u, v, tt)) {
                    if (tt > 0.0f && tt < dist) {
                        dist = tt;
                        bu = u;
                        bv = v;
                        bvIdx = e.node;
                        tri = t;
                    }
                }
            }
        } else {
            ++innerPops;
            const float da = box(nodes[n.a]);
            const float db = box(nodes[n.b]);
            const bool pa = da >= 0.0f && da <= dist + minDelta;
            const bool pb = db >= 0.0f && db <= dist + minDelta;
            if (pa && pb) {
                if (da < db) {
                    stack.push_back({n.b, db});
                    stack.push_back({n.a, da});
                } else {
                    stack.push_back({n.a, da});
                    stack.push_back({n.b, db});
                }
            } else if (pa) {
                stack.push_back({n.a, da});
            } else if (pb) {
                stack.push_back({n.b, db});
            }
        }
    }
}

// IntersectMeshInstance, Intersect.cpp:143-199
bool intersect_instance(const orc_scene& s, uint32_t ii, V3 o, V3 d, Hit& h,
                        std::vector<StackEntry>& stack, uint32_t* totB, uint32_t* totT, uint32_t* totI)
{
    const Instance& in = s.instances[ii];
    if (ray_aabb(o, d, in.wlo, in.whi) < 0.0f) return false;
#ifdef ORC_FAITHFUL_COST
    const M4 inv = inverse4(in.model);
#else
    const M4& inv = in.inv;
#endif
    const V3 lo = xyz(mul(inv, V4{o.x, o.y, o.z, 1.0f}));
    const V3 ld = normalize(xyz(mul(inv, V4{d.x, d.y, d.z, 0.0f})));
    const Mesh& m = s.meshes[in.mesh];
    float dist = std::numeric_limits<float>::max();
    float bu = 0, bv = 0;
    uint32_t bvIdx = 0, tri = 0, bvhTests = 0, triTests = 0, innerPops = 0;
    if (m.hasBVH)
        tris_bvh(m, lo, ld, dist, bu, bv, bvIdx, tri, bvhTests, triTests, innerPops, stack);
    else
        tris_linear(m, lo, ld, dist, bu, bv, tri, triTests);
    if (totB) *totB += bvhTests;
    if (totT) *totT += triTests;
    if (totI) *totI += innerPops;
    if (!(dist < std::numeric_limits<float>::max())) return false;
    const V3 lp = lo + dist * ld;
    h.worldPos = xyz(mul(in.model, V4{lp.x, lp.y, lp.z, 1.0f}));
    h.dist = length(h.worldPos - o);
    h.tri = tri;
    h.bv = bvIdx;
    h.u = bu;
    h.v = bv;
    h.bvhTests = bvhTests;
    h.triTests = triTests;
    h.inst = ii;
    h.hit = true;
    return true;
}

// IntersectScene, Intersect.cpp:201-219: strict '<' keeps the first instance.
Hit intersect_scene(const orc_scene& s, V3 o, V3 d, std::vector<StackEntry>& stack,
                    uint32_t* totB = nullptr, uint32_t* totT = nullptr, uint32_t* totI = nullptr)
{
    float best = std::numeric_limits<float>::max();
    Hit bestHit;
    const uint32_t n = static_cast<uint32_t>(s.instances.size());
    for (uint32_t i = 0; i < n; ++i) {
        Hit h;
        if (intersect_instance(s, i, o, d, h, stack, totB, totT, totI)) {
            if (h.dist < best) {
                best = h.dist;
                bestHit = h;
            }
        }
    }
    return bestHit;
}

// ----------------------------------------------------------------------------
// Textures and materials (Image.cpp:11-75, Texture.cpp:12-61, Material.hpp:82-135)
// ----------------------------------------------------------------------------
V4 texel(const Texture& t, int x, int y)
{
    // SamplePixel, Image.cpp:11-15.  The reference can read one texel past a
    // row (x == W after rounding); the index is clamped to the image here.
    long long idx = (static_cast<long long>(y) * t.w + x) * 3;
    const long long maxIdx = static_cast<long long>(t.w) * t.h * 3 - 3;
    if (idx < 0) idx = 0;
    if (idx > maxIdx) idx = maxIdx;
    if (!t.rgbf.empty())
        return {t.rgbf[idx], t.rgbf[idx + 1], t.rgbf[idx + 2], 1.0f};
    return V4{static_cast<float>(t.rgb8[idx]) / 255.0f, static_cast<float>(t.rgb8[idx + 1]) / 255.0f,
              static_cast<float>(t.rgb8[idx + 2]) / 255.0f, 255.0f / 255.0f};
}

inline V4 mix4(V4 a, V4 b, float s)
{
    const float r = 1.0f - s;
    return {a.x * r + b.x * s, a.y * r + b.y * s, a.z * r + b.z * s, a.w * r + b.w * s};
}

// Image::Sample with SampleNearest / SampleLinear (the latter keeps the
// reference's weight bug: sx = u - x0/W, Image.cpp:26-44).
V4 image_sample(const Texture& t, float uvx, float uvy)
{
    const float u = uvx - std::floor(uvx);
    const float v = uvy - std::floor(uvy);
    const int W = static_cast<int>(t.w), H = static_cast<int>(t.h);
    if (t.filter == MT_FILTER_LINEAR) {
        const int x0 = static_cast<int>(std::floor(u * static_cast<float>(W)));
        const int x1 = std::min(x0 + 1, W - 1);
        const int y0 = static_cast<int>(std::floor(v * static_cast<float>(H)));
        const int y1 = std::min(y0 + 1, H - 1);
        const float sx = u - static_cast<float>(x0) / static_cast<float>(W);
        const float sy = v - static_cast<float>(y0) / static_cast<float>(H);
        const V4 c00 = texel(t, x0, y0), c10 = texel(t, x1, y0);
        const V4 c01 = texel(t, x0, y1), c11 = texel(t, x1, y1);
        return mix4(mix4(c00, c10, sx), mix4(c01, c11, sx), sy);
    }
    int ix = static_cast<int>(u * static_cast<float>(W)) % W;
    int iy = static_cast<int>(v * static_cast<float>(H)) % H;
    if (ix < 0) ix += W;
    if (iy < 0) iy += H;
    return texel(t, ix, iy);
}

// Texture::Sample, Texture.cpp:52-56 (uv * scale + offset)
V4 tex_sample(const orc_scene& s, int ti, V2 uv)
{
    const Texture& t = s.textures[ti];
    return image_sample(t, uv.x * t.scale.x + t.offset.x, uv.y * t.scale.y + t.offset.y);
}

struct MatPoint {
    V4 base;
    float metallic, roughness;
    V3 normal, emission;
};

// Material::SampleMaterial, Material.hpp:82-135
MatPoint sample_material(const orc_scene& s, const Material& m, V2 uv)
{
    MatPoint p;
    if (m.baseTex >= 0) {
        const V4 t = tex_sample(s, m.baseTex, uv);
        p.base = {t.x * m.baseFactor.x, t.y * m.baseFactor.y, t.z * m.baseFactor.z,
                  t.w * m.baseFactor.w};
    } else {
        p.base = m.baseFactor;
    }
    if (m.mrTex >= 0) {
        const V4 t = tex_sample(s, m.mrTex, uv);
        p.metallic = t.z * m.metallic;
        p.roughness = t.y * m.roughness;
    } else {
        p.metallic = m.metallic;
        p.roughness = m.roughness;
    }
    if (m.nrmTex >= 0) {
        const V4 t = tex_sample(s, m.nrmTex, uv);
        const V3 c{t.x, t.y, t.z};
        p.normal = normalize(c * m.normalScale * 2.0f + (-1.0f));
    } else {
        p.normal = V3{0.0f, 0.0f, 1.0f};
    }
    if (m.emTex >= 0) {
        const V4 t = tex_sample(s, m.emTex, uv);
        p.emission = V3{t.x, t.y, t.z} * m.emissive;
    } else {
        p.emission = m.emissive;
    }
    return p;
}

// Scene::SampleSkybox + Image::SampleEquirectangular (Scene.cpp:61-73,
// Image.cpp:63-75); the texture offset (hdriRotation) is not applied.
V3 sample_sky(const orc_scene& s, V3 d, bool primary)
{
    const float mult = primary ? s.cfg.hdri_primary_intensity : s.cfg.hdri_secondary_intensity;
    if (s.env < 0) return v3(0.0f);
    const Texture& t = s.textures[s.env];
    const float theta = std::atan2(d.z, d.x);
    const float phi = std::acos(d.y / length(d));
    const float u = (theta + kPi) / (2.0f * kPi);
    const float v = phi / kPi;
    const V4 c = image_sample(t, u, v);
    return V3{c.x * mult, c.y * mult, c.z * mult};
}

// ----------------------------------------------------------------------------
// BRDF, restated from src/Tracer/BRDF.hpp
// ----------------------------------------------------------------------------
V3 fresnel_schlick(float c, V3 f0)
{
    c = gclamp(c, 0.0f, 1.0f);
    const float p = std::pow(1.0f - c, 5.0f);
    return f0 + (v3(1.0f) - f0) * v3(p);
}

V3 base_reflectivity(V3 base, float metallic)
{
    metallic = gclamp(metallic, 0.0f, 1.0f);
    const float r = 1.0f - metallic;
    return v3(0.04f) * r + base * metallic;
}

float distribution_ggx(float nh, float roughness)
{
    nh = gclamp(nh, 0.0f, 1.0f);
    const float a = roughness * roughness;
    const float a2 = a * a;
    const float nh2 = nh * nh;
    float denom = nh2 * (a2 - 1.0f) + 1.0f;
    denom = kPi * denom * denom;
    return a2 / denom;
}

float geometry_schlick_ggx(float nv, float roughness)
{
    nv = gclamp(nv, 0.0f, 1.0f);
    const float r = roughness + 1.0f;
    const float k = (r * r) / 8.0f;
    const float denom = nv * (1.0f - k) + k;
    return nv / denom;
}

V3 eval_brdf(V3 L, V3 V, V3 N, V3 base, float roughness, float metallic)
{
    roughness = gmax(roughness, 0.05f);
    const float nl = gmax(dot(N, L), 0.0f);
    const float nv = gmax(dot(N, V), 0.0f);
    if (nl <= 0.0f || nv <= 0.0f) return v3(0.0f);
    const V3 h = normalize(V + L);
    const float nh = gmax(dot(N, h), 0.0f);
    const float hv = gmax(dot(h, V), 0.0f);
    const V3 f0 = base_reflectivity(base, metallic);
    const V3 f = fresnel_schlick(hv, f0);
    const float d = distribution_ggx(nh, roughness);
    const float g = geometry_schlick_ggx(nv, roughness) * geometry_schlick_ggx(nl, roughness);
    const V3 kd = (v3(1.0f) - f) * (1.0f - metallic);
    const V3 diffuse = kd * base / kPi;
    const V3 spec = (d * g * f) / gmax(4.0f * nv * nl, 0.001f);
    return vmax(diffuse + spec, v3(0.0f));
}

float diffuse_pdf(V3 L, V3 N) { return gmax(dot(N, L), 0.0f) / kPi; }

float specular_pdf(V3 L, V3 V, V3 N, float roughness)
{
    const float nl = gmax(dot(N, L), 0.0f);
    const float nv = gmax(dot(N, V), 0.0f);
    if (nl <= 0.0f || nv <= 0.0f) return 0.0f;
    const V3 h = normalize(V + L);
    const float nh = gmax(dot(N, h), 0.0f);
    const float vh = gmax(dot(V, h), 0.0f);
    if (vh <= 0.0f) return 0.0f;
    return distribution_ggx(nh, gmax(roughness, 0.05f)) * nh / (4.0f * vh);
}

// ----------------------------------------------------------------------------
// Sampling helpers, restated from src/Tracer/Tracer.cpp:26-121
// ----------------------------------------------------------------------------
void build_tbn(V3 n, V3& t, V3& b)
{
    const V3 up = (std::fabs(n.z) < 0.999f) ? V3{0, 0, 1} : V3{1, 0, 0};
    t = normalize(cross(up, n));
    b = cross(n, t);
}

V3 cosine_hemisphere(float u1, float u2, V3 n)
{
    const float r = std::sqrt(u1);
    const float phi = 2.0f * kPi * u2;
    V3 t, b;
    build_tbn(n, t, b);
    const V3 l{r * std::cos(phi), r * std::sin(phi), std::sqrt(gmax(0.0f, 1.0f - u1))};
    return normalize(t * l.x + b * l.y + n * l.z);
}

V3 sample_cosine(Rng& rng, uint32_t bounce, uint32_t slot, uint32_t c0, V3 n)
{
    const float u1 = rng.uniform(0.0f, 1.0f, bounce, slot, c0);
    const float u2 = rng.uniform(0.0f, 1.0f, bounce, slot, c0 + 1);
    return cosine_hemisphere(u1, u2, n);
}

// SampleGGXDirection's reflection for given uniforms; false when it points
// below the surface.
bool ggx_reflection(V3 incident, V3 n, float roughness, float u1, float u2, V3& out);

V3 sample_ggx(Rng& rng, uint32_t bounce, V3 incident, V3 n, float roughness)
{
    const float u1 = rng.uniform(0.0f, 1.0f, bounce, SLOT_LOBE, 1);
    const float u2 = rng.uniform(0.0f, 1.0f, bounce, SLOT_LOBE, 2);
    V3 r;
    return ggx_reflection(incident, n, roughness, u1, u2, r) ? r : sample_cosine(rng, bounce, SLOT_FALLBACK, 0, n);
}

bool ggx_reflection(V3 incident, V3 n, float roughness, float u1, float u2, V3& out)
{
    const float alpha = gmax(roughness * roughness, 0.0025f);
    const float alpha2 = alpha * alpha;
    const float phi = 2.0f * kPi * u2;
    const float tan2 = alpha2 * u1 / gmax(1.0f - u1, 0.0001f);
    const float cosT = 1.0f / std::sqrt(1.0f + tan2);
    const float sinT = std::sqrt(gmax(0.0f, 1.0f - cosT * cosT));
    V3 t, b;
    build_tbn(n, t, b);
    V3 h = normalize(t * (sinT * std::cos(phi)) + b * (sinT * std::sin(phi)) + n * cosT);
    if (dot(h, -incident) < 0.0f) h = -h;
    const V3 r = reflect(incident, h);
    if (!(dot(r, n) > 0.0f)) return false;
    out = normalize(r);
    return true;
}

float specular_probability(V3 view, V3 n, V3 base, float metallic)
{
    const V3 f0 = base_reflectivity(base, metallic);
    const V3 f = fresnel_schlick(gmax(dot(n, view), 0.0f), f0);
    const float p = (f.x + f.y + f.z) / 3.0f;
    return gclamp(p, 0.05f, 0.95f);
}

V3 random_direction(Rng& rng, uint32_t bounce)
{
    const float u = rng.uniform(0.0f, 2.0f * kPi, bounce, SLOT_LIGHT_JITTER, 0);
    const float v = rng.uniform(-kPi / 2.0f, kPi / 2.0f, bounce, SLOT_LIGHT_JITTER, 1);
    return normalize(V3{cosf(u) * cosf(v), sinf(v), sinf(u) * cosf(v)});
}

// ComputeNormal, Tracer.cpp:95-105
V3 compute_normal(V3 surf, V3 tex)
{
    const V3 n = normalize(surf);
    const V3 up = (std::fabs(n.y) < 0.9f) ? V3{0, 1, 0} : V3{1, 0, 0};
    const V3 t = normalize(cross(n, up));
    const V3 b = normalize(cross(t, n));
    return normalize(V3{t.x * tex.x + b.x * tex.y + n.x * tex.z,
                        t.y * tex.x + b.y * tex.y + n.y * tex.z,
                        t.z * tex.x + b.z * tex.y + n.z * tex.z});
}

V3 aces(V3 c, float expo)
{
    const V3 col = c * expo;
    const float a = 2.51f, b = 0.03f, cc = 2.43f, d = 0.59f, e = 0.14f;
    return (col * (col * a + b)) / (col * (col * cc + d) + e);
}

// ----------------------------------------------------------------------------
// Path generation and shading walk (Tracer.cpp:134-210, 229-348)
// ----------------------------------------------------------------------------
struct PathStep {
    V3 rayO, rayD;
    V3 hitPos, base, normal, energy, emission;
    float metallic, roughness;
    bool didHit;
    // debug information (Tracer.hpp:46-53); a miss step keeps zeros here, where
    // the reference leaves these members uninitialised
    V3 geomN{0, 0, 0};
    float brdfIntensity = 0.0f, pdf = 0.0f;
    uint32_t bvhTests = 0, triTests = 0, triIndex = 0, bvIndex = 0, inst = 0;
    // kept for the adjoint replay
    uint32_t mat = 0;
    V2 uv{0.0f, 0.0f};
    V3 nextDir{0, 0, 0};
    float facNext = 0.0f;  // energy = brdf(nextDir) * facNext
    bool chosen = false, visible = false;
    uint32_t light = 0;
    V3 ldir{0, 0, 0};
    float facLight = 0.0f;  // NEE = cur * brdf(ldir) * color * spot * facLight
    float spot = 1.0f;
    V3 sky{0, 0, 0};       // sky sample of a miss step
};

struct Worker {
    std::vector<StackEntry> stack;
    std::vector<PathStep> path;
    uint64_t rays = 0;
};

void generate_path(const orc_scene& s, Worker& w, Rng& rng, V3 o0, V3 d0)
{
    const mt_config& cfg = s.cfg;
    V3 o = o0, d = d0;
    V3 total = v3(1.0f);
    w.path.clear();
    uint32_t bounce = 0;
    while (w.path.size() < cfg.bounces) {
        PathStep st;
        const Hit hit = intersect_scene(s, o, d, w.stack);
        ++w.rays;
        st.rayO = o;
        st.rayD = d;
        if (!hit.hit) {
            st.didHit = false;
            w.path.push_back(st);
            break;
        }
        // RayHitGeometryInfo (Ray.cpp:7-48)
        const Instance& in = s.instances[hit.inst];
        const Mesh& m = s.meshes[in.mesh];
        const float wgt = 1.0f - hit.u - hit.v;
        const uint32_t t3 = hit.tri * 3;
        const V3 ni = normalize(wgt * m.nrm[t3] + hit.u * m.nrm[t3 + 1] + hit.v * m.nrm[t3 + 2]);
        const V4 nw = normalize4(mul(in.model, V4{ni.x, ni.y, ni.z, 0.0f}));
        const V3 geomN{nw.x, nw.y, nw.z};
        V2 uv{0.0f, 0.0f};
        if (!m.uv0.empty()) {
            const V2 a = m.uv0[t3], b = m.uv0[t3 + 1], c = m.uv0[t3 + 2];
            uv = {wgt * a.x + hit.u * b.x + hit.v * c.x, wgt * a.y + hit.u * b.y + hit.v * c.y};
        }
        MatPoint mp = sample_material(s, s.materials[in.material], uv);
        mp.base = {mp.base.x * 0.96f + 0.04f, mp.base.y * 0.96f + 0.04f, mp.base.z * 0.96f + 0.04f,
                   mp.base.w * 0.96f + 0.04f};
        st.hitPos = hit.worldPos;
        st.base = {mp.base.x, mp.base.y, mp.base.z};
        st.roughness = mp.roughness;
        st.metallic = mp.metallic;
        st.normal = compute_normal(geomN, mp.normal);
        st.emission = mp.emission;
        st.didHit = true;
        st.mat = in.material;
        st.uv = uv;
        st.geomN = geomN;
        st.bvhTests = hit.bvhTests;
        st.triTests = hit.triTests;
        st.bvIndex = hit.bv & 0xffffu;
        st.triIndex = hit.tri & 0xffffu;
        st.inst = hit.inst;

        const V3 view = -d;
        const float ps = specular_probability(view, st.normal, st.base, st.metallic);
        V3 nd;
        if (rng.uniform(0.0f, 1.0f, bounce, SLOT_LOBE, 0) < ps)
            nd = sample_ggx(rng, bounce, d, st.normal, mp.roughness);
        else
            nd = sample_cosine(rng, bounce, SLOT_LOBE, 1, st.normal);
        const V3 no = (o + d * hit.dist) + st.normal * 0.0001f;
        const float dp = diffuse_pdf(nd, st.normal);
        const float sp = specular_pdf(nd, view, st.normal, st.roughness);
        const float pdf = (1.0f - ps) * dp + ps * sp;
        const V3 brdf = eval_brdf(nd, view, st.normal, st.base, st.roughness, st.metallic);
        const float nl = gmax(dot(st.normal, nd), 0.0f);
        st.energy = (pdf > 0.0f) ? brdf * (nl / pdf) : v3(0.0f);
        st.brdfIntensity = (brdf.x + brdf.y) + brdf.z;
        st.pdf = pdf;
        st.nextDir = nd;
        st.facNext = (pdf > 0.0f) ? nl / pdf : 0.0f;
        w.path.push_back(st);
        o = no;
        d = nd;
        total = total * st.energy;
        if (length(total) < cfg.terminate_energy) break;
        ++bounce;
    }
}

struct LightOut {
    V3 emitted, direct, indirect, sky;
};

V3 process_ray_forward(const orc_scene& s, Worker& w, Rng& rng, V3 o, V3 d, float expo,
                       V3* total_out = nullptr, LightOut* parts = nullptr)
{
    const mt_config& cfg = s.cfg;
    generate_path(s, w, rng, o, d);
    V3 cur = v3(1.0f);
    V3 emitted = v3(0.0f), direct = v3(0.0f), indirect = v3(0.0f), sky = v3(0.0f);
    for (size_t i = 0; i < w.path.size(); ++i) {
        PathStep& st = w.path[i];
        const uint32_t bounce = static_cast<uint32_t>(i);
        if (!st.didHit) {
            const V3 color = (i > 0) ? w.path[i - 1].base : v3(1.0f);
            st.sky = sample_sky(s, st.rayD, i == 0);
            sky = sky + color * cur * st.sky;
            break;
        }
        emitted = emitted + cur * cfg.emission_base_intensity * st.emission;
        int chosen = -1;
        float pickPdf = 0.0f, totalScore = 0.0f;
        for (size_t li = 0; li < s.lights.size(); ++li) {
            const V3 lp = s.lights[li].pos - st.hitPos;
            const float d2 = dot(lp, lp);
            const float score = s.lights[li].simpleIntensity / (d2 + 1.0f);
            totalScore += score;
            const uint32_t slot = SLOT_LIGHT_PICK + static_cast<uint32_t>(li >> 2);
            if (rng.uniform(0.0f, 1.0f, bounce, slot, static_cast<uint32_t>(li & 3)) * totalScore <
                score) {
                chosen = static_cast<int>(li);
                pickPdf = score;
            }
        }
        pickPdf /= totalScore;
        if (chosen == -1) continue;  // skips the energy update (Tracer.cpp:279)
        const Light& L = s.lights[chosen];
        V3 lpos;
        if (L.type == MT_LIGHT_POINT || L.type == MT_LIGHT_SPOT)
            lpos = L.pos + random_direction(rng, bounce) * L.pointSize;
        else
            lpos = L.pos;
        const V3 lvec = lpos - st.hitPos;
        const V3 ldir = normalize(lvec);
        V3 lcol;
        st.spot = 1.0f;
        if (L.type == MT_LIGHT_SPOT) {
            const float dd = dot(-ldir, L.dir);
            const float inten = (dd - L.outerCos) / (L.innerCos - L.outerCos);
            st.spot = gclamp(inten, 0.0f, 1.0f);
            lcol = L.color * st.spot;
        } else {
            lcol = L.color;
        }
        st.chosen = true;
        st.light = static_cast<uint32_t>(chosen);
        st.ldir = ldir;
        const V3 so = st.hitPos + lvec * 0.0001f;
        const Hit sh = intersect_scene(s, so, ldir, w.stack);
        ++w.rays;
        if (!sh.hit || sh.dist > length(lvec)) {
            const V3 brdf = eval_brdf(ldir, -st.rayD, st.normal, st.base, st.roughness, st.metallic);
            const float nl = gmax(dot(st.normal, ldir), 0.0f);
            const float fall = 1.0f / (length(lvec) * length(lvec) + 1.0f);
            const V3 le = brdf * nl * fall;
            const V3 c = cur * le * lcol / pickPdf;
            st.visible = true;
            st.facLight = nl * fall / pickPdf;
            if (i == 0)
                direct = direct + c;
            else
                indirect = indirect + c;
        }
        cur = cur * st.energy;
    }
    const V3 total = ((emitted + direct) + indirect) + sky;
    if (total_out) *total_out = total;
    if (parts) *parts = {emitted, direct, indirect, sky};
    return aces(total, expo);
}

// RandomColorFromU16, Tracer.cpp:350-364
V3 random_color_u16(uint32_t value)
{
    uint32_t x = value & 0xffffu;
    x ^= x >> 7;
    x *= 0x2C1B3C6Du;
    x ^= x >> 12;
    x *= 0x297A2D39u;
    x ^= x >> 15;
    const uint32_t v = x & 0xffffu;
    return {static_cast<float>((v & 0x01C0u) >> 6) / 7.0f, static_cast<float>((v & 0x0038u) >> 3) / 7.0f,
            static_cast<float>(v & 0x0007u) / 7.0f};
}

// Config::DebugMode values (src/CLI/Config.hpp:16-40)
enum DebugMode {
    DBG_NONE = 0, DBG_PRIMARY_BVH, DBG_TOTAL_BVH, DBG_PRIMARY_TRI, DBG_TOTAL_TRI, DBG_ALBEDO,
    DBG_METALLIC_ROUGHNESS, DBG_GEOM_NORMAL, DBG_SHADING_NORMAL, DBG_DIRECT, DBG_INDIRECT, DBG_EMISSION,
    DBG_COLOR_MESH, DBG_COLOR_TRIANGLE, DBG_COLOR_BV, DBG_BOUNCES, DBG_DEPTH, DBG_FRESNEL, DBG_BRDF, DBG_PDF,
    DBG_REFLECTED, DBG_PIXEL_STDDEV, DBG_FIREFLY, DBG_COUNT
};

// ProcessDebugRay, Tracer.cpp:366-488.  The colour per mesh is keyed by the
// instance index: the reference keys it by the low 16 bits of the
// MeshInstance's address, which change from run to run.
V3 process_debug_ray(const orc_scene& s, Worker& w, Rng& rng, V3 o, V3 d, float expo, int mode)
{
    LightOut lo;
    const V3 total = process_ray_forward(s, w, rng, o, d, expo, nullptr, &lo);
    const PathStep& f = w.path.front();
    const bool hit = f.didHit;
    const V3 black = v3(0.0f);
    auto sum_steps = [&](bool tris) {
        float acc = 0.0f;
        for (const PathStep& st : w.path) acc = acc + static_cast<float>(tris ? st.triTests : st.bvhTests);
        return acc;
    };
    switch (mode) {
        case DBG_PRIMARY_BVH: return hit ? v3(static_cast<float>(f.bvhTests)) : black;
        case DBG_TOTAL_BVH: return hit ? v3(sum_steps(false)) : black;
        case DBG_PRIMARY_TRI: return hit ? v3(static_cast<float>(f.triTests)) : black;
        case DBG_TOTAL_TRI: return hit ? v3(sum_steps(true)) : black;
        case DBG_BOUNCES: return hit ? v3(static_cast<float>(w.path.size())) : black;
        case DBG_ALBEDO: return hit ? f.base : black;
        case DBG_METALLIC_ROUGHNESS: return hit ? V3{0.0f, f.metallic, f.roughness} : black;
        case DBG_GEOM_NORMAL: return hit ? f.geomN * 0.5f + v3(0.5f) : black;
        case DBG_SHADING_NORMAL: return hit ? f.normal * 0.5f + v3(0.5f) : black;
        case DBG_DIRECT: return aces(lo.direct, expo);
        case DBG_INDIRECT: return aces(lo.indirect + lo.sky, expo);
        case DBG_EMISSION: return aces(lo.emitted, expo);
        case DBG_COLOR_MESH: return hit ? random_color_u16(f.inst) : black;
        case DBG_COLOR_TRIANGLE: return hit ? random_color_u16(f.triIndex) : black;
        case DBG_COLOR_BV: return hit ? random_color_u16(f.bvIndex) : black;
        case DBG_DEPTH: return hit ? v3(length(f.hitPos - o)) : black;
        case DBG_FRESNEL: {
            const V3 f0 = base_reflectivity(f.base, f.metallic);
            const float c = dot(f.normal, -d);
            return hit ? fresnel_schlick(gmax(c, 0.0f), f0) : black;
        }
        case DBG_BRDF: return hit ? v3(f.brdfIntensity) : black;
        case DBG_PDF: return hit ? v3(f.pdf) : black;
        case DBG_REFLECTED: return w.path.size() > 1 ? w.path[1].rayD * 0.5f + v3(0.5f) : black;
        default: return total;
    }
}

// Heatmap, Tracer.cpp:650-670 (glm::mix(a, b, f) = a * (1 - f) + b * f)
V3 heatmap(float t)
{
    t = gclamp(t, 0.0f, 1.0f);
    static const V3 colors[5] = {{0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0}};
    const float x = t * 4.0f;
    const int i = std::min(static_cast<int>(x), 3);
    const float fr = x - static_cast<float>(i);
    const float r = 1.0f - fr;
    const V3 a = colors[i], b = colors[i + 1];
    return {a.x * r + b.x * fr, a.y * r + b.y * fr, a.z * r + b.z * fr};
}

// ApplyDebugPostProcessing, Tracer.cpp:695-716: heatmap modes map the image's
// intensity (r+g+b)/3, divided by its maximum, to a colour ramp or to grey.
void debug_postprocess(float* rgb, uint32_t W, uint32_t H, int mode)
{
    bool colorful;
    switch (mode) {
        case DBG_PRIMARY_BVH: case DBG_TOTAL_BVH: case DBG_PRIMARY_TRI: case DBG_TOTAL_TRI:
        case DBG_BOUNCES: case DBG_FIREFLY: colorful = true; break;
        case DBG_DEPTH: case DBG_BRDF: case DBG_PIXEL_STDDEV: colorful = false; break;
        default: return;
    }
    const size_t n = static_cast<size_t>(W) * H;
    float maxI = 0.0f;
    for (size_t i = 0; i < n; ++i) {
        const float in = ((rgb[3 * i] + rgb[3 * i + 1]) + rgb[3 * i + 2]) / 3.0f;
        maxI = std::max(maxI, in);
    }
    for (size_t i = 0; i < n; ++i) {
        const float in = ((rgb[3 * i] + rgb[3 * i + 1]) + rgb[3 * i + 2]) / 3.0f;
        const float t = maxI > 0.0f ? in / maxI : 0.0f;
        const V3 c = colorful ? heatmap(t) : v3(t);
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
    }
}

// CleanupFireflies (Tracer.cpp:490-548) + average (Tracer.cpp:593-600).
// The two debug modes that read the clamp's own statistics replace every
// sample and divide by the sample count (CleanupFireflies returns
// buffer.size() for them): DebugPixelStandardDeviation writes sqrt of the
// population variance of the intensities (Tracer.cpp:516-523), computed before
// any sample is dropped; DebugFireflyElimination writes the number of samples
// the threshold dropped (Tracer.cpp:537-544).  Without the clamp the reference
// never calls CleanupFireflies, so both modes then average the plain samples.
V3 resolve_pixel(std::vector<V3>& buf, bool enable, float k, int debug_mode)
{
    size_t n = buf.size();
    if (enable) {
        auto inten = [](V3 c) { return (c.x + c.y + c.z) / 3.0f; };
        float sum = 0.0f;
        for (const V3& c : buf) sum = sum + inten(c);
        const float mean = sum / static_cast<float>(buf.size());
        float var = 0.0f;
        for (const V3& c : buf) {
            const float df = inten(c) - mean;
            var = var + df * df;
        }
        var = var / static_cast<float>(buf.size());
        const float sigma = std::sqrt(var);
        if (debug_mode == MT_DEBUG_PIXEL_STANDARD_DEVIATION) {
            for (V3& c : buf) c = v3(sigma);
        } else {
            const float thr = k * sigma;
            for (V3& c : buf) {
                if (std::fabs(inten(c) - mean) > thr) {
                    c = v3(0.0f);
                    --n;
                }
            }
            if (debug_mode == MT_DEBUG_FIREFLY_ELIMINATION) {
                const float dropped = static_cast<float>(buf.size() - n);
                for (V3& c : buf) c = v3(dropped);
                n = buf.size();
            }
        }
        if (n == 0) n = 1;
    }
    V3 acc = v3(0.0f);
    for (const V3& c : buf) acc = acc + c;
    return acc / static_cast<float>(n);
}

// Camera::GeneratePerspectiveRay / GenerateOrthogonalRay, Camera.cpp:17-44
void camera_ray(const Camera& c, float u, float v, float aspect, V3& o, V3& d)
{
    if (c.type == 0) {
        const float fs = std::tan(c.fov * 0.5f);
        const float px = (2.0f * u - 1.0f) * fs * aspect;
        const float py = (2.0f * v - 1.0f) * fs;
        const V4 dc = normalize4(V4{px, -py, -1.0f, 0.0f});
        o = xyz(mul(c.c2w, V4{0, 0, 0, 1}));
        d = normalize(xyz(mul(c.c2w, dc)));
    } else {
        const float px = (2.0f * u - 1.0f) * c.ortho.x * aspect / c.aspect;
        const float py = (2.0f * v - 1.0f) * c.ortho.y;
        o = xyz(mul(c.c2w, V4{px, -py, 0.0f, 1.0f}));
        d = normalize(xyz(mul(c.c2w, V4{0.0f, 0.0f, -1.0f, 0.0f})));
    }
}

// Platform::SetThreadAffinity (src/Platform/Platform.cpp:7-18): core
// coreId modulo the hardware threads; a failure only costs speed.
void pin_thread(std::thread& th, unsigned core)
{
#ifdef __linux__
    const unsigned n = std::max(1u, std::thread::hardware_concurrency());
    cpu_set_t set;
    CPU_ZERO(&set);
    CPU_SET(core % n, &set);
    (void)pthread_setaffinity_np(th.native_handle(), sizeof(cpu_set_t), &set);
#else
    (void)th;
    (void)core;
#endif
}

unsigned hw_threads(int threads)
{
    if (threads > 0) return static_cast<unsigned>(threads);
    const unsigned h = std::thread::hardware_concurrency();
    return h ? h : 1;
}

template <class F>
void parallel_for(uint64_t n, int threads, F&& f)
{
    const unsigned T = hw_threads(threads);
    if (T <= 1 || n < 64) {
        for (uint64_t i = 0; i < n; ++i) f(i, 0u);
        return;
    }
    std::atomic<uint64_t> next{0};
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < T; ++t)
        pool.emplace_back([&, t]() {
            for (;;) {
                const uint64_t b = next.fetch_add(256);
                if (b >= n) break;
                const uint64_t e = std::min<uint64_t>(n, b + 256);
                for (uint64_t i = b; i < e; ++i) f(i, t);
            }
        });
    for (auto& th : pool) th.join();
}

void seed_counter(Rng& rng, const orc_scene& s)
{
    rng.mode = ORC_RNG_COUNTER;
    rng.key[0] = static_cast<uint32_t>(s.cfg.seed);
    rng.key[1] = static_cast<uint32_t>(s.cfg.seed >> 32);
}

// ----------------------------------------------------------------------------
// Adjoint check: derivatives of EvaluateBRDF (BRDF.hpp:52-77) by forward-mode
// dual numbers over (base r, g, b, roughness, metallic).
// ----------------------------------------------------------------------------
struct Dual {
    float v;
    float d[5];
    static Dual c(float x)
    {
        Dual r{x, {0, 0, 0, 0, 0}};
        return r;
    }
    static Dual var(float x, int k)
    {
        Dual r = c(x);
        r.d[k] = 1.0f;
        return r;
    }
};
Dual operator+(const Dual& a, const Dual& b)
{
    Dual r{a.v + b.v, {}};
    for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
Dual operator-(const Dual& a, const Dual& b)
{
    Dual r{a.v - b.v, {}};
    for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
Dual operator*(const Dual& a, const Dual& b)
{
    Dual r{a.v * b.v, {}};
    for (int k = 0; k < 5; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
Dual operator/(const Dual& a, const Dual& b)
{
    Dual r{a.v / b.v, {}};
    for (int k = 0; k < 5; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
    return r;
}

void brdf_grad(V3 L, V3 V, V3 N, V3 base, float rough, float metal, V3 adj, double* g)
{
    const float nl = gmax(dot(N, L), 0.0f), nv = gmax(dot(N, V), 0.0f);
    if (nl <= 0.0f || nv <= 0.0f) return;
    const V3 h = normalize(V + L);
    const float nh = gclamp(gmax(dot(N, h), 0.0f), 0.0f, 1.0f);
    const float hv = gclamp(gmax(dot(h, V), 0.0f), 0.0f, 1.0f);
    const Dual one = Dual::c(1.0f);
    const Dual r = rough < 0.05f ? Dual::c(0.05f) : Dual::var(rough, 3);
    const Dual m = Dual::var(metal, 4);
    const Dual mc = metal < 0.0f ? Dual::c(0.0f) : (metal > 1.0f ? Dual::c(1.0f) : m);
    const Dual p5 = Dual::c(std::pow(1.0f - hv, 5.0f));
    const Dual a = r * r, a2 = a * a;
    const Dual q = Dual::c(nh * nh) * (a2 - one) + one;
    const Dual D = a2 / (Dual::c(kPi) * q * q);
    const Dual rr = r + one;
    const Dual k = rr * rr / Dual::c(8.0f);
    const Dual G = (Dual::c(nv) / (Dual::c(nv) * (one - k) + k)) * (Dual::c(nl) / (Dual::c(nl) * (one - k) + k));
    const Dual sden = Dual::c(gmax(4.0f * nv * nl, 0.001f));
    const float b[3] = {base.x, base.y, base.z}, ad[3] = {adj.x, adj.y, adj.z};
    for (int ch = 0; ch < 3; ++ch) {
        const Dual bc = Dual::var(b[ch], ch);
        const Dual f0 = Dual::c(0.04f) * (one - mc) + bc * mc;
        const Dual F = f0 + (one - f0) * p5;
        const Dual f = (one - F) * (one - m) * bc / Dual::c(kPi) + D * G * F / sden;
        if (f.v < 0.0f) continue;
        for (int kk = 0; kk < 5; ++kk) g[kk] += static_cast<double>(ad[ch]) * f.d[kk];
    }
}

// Texel indices and weights Image::Sample blends (Image.cpp:17-61).
int texel_taps(const Texture& t, float uvx, float uvy, long long idx[4], float w[4])
{
    const float u = uvx - std::floor(uvx), v = uvy - std::floor(uvy);
    const int W = static_cast<int>(t.w), H = static_cast<int>(t.h);
    const long long maxIdx = static_cast<long long>(t.w) * t.h - 1;
    auto at = [&](int x, int y) {
        const long long i = static_cast<long long>(y) * t.w + x;
        return i < 0 ? 0 : (i > maxIdx ? maxIdx : i);
    };
    if (t.filter == MT_FILTER_LINEAR) {
        const int x0 = static_cast<int>(std::floor(u * static_cast<float>(W)));
        const int x1 = std::min(x0 + 1, W - 1);
        const int y0 = static_cast<int>(std::floor(v * static_cast<float>(H)));
        const int y1 = std::min(y0 + 1, H - 1);
        const float sx = u - static_cast<float>(x0) / static_cast<float>(W);
        const float sy = v - static_cast<float>(y0) / static_cast<float>(H);
        idx[0] = at(x0, y0), w[0] = (1 - sx) * (1 - sy);
        idx[1] = at(x1, y0), w[1] = sx * (1 - sy);
        idx[2] = at(x0, y1), w[2] = (1 - sx) * sy;
        idx[3] = at(x1, y1), w[3] = sx * sy;
        return 4;
    }
    int ix = static_cast<int>(u * static_cast<float>(W)) % W;
    int iy = static_cast<int>(v * static_cast<float>(H)) % H;
    if (ix < 0) ix += W;
    if (iy < 0) iy += H;
    idx[0] = at(ix, iy);
    w[0] = 1.0f;
    return 1;
}

float aces_slope(float x)
{
    const double a = 2.51, b = 0.03, c = 2.43, d = 0.59, e = 0.14, X = x;
    const double n = X * (a * X + b), dn = X * (c * X + d) + e;
    return static_cast<float>(((2 * a * X + b) * dn - n * (2 * c * X + d)) / (dn * dn));
}

struct GradAcc {
    std::vector<double> mat;  // materials * 5
    std::vector<double> light;
    std::vector<double> texel;
    double loss = 0.0;
};

// Replays one kept sample's recorded path backwards (adjoint of
// ProcessRayForward with the path's decisions held fixed).
void sample_backward(const orc_scene& s, const std::vector<PathStep>& path, V3 gv,
                     const std::vector<long long>& texOff, GradAcc& acc)
{
    size_t nv = 0;
    while (nv < path.size() && path[nv].didHit) ++nv;
    const bool miss = nv < path.size();
    std::vector<V3> cur(nv + 1, v3(1.0f));
    for (size_t i = 0; i < nv; ++i) cur[i + 1] = path[i].chosen ? cur[i] * path[i].energy : cur[i];
    V3 adj = v3(0.0f), adjBaseSky = v3(0.0f);
    if (miss && nv > 0) {
        adj = gv * path[nv - 1].base * path[nv].sky;
        adjBaseSky = gv * cur[nv] * path[nv].sky;
    }
    for (size_t ii = nv; ii-- > 0;) {
        const PathStep& st = path[ii];
        double g[5] = {0, 0, 0, 0, 0};
        if (ii + 1 == nv) {
            g[0] += adjBaseSky.x;
            g[1] += adjBaseSky.y;
            g[2] += adjBaseSky.z;
        }
        const V3 adjNext = adj;
        const V3 V = -st.rayD;
        if (st.chosen) {
            adj = adjNext * st.energy;
            brdf_grad(st.nextDir, V, st.normal, st.base, st.roughness, st.metallic,
                      adjNext * cur[ii] * st.facNext, g);
        }
        adj = adj + gv * s.cfg.emission_base_intensity * st.emission;
        if (st.chosen && st.visible) {
            const Light& L = s.lights[st.light];
            const V3 lc = L.color * (st.spot * st.facLight);
            const V3 fl = eval_brdf(st.ldir, V, st.normal, st.base, st.roughness, st.metallic);
            adj = adj + gv * fl * lc;
            brdf_grad(st.ldir, V, st.normal, st.base, st.roughness, st.metallic, gv * cur[ii] * lc, g);
            const V3 c = cur[ii] * fl * lc;
            acc.light[st.light] += static_cast<double>(gv.x) * c.x + static_cast<double>(gv.y) * c.y +
                                   static_cast<double>(gv.z) * c.z;
        }
        const Material& M = s.materials[st.mat];
        V3 tb = v3(1.0f);
        float tr = 1.0f, tm = 1.0f;
        if (M.baseTex >= 0) {
            const V4 t = tex_sample(s, M.baseTex, st.uv);
            tb = {t.x, t.y, t.z};
        }
        if (M.mrTex >= 0) {
            const V4 t = tex_sample(s, M.mrTex, st.uv);
            tr = t.y;
            tm = t.z;
        }
        double* dm = &acc.mat[5 * st.mat];
        dm[0] += g[0] * 0.96 * tb.x;
        dm[1] += g[1] * 0.96 * tb.y;
        dm[2] += g[2] * 0.96 * tb.z;
        dm[3] += g[3] * tr;
        dm[4] += g[4] * tm;
        if (M.baseTex >= 0 && texOff[M.baseTex] >= 0) {
            const Texture& t = s.textures[M.baseTex];
            long long idx[4];
            float w[4];
            const int n = texel_taps(t, st.uv.x * t.scale.x + t.offset.x, st.uv.y * t.scale.y + t.offset.y, idx, w);
            double* dt = &acc.texel[texOff[M.baseTex]];
            for (int q = 0; q < n; ++q) {
                dt[3 * idx[q]] += g[0] * 0.96 * M.baseFactor.x * w[q];
                dt[3 * idx[q] + 1] += g[1] * 0.96 * M.baseFactor.y * w[q];
                dt[3 * idx[q] + 2] += g[2] * 0.96 * M.baseFactor.z * w[q];
            }
        }
    }
}

}  // namespace

// ============================================================================
// C API
// ============================================================================
extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

void orc_free(void* p) { std::free(p); }

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    philox4x32_10(ctr, key, out);
}

int orc_bvh_build(const float* positions, uint32_t T, uint32_t max_triangles, uint32_t max_depth,
                  mt_bvh_node** nodes, uint32_t* num_nodes, uint32_t** indices,
                  uint32_t* num_indices)
{
    if (!positions || !nodes || !num_nodes || !indices || !num_indices) return fail("null arg");
    FlatBVH f;
    const int rc = build_bvh(reinterpret_cast<const V3*>(positions), T, max_triangles, max_depth, f);
    if (rc != MT_OK) return rc;
    *nodes = static_cast<mt_bvh_node*>(std::malloc(f.nodes.size() * sizeof(mt_bvh_node)));
    *indices = static_cast<uint32_t*>(std::malloc(std::max<size_t>(1, f.indices.size()) * 4));
    if (!*nodes || !*indices) return fail("oom", MT_ERR_OOM);
    std::memcpy(*nodes, f.nodes.data(), f.nodes.size() * sizeof(mt_bvh_node));
    std::memcpy(*indices, f.indices.data(), f.indices.size() * 4);
    *num_nodes = static_cast<uint32_t>(f.nodes.size());
    *num_indices = static_cast<uint32_t>(f.indices.size());
    return MT_OK;
}

int orc_scene_create(const mt_scene_desc* d, const mt_config* cfg, orc_scene** out)
{
    if (!d || !cfg || !out) return fail("null arg");
    *out = nullptr;
    auto s = std::make_unique<orc_scene>();
    s->cfg = *cfg;
    for (uint32_t i = 0; i < d->num_textures; ++i) {
        const mt_texture_desc& t = d->textures[i];
        Texture x;
        x.w = t.width;
        x.h = t.height;
        x.filter = t.filter;
        x.offset = {t.offset[0], t.offset[1]};
        x.scale = {t.scale[0], t.scale[1]};
        const size_t n = static_cast<size_t>(t.width) * t.height * 3;
        if (n == 0 || (!t.rgb8 && !t.rgb32f)) return fail("texture without texels");
        if (t.rgb32f)
            x.rgbf.assign(t.rgb32f, t.rgb32f + n);
        else
            x.rgb8.assign(t.rgb8, t.rgb8 + n);
        s->textures.push_back(std::move(x));
    }
    for (uint32_t i = 0; i < d->num_meshes; ++i) {
        const mt_mesh_desc& md = d->meshes[i];
        Mesh m;
        const size_t nv = static_cast<size_t>(md.num_triangles) * 3;
        if (!md.positions || !md.normals || md.num_triangles == 0)
            return fail("mesh needs positions and normals");
        m.pos.resize(nv);
        m.nrm.resize(nv);
        std::memcpy(m.pos.data(), md.positions, nv * 12);
        std::memcpy(m.nrm.data(), md.normals, nv * 12);
        if (md.uv0) {
            m.uv0.resize(nv);
            std::memcpy(m.uv0.data(), md.uv0, nv * 8);
        }
        m.lo = v3(std::numeric_limits<float>::max());
        m.hi = v3(std::numeric_limits<float>::lowest());
        for (const V3& p : m.pos) {
            m.lo = vmin(m.lo, p);
            m.hi = vmax(m.hi, p);
        }
        const bool want = !cfg->bvh_disable && md.num_triangles > cfg->bvh_max_triangles;
        if (want) {
            if (md.bvh_nodes && md.bvh_indices) {
                m.bvh.nodes.assign(md.bvh_nodes, md.bvh_nodes + md.num_bvh_nodes);
                m.bvh.indices.assign(md.bvh_indices, md.bvh_indices + md.num_bvh_indices);
            } else {
                const int rc = build_bvh(m.pos.data(), md.num_triangles, cfg->bvh_max_triangles,
                                         cfg->bvh_max_depth, m.bvh);
                if (rc != MT_OK) return rc;
            }
            m.hasBVH = true;
        }
        s->meshes.push_back(std::move(m));
    }
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const mt_material_desc& m = d->materials[i];
        Material x;
        x.baseFactor = {m.base_color_factor[0], m.base_color_factor[1], m.base_color_factor[2],
                        m.base_color_factor[3]};
        x.emissive = {m.emissive_factor[0], m.emissive_factor[1], m.emissive_factor[2]};
        x.normalScale = m.normal_scale;
        x.metallic = m.metallic_factor;
        x.roughness = m.roughness_factor;
        x.baseTex = m.base_color_tex;
        x.mrTex = m.metallic_roughness_tex;
        x.nrmTex = m.normal_tex;
        x.emTex = m.emissive_tex;
        for (int ti : {x.baseTex, x.mrTex, x.nrmTex, x.emTex})
            if (ti >= static_cast<int>(d->num_textures)) return fail("texture index out of range");
        s->materials.push_back(x);
    }
    for (uint32_t i = 0; i < d->num_instances; ++i) {
        const mt_instance_desc& id = d->instances[i];
        if (id.mesh >= d->num_meshes || id.material >= d->num_materials)
            return fail("instance references a missing mesh or material");
        Instance in;
        in.mesh = id.mesh;
        in.material = id.material;
        std::memcpy(in.model.m, id.transform, 64);
        in.inv = inverse4(in.model);
        // MeshInstance::CalculateWorldAABB, Mesh.cpp:56-80
        const Mesh& m = s->meshes[id.mesh];
        const V3 a = m.lo, b = m.hi;
        const V3 corners[8] = {{a.x, a.y, a.z}, {a.x, a.y, b.z}, {a.x, b.y, a.z}, {a.x, b.y, b.z},
                               {b.x, a.y, a.z}, {b.x, a.y, b.z}, {b.x, b.y, a.z}, {b.x, b.y, b.z}};
        in.wlo = v3(std::numeric_limits<float>::max());
        in.whi = v3(std::numeric_limits<float>::lowest());
        for (const V3& c : corners) {
            const V3 w = xyz(mul(in.model, V4{c.x, c.y, c.z, 1.0f}));
            in.wlo = vmin(in.wlo, w);
            in.whi = vmax(in.whi, w);
        }
        s->instances.push_back(in);
    }
    for (uint32_t i = 0; i < d->num_lights; ++i) {
        const mt_light_desc& l = d->lights[i];
        Light x;
        x.type = l.type;
        x.pos = {l.position[0], l.position[1], l.position[2]};
        x.color = {l.color[0], l.color[1], l.color[2]};
        x.dir = {l.direction[0], l.direction[1], l.direction[2]};
        x.pointSize = l.point_size;
        x.innerCos = l.spot_inner_cos;
        x.outerCos = l.spot_outer_cos;
        x.simpleIntensity = (x.color.x + x.color.y + x.color.z) / 3.0f;
        s->lights.push_back(x);
    }
    s->cam.type = d->camera.type;
    std::memcpy(s->cam.c2w.m, d->camera.camera_to_world, 64);
    s->cam.fov = d->camera.yfov;
    s->cam.aspect = d->camera.aspect;
    s->cam.ortho = {d->camera.ortho_size[0], d->camera.ortho_size[1]};
    s->env = d->env_texture;
    if (s->env >= static_cast<int>(d->num_textures)) return fail("env texture out of range");
    *out = s.release();
    return MT_OK;
}

void orc_scene_destroy(orc_scene* s) { delete s; }

int orc_scene_mesh_bvh(const orc_scene* s, uint32_t mesh, const mt_bvh_node** nodes,
                       uint32_t* num_nodes, const uint32_t** indices, uint32_t* num_indices)
{
    if (!s || mesh >= s->meshes.size()) return fail("bad mesh");
    const Mesh& m = s->meshes[mesh];
    *nodes = m.hasBVH ? m.bvh.nodes.data() : nullptr;
    *num_nodes = m.hasBVH ? static_cast<uint32_t>(m.bvh.nodes.size()) : 0;
    *indices = m.hasBVH ? m.bvh.indices.data() : nullptr;
    *num_indices = m.hasBVH ? static_cast<uint32_t>(m.bvh.indices.size()) : 0;
    return MT_OK;
}

int orc_trace_rays(const orc_scene* s, const mt_ray* rays, uint64_t n, mt_hit* hits, int query,
                   uint32_t* totals, int threads)
{
    if (!s || (!rays && n) || (!hits && n)) return fail("null arg");
    const unsigned T = hw_threads(threads);
    std::vector<std::vector<StackEntry>> stacks(T);
    parallel_for(n, threads, [&](uint64_t i, unsigned t) {
        const mt_ray& r = rays[i];
        const V3 o{r.origin[0], r.origin[1], r.origin[2]};
        const V3 d{r.direction[0], r.direction[1], r.direction[2]};
        uint32_t tb = 0, tt = 0, ti = 0;
        const Hit h = intersect_scene(*s, o, d, stacks[t], &tb, &tt, &ti);
        mt_hit& o_ = hits[i];
        if (query == MT_QUERY_ANY) {
            std::memset(&o_, 0, sizeof(o_));
            o_.instance = (h.hit && !(h.dist > r.tmax)) ? 1u : 0u;
            o_.distance = h.hit ? h.dist : 0.0f;
        } else if (!h.hit) {
            std::memset(&o_, 0, sizeof(o_));
            o_.instance = MT_NO_HIT;
        } else {
            o_.distance = h.dist;
            o_.u = h.u;
            o_.v = h.v;
            o_.instance = h.inst;
            o_.triangle = h.tri;
            o_.bv_index = h.bv;
            o_.bvh_tests = query == MT_QUERY_CLOSEST_COUNT ? h.bvhTests : 0;
            o_.tri_tests = query == MT_QUERY_CLOSEST_COUNT ? h.triTests : 0;
        }
        if (totals) {
            totals[3 * i] = tb;
            totals[3 * i + 1] = ti;
            totals[3 * i + 2] = tt;
        }
    });
    return MT_OK;
}

int orc_trace_f64(const orc_scene* s, const mt_ray* rays, const mt_hit* hits, uint64_t n,
                  double* out)
{
    for (uint64_t i = 0; i < n; ++i) {
        double* r = out + 3 * i;
        if (hits[i].instance == MT_NO_HIT || hits[i].instance >= s->instances.size()) {
            r[0] = r[1] = r[2] = std::nan("");
            continue;
        }
        const Instance& in = s->instances[hits[i].instance];
        const Mesh& m = s->meshes[in.mesh];
        const double o[3] = {rays[i].origin[0], rays[i].origin[1], rays[i].origin[2]};
        const double dw[3] = {rays[i].direction[0], rays[i].direction[1], rays[i].direction[2]};
        const float* A = in.inv.m;
        double lo[3], ld[3];
        for (int k = 0; k < 3; ++k) {
            lo[k] = A[k] * o[0] + A[4 + k] * o[1] + A[8 + k] * o[2] + A[12 + k];
            ld[k] = A[k] * dw[0] + A[4 + k] * dw[1] + A[8 + k] * dw[2];
        }
        const double ln = std::sqrt(ld[0] * ld[0] + ld[1] * ld[1] + ld[2] * ld[2]);
        for (double& x : ld) x /= ln;
        const V3 a = m.pos[hits[i].triangle * 3], b = m.pos[hits[i].triangle * 3 + 1],
                 c = m.pos[hits[i].triangle * 3 + 2];
        const double v0[3] = {a.x, a.y, a.z};
        const double e1[3] = {(double)b.x - a.x, (double)b.y - a.y, (double)b.z - a.z};
        const double e2[3] = {(double)c.x - a.x, (double)c.y - a.y, (double)c.z - a.z};
        auto crs = [](const double* p, const double* q, double* r_) {
            r_[0] = p[1] * q[2] - p[2] * q[1];
            r_[1] = p[2] * q[0] - p[0] * q[2];
            r_[2] = p[0] * q[1] - p[1] * q[0];
        };
        auto dt = [](const double* p, const double* q) { return p[0] * q[0] + p[1] * q[1] + p[2] * q[2]; };
        double p[3], q[3], sv[3];
        crs(ld, e2, p);
        const double det = dt(e1, p);
        for (int k = 0; k < 3; ++k) sv[k] = lo[k] - v0[k];
        crs(sv, e1, q);
        const double u = dt(sv, p) / det, v = dt(ld, q) / det, t = dt(e2, q) / det;
        double lp[3], wp[3];
        for (int k = 0; k < 3; ++k) lp[k] = lo[k] + t * ld[k];
        const float* M = in.model.m;
        for (int k = 0; k < 3; ++k) wp[k] = M[k] * lp[0] + M[4 + k] * lp[1] + M[8 + k] * lp[2] + M[12 + k];
        const double dx = wp[0] - o[0], dy = wp[1] - o[1], dz = wp[2] - o[2];
        r[0] = std::sqrt(dx * dx + dy * dy + dz * dz);
        r[1] = u;
        r[2] = v;
    }
    return MT_OK;
}

// GeneratePath's bounce sampling (Tracer.cpp:177-203) with explicit uniforms.
int orc_brdf_sample(const mt_brdf_sample_query* q, uint64_t n, mt_brdf_sample_result* out)
{
    if (!q || !out) return fail("null arg");
    for (uint64_t i = 0; i < n; ++i) {
        const mt_brdf_sample_query& x = q[i];
        const V3 V{x.V[0], x.V[1], x.V[2]}, N{x.N[0], x.N[1], x.N[2]};
        const V3 B{x.base_color[0], x.base_color[1], x.base_color[2]};
        const float ps = specular_probability(V, N, B, x.metallic);
        V3 nd;
        int lobe = 0;
        if (x.u[0] < ps) {
            lobe = 1;
            if (!ggx_reflection(-V, N, x.roughness, x.u[1], x.u[2], nd)) {
                lobe = 2;
                nd = cosine_hemisphere(x.u[3], x.u[4], N);
            }
        } else {
            nd = cosine_hemisphere(x.u[1], x.u[2], N);
        }
        mt_brdf_sample_result& r = out[i];
        r.L[0] = nd.x;
        r.L[1] = nd.y;
        r.L[2] = nd.z;
        r.pdf = (1.0f - ps) * diffuse_pdf(nd, N) + ps * specular_pdf(nd, V, N, x.roughness);
        r.specular_probability = ps;
        r.lobe = lobe;
    }
    return MT_OK;
}

int orc_brdf_batch(const mt_brdf_query* q, uint64_t n, mt_brdf_result* out)
{
    for (uint64_t i = 0; i < n; ++i) {
        const mt_brdf_query& x = q[i];
        const V3 L{x.L[0], x.L[1], x.L[2]}, V{x.V[0], x.V[1], x.V[2]}, N{x.N[0], x.N[1], x.N[2]};
        const V3 B{x.base_color[0], x.base_color[1], x.base_color[2]};
        const V3 f = eval_brdf(L, V, N, B, x.roughness, x.metallic);
        out[i].f[0] = f.x;
        out[i].f[1] = f.y;
        out[i].f[2] = f.z;
        out[i].diffuse_pdf = diffuse_pdf(L, N);
        out[i].specular_pdf = specular_pdf(L, V, N, x.roughness);
    }
    return MT_OK;
}

int orc_camera_rays(const orc_scene* s, const float* uv, uint64_t n, mt_ray* out)
{
    const float aspect = static_cast<float>(s->cfg.width) / static_cast<float>(s->cfg.height);
    for (uint64_t i = 0; i < n; ++i) {
        V3 o, d;
        camera_ray(s->cam, uv[2 * i], uv[2 * i + 1], aspect, o, d);
        out[i] = mt_ray{{o.x, o.y, o.z}, std::numeric_limits<float>::max(), {d.x, d.y, d.z}, 0.0f};
    }
    return MT_OK;
}

void orc_aces(const float in_rgb[3], float expo, float out_rgb[3])
{
    const V3 r = aces(V3{in_rgb[0], in_rgb[1], in_rgb[2]}, expo);
    out_rgb[0] = r.x;
    out_rgb[1] = r.y;
    out_rgb[2] = r.z;
}

int orc_resolve_pixel(const float* samples_rgb, uint32_t n, int firefly_enable, float k,
                      int debug_mode, float out_rgb[3])
{
    if (n == 0) return fail("no samples");
    std::vector<V3> buf(n);
    std::memcpy(buf.data(), samples_rgb, static_cast<size_t>(n) * 12);
    const V3 r = resolve_pixel(buf, firefly_enable != 0, k, debug_mode);
    out_rgb[0] = r.x;
    out_rgb[1] = r.y;
    out_rgb[2] = r.z;
    return MT_OK;
}

// Tracer::StartRender tile queue (Tracer.cpp:718-779) + RenderBlock
// (Tracer.cpp:550-616), over the tiles that meet rows [row0, row1).
int orc_render(const orc_scene* s, int rng_mode, int threads, uint32_t row0, uint32_t row1,
               float* rgb_out, uint64_t* rays_out, uint64_t* samples_out)
{
    if (!s || !rgb_out) return fail("null arg");
    const mt_config& cfg = s->cfg;
    const uint32_t W = cfg.width, H = cfg.height, B = 32;
    row1 = std::min(row1, H);
    if (row0 >= row1) return fail("empty row range");
    struct Block {
        uint32_t x, y, w, h, id;
    };
    std::vector<Block> blocks;
    uint32_t id = 0;
    for (uint32_t y = 0; y < H; y += B)
        for (uint32_t x = 0; x < W; x += B, ++id) {
            const uint32_t y0 = std::max(y, row0), y1 = std::min(std::min(y + B, H), row1);
            if (y0 >= y1) continue;
            blocks.push_back({x, y0, std::min(B, W - x), y1 - y0, id});
        }
    const float aspect = static_cast<float>(W) / static_cast<float>(H);
    const float pxW = 1.0f / static_cast<float>(W), pxH = 1.0f / static_cast<float>(H);
    const float expo = std::pow(2.0f, -cfg.ev_exposure);
    std::atomic<size_t> next{0};
    std::atomic<uint64_t> rays{0}, samples{0};
    auto work = [&]() {
        Worker w;
        std::vector<V3> sampleBuf;
        for (;;) {
            const size_t bi = next.fetch_add(1);
            if (bi >= blocks.size()) break;
            const Block& b = blocks[bi];
            Rng rng;
            if (rng_mode == ORC_RNG_MT19937) {
                rng.mode = ORC_RNG_MT19937;
                rng.gen.seed(static_cast<uint32_t>(cfg.seed + b.id));
            } else {
                seed_counter(rng, *s);
            }
            uint64_t localSamples = 0;
            for (uint32_t y = b.y; y < b.y + b.h; ++y)
                for (uint32_t x = b.x; x < b.x + b.w; ++x) {
                    sampleBuf.clear();
                    const float bu = static_cast<float>(x) * pxW;
                    const float bv = static_cast<float>(y) * pxH;
                    rng.pixel = y * W + x;
                    for (uint32_t sm = 0; sm < cfg.samples; ++sm) {
                        rng.sample = sm;
                        const float u = bu + rng.uniform(0.0f, pxW, 0, SLOT_JITTER, 0);
                        const float v = bv + rng.uniform(0.0f, pxH, 0, SLOT_JITTER, 1);
                        V3 o, d;
                        camera_ray(s->cam, u, v, aspect, o, d);
                        sampleBuf.push_back(cfg.debug_mode
                                                ? process_debug_ray(*s, w, rng, o, d, expo, cfg.debug_mode)
                                                : process_ray_forward(*s, w, rng, o, d, expo));
                        ++localSamples;
                    }
                    const V3 c = resolve_pixel(sampleBuf, cfg.firefly_enable != 0,
                                               cfg.firefly_threshold, cfg.debug_mode);
                    float* px = rgb_out + (static_cast<size_t>(y) * W + x) * 3;
                    px[0] = c.x;
                    px[1] = c.y;
                    px[2] = c.z;
                }
            rays += w.rays;
            w.rays = 0;
            samples += localSamples;
        }
    };
    const unsigned T = hw_threads(threads);
    std::vector<std::thread> pool;
    // Tracer::StartRender pins worker i to core i * (cores / workers) when the
    // workers fit the cores (Tracer.cpp:755-775)
    const unsigned cores = std::max(1u, std::thread::hardware_concurrency());
    for (unsigned t = 0; t < T; ++t) {
        pool.emplace_back(work);
        if (T <= cores) pin_thread(pool.back(), t * (cores / T));
    }
    for (auto& th : pool) th.join();
    if (rays_out) *rays_out = rays.load();
    if (samples_out) *samples_out = samples.load();
    // WaitForRender's post-processing needs the whole image
    if (cfg.debug_mode && row0 == 0 && row1 == H) debug_postprocess(rgb_out, W, H, cfg.debug_mode);
    return MT_OK;
}

int orc_render_samples(const orc_scene* s, int threads, uint32_t row0, uint32_t row1, float* out)
{
    if (!s || !out) return fail("null arg");
    const mt_config& cfg = s->cfg;
    const uint32_t W = cfg.width, H = cfg.height;
    row1 = std::min(row1, H);
    if (row0 >= row1) return fail("empty row range");
    const uint32_t rows = row1 - row0;
    const float aspect = static_cast<float>(W) / static_cast<float>(H);
    const float pxW = 1.0f / static_cast<float>(W), pxH = 1.0f / static_cast<float>(H);
    const float expo = std::pow(2.0f, -cfg.ev_exposure);
    const uint64_t npix = static_cast<uint64_t>(rows) * W;
    const unsigned T = hw_threads(threads);
    std::vector<Worker> workers(T);
    parallel_for(npix, threads, [&](uint64_t p, unsigned t) {
        const uint32_t y = row0 + static_cast<uint32_t>(p / W), x = static_cast<uint32_t>(p % W);
        Rng rng;
        seed_counter(rng, *s);
        rng.pixel = y * W + x;
        for (uint32_t sm = 0; sm < cfg.samples; ++sm) {
            rng.sample = sm;
            const float u = static_cast<float>(x) * pxW + rng.uniform(0.0f, pxW, 0, SLOT_JITTER, 0);
            const float v = static_cast<float>(y) * pxH + rng.uniform(0.0f, pxH, 0, SLOT_JITTER, 1);
            V3 o, d;
            camera_ray(s->cam, u, v, aspect, o, d);
            const V3 c = process_ray_forward(*s, workers[t], rng, o, d, expo);
            float* dst = out + ((static_cast<uint64_t>(sm) * rows + (y - row0)) * W + x) * 3;
            dst[0] = c.x;
            dst[1] = c.y;
            dst[2] = c.z;
        }
    });
    return MT_OK;
}

int orc_render_grad(const orc_scene* s, const float* target, float* image, float* loss, float* d_base,
                    float* d_rough, float* d_metal, float* d_light, float* d_texels, int threads)
{
    if (!s || !target || !image || !loss || !d_base || !d_rough || !d_metal) return fail("null arg");
    const mt_config& cfg = s->cfg;
    const uint32_t W = cfg.width, H = cfg.height, S = cfg.samples;
    const float aspect = static_cast<float>(W) / static_cast<float>(H);
    const float pxW = 1.0f / static_cast<float>(W), pxH = 1.0f / static_cast<float>(H);
    const float expo = std::pow(2.0f, -cfg.ev_exposure);
    // RGB32F textures used as a base colour, in texture order
    std::vector<long long> texOff(s->textures.size(), -1);
    std::vector<char> used(s->textures.size(), 0);
    for (const Material& m : s->materials)
        if (m.baseTex >= 0) used[m.baseTex] = 1;
    long long ntex = 0;
    for (size_t i = 0; i < s->textures.size(); ++i)
        if (used[i] && !s->textures[i].rgbf.empty()) {
            texOff[i] = ntex;
            ntex += 3ll * s->textures[i].w * s->textures[i].h;
        }
    const unsigned T = hw_threads(threads);
    std::vector<GradAcc> acc(T);
    for (GradAcc& a : acc) {
        a.mat.assign(5 * s->materials.size(), 0.0);
        a.light.assign(s->lights.size(), 0.0);
        a.texel.assign(static_cast<size_t>(ntex), 0.0);
    }
    std::vector<Worker> workers(T);
    parallel_for(static_cast<uint64_t>(W) * H, threads, [&](uint64_t p, unsigned t) {
        const uint32_t y = static_cast<uint32_t>(p / W), x = static_cast<uint32_t>(p % W);
        Worker& w = workers[t];
        Rng rng;
        seed_counter(rng, *s);
        rng.pixel = y * W + x;
        std::vector<std::vector<PathStep>> paths(S);
        std::vector<V3> vals(S), totals(S);
        for (uint32_t sm = 0; sm < S; ++sm) {
            rng.sample = sm;
            const float u = static_cast<float>(x) * pxW + rng.uniform(0.0f, pxW, 0, SLOT_JITTER, 0);
            const float v = static_cast<float>(y) * pxH + rng.uniform(0.0f, pxH, 0, SLOT_JITTER, 1);
            V3 o, d;
            camera_ray(s->cam, u, v, aspect, o, d);
            vals[sm] = process_ray_forward(*s, w, rng, o, d, expo, &totals[sm]);
            paths[sm] = w.path;
        }
        std::vector<V3> buf = vals;
        const V3 img = resolve_pixel(buf, cfg.firefly_enable != 0, cfg.firefly_threshold, MT_DEBUG_NONE);
        float* ip = image + 3 * p;
        ip[0] = img.x, ip[1] = img.y, ip[2] = img.z;
        const V3 r{img.x - target[3 * p], img.y - target[3 * p + 1], img.z - target[3 * p + 2]};
        acc[t].loss += static_cast<double>(r.x) * r.x + static_cast<double>(r.y) * r.y +
                       static_cast<double>(r.z) * r.z;
        // firefly mask (CleanupFireflies, Tracer.cpp:490-548)
        auto inten = [](V3 c) { return (c.x + c.y + c.z) / 3.0f; };
        float mean = 0.0f, thr = std::numeric_limits<float>::max();
        uint32_t kept = S;
        if (cfg.firefly_enable) {
            float sum = 0.0f;
            for (const V3& c : vals) sum = sum + inten(c);
            mean = sum / static_cast<float>(S);
            float var = 0.0f;
            for (const V3& c : vals) {
                const float df = inten(c) - mean;
                var = var + df * df;
            }
            var = var / static_cast<float>(S);
            thr = cfg.firefly_threshold * std::sqrt(var);
            for (const V3& c : vals)
                if (std::fabs(inten(c) - mean) > thr) --kept;
            if (kept == 0) kept = 1;
        }
        const float scale = 2.0f / static_cast<float>(kept);
        for (uint32_t sm = 0; sm < S; ++sm) {
            if (cfg.firefly_enable && std::fabs(inten(vals[sm]) - mean) > thr) continue;
            const V3 tt = totals[sm];
            const V3 gv{r.x * scale * aces_slope(tt.x * expo) * expo, r.y * scale * aces_slope(tt.y * expo) * expo,
                        r.z * scale * aces_slope(tt.z * expo) * expo};
            sample_backward(*s, paths[sm], gv, texOff, acc[t]);
        }
    });
    double L = 0.0;
    for (const GradAcc& a : acc) L += a.loss;
    *loss = static_cast<float>(L);
    for (size_t m = 0; m < s->materials.size(); ++m) {
        double g[5] = {0, 0, 0, 0, 0};
        for (const GradAcc& a : acc)
            for (int k = 0; k < 5; ++k) g[k] += a.mat[5 * m + k];
        d_base[3 * m] += static_cast<float>(g[0]);
        d_base[3 * m + 1] += static_cast<float>(g[1]);
        d_base[3 * m + 2] += static_cast<float>(g[2]);
        d_rough[m] += static_cast<float>(g[3]);
        d_metal[m] += static_cast<float>(g[4]);
    }
    if (d_light)
        for (size_t l = 0; l < s->lights.size(); ++l) {
            double g = 0;
            for (const GradAcc& a : acc) g += a.light[l];
            d_light[l] += static_cast<float>(g);
        }
    if (d_texels)
        for (long long i = 0; i < ntex; ++i) {
            double g = 0;
            for (const GradAcc& a : acc) g += a.texel[static_cast<size_t>(i)];
            d_texels[i] += static_cast<float>(g);
        }
    return MT_OK;
}

}  // extern "C"
