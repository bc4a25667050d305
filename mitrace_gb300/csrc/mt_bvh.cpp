// mt_bvh.cpp - host BVH builder producing the reference's BVH topology.
//
// Same rule as Scene::BVHTreeNode::Subdivide (src/Scene/BVH.cpp:117-195):
// split at the mean of the vertex positions on each axis, send a triangle left
// if its min < split and right if its max >= split (straddlers go to both),
// score (nL + nR) / n (FLT_MAX when one side gets everything), prefer x, then
// y, then z on ties, give each child the parent box clipped at the split
// plane, and stop at <= max_triangles or when the depth budget is used up.
// Flattening follows BVH::Flatten (BVH.cpp:214-272): root at 0, slot 1 unused,
// sibling pairs adjacent, A's subtree before B's.
//
// Differences from the reference that do not change the output: per-triangle
// bounds and vertex sums are computed once instead of at every level; only the
// winning axis' child lists are materialised (the reference builds all three);
// inner nodes drop their index lists once split; large subtrees are built on
// separate threads (each node's sums stay sequential in index order, so every
// float result is the same).
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mitrace_gpu.h"

namespace mt {
namespace {

struct P3 {
    float v[3];
};

inline float fmin_g(float x, float y) { return (y < x) ? y : x; }
inline float fmax_g(float x, float y) { return (x < y) ? y : x; }

struct Node {
    std::vector<uint32_t> tris;
    float lo[3], hi[3];
    std::unique_ptr<Node> a, b;
    bool leaf = true;
};

struct Builder {
    const P3* pos;
    std::vector<P3> tmin, tmax, vsum;
    uint32_t max_tri;
    std::atomic<int> threads{0};
    int thread_cap = 1;

    void prepare(uint32_t T)
    {
        tmin.resize(T);
        tmax.resize(T);
        vsum.resize(T);
        for (uint32_t t = 0; t < T; ++t) {
            const P3 &a = pos[3 * t], &b = pos[3 * t + 1], &c = pos[3 * t + 2];
            for (int k = 0; k < 3; ++k) {
                tmin[t].v[k] = fmin_g(a.v[k], fmin_g(b.v[k], c.v[k]));
                tmax[t].v[k] = fmax_g(a.v[k], fmax_g(b.v[k], c.v[k]));
                vsum[t].v[k] = (a.v[k] + b.v[k]) + c.v[k];
            }
        }
    }

    void subdivide(Node& n, unsigned depth_budget)
    {
        const size_t N = n.tris.size();
        if (N <= static_cast<size_t>(max_tri)) return;
        float sum[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t t : n.tris)
            for (int k = 0; k < 3; ++k) sum[k] = sum[k] + vsum[t].v[k];
        float com[3];
        const float denom = static_cast<float>(N * 3);
        for (int k = 0; k < 3; ++k) com[k] = sum[k] / denom;
        size_t nl[3] = {0, 0, 0}, nr[3] = {0, 0, 0};
        for (uint32_t t : n.tris)
            for (int k = 0; k < 3; ++k) {
                nl[k] += tmin[t].v[k] < com[k];
                nr[k] += tmax[t].v[k] >= com[k];
            }
        const float big = std::numeric_limits<float>::max();
        float score[3];
        for (int k = 0; k < 3; ++k)
            score[k] = (nl[k] == N || nr[k] == N) ? big
                                                  : static_cast<float>(nl[k] + nr[k]) / static_cast<float>(N);
        if (score[0] == big && score[1] == big && score[2] == big) return;
        int ax;
        if (score[0] < score[1] && score[0] < score[2])
            ax = 0;
        else if (score[1] < score[2])
            ax = 1;
        else
            ax = 2;
        n.a = std::make_unique<Node>();
        n.b = std::make_unique<Node>();
        n.a->tris.reserve(nl[ax]);
        n.b->tris.reserve(nr[ax]);
        for (uint32_t t : n.tris) {
            if (tmin[t].v[ax] < com[ax]) n.a->tris.push_back(t);
            if (tmax[t].v[ax] >= com[ax]) n.b->tris.push_back(t);
        }
        std::memcpy(n.a->lo, n.lo, 12);
        std::memcpy(n.a->hi, n.hi, 12);
        std::memcpy(n.b->lo, n.lo, 12);
        std::memcpy(n.b->hi, n.hi, 12);
        n.a->hi[ax] = com[ax];
        n.b->lo[ax] = com[ax];
        n.leaf = false;
        std::vector<uint32_t>().swap(n.tris);
        if (depth_budget == 0) return;
        const size_t big_subtree = 1u << 15;
        bool spawn = false;
        if (n.a->tris.size() > big_subtree && n.b->tris.size() > big_subtree) {
            if (threads.fetch_add(1) < thread_cap)
                spawn = true;
            else
                threads.fetch_sub(1);
        }
        if (spawn) {
            std::thread th([&] { subdivide(*n.a, depth_budget - 1); });
            subdivide(*n.b, depth_budget - 1);
            th.join();
            threads.fetch_sub(1);
        } else {
            subdivide(*n.a, depth_budget - 1);
            subdivide(*n.b, depth_budget - 1);
        }
    }
};

void set_box(mt_bvh_node& d, const Node& n)
{
    std::memcpy(d.lo, n.lo, 12);
    std::memcpy(d.hi, n.hi, 12);
}

void flatten_pair(std::vector<mt_bvh_node>& nodes, std::vector<uint32_t>& idx, const Node& A,
                  const Node& B, uint32_t& ia, uint32_t& ib)
{
    ia = static_cast<uint32_t>(nodes.size());
    ib = ia + 1;
    nodes.push_back(mt_bvh_node{});
    nodes.push_back(mt_bvh_node{});
    set_box(nodes[ia], A);
    set_box(nodes[ib], B);
    const Node* kids[2] = {&A, &B};
    const uint32_t at[2] = {ia, ib};
    for (int k = 0; k < 2; ++k) {
        const Node& n = *kids[k];
        if (n.leaf) {
            nodes[at[k]].a = static_cast<uint32_t>(idx.size()) | MT_BVH_LEAF_BIT;
            nodes[at[k]].b = static_cast<uint32_t>(n.tris.size());
            idx.insert(idx.end(), n.tris.begin(), n.tris.end());
        } else {
            uint32_t ca, cb;
            flatten_pair(nodes, idx, *n.a, *n.b, ca, cb);
            nodes[at[k]].a = ca;
            nodes[at[k]].b = cb;
        }
    }
}

}  // namespace

int build_bvh(const float* positions, uint32_t T, uint32_t max_triangles, uint32_t cfg_max_depth,
              std::vector<mt_bvh_node>& nodes, std::vector<uint32_t>& indices, std::string& err)
{
    if (T == 0) {
        err = "Cannot compute AABB for a BVH node with no triangles.";
        return MT_ERR_INVALID;
    }
    Builder b;
    b.pos = reinterpret_cast<const P3*>(positions);
    b.max_tri = max_triangles;
    const unsigned hw = std::thread::hardware_concurrency();
    b.thread_cap = hw > 1 ? static_cast<int>(hw) - 1 : 0;
    b.prepare(T);
    Node root;
    root.tris.resize(T);
    for (uint32_t i = 0; i < T; ++i) root.tris[i] = i;
    // ComputeAABB (BVH.cpp:29-50)
    for (int k = 0; k < 3; ++k) {
        root.lo[k] = std::numeric_limits<float>::max();
        root.hi[k] = std::numeric_limits<float>::lowest();
    }
    for (uint32_t t = 0; t < T; ++t)
        for (int k = 0; k < 3; ++k) {
            root.lo[k] = fmin_g(root.lo[k], b.tmin[t].v[k]);
            root.hi[k] = fmax_g(root.hi[k], b.tmax[t].v[k]);
        }
    // Mesh.cpp:40 passes bvhMaxDepth - 1, BVH.cpp:211 subtracts 1 again (unsigned).
    const unsigned budget = (cfg_max_depth - 1u) - 1u;
    b.subdivide(root, budget);
    if (root.leaf) {
        err = "BVH root could not be split (the reference flattens null children here, "
              "BVH.cpp:264-265)";
        return MT_ERR_INVALID;
    }
    nodes.clear();
    indices.clear();
    nodes.push_back(mt_bvh_node{});
    nodes.push_back(mt_bvh_node{});
    uint32_t ca, cb;
    flatten_pair(nodes, indices, *root.a, *root.b, ca, cb);
    set_box(nodes[0], root);
    nodes[0].a = ca;
    nodes[0].b = cb;
    return MT_OK;
}

}  // namespace mt
