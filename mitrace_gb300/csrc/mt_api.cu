// mt_api.cu - the C ABI (include/mitrace_gpu.h): scene upload, render
// orchestration and ray queries.  Host code here is compiled with
// -ffp-contract=off so the instance bounds and inverses it precomputes carry
// the same float values as a plain IEEE evaluation.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/mitrace_gpu.h"
#include "mt_device.cuh"
#include "mt_adjoint.h"
#include "mt_internal.h"
#include "mt_kernels.h"
#include "mt_nrc.h"

using namespace mt;

namespace {

thread_local std::string g_err;

mt_status set_err(mt_status code, const std::string& msg)
{
    g_err = msg;
    return code;
}

#define MT_CUDA(call)                                                                             \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            return set_err(e_ == cudaErrorMemoryAllocation ? MT_ERR_OOM : MT_ERR_CUDA,            \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                   \
        }                                                                                         \
    } while (0)

inline float hmin(float x, float y) { return (y < x) ? y : x; }
inline float hmax(float x, float y) { return (x < y) ? y : x; }

// Column-major 4x4 times (x,y,z,w) with GLM's pairing (c0*x + c1*y) + (c2*z + c3*w).
void mat_vec(const float* m, const float v[4], float r[4])
{
    for (int k = 0; k < 4; ++k)
        r[k] = (m[k] * v[0] + m[4 + k] * v[1]) + (m[8 + k] * v[2] + m[12 + k] * v[3]);
}

// 4x4 inverse by cofactor expansion, evaluated once per instance (the
// reference evaluates glm::inverse per ray per instance, Intersect.cpp:151-152;
// the value is ray-independent).
void inverse4(const float* a, float* out)
{
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
    const float s = 1.0f / det;
    for (int i = 0; i < 16; ++i) out[i] = inv[i] * s;
}

// Device blocks released by a handle are kept for the next handle on the same
// device instead of going back to the driver: a render's wavefront state is
// gigabytes (3.4 GB for a 1080p 7-spp image), and cudaFree / cudaMalloc of it
// cost milliseconds per mt_destroy / mt_create.  A request takes the smallest
// cached block of at least its size and at most twice it.  The cache holds at
// most MT_DEVICE_CACHE_BYTES per device (default: an eighth of the device's
// memory; 0 disables it); mt_release_cached_memory gives every cached block
// back.  A block enters the cache only once the device has finished with it
// (mt_destroy synchronizes the device first, as cudaFree would).
struct BlockCache {
    std::mutex mu;
    std::multimap<size_t, void*> free_blocks[64];
    size_t cached[64] = {};
    size_t cap[64] = {};
    bool cap_known[64] = {};
    std::unordered_map<void*, std::pair<int, size_t>> size_of;  // every live or cached block
};
// Set while mt_destroy deletes a handle after synchronizing the device: its
// blocks can enter the cache without another synchronization.
thread_local bool g_device_idle = false;
BlockCache& block_cache()
{
    static BlockCache* c = new BlockCache();  // outlives static destruction at exit
    return *c;
}
// (called with the cache's lock held)
size_t cache_cap(BlockCache& c, int dev)
{
    const char* v = std::getenv("MT_DEVICE_CACHE_BYTES");
    if (v && *v) return static_cast<size_t>(std::strtoull(v, nullptr, 10));
    if (!c.cap_known[dev]) {
        cudaDeviceProp prop{};
        c.cap[dev] = cudaGetDeviceProperties(&prop, dev) == cudaSuccess ? prop.totalGlobalMem / 8 : 0;
        c.cap_known[dev] = true;
    }
    return c.cap[dev];
}

// Every device allocation of a handle goes through here.  Fault injection for
// tests: when MT_DEVICE_ALLOC_LIMIT holds a byte count, a single allocation
// larger than that fails with cudaErrorMemoryAllocation, as if the device were
// out of memory, so the MT_ERR_OOM paths can be exercised without exhausting
// a shared GPU.
cudaError_t dev_malloc(void** p, size_t bytes)
{
    const char* lim = std::getenv("MT_DEVICE_ALLOC_LIMIT");
    if (lim && *lim && bytes > std::strtoull(lim, nullptr, 10)) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaMalloc(p, bytes);
    BlockCache& c = block_cache();
    {
        std::lock_guard<std::mutex> lk(c.mu);
        auto it = c.free_blocks[dev].lower_bound(bytes);
        if (it != c.free_blocks[dev].end() && it->first <= 2 * bytes) {
            *p = it->second;
            c.cached[dev] -= it->first;
            c.free_blocks[dev].erase(it);
            return cudaSuccess;
        }
    }
    e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation) {
        // give the cached blocks back to the driver and try once more
        mt_release_cached_memory();
        (void)cudaGetLastError();
        e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(c.mu);
    c.size_of[*p] = {dev, bytes};
    return cudaSuccess;
}

// Releases a block of dev_malloc: into the cache of its device while that has
// room, else back to the driver.  Work still in flight may use the block, so
// unless the device was just synchronized (mt_destroy) the device is
// synchronized first, as cudaFree does.
void dev_free(void* p)
{
    if (!p) return;
    BlockCache& c = block_cache();
    std::unique_lock<std::mutex> lk(c.mu);
    auto it = c.size_of.find(p);
    if (it == c.size_of.end()) {
        lk.unlock();
        cudaFree(p);
        return;
    }
    const int dev = it->second.first;
    const size_t bytes = it->second.second;
    if (c.cached[dev] + bytes <= cache_cap(c, dev)) {
        if (!g_device_idle) {
            lk.unlock();
            int cur = 0;
            cudaGetDevice(&cur);
            if (cur != dev) cudaSetDevice(dev);
            const cudaError_t e = cudaDeviceSynchronize();
            if (cur != dev) cudaSetDevice(cur);
            lk.lock();
            if (e != cudaSuccess) {  // a faulted context: hand the block back to the driver
                c.size_of.erase(p);
                lk.unlock();
                cudaFree(p);
                return;
            }
        }
        c.free_blocks[dev].emplace(bytes, p);
        c.cached[dev] += bytes;
        return;
    }
    c.size_of.erase(it);
    lk.unlock();
    cudaFree(p);
}

// Pinned host words for the per-render counters, carved from pages allocated
// once (cudaMallocHost / cudaFreeHost per handle cost far more than the
// handle's whole scene upload).
struct PinnedSlots {
    std::mutex mu;
    std::vector<unsigned long long*> free_slots;
};
PinnedSlots& pinned_slots()
{
    static PinnedSlots* s = new PinnedSlots();
    return *s;
}
cudaError_t pinned_slot_alloc(unsigned long long** out)
{
    PinnedSlots& ps = pinned_slots();
    std::lock_guard<std::mutex> lk(ps.mu);
    if (ps.free_slots.empty()) {
        constexpr size_t kSlots = 256, kWords = 4;
        unsigned long long* page = nullptr;
        const cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&page), kSlots * kWords * sizeof(*page));
        if (e != cudaSuccess) return e;
        for (size_t i = 0; i < kSlots; ++i) ps.free_slots.push_back(page + kWords * i);
    }
    *out = ps.free_slots.back();
    ps.free_slots.pop_back();
    return cudaSuccess;
}
void pinned_slot_free(unsigned long long* p)
{
    if (!p) return;
    PinnedSlots& ps = pinned_slots();
    std::lock_guard<std::mutex> lk(ps.mu);
    ps.free_slots.push_back(p);
}

template <class T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    DevArray(DevArray&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    ~DevArray() { reset(); }
    void reset()
    {
        if (p) dev_free(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count)
    {
        reset();
        n = count;
        if (count == 0) return cudaSuccess;
        return dev_malloc(reinterpret_cast<void**>(&p), count * sizeof(T));
    }
    cudaError_t upload(const T* src, size_t count, cudaStream_t st)
    {
        cudaError_t e = alloc(count);
        if (e != cudaSuccess || count == 0) return e;
        return cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, st);
    }
};

// Maximum BVH depth (edges from the root to the deepest leaf) of a flattened BVH.
bool bvh_depth(const std::vector<mt_bvh_node>& nodes, const std::vector<uint32_t>& idx,
               uint32_t num_tris, uint32_t& depth, std::string& why)
{
    depth = 0;
    if (nodes.empty()) {
        why = "empty BVH";
        return false;
    }
    if (nodes.size() >= MT_BVH_LEAF_BIT) {  // traversal stack entries flag leaves with that bit
        why = "BVH with 2^31 nodes or more";
        return false;
    }
    std::vector<std::pair<uint32_t, uint32_t>> st{{0u, 0u}};
    size_t visited = 0;
    while (!st.empty()) {
        const auto [ni, d] = st.back();
        st.pop_back();
        if (ni >= nodes.size() || ++visited > nodes.size()) {
            why = "BVH node index out of range or cyclic";
            return false;
        }
        depth = std::max(depth, d);
        const mt_bvh_node& n = nodes[ni];
        if (n.a & MT_BVH_LEAF_BIT) {
            const uint64_t first = n.a & ~MT_BVH_LEAF_BIT, count = n.b & ~MT_BVH_LEAF_BIT;
            if (first + count > idx.size()) {
                why = "BVH leaf range outside the index array";
                return false;
            }
            for (uint64_t i = first; i < first + count; ++i)
                if (idx[i] >= num_tris) {
                    why = "BVH index names a missing triangle";
                    return false;
                }
        } else {
            if (n.b != n.a + 1) {
                why = "BVH siblings are not adjacent";
                return false;
            }
            st.push_back({n.a, d + 1});
            st.push_back({n.b, d + 1});
        }
    }
    return true;
}

// Everything mt_create can reject without touching the device: missing
// arrays, prebuilt BVHs that are malformed or deeper than the traversal stack,
// empty textures, and indices naming missing meshes, materials, textures or
// light types.  Runs before the first CUDA call, so a bad scene never reaches
// an upload.
mt_status validate_scene(const mt_scene_desc* d, const mt_config& cfg, std::string& why)
{
    for (uint32_t mi = 0; mi < d->num_meshes; ++mi) {
        const mt_mesh_desc& md = d->meshes[mi];
        const std::string tag = "mesh " + std::to_string(mi) + ": ";
        if (!md.positions || !md.normals || md.num_triangles == 0) {
            why = tag + "positions and normals are required (GLTF.cpp:328-329)";
            return MT_ERR_INVALID;
        }
        const bool want_bvh = !cfg.bvh_disable && md.num_triangles > cfg.bvh_max_triangles;  // Mesh.cpp:37-40
        if (!want_bvh || !(md.bvh_nodes && md.bvh_indices)) continue;
        if (md.num_bvh_nodes == 0 || md.num_bvh_indices == 0) {
            why = tag + "prebuilt BVH with no nodes or no indices";
            return MT_ERR_INVALID;
        }
        std::vector<mt_bvh_node> bn(md.bvh_nodes, md.bvh_nodes + md.num_bvh_nodes);
        std::vector<uint32_t> bi(md.bvh_indices, md.bvh_indices + md.num_bvh_indices);
        uint32_t depth = 0;
        std::string w;
        if (!bvh_depth(bn, bi, md.num_triangles, depth, w)) {
            why = tag + w;
            return MT_ERR_INVALID;
        }
        if (depth + 2 > MT_STACK_SIZE) {
            why = tag + "BVH depth " + std::to_string(depth) + " exceeds the traversal stack (" +
                  std::to_string(MT_STACK_SIZE - 2) + ")";
            return MT_ERR_INVALID;
        }
    }
    for (uint32_t ti = 0; ti < d->num_textures; ++ti) {
        const mt_texture_desc& t = d->textures[ti];
        if (static_cast<uint64_t>(t.width) * t.height == 0 || (!t.rgb8 && !t.rgb32f)) {
            why = "texture " + std::to_string(ti) + " has no texels";
            return MT_ERR_INVALID;
        }
    }
    const int nt = static_cast<int>(d->num_textures);
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const mt_material_desc& m = d->materials[i];
        for (int ti : {m.base_color_tex, m.metallic_roughness_tex, m.normal_tex, m.emissive_tex})
            if (ti < -1 || ti >= nt) {
                why = "material " + std::to_string(i) + " names a missing texture";
                return MT_ERR_INVALID;
            }
    }
    for (uint32_t i = 0; i < d->num_instances; ++i)
        if (d->instances[i].mesh >= d->num_meshes || d->instances[i].material >= d->num_materials) {
            why = "instance " + std::to_string(i) + " names a missing mesh or material";
            return MT_ERR_INVALID;
        }
    for (uint32_t i = 0; i < d->num_lights; ++i)
        if (d->lights[i].type < MT_LIGHT_POINT || d->lights[i].type > MT_LIGHT_AREA) {
            why = "light " + std::to_string(i) + " has an unknown type";
            return MT_ERR_INVALID;
        }
    if (d->env_texture < -1 || d->env_texture >= nt) {
        why = "env texture index out of range";
        return MT_ERR_INVALID;
    }
    return MT_OK;
}

}  // namespace

struct mt_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    // a second stream and two events for the shadow stages that run beside the
    // next bounce's extension (launch_batch)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_shaded = nullptr, ev_shadowed = nullptr;
    mt_config cfg{};
    DevScene S{};
    // scene storage
    DevArray<float4> nodes, slots;
    DevArray<float> normals, uvs;
    DevArray<DevMesh> meshes;
    DevArray<DevInstance> instances;
    DevArray<DevMaterial> materials;
    DevArray<DevTexture> textures;
    DevArray<DevLight> lights;
    std::vector<DevArray<uint8_t>> tex8;
    std::vector<DevArray<float>> texf;
    std::vector<DevMaterial> host_mats;  // as uploaded (mt_update_* keep the texture slots and light types)
    std::vector<DevLight> host_lights;
    DevArray<int> error_flag;
    uint64_t scene_bytes = 0;
    float world_lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                         std::numeric_limits<float>::max()};
    float world_hi[3] = {std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(),
                         std::numeric_limits<float>::lowest()};
    // wavefront storage (allocated on first render)
    uint32_t batch = 0;
    uint64_t band_capacity = 0;  // samples the band planes hold
    uint32_t wave_spp = 0;       // paths per pixel the batch is sized for (0: cfg.samples)
    DevArray<float4> pstate;     // 10 float4 planes
    DevArray<uint4> phit;
    DevArray<float4> sq;         // 3 float4 planes
    DevArray<uint32_t> queues;   // 2 planes
    DevArray<uint32_t> counts;
    DevArray<unsigned long long> rays;  // [0] extension, [1] shadow
    DevArray<float> samples;     // 3 planes
    DevArray<float4> dval;       // debug render modes only
    DevArray<uint4> dcnt;
    DevArray<float> image;
    // pinned, 4 words: [0] extension rays, [1] shadow rays of the last render,
    // [2] the device error word after it
    unsigned long long* rays_host = nullptr;
    cudaEvent_t render_done = nullptr;        // end of the last enqueued render
    std::atomic<bool> render_pending{false};
    // serialises settle_render (the stat thread's mt_get_stats, the render
    // thread's next render and the profiler calls may all settle a render)
    std::mutex settle_mu;
    // profiling
    Profiler prof;
    DevArray<unsigned long long> prof_counts;  // 6 words
    double prof_ms[MT_NUM_STAGES] = {};
    uint64_t prof_launches[MT_NUM_STAGES] = {};
    uint64_t prof_rays[2] = {};
    // adjoint
    uint32_t grad_batch = 0;
    DevArray<float4> rec_vert, rec_path, grad_pix;
    DevArray<uint32_t> grad_order, grad_bins;
    DevArray<long long> texel_off;
    uint64_t grad_texels = 0;
    // neural radiance cache (mt_nrc_enable)
    struct Nrc {
        bool on = false;
        mt_nrc_config cfg{};
        DevArray<float> master, m, v, partial, planes, frame;
        DevArray<uint16_t> fwd, infer;
        DevArray<float> ema;
        DevArray<float4> qrec, trec, samples;
        // [0] cache queries of a batch, [1] training samples, [2] queries of the
        // frame, [3] summed step losses of the frame (float bits)
        DevArray<uint32_t> counters;
        DevArray<uint32_t> step;  // device Adam step counter
        cudaGraphExec_t steps_graph = nullptr;  // a frame's training steps, replayed
        uint32_t graph_steps = 0;
        NrcOptimizer opt{};
        uint64_t frames = 0;          // frames rendered (sample indices continue)
        uint64_t plane_capacity = 0;  // samples the cached render's band planes hold
        uint32_t train_chunk = 0;     // training paths per wavefront batch
        uint32_t sample_cap = 0;
        // the training paths' own wavefront state and stream: a frame traces
        // them and trains beside the cached render, whose cache queries wait
        // for the training (ev_trained)
        DevArray<float4> tstate, tsq;
        DevArray<uint4> thit;
        DevArray<uint32_t> tqueues, tcounts;
        DevArray<unsigned long long> trays;
        cudaStream_t tstream = nullptr;
        cudaEvent_t ev_fork = nullptr, ev_trained = nullptr;
    } nrc;
    // query scratch
    DevArray<mt_ray> qrays;
    DevArray<mt_hit> qhits;
    DevArray<uint32_t> qfetch;  // ray fetch counter of the query kernels
    // async render
    std::mutex mu;
    std::thread worker;
    std::atomic<int> running{0};
    std::atomic<int> started{0};
    std::atomic<int> done{0};
    std::atomic<int> kill{0};
    std::atomic<int> result{MT_OK};
    std::string worker_err;
    std::atomic<uint64_t> stat_rays{0}, stat_samples{0};
    std::atomic<uint64_t> work_total{1}, work_done{0};
    std::chrono::steady_clock::time_point t0;
    std::atomic<uint64_t> launches{0};

    ~mt_handle()
    {
        if (worker.joinable()) worker.join();
        if (nrc.steps_graph) cudaGraphExecDestroy(nrc.steps_graph);
        pinned_slot_free(rays_host);
        if (render_done) cudaEventDestroy(render_done);
        if (nrc.ev_fork) cudaEventDestroy(nrc.ev_fork);
        if (nrc.ev_trained) cudaEventDestroy(nrc.ev_trained);
        if (nrc.tstream) cudaStreamDestroy(nrc.tstream);
        if (ev_shaded) cudaEventDestroy(ev_shaded);
        if (ev_shadowed) cudaEventDestroy(ev_shadowed);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

DevMaterial dev_material(const mt_material_desc& m)
{
    DevMaterial x{};
    std::memcpy(x.base, m.base_color_factor, 16);
    std::memcpy(x.emissive, m.emissive_factor, 12);
    x.normal_scale = m.normal_scale;
    x.metallic = m.metallic_factor;
    x.roughness = m.roughness_factor;
    x.base_tex = m.base_color_tex;
    x.mr_tex = m.metallic_roughness_tex;
    x.nrm_tex = m.normal_tex;
    x.em_tex = m.emissive_tex;
    return x;
}

DevLight dev_light(const mt_light_desc& l)
{
    DevLight x{};
    x.type = l.type;
    std::memcpy(x.pos, l.position, 12);
    std::memcpy(x.color, l.color, 12);
    std::memcpy(x.dir, l.direction, 12);
    x.point_size = l.point_size;
    x.inner_cos = l.spot_inner_cos;
    x.outer_cos = l.spot_outer_cos;
    x.simple = (l.color[0] + l.color[1] + l.color[2]) / 3.0f;  // PrepareLights, Tracer.cpp:123-132
    return x;
}

mt_status upload_scene(mt_handle* h, const mt_scene_desc* d)
{
    const mt_config& cfg = h->cfg;
    cudaStream_t st = h->stream;
    std::vector<float4> nodes, slots;
    std::vector<float> normals, uvs;
    std::vector<DevMesh> meshes(d->num_meshes);
    std::vector<std::pair<std::vector<float>, std::vector<float>>> bounds(d->num_meshes);
    std::vector<float> mesh_lo(3 * d->num_meshes), mesh_hi(3 * d->num_meshes);
    uint32_t attr = 0;
    for (uint32_t mi = 0; mi < d->num_meshes; ++mi) {
        const mt_mesh_desc& md = d->meshes[mi];
        if (!md.positions || !md.normals || md.num_triangles == 0)
            return set_err(MT_ERR_INVALID, "mesh " + std::to_string(mi) +
                                               ": positions and normals are required (GLTF.cpp:328-329)");
        const uint32_t T = md.num_triangles;
        const float* P = md.positions;
        // Mesh::CalculateAABB (Mesh.cpp:43-54)
        float lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                       std::numeric_limits<float>::max()};
        float hi[3] = {std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(),
                       std::numeric_limits<float>::lowest()};
        for (uint64_t v = 0; v < 3ull * T; ++v)
            for (int k = 0; k < 3; ++k) {
                lo[k] = hmin(lo[k], P[3 * v + k]);
                hi[k] = hmax(hi[k], P[3 * v + k]);
            }
        std::memcpy(&mesh_lo[3 * mi], lo, 12);
        std::memcpy(&mesh_hi[3 * mi], hi, 12);

        DevMesh m{};
        m.node_off = static_cast<uint32_t>(nodes.size() / 2);
        m.slot_off = static_cast<uint32_t>(slots.size() / 3);
        m.attr_off = attr;
        m.num_tris = T;
        m.has_uv = md.uv0 != nullptr;
        const bool want_bvh = !cfg.bvh_disable && T > cfg.bvh_max_triangles;  // Mesh.cpp:37-40
        std::vector<mt_bvh_node> bn;
        std::vector<uint32_t> bi;
        if (want_bvh) {
            if (md.bvh_nodes && md.bvh_indices) {
                bn.assign(md.bvh_nodes, md.bvh_nodes + md.num_bvh_nodes);
                bi.assign(md.bvh_indices, md.bvh_indices + md.num_bvh_indices);
            } else {
                std::string err;
                const int rc = build_bvh(P, T, cfg.bvh_max_triangles, cfg.bvh_max_depth, bn, bi, err);
                if (rc != MT_OK) return set_err(static_cast<mt_status>(rc), "mesh " + std::to_string(mi) + ": " + err);
            }
            uint32_t depth = 0;
            std::string why;
            // prebuilt BVHs passed validate_scene; this checks the library's own build
            if (!bvh_depth(bn, bi, T, depth, why))
                return set_err(MT_ERR_INVALID, "mesh " + std::to_string(mi) + ": " + why);
            if (depth + 2 > MT_STACK_SIZE)
                return set_err(MT_ERR_INVALID, "mesh " + std::to_string(mi) + ": BVH depth " +
                                                   std::to_string(depth) + " exceeds the traversal stack (" +
                                                   std::to_string(MT_STACK_SIZE - 2) + ")");
            m.has_bvh = 1;
            for (const mt_bvh_node& n : bn) {
                float4 a, b;
                a.x = n.lo[0]; a.y = n.lo[1]; a.z = n.lo[2];
                b.x = n.hi[0]; b.y = n.hi[1]; b.z = n.hi[2];
                std::memcpy(&a.w, &n.a, 4);
                std::memcpy(&b.w, &n.b, 4);
                nodes.push_back(a);
                nodes.push_back(b);
            }
        } else {
            bi.resize(T);
            for (uint32_t t = 0; t < T; ++t) bi[t] = t;
        }
        m.num_slots = static_cast<uint32_t>(bi.size());
        for (uint32_t t : bi) {
            const float* v0 = P + 9ull * t;
            const float* v1 = v0 + 3;
            const float* v2 = v0 + 6;
            float4 A, B, C;
            A.x = v0[0]; A.y = v0[1]; A.z = v0[2];
            std::memcpy(&A.w, &t, 4);
            B.x = v1[0] - v0[0]; B.y = v1[1] - v0[1]; B.z = v1[2] - v0[2]; B.w = 0.0f;
            C.x = v2[0] - v0[0]; C.y = v2[1] - v0[1]; C.z = v2[2] - v0[2]; C.w = 0.0f;
            slots.push_back(A);
            slots.push_back(B);
            slots.push_back(C);
        }
        normals.insert(normals.end(), md.normals, md.normals + 9ull * T);
        if (md.uv0)
            uvs.insert(uvs.end(), md.uv0, md.uv0 + 6ull * T);
        else
            uvs.insert(uvs.end(), 6ull * T, 0.0f);
        attr += T;
        meshes[mi] = m;
    }

    std::vector<DevTexture> texs(d->num_textures);
    h->tex8.resize(d->num_textures);
    h->texf.resize(d->num_textures);
    for (uint32_t ti = 0; ti < d->num_textures; ++ti) {
        const mt_texture_desc& t = d->textures[ti];
        const size_t n = static_cast<size_t>(t.width) * t.height * 3;
        if (n == 0 || (!t.rgb8 && !t.rgb32f))
            return set_err(MT_ERR_INVALID, "texture " + std::to_string(ti) + " has no texels");
        DevTexture x{};
        x.w = t.width;
        x.h = t.height;
        x.filter = t.filter;
        x.offx = t.offset[0];
        x.offy = t.offset[1];
        x.sclx = t.scale[0];
        x.scly = t.scale[1];
        if (t.rgb32f) {
            MT_CUDA(h->texf[ti].upload(t.rgb32f, n, st));
            x.rgbf = h->texf[ti].p;
            h->scene_bytes += n * 4;
        } else {
            MT_CUDA(h->tex8[ti].upload(t.rgb8, n, st));
            x.rgb8 = h->tex8[ti].p;
            h->scene_bytes += n;
        }
        texs[ti] = x;
    }

    std::vector<DevMaterial> mats(d->num_materials);
    for (uint32_t i = 0; i < d->num_materials; ++i) {
        const DevMaterial x = dev_material(d->materials[i]);
        for (int ti : {x.base_tex, x.mr_tex, x.nrm_tex, x.em_tex})
            if (ti >= static_cast<int>(d->num_textures))
                return set_err(MT_ERR_INVALID, "material " + std::to_string(i) + " names a missing texture");
        mats[i] = x;
    }

    std::vector<DevInstance> insts(d->num_instances);
    for (uint32_t i = 0; i < d->num_instances; ++i) {
        const mt_instance_desc& id = d->instances[i];
        if (id.mesh >= d->num_meshes || id.material >= d->num_materials)
            return set_err(MT_ERR_INVALID, "instance " + std::to_string(i) + " names a missing mesh or material");
        DevInstance x{};
        std::memcpy(x.model, id.transform, 64);
        inverse4(id.transform, x.inv);
        x.mesh = id.mesh;
        x.material = id.material;
        // MeshInstance::CalculateWorldAABB (Mesh.cpp:56-80)
        const float* a = &mesh_lo[3 * id.mesh];
        const float* b = &mesh_hi[3 * id.mesh];
        const float corners[8][3] = {{a[0], a[1], a[2]}, {a[0], a[1], b[2]}, {a[0], b[1], a[2]},
                                     {a[0], b[1], b[2]}, {b[0], a[1], a[2]}, {b[0], a[1], b[2]},
                                     {b[0], b[1], a[2]}, {b[0], b[1], b[2]}};
        for (int k = 0; k < 3; ++k) {
            x.wlo[k] = std::numeric_limits<float>::max();
            x.whi[k] = std::numeric_limits<float>::lowest();
        }
        for (const auto& c : corners) {
            const float v[4] = {c[0], c[1], c[2], 1.0f};
            float w[4];
            mat_vec(id.transform, v, w);
            for (int k = 0; k < 3; ++k) {
                x.wlo[k] = hmin(x.wlo[k], w[k]);
                x.whi[k] = hmax(x.whi[k], w[k]);
            }
        }
        insts[i] = x;
        for (int k = 0; k < 3; ++k) {
            h->world_lo[k] = std::min(h->world_lo[k], x.wlo[k]);
            h->world_hi[k] = std::max(h->world_hi[k], x.whi[k]);
        }
    }

    std::vector<DevLight> lights(d->num_lights);
    for (uint32_t i = 0; i < d->num_lights; ++i) lights[i] = dev_light(d->lights[i]);
    if (d->env_texture >= static_cast<int>(d->num_textures))
        return set_err(MT_ERR_INVALID, "env texture index out of range");
    // gradient layout: RGB32F textures used as a base colour, in texture order
    {
        std::vector<long long> off(std::max<uint32_t>(1, d->num_textures), -1);
        std::vector<char> used(d->num_textures, 0);
        for (uint32_t i = 0; i < d->num_materials; ++i)
            if (d->materials[i].base_color_tex >= 0) used[d->materials[i].base_color_tex] = 1;
        uint64_t total = 0;
        for (uint32_t ti = 0; ti < d->num_textures; ++ti)
            if (used[ti] && d->textures[ti].rgb32f) {
                off[ti] = static_cast<long long>(total);
                total += 3ull * d->textures[ti].width * d->textures[ti].height;
            }
        h->grad_texels = total;
        MT_CUDA(h->texel_off.upload(off.data(), off.size(), st));
    }

    MT_CUDA(h->nodes.upload(nodes.data(), nodes.size(), st));
    MT_CUDA(h->slots.upload(slots.data(), slots.size(), st));
    MT_CUDA(h->normals.upload(normals.data(), normals.size(), st));
    MT_CUDA(h->uvs.upload(uvs.data(), uvs.size(), st));
    MT_CUDA(h->meshes.upload(meshes.data(), meshes.size(), st));
    MT_CUDA(h->instances.upload(insts.data(), insts.size(), st));
    MT_CUDA(h->materials.upload(mats.data(), mats.size(), st));
    h->host_mats = mats;
    h->host_lights = lights;
    MT_CUDA(h->textures.upload(texs.data(), texs.size(), st));
    MT_CUDA(h->lights.upload(lights.data(), lights.size(), st));
    // [0] render and ray-query traversal (MT_ERRBIT_STACK), cleared per render;
    // [1] the radiance cache's bounded tensor-core waits (MT_ERRBIT_TIMEOUT)
    MT_CUDA(h->error_flag.alloc(2));
    MT_CUDA(h->qfetch.alloc(1));
    MT_CUDA(cudaMemsetAsync(h->error_flag.p, 0, 2 * sizeof(int), st));
    h->scene_bytes += nodes.size() * 16 + slots.size() * 16 + normals.size() * 4 + uvs.size() * 4 +
                      insts.size() * sizeof(DevInstance);
    MT_CUDA(cudaStreamSynchronize(st));

    DevScene& S = h->S;
    S.nodes = h->nodes.p;
    S.slots = h->slots.p;
    {
        int dev = 0, l2 = 0;
        MT_CUDA(cudaGetDevice(&dev));
        MT_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev));
        const double bvh_bytes = (nodes.size() + slots.size()) * 16.0;
        const bool resident = bvh_bytes <= MT_TRAVERSE_RESIDENT_L2_FRACTION * l2;
        S.trav_pops = resident ? MT_TRAVERSE_POPS_RESIDENT : 1;
        S.trav_prefetch = resident ? 0 : 1;
        // an L2-resident scene's rays are short (tens of triangle tests), so
        // instance switches are frequent and worth batching; a large scene's
        // rays run thousands of tests between switches (measured on the 6.1 M
        // triangle scene: 8 lanes 45.9 against 45.6 Mrays/s unbatched, 16
        // lanes 2% slower)
        S.trav_switch = resident ? MT_TRAVERSE_SWITCH_RESIDENT : 1;
    }
    S.normals = h->normals.p;
    S.uvs = h->uvs.p;
    S.meshes = h->meshes.p;
    S.instances = h->instances.p;
    S.materials = h->materials.p;
    S.textures = h->textures.p;
    S.lights = h->lights.p;
    S.num_instances = d->num_instances;
    S.num_lights = d->num_lights;
    S.env = d->env_texture;
    S.hdri_prim = cfg.hdri_primary_intensity;
    S.hdri_sec = cfg.hdri_secondary_intensity;
    S.emission_base = cfg.emission_base_intensity;
    S.cam_type = d->camera.type;
    std::memcpy(S.c2w, d->camera.camera_to_world, 64);
    S.fov_scale = tanf(d->camera.yfov * 0.5f);
    S.cam_aspect = d->camera.aspect;
    S.ortho_x = d->camera.ortho_size[0];
    S.ortho_y = d->camera.ortho_size[1];
    S.width = cfg.width;
    S.height = cfg.height;
    S.bounces = cfg.bounces;
    S.spp = cfg.samples;
    S.terminate_energy = cfg.terminate_energy;
    S.exposure = powf(2.0f, -cfg.ev_exposure);
    S.px_w = 1.0f / static_cast<float>(cfg.width);
    S.px_h = 1.0f / static_cast<float>(cfg.height);
    S.render_aspect = static_cast<float>(cfg.width) / static_cast<float>(cfg.height);
    S.key0 = static_cast<uint32_t>(cfg.seed);
    S.key1 = static_cast<uint32_t>(cfg.seed >> 32);
    S.firefly_enable = cfg.firefly_enable;
    S.firefly_k = cfg.firefly_threshold;
    S.error_flag = h->error_flag.p;
    S.debug_mode = cfg.debug_mode;
    return MT_OK;
}

uint64_t env_u64(const char* name, uint64_t dflt)
{
    const char* v = std::getenv(name);
    if (!v || !*v) return dflt;
    return std::strtoull(v, nullptr, 10);
}

mt_status alloc_wave(mt_handle* h, uint64_t batch)
{
    const mt_config& c = h->cfg;
    const uint64_t npix = static_cast<uint64_t>(c.width) * c.height;
    MT_CUDA(h->pstate.alloc(10ull * batch));
    MT_CUDA(h->phit.alloc(batch));
    MT_CUDA(h->sq.alloc(3ull * batch));
    MT_CUDA(h->queues.alloc(2ull * batch));
    MT_CUDA(h->counts.alloc(8));
    MT_CUDA(cudaMemset(h->counts.p, 0, 8 * sizeof(uint32_t)));
    MT_CUDA(h->rays.alloc(2));
    MT_CUDA(h->samples.alloc(3ull * h->band_capacity));
    MT_CUDA(h->image.alloc(npix * 3));
    if (c.debug_mode) {
        MT_CUDA(h->dval.alloc(batch));
        MT_CUDA(h->dcnt.alloc(batch));
    }
    if (!h->rays_host) {
        MT_CUDA(pinned_slot_alloc(&h->rays_host));
        h->rays_host[0] = h->rays_host[1] = h->rays_host[2] = h->rays_host[3] = 0;
    }
    if (!h->render_done) MT_CUDA(cudaEventCreateWithFlags(&h->render_done, cudaEventDisableTiming));
    return MT_OK;
}

// Sizes the wavefront: a batch of paths and the per-sample planes of one band
// of image rows (the firefly clamp needs every sample of a pixel at once).
mt_status ensure_wave(mt_handle* h)
{
    if (h->batch) return MT_OK;
    const mt_config& c = h->cfg;
    const uint64_t npix = static_cast<uint64_t>(c.width) * c.height;
    const uint64_t total = npix * std::max<uint32_t>(c.samples, h->wave_spp);
    // Paths in flight per batch.  Every bounce launches the persistent
    // traversal kernels once per batch, and each launch ends with a tail in
    // which a few long rays keep their warps busy while the rest of the GPU
    // idles; the larger the batch, the smaller that tail's share (measured on
    // the 1080p 256-spp material grid, Mrays/s: 4 M paths 1058, 8 M 1159,
    // 16 M 1213, 32 M 1240, 64 M 1254).  A path's wave state takes 232 bytes,
    // so the default of 64 M paths holds 15.6 GB; it is cut to a quarter of
    // the free device memory.
    const uint64_t kWaveBytesPerPath = 10 * 16 + 16 + 3 * 16 + 2 * 4;
    uint64_t batch = env_u64("MT_BATCH_PATHS", 1ull << 26);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && free_b > 0)
        batch = std::min<uint64_t>(batch, free_b / 4 / kWaveBytesPerPath);
    batch = std::max<uint64_t>(1024, std::min<uint64_t>(batch, total));
    const uint64_t budget = env_u64("MT_SAMPLE_BUDGET_MB", 12288) << 20;
    uint64_t rows = budget / (static_cast<uint64_t>(c.width) * c.samples * 12ull);
    rows = std::max<uint64_t>(1, std::min<uint64_t>(rows, c.height));
    h->band_capacity = rows * c.width * c.samples;
    // h->batch stays 0 (wave not ready) until every buffer exists: a failed
    // allocation releases what was taken and a later call tries again
    const mt_status rc = alloc_wave(h, batch);
    if (rc != MT_OK) {
        h->pstate.reset();
        h->phit.reset();
        h->sq.reset();
        h->queues.reset();
        h->counts.reset();
        h->rays.reset();
        h->samples.reset();
        h->image.reset();
        h->dval.reset();
        h->dcnt.reset();
        return rc;
    }
    h->batch = static_cast<uint32_t>(batch);
    return MT_OK;
}

mt_status settle_render(mt_handle* h);

// Drops the wavefront state so that the next ensure_wave sizes it afresh
// (the last render's counters are folded in first; the NRC and adjoint
// buffers sized from the old batch are released too).
void rc_settle_and_release_wave(mt_handle* h)
{
    (void)settle_render(h);
    h->batch = 0;
    h->pstate.reset();
    h->phit.reset();
    h->sq.reset();
    h->queues.reset();
    h->counts.reset();
    h->rays.reset();
    h->samples.reset();
    h->image.reset();
    h->dval.reset();
    h->dcnt.reset();
    h->grad_batch = 0;
    h->rec_vert.reset();
    h->rec_path.reset();
    h->grad_pix.reset();
    h->grad_order.reset();
    h->grad_bins.reset();
}

struct WaveViews {
    PathState P;
    ShadowQueue SQ;
    WaveBuffers W;
};

WaveViews views(mt_handle* h)
{
    WaveViews v{};
    const uint64_t B = h->batch;
    float4* s = h->pstate.p;
    v.P.ro = s + 0 * B;
    v.P.rd = s + 1 * B;
    v.P.cur = s + 2 * B;
    v.P.tot = s + 3 * B;
    v.P.prev = s + 4 * B;
    v.P.emit = s + 5 * B;
    v.P.direct = s + 6 * B;
    v.P.indirect = s + 7 * B;
    v.P.sky = s + 8 * B;
    v.P.hitA = s + 9 * B;
    v.P.hitB = h->phit.p;
    v.P.dval = h->dval.p;
    v.P.dcnt = h->dcnt.p;
    v.SQ.o = h->sq.p;
    v.SQ.d = h->sq.p + B;
    v.SQ.c = h->sq.p + 2 * B;
    v.W.q[0] = h->queues.p;
    v.W.q[1] = h->queues.p + B;
    v.W.counts = h->counts.p;
    v.W.rays = h->rays.p;
    v.W.sr = h->samples.p;
    v.W.sg = h->samples.p + h->band_capacity;
    v.W.sb = h->samples.p + 2 * h->band_capacity;
    v.W.side = h->side;
    v.W.ev_shaded = h->ev_shaded;
    v.W.ev_shadowed = h->ev_shadowed;
    return v;
}

mt_status settle_render(mt_handle* h);

// Enqueues a render of rows [row0, row1) (the whole image by default) into
// `out` on `st`.  With sync_each_batch the host waits for every batch
// (progress/kill granularity for the async API).
mt_status render_into(mt_handle* h, float* out, cudaStream_t st, bool sync_each_batch, uint32_t row0 = 0,
                      uint32_t row1 = 0xFFFFFFFFu)
{
    mt_status rc = ensure_wave(h);
    if (rc != MT_OK) return rc;
    // the previous render's counters and error word share the pinned words
    // this render copies back into: fold them in first
    rc = settle_render(h);
    if (rc != MT_OK) return rc;
    const mt_config& c = h->cfg;
    row1 = std::min<uint32_t>(row1, c.height);
    const bool whole = row0 == 0 && row1 == c.height;
    const WaveViews v = views(h);
    MT_CUDA(cudaMemsetAsync(h->rays.p, 0, 2 * sizeof(unsigned long long), st));
    MT_CUDA(cudaMemsetAsync(h->error_flag.p, 0, sizeof(int), st));
    Profiler* prof = (h->prof.timing || h->prof.counting) ? &h->prof : nullptr;
    const uint64_t rows_per_band = h->band_capacity / (static_cast<uint64_t>(c.width) * c.samples);
    uint64_t total_batches = 0;
    for (uint64_t r0 = row0; r0 < row1; r0 += rows_per_band) {
        const uint64_t rows = std::min<uint64_t>(rows_per_band, row1 - r0);
        total_batches += (rows * c.width * c.samples + h->batch - 1) / h->batch;
    }
    h->work_total = std::max<uint64_t>(1, total_batches);
    h->work_done = 0;
    uint64_t launches = 0;
    for (uint64_t r0 = row0; r0 < row1; r0 += rows_per_band) {
        const uint64_t rows = std::min<uint64_t>(rows_per_band, row1 - r0);
        const uint32_t band_pix = static_cast<uint32_t>(rows * c.width);
        const uint32_t pix_base = static_cast<uint32_t>(r0 * c.width);
        const uint64_t paths = static_cast<uint64_t>(band_pix) * c.samples;
        for (uint64_t g0 = 0; g0 < paths; g0 += h->batch) {
            if (h->kill.load()) {
                h->launches += launches;
                return set_err(MT_ERR_KILLED, "render killed");
            }
            const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(h->batch, paths - g0));
            MT_CUDA(launch_batch(h->S, v.P, v.SQ, v.W, g0, n, band_pix, pix_base, st, &launches, prof));
            if (sync_each_batch) {
                MT_CUDA(cudaMemcpyAsync(h->rays_host, h->rays.p, 2 * sizeof(unsigned long long),
                                        cudaMemcpyDeviceToHost, st));
                MT_CUDA(cudaStreamSynchronize(st));
                h->stat_rays = h->rays_host[0] + h->rays_host[1];
                h->stat_samples += n;
            }
            h->work_done += 1;
        }
        MT_CUDA(launch_resolve(h->S, v.W, band_pix, pix_base, out, st, prof));
        ++launches;
    }
    if (whole && debug_needs_post(c.debug_mode)) {
        // WaitForRender's post-processing (Tracer.cpp:781-799) over the whole image
        MT_CUDA(launch_debug_post(out, static_cast<uint64_t>(c.width) * c.height, c.debug_mode, h->counts.p + 7, st));
        launches += 2;
    }
    MT_CUDA(cudaMemcpyAsync(h->rays_host, h->rays.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    MT_CUDA(cudaMemcpyAsync(h->rays_host + 2, h->error_flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    {
        std::lock_guard<std::mutex> lk(h->settle_mu);
        MT_CUDA(cudaEventRecord(h->render_done, st));
        h->render_pending = true;
    }
    h->launches += launches;
    return MT_OK;
}

// Folds the finished render's ray counters (and profile) into the handle and
// reports a device error word the render left set (a traversal stack overflow:
// MT_ERR_INVALID).  Thread-safe; blocks until that render has finished.
mt_status settle_render(mt_handle* h)
{
    std::lock_guard<std::mutex> lk(h->settle_mu);
    if (!h->render_pending) return MT_OK;
    MT_CUDA(cudaEventSynchronize(h->render_done));
    h->render_pending = false;
    h->stat_rays = h->rays_host[0] + h->rays_host[1];
    h->prof_rays[0] += h->rays_host[0];
    h->prof_rays[1] += h->rays_host[1];
    if (h->prof.timing) MT_CUDA(h->prof.collect(h->prof_ms, h->prof_launches));
    const unsigned long long flag = h->rays_host[2];
    h->rays_host[2] = 0;
    if (flag & MT_ERRBIT_STACK)
        return set_err(MT_ERR_INVALID, "device error flag set (traversal stack overflow)");
    return MT_OK;
}

void worker_main(mt_handle* h)
{
    cudaSetDevice(h->device);
    mt_status rc = render_into(h, h->image.p ? h->image.p : nullptr, h->stream, true);
    if (rc == MT_OK) {
        cudaError_t e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) rc = set_err(MT_ERR_CUDA, cudaGetErrorString(e));
    }
    if (rc == MT_OK) rc = settle_render(h);
    if (rc == MT_OK) {
        int flag = 0;
        if (cudaMemcpy(&flag, h->error_flag.p, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && flag)
            rc = set_err(MT_ERR_INVALID, "device error flag set (traversal stack overflow)");
    }
    if (rc != MT_OK) h->worker_err = g_err;
    h->result = rc;
    h->done = 1;
    h->running = 0;
}

mt_status check_handle(const mt_handle* h)
{
    if (!h) return set_err(MT_ERR_INVALID, "null handle");
    return MT_OK;
}

}  // namespace

namespace mt {

const DevScene* internal_scene(const mt_handle* h) { return h ? &h->S : nullptr; }
bool internal_busy(const mt_handle* h) { return h && h->running.load() != 0; }
void internal_count_samples(mt_handle* h, uint64_t n)
{
    if (h) h->stat_samples += n;
}
mt_status internal_error(mt_status code, const std::string& msg) { return set_err(code, msg); }

}  // namespace mt

namespace {

// Xavier-uniform initial weights, bound sqrt(6 / (fan_in + fan_out)), from a
// splitmix64 stream of the seed.
void nrc_init_weights(uint32_t seed, std::vector<float>& w)
{
    w.assign(kNrcParams, 0.0f);
    uint64_t x = 0x9E3779B97F4A7C15ull ^ seed;
    auto next = [&x]() {
        x += 0x9E3779B97F4A7C15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    const int ins[5] = {80, 64, 64, 64, 64}, outs[5] = {64, 64, 64, 64, 3};
    size_t off = 0;
    for (int l = 0; l < 5; ++l) {
        const double bound = std::sqrt(6.0 / (ins[l] + outs[l]));
        for (int k = 0; k < ins[l] * outs[l]; ++k) {
            const double u = static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0);
            w[off + k] = static_cast<float>((2.0 * u - 1.0) * bound);
        }
        off += static_cast<size_t>(ins[l]) * outs[l];
    }
}

uint64_t gcd64(uint64_t a, uint64_t b)
{
    while (b) {
        const uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

// The frame's training steps recorded once as a CUDA graph (the launches are
// fixed; step numbers live on the device), when the cache is enabled and again
// whenever the step count changes.
mt_status nrc_steps_graph(mt_handle* h)
{
    auto& N = h->nrc;
    const mt_nrc_config& nc = N.cfg;
    if (N.steps_graph && N.graph_steps == nc.train_steps) return MT_OK;
    if (N.steps_graph) cudaGraphExecDestroy(N.steps_graph);
    N.steps_graph = nullptr;
    cudaStream_t cs = nullptr;
    MT_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    const uint64_t host_step = N.opt.step;
    for (uint32_t s = 0; s < nc.train_steps && e == cudaSuccess; ++s) {
        NrcTrainArgs a{};
        a.feat = N.samples.p;
        a.fstride = 6;
        a.targets = reinterpret_cast<const float*>(N.samples.p + 5);
        a.tstride = 24;
        a.count = N.counters.p + 1;
        a.count_cap = N.sample_cap;
        a.rows = nc.train_batch;
        e = launch_nrc_train_step(N.opt, a, reinterpret_cast<float*>(N.counters.p + 3), nullptr, cs);
    }
    N.opt.step = host_step;  // captured, not run
    const cudaError_t e2 = cudaStreamEndCapture(cs, &graph);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&N.steps_graph, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    MT_CUDA(e);
    N.graph_steps = nc.train_steps;
    return MT_OK;
}

mt_status nrc_alloc(mt_handle* h, const mt_nrc_config& c)
{
    auto& N = h->nrc;
    N.on = false;
    N.cfg = c;
    const mt_config& cfg = h->cfg;
    const cudaStream_t st = h->stream;
    NrcOptimizer& O = N.opt;
    O.max_splits = 128;
    O.max_rows = 4u * c.train_batch;
    MT_CUDA(N.master.alloc(kNrcParams));
    MT_CUDA(N.m.alloc(kNrcParams));
    MT_CUDA(N.v.alloc(kNrcParams));
    MT_CUDA(N.partial.alloc(static_cast<size_t>(O.max_splits) * kNrcParams));
    MT_CUDA(N.fwd.alloc(kNrcFwdElems));
    MT_CUDA(N.infer.alloc(kNrcFwdElems));
    MT_CUDA(N.ema.alloc(kNrcParams));
    MT_CUDA(cudaMemsetAsync(N.fwd.p, 0, kNrcFwdElems * 2, st));
    MT_CUDA(cudaMemsetAsync(N.infer.p, 0, kNrcFwdElems * 2, st));
    O.master = N.master.p;
    O.m = N.m.p;
    O.v = N.v.p;
    O.partial = N.partial.p;
    O.fwd = N.fwd.p;
    O.infer = N.infer.p;
    O.ema = N.ema.p;
    O.ema_decay = c.ema_decay;
    O.lr = c.learning_rate;
    O.beta1 = c.beta1;
    O.beta2 = c.beta2;
    O.eps = c.epsilon;
    O.step = 0;
    // [0] Adam steps taken, [1] Adam blocks done with the current step
    MT_CUDA(N.step.alloc(2));
    MT_CUDA(cudaMemsetAsync(N.step.p, 0, 2 * sizeof(uint32_t), st));
    O.d_step = N.step.p;
    O.d_done = N.step.p + 1;
    O.err = h->error_flag.p + 1;
    if (N.steps_graph) {
        cudaGraphExecDestroy(N.steps_graph);
        N.steps_graph = nullptr;
    }
    MT_CUDA(nrc_prepare());
    // training paths and their samples
    const uint32_t bounces = std::max<uint32_t>(1, cfg.bounces);
    N.train_chunk = std::min<uint32_t>(c.train_paths, h->batch);
    MT_CUDA(N.trec.alloc(static_cast<size_t>(N.train_chunk) * bounces * 8));
    MT_CUDA(cudaMemsetAsync(N.trec.p, 0, N.trec.n * sizeof(float4), st));
    MT_CUDA(N.tstate.alloc(10ull * N.train_chunk));
    MT_CUDA(N.thit.alloc(N.train_chunk));
    MT_CUDA(N.tsq.alloc(3ull * N.train_chunk));
    MT_CUDA(N.tqueues.alloc(2ull * N.train_chunk));
    MT_CUDA(N.tcounts.alloc(8));
    MT_CUDA(cudaMemsetAsync(N.tcounts.p, 0, 8 * sizeof(uint32_t), st));
    MT_CUDA(N.trays.alloc(2));
    MT_CUDA(cudaMemsetAsync(N.trays.p, 0, 2 * sizeof(unsigned long long), st));
    if (!N.tstream) {
        // the training is on the frame's critical path (the cache queries wait
        // for it): its kernels take free SMs before the render's
        int lo = 0, hi = 0;
        MT_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        MT_CUDA(cudaStreamCreateWithPriority(&N.tstream, cudaStreamNonBlocking, hi));
    }
    if (!N.ev_fork) MT_CUDA(cudaEventCreateWithFlags(&N.ev_fork, cudaEventDisableTiming));
    if (!N.ev_trained) MT_CUDA(cudaEventCreateWithFlags(&N.ev_trained, cudaEventDisableTiming));
    N.sample_cap = c.train_paths * bounces;
    MT_CUDA(N.samples.alloc(static_cast<size_t>(N.sample_cap) * 6));
    MT_CUDA(N.qrec.alloc(static_cast<size_t>(h->batch) * 6));
    MT_CUDA(N.counters.alloc(4));
    MT_CUDA(cudaMemsetAsync(N.counters.p, 0, 4 * sizeof(uint32_t), st));
    // band planes of the cached render and its frame image
    const uint64_t npix = static_cast<uint64_t>(cfg.width) * cfg.height;
    const uint64_t budget = env_u64("MT_SAMPLE_BUDGET_MB", 12288) << 20;
    uint64_t rows = budget / (static_cast<uint64_t>(cfg.width) * c.spp * 12ull);
    rows = std::max<uint64_t>(1, std::min<uint64_t>(rows, cfg.height));
    N.plane_capacity = rows * cfg.width * c.spp;
    MT_CUDA(N.planes.alloc(3 * N.plane_capacity));
    MT_CUDA(N.frame.alloc(npix * 3));
    // weights
    std::vector<float> w;
    nrc_init_weights(c.seed, w);
    MT_CUDA(cudaMemcpyAsync(N.master.p, w.data(), kNrcParams * sizeof(float), cudaMemcpyHostToDevice, st));
    MT_CUDA(cudaMemsetAsync(N.m.p, 0, kNrcParams * sizeof(float), st));
    MT_CUDA(cudaMemsetAsync(N.v.p, 0, kNrcParams * sizeof(float), st));
    MT_CUDA(launch_nrc_publish(O, st));
    MT_CUDA(cudaStreamSynchronize(st));
    N.frames = 0;
    if (c.train_steps) {
        const mt_status rg = nrc_steps_graph(h);
        if (rg != MT_OK) return rg;
    }
    N.on = true;
    return MT_OK;
}

mt_status nrc_ready(mt_handle* h)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    if (!h->nrc.on) return set_err(MT_ERR_STATE, "the radiance cache is not enabled (mt_nrc_enable)");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    return MT_OK;
}

}  // namespace

extern "C" {

const char* mt_last_error(void) { return g_err.c_str(); }
int mt_abi_version(void) { return MT_ABI_VERSION; }

void mt_config_defaults(mt_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->width = 1280;
    c->height = 720;
    c->samples = 64;
    c->bounces = 5;
    c->ev_exposure = 8.0f;
    c->hdri_primary_intensity = 350.0f;
    c->hdri_secondary_intensity = 350.0f;
    c->emission_base_intensity = 1.0f;
    c->bvh_disable = 0;
    c->bvh_max_triangles = 32;
    c->bvh_max_depth = 32;
    c->firefly_enable = 1;
    c->firefly_threshold = 6.0f;
    c->terminate_energy = 0.01f;
    c->debug_mode = 0;
    c->seed = 0;
}

mt_status mt_create(const mt_scene_desc* scene, const mt_config* cfg, mt_handle** out)
{
    if (!out) return set_err(MT_ERR_INVALID, "out is null");
    *out = nullptr;
    if (!scene || !cfg) return set_err(MT_ERR_INVALID, "scene and config are required");
    if (cfg->width == 0 || cfg->height == 0 || cfg->samples == 0)
        return set_err(MT_ERR_INVALID, "width, height and samples must be positive");
    if (static_cast<uint64_t>(cfg->width) * cfg->height > 0xFFFFFFFFull / 2)
        return set_err(MT_ERR_INVALID, "image too large");
    if (cfg->debug_mode < 0 || cfg->debug_mode >= MT_DEBUG_COUNT)
        return set_err(MT_ERR_INVALID, "debug_mode is not a Config::DebugMode value");
    if (scene->num_meshes && !scene->meshes) return set_err(MT_ERR_INVALID, "meshes is null");
    if (scene->num_instances && !scene->instances) return set_err(MT_ERR_INVALID, "instances is null");
    if (scene->num_materials && !scene->materials) return set_err(MT_ERR_INVALID, "materials is null");
    if (scene->num_textures && !scene->textures) return set_err(MT_ERR_INVALID, "textures is null");
    if (scene->num_lights && !scene->lights) return set_err(MT_ERR_INVALID, "lights is null");
    {
        std::string why;
        const mt_status v = validate_scene(scene, *cfg, why);
        if (v != MT_OK) return set_err(v, why);
    }
    mt_handle* h = new (std::nothrow) mt_handle();
    if (!h) return set_err(MT_ERR_OOM, "host allocation failed");
    h->cfg = *cfg;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_shaded, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_shadowed, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete h;
        return set_err(MT_ERR_CUDA, std::string("CUDA unavailable: ") + cudaGetErrorString(e));
    }
    const mt_status rc = upload_scene(h, scene);
    if (rc != MT_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return MT_OK;
}

void mt_destroy(mt_handle* h)
{
    if (!h) return;
    h->kill = 1;
    if (h->worker.joinable()) h->worker.join();
    // work the caller enqueued on its own streams (mt_render_device, ray
    // queries, the adjoint) may still read the handle's buffers: finish it
    // before they are reused, as cudaFree would
    int cur = 0;
    cudaGetDevice(&cur);
    const int dev = h->device;
    if (cur != dev) cudaSetDevice(dev);
    g_device_idle = cudaDeviceSynchronize() == cudaSuccess;
    delete h;
    g_device_idle = false;
    if (cur != dev) cudaSetDevice(cur);
}

void mt_release_cached_memory(void)
{
    BlockCache& c = block_cache();
    std::vector<void*> blocks;
    {
        std::lock_guard<std::mutex> lk(c.mu);
        for (int d = 0; d < 64; ++d) {
            for (auto& kv : c.free_blocks[d]) {
                blocks.push_back(kv.second);
                c.size_of.erase(kv.second);
            }
            c.free_blocks[d].clear();
            c.cached[d] = 0;
        }
    }
    for (void* p : blocks) cudaFree(p);
}

mt_status mt_start(mt_handle* h)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(h->mu);
    if (h->running) return set_err(MT_ERR_STATE, "a render is already running");
    if (h->worker.joinable()) h->worker.join();
    mt_status rc = ensure_wave(h);
    if (rc != MT_OK) return rc;
    h->kill = 0;
    h->done = 0;
    h->result = MT_OK;
    h->stat_rays = 0;
    h->stat_samples = 0;
    h->work_done = 0;
    h->t0 = std::chrono::steady_clock::now();
    h->running = 1;
    h->started = 1;
    h->worker = std::thread(worker_main, h);
    return MT_OK;
}

mt_status mt_wait(mt_handle* h, float* rgb_out)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->started) return set_err(MT_ERR_STATE, "no render was started");
    if (h->worker.joinable()) h->worker.join();
    const mt_status rc = static_cast<mt_status>(h->result.load());
    if (rc != MT_OK) return set_err(rc, h->worker_err);
    if (rgb_out) {
        const size_t bytes = static_cast<size_t>(h->cfg.width) * h->cfg.height * 3 * sizeof(float);
        MT_CUDA(cudaMemcpy(rgb_out, h->image.p, bytes, cudaMemcpyDeviceToHost));
    }
    return MT_OK;
}

mt_status mt_kill(mt_handle* h)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    h->kill = 1;
    return MT_OK;
}

mt_status mt_get_stats(const mt_handle* h, mt_stats* out)
{
    if (check_handle(h) != MT_OK || !out) return set_err(MT_ERR_INVALID, "null argument");
    // a finished render's counters are folded in here (under the handle's
    // settle lock); a render still on the GPU is left alone, never waited for
    mt_status settled = MT_OK;
    if (!h->running && h->render_pending && cudaEventQuery(h->render_done) == cudaSuccess)
        settled = settle_render(const_cast<mt_handle*>(h));
    mt_stats s{};
    const double el = h->started ? std::chrono::duration<double>(std::chrono::steady_clock::now() - h->t0).count() : 0.0;
    s.progress = static_cast<float>(static_cast<double>(h->work_done.load()) / static_cast<double>(h->work_total.load()));
    if (s.progress > 1.0f) s.progress = 1.0f;
    s.time_elapsed = static_cast<float>(el);
    s.estimated_time_remaining = s.progress > 0.0f ? s.time_elapsed / s.progress * (1.0f - s.progress) : 0.0f;
    s.rays = h->stat_rays.load();
    s.samples = h->stat_samples.load();
    *out = s;
    return settled;
}

int mt_is_done(const mt_handle* h) { return h && h->started && h->done ? 1 : 0; }

uint64_t mt_kernel_launches(const mt_handle* h) { return h ? h->launches.load() : 0; }

mt_status mt_profile_enable(mt_handle* h, int timing, int counting)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    if (h->running) return set_err(MT_ERR_STATE, "a render is running");
    if (counting && !h->prof_counts.p) {
        MT_CUDA(h->prof_counts.alloc(6));
        MT_CUDA(cudaMemset(h->prof_counts.p, 0, 6 * sizeof(unsigned long long)));
    }
    h->prof.timing = timing != 0;
    h->prof.counting = counting != 0;
    h->prof.d_counts = h->prof_counts.p;
    return MT_OK;
}

mt_status mt_profile_reset(mt_handle* h)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    if (h->running) return set_err(MT_ERR_STATE, "a render is running");
    mt_status rc = settle_render(h);
    if (rc != MT_OK) return rc;
    std::lock_guard<std::mutex> lk(h->settle_mu);
    for (int i = 0; i < MT_NUM_STAGES; ++i) {
        h->prof_ms[i] = 0.0;
        h->prof_launches[i] = 0;
    }
    h->prof_rays[0] = h->prof_rays[1] = 0;
    if (h->prof_counts.p) MT_CUDA(cudaMemset(h->prof_counts.p, 0, 6 * sizeof(unsigned long long)));
    return MT_OK;
}

mt_status mt_profile_read(mt_handle* h, mt_profile* out)
{
    if (check_handle(h) != MT_OK || !out) return set_err(MT_ERR_INVALID, "null argument");
    if (h->running) return set_err(MT_ERR_STATE, "a render is running");
    mt_status rc = settle_render(h);
    if (rc != MT_OK) return rc;
    std::lock_guard<std::mutex> lk(h->settle_mu);
    std::memset(out, 0, sizeof(*out));
    for (int i = 0; i < MT_NUM_STAGES; ++i) {
        out->stage[i].launches = h->prof_launches[i];
        out->stage[i].milliseconds = h->prof_ms[i];
    }
    out->stage[MT_STAGE_EXTEND].rays = h->prof_rays[0];
    out->stage[MT_STAGE_SHADOW].rays = h->prof_rays[1];
    if (h->prof_counts.p) {
        unsigned long long c[6];
        MT_CUDA(cudaMemcpy(c, h->prof_counts.p, sizeof(c), cudaMemcpyDeviceToHost));
        out->stage[MT_STAGE_EXTEND].node_pops = c[0];
        out->stage[MT_STAGE_EXTEND].inner_pops = c[1];
        out->stage[MT_STAGE_EXTEND].tri_tests = c[2];
        out->stage[MT_STAGE_SHADOW].node_pops = c[3];
        out->stage[MT_STAGE_SHADOW].inner_pops = c[4];
        out->stage[MT_STAGE_SHADOW].tri_tests = c[5];
    }
    return MT_OK;
}

mt_status mt_render_device(mt_handle* h, float* d_rgb_out, void* cuda_stream)
{
    if (check_handle(h) != MT_OK || !d_rgb_out) return set_err(MT_ERR_INVALID, "null argument");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);  // 0: the legacy default stream
    h->kill = 0;
    const mt_status rc = render_into(h, d_rgb_out, st, false);
    if (rc == MT_OK) h->stat_samples += static_cast<uint64_t>(h->cfg.width) * h->cfg.height * h->cfg.samples;
    return rc;
}

mt_status mt_set_seed(mt_handle* h, uint64_t seed)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    h->cfg.seed = seed;
    h->S.key0 = static_cast<uint32_t>(seed);
    h->S.key1 = static_cast<uint32_t>(seed >> 32);
    return MT_OK;
}

mt_status mt_render_rows_device(mt_handle* h, uint32_t row0, uint32_t row1, float* d_rgb_out, void* cuda_stream)
{
    if (check_handle(h) != MT_OK || !d_rgb_out) return set_err(MT_ERR_INVALID, "null argument");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    if (row0 >= row1 || row1 > h->cfg.height) return set_err(MT_ERR_INVALID, "rows must satisfy row0 < row1 <= height");
    if ((row0 != 0 || row1 != h->cfg.height) && debug_needs_post(h->cfg.debug_mode))
        return set_err(MT_ERR_INVALID, "heatmap debug modes normalise over the whole image: render every row");
    h->kill = 0;
    const mt_status rc = render_into(h, d_rgb_out, static_cast<cudaStream_t>(cuda_stream), false, row0, row1);
    if (rc == MT_OK) h->stat_samples += static_cast<uint64_t>(row1 - row0) * h->cfg.width * h->cfg.samples;
    return rc;
}

mt_status mt_render_grad(mt_handle* h, const mt_grad_buffers* g, void* cuda_stream)
{
    if (check_handle(h) != MT_OK || !g) return set_err(MT_ERR_INVALID, "null argument");
    if ((!g->target && !g->d_image) || !g->image || (!g->loss && !g->d_image) || !g->d_base || !g->d_roughness ||
        !g->d_metallic ||
        (!g->d_light && h->S.num_lights))
        return set_err(MT_ERR_INVALID, "target, image, loss and the material/light gradient buffers are required");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    if (h->cfg.bounces > MT_GRAD_MAX_BOUNCES)
        return set_err(MT_ERR_INVALID, "mt_render_grad supports at most MT_GRAD_MAX_BOUNCES bounces");
    if (h->cfg.debug_mode) return set_err(MT_ERR_INVALID, "mt_render_grad needs debug_mode 0");
    mt_status rc = ensure_wave(h);
    if (rc != MT_OK) return rc;
    const mt_config& c = h->cfg;
    const uint64_t rows_per_band = h->band_capacity / (static_cast<uint64_t>(c.width) * c.samples);
    if (!h->grad_batch) {
        // Paths replayed per batch: their vertex records (5 float4 per bounce
        // plus 2 per path, and the path's place in the grouping by length) are
        // the adjoint's only storage, O(batch).  Sixteen
        // samples per pixel of a band (at least 2^20 paths) keep the memory
        // proportional to the pixels, not to the samples, while batches stay
        // large enough that the replay's traversal launches are not dominated
        // by their tails; capped at an eighth of the free device memory.
        const uint64_t rec_bytes = (static_cast<uint64_t>(std::max<uint32_t>(1, c.bounces)) * 5 + 2) * 16 + 4;
        uint64_t want = std::max<uint64_t>(1ull << 20, 16ull * rows_per_band * c.width);
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && free_b > 0)
            want = std::min<uint64_t>(want, std::max<uint64_t>(1024, free_b / 8 / rec_bytes));
        const uint64_t gb = std::min<uint64_t>(h->batch, env_u64("MT_GRAD_BATCH_PATHS", want));
        MT_CUDA(h->rec_vert.alloc(gb * std::max<uint32_t>(1, c.bounces) * 5));
        MT_CUDA(h->rec_path.alloc(gb * 2));
        MT_CUDA(h->grad_pix.alloc(2 * rows_per_band * c.width));
        MT_CUDA(h->grad_order.alloc(gb));
        MT_CUDA(h->grad_bins.alloc(2 * kAdjointBins));
        h->grad_batch = static_cast<uint32_t>(gb);  // set once every record buffer exists
    }
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    const WaveViews v = views(h);
    GradParams G{};
    G.target = g->target;
    G.d_image = g->d_image;
    G.loss = g->loss;
    G.d_base = g->d_base;
    G.d_rough = g->d_roughness;
    G.d_metal = g->d_metallic;
    G.d_light = g->d_light;
    G.d_texels = h->grad_texels ? g->d_texels : nullptr;
    G.texel_off = h->texel_off.p;
    G.pix = h->grad_pix.p;
    G.order = h->grad_order.p;
    G.bins = h->grad_bins.p;
    const uint32_t nmat = static_cast<uint32_t>(h->materials.n);
    G.smem_materials = nmat <= 1024 ? nmat : 0;
    G.smem_lights = h->S.num_lights <= 256 ? h->S.num_lights : 0;
    RecordBuffers R;
    R.vert = h->rec_vert.p;
    R.path = h->rec_path.p;
    if (!g->d_image) MT_CUDA(cudaMemsetAsync(g->loss, 0, sizeof(float), st));
    MT_CUDA(cudaMemsetAsync(h->rays.p, 0, 2 * sizeof(unsigned long long), st));
    uint64_t launches = 0;
    for (uint64_t r0 = 0; r0 < c.height; r0 += rows_per_band) {
        const uint64_t rows = std::min<uint64_t>(rows_per_band, c.height - r0);
        const uint32_t band_pix = static_cast<uint32_t>(rows * c.width);
        const uint32_t pix_base = static_cast<uint32_t>(r0 * c.width);
        const uint64_t paths = static_cast<uint64_t>(band_pix) * c.samples;
        for (uint64_t g0 = 0; g0 < paths; g0 += h->batch) {
            const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(h->batch, paths - g0));
            MT_CUDA(launch_batch(h->S, v.P, v.SQ, v.W, g0, n, band_pix, pix_base, st, &launches, nullptr));
        }
        MT_CUDA(launch_resolve(h->S, v.W, band_pix, pix_base, g->image, st, nullptr));
        MT_CUDA(launch_grad_pixel(h->S, v.W, band_pix, pix_base, g->image, G, st));
        launches += 2;
        for (uint64_t g0 = 0; g0 < paths; g0 += h->grad_batch) {
            const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(h->grad_batch, paths - g0));
            MT_CUDA(launch_batch(h->S, v.P, v.SQ, v.W, g0, n, band_pix, pix_base, st, &launches, nullptr, &R));
            MT_CUDA(launch_adjoint(h->S, G, R, v.W, g0, n, band_pix, st));
            launches += 3;
        }
    }
    h->launches += launches;
    return MT_OK;
}

mt_status mt_trace_rays_device(mt_handle* h, const mt_ray* d_rays, uint64_t n, mt_hit* d_hits, int query,
                               void* cuda_stream)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    if (n && (!d_rays || !d_hits)) return set_err(MT_ERR_INVALID, "null ray or hit buffer");
    if (query < MT_QUERY_CLOSEST || query > MT_QUERY_CLOSEST_TOTALS)
        return set_err(MT_ERR_INVALID, "unknown query");
    if ((reinterpret_cast<uintptr_t>(d_rays) | reinterpret_cast<uintptr_t>(d_hits)) & 15)
        return set_err(MT_ERR_INVALID, "ray and hit buffers must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);  // 0: the legacy default stream
    MT_CUDA(launch_trace(h->S, d_rays, n, d_hits, query, h->qfetch.p, st));
    h->launches += n ? 1 : 0;
    return MT_OK;
}

mt_status mt_trace_rays(mt_handle* h, const mt_ray* rays, uint64_t n, mt_hit* hits, int query)
{
    if (check_handle(h) != MT_OK) return MT_ERR_INVALID;
    if (n == 0) return MT_OK;
    if (!rays || !hits) return set_err(MT_ERR_INVALID, "null ray or hit buffer");
    if (h->qrays.n < n) {
        MT_CUDA(h->qrays.alloc(n));
        MT_CUDA(h->qhits.alloc(n));
    }
    MT_CUDA(cudaMemcpyAsync(h->qrays.p, rays, n * sizeof(mt_ray), cudaMemcpyHostToDevice, h->stream));
    const mt_status rc = mt_trace_rays_device(h, h->qrays.p, n, h->qhits.p, query, h->stream);
    if (rc != MT_OK) return rc;
    MT_CUDA(cudaMemcpyAsync(hits, h->qhits.p, n * sizeof(mt_hit), cudaMemcpyDeviceToHost, h->stream));
    MT_CUDA(cudaStreamSynchronize(h->stream));
    int flag = 0;
    MT_CUDA(cudaMemcpy(&flag, h->error_flag.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return set_err(MT_ERR_INVALID, "device error flag set (traversal stack overflow)");
    return MT_OK;
}

mt_status mt_brdf_sample_batch(const mt_brdf_sample_query* q, uint64_t n, mt_brdf_sample_result* out)
{
    if (n == 0) return MT_OK;
    if (!q || !out) return set_err(MT_ERR_INVALID, "null argument");
    mt_brdf_sample_query* dq = nullptr;
    mt_brdf_sample_result* dr = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&dq), n * sizeof(mt_brdf_sample_query));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&dr), n * sizeof(mt_brdf_sample_result));
    if (e == cudaSuccess) e = cudaMemcpy(dq, q, n * sizeof(mt_brdf_sample_query), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_brdf_sample(dq, n, dr, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, dr, n * sizeof(mt_brdf_sample_result), cudaMemcpyDeviceToHost);
    if (dq) cudaFree(dq);
    if (dr) cudaFree(dr);
    if (e != cudaSuccess) return set_err(MT_ERR_CUDA, cudaGetErrorString(e));
    return MT_OK;
}

mt_status mt_brdf_batch(const mt_brdf_query* q, uint64_t n, mt_brdf_result* out)
{
    if (n == 0) return MT_OK;
    if (!q || !out) return set_err(MT_ERR_INVALID, "null argument");
    mt_brdf_query* dq = nullptr;
    mt_brdf_result* dr = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&dq), n * sizeof(mt_brdf_query));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&dr), n * sizeof(mt_brdf_result));
    if (e == cudaSuccess) e = cudaMemcpy(dq, q, n * sizeof(mt_brdf_query), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_brdf(dq, n, dr, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, dr, n * sizeof(mt_brdf_result), cudaMemcpyDeviceToHost);
    if (dq) cudaFree(dq);
    if (dr) cudaFree(dr);
    if (e != cudaSuccess) return set_err(MT_ERR_CUDA, cudaGetErrorString(e));
    return MT_OK;
}

mt_status mt_resolve_batch(const float* samples_rgb, uint32_t npix, uint32_t spp, int firefly_enable, float k,
                           int debug_mode, float* rgb_out)
{
    if (npix == 0) return MT_OK;
    if (!samples_rgb || !rgb_out) return set_err(MT_ERR_INVALID, "null argument");
    if (spp == 0) return set_err(MT_ERR_INVALID, "spp must be positive");
    if (debug_mode < 0 || debug_mode >= MT_DEBUG_COUNT)
        return set_err(MT_ERR_INVALID, "debug_mode is not a Config::DebugMode value");
    const uint64_t n = static_cast<uint64_t>(npix) * spp;
    // pixel-major host samples -> the render's sample-major R, G, B planes
    std::vector<float> planes;
    try {
        planes.resize(3 * n);
    } catch (const std::bad_alloc&) {
        return set_err(MT_ERR_OOM, "host allocation failed");
    }
    for (uint64_t p = 0; p < npix; ++p)
        for (uint64_t s = 0; s < spp; ++s)
            for (int c = 0; c < 3; ++c) planes[c * n + s * npix + p] = samples_rgb[(p * spp + s) * 3 + c];
    float* dp = nullptr;
    float* dout = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&dp), 3 * n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&dout), 3ull * npix * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dp, planes.data(), 3 * n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = launch_resolve_planes(dp, dp + n, dp + 2 * n, npix, spp, firefly_enable, k, debug_mode, dout, 0);
    if (e == cudaSuccess) e = cudaMemcpy(rgb_out, dout, 3ull * npix * sizeof(float), cudaMemcpyDeviceToHost);
    if (dp) cudaFree(dp);
    if (dout) cudaFree(dout);
    if (e != cudaSuccess)
        return set_err(e == cudaErrorMemoryAllocation ? MT_ERR_OOM : MT_ERR_CUDA, cudaGetErrorString(e));
    return MT_OK;
}

mt_status mt_bvh_build(const float* positions, uint32_t num_triangles, uint32_t max_triangles,
                       uint32_t max_depth, mt_bvh_node** nodes, uint32_t* num_nodes, uint32_t** indices,
                       uint32_t* num_indices)
{
    if (!positions || !nodes || !num_nodes || !indices || !num_indices)
        return set_err(MT_ERR_INVALID, "null argument");
    std::vector<mt_bvh_node> bn;
    std::vector<uint32_t> bi;
    std::string err;
    const int rc = build_bvh(positions, num_triangles, max_triangles, max_depth, bn, bi, err);
    if (rc != MT_OK) return set_err(static_cast<mt_status>(rc), err);
    *nodes = static_cast<mt_bvh_node*>(std::malloc(bn.size() * sizeof(mt_bvh_node)));
    *indices = static_cast<uint32_t*>(std::malloc(std::max<size_t>(1, bi.size()) * sizeof(uint32_t)));
    if (!*nodes || !*indices) {
        std::free(*nodes);
        std::free(*indices);
        return set_err(MT_ERR_OOM, "host allocation failed");
    }
    std::memcpy(*nodes, bn.data(), bn.size() * sizeof(mt_bvh_node));
    std::memcpy(*indices, bi.data(), bi.size() * sizeof(uint32_t));
    *num_nodes = static_cast<uint32_t>(bn.size());
    *num_indices = static_cast<uint32_t>(bi.size());
    return MT_OK;
}

void mt_bvh_free(mt_bvh_node* nodes, uint32_t* indices)
{
    std::free(nodes);
    std::free(indices);
}

void mt_nrc_config_defaults(mt_nrc_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->train_paths = 65536;
    c->train_batch = 16384;
    c->train_steps = 128;
    c->spp = 4;
    c->learning_rate = 1e-2f;
    c->beta1 = 0.9f;
    c->beta2 = 0.99f;
    c->epsilon = 1e-15f;
    c->rough_min = 0.3f;
    c->seed = 1337;
    c->ema_decay = 0.9f;
    c->target_cap = 0.5f;
}

mt_status mt_nrc_enable(mt_handle* h, const mt_nrc_config* c)
{
    if (check_handle(h) != MT_OK || !c) return set_err(MT_ERR_INVALID, "null argument");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    if (c->train_paths == 0 || c->train_batch == 0 || c->train_batch > (1u << 24) || c->spp == 0 ||
        !(c->learning_rate > 0.0f) || !(c->beta1 >= 0.0f && c->beta1 < 1.0f) || !(c->beta2 >= 0.0f && c->beta2 < 1.0f) ||
        !(c->epsilon >= 0.0f) || !(c->ema_decay >= 0.0f && c->ema_decay < 1.0f) ||
        c->end_at > MT_NRC_END_AT_DIFFUSE || std::isnan(c->target_cap))
        return set_err(MT_ERR_INVALID, "invalid radiance-cache configuration");
    if (static_cast<uint64_t>(c->train_paths) * std::max<uint32_t>(1, h->cfg.bounces) > 0xFFFFFFFFull)
        return set_err(MT_ERR_INVALID, "train_paths * bounces exceeds 2^32");
    if (h->cfg.debug_mode) return set_err(MT_ERR_INVALID, "the radiance cache needs debug_mode 0");
    // a cached frame renders c->spp samples per pixel: size the wavefront so
    // that a frame is one batch when the device allows it (a batch holds at
    // most 2^26 paths), rather than the mt_config samples it was sized for
    if (c->spp > std::max<uint32_t>(h->cfg.samples, h->wave_spp)) {
        const uint64_t npix = static_cast<uint64_t>(h->cfg.width) * h->cfg.height;
        const bool grow = h->batch && h->batch < std::min<uint64_t>(1ull << 26, npix * c->spp);
        h->wave_spp = c->spp;
        if (grow) {
            MT_CUDA(cudaStreamSynchronize(h->stream));
            rc_settle_and_release_wave(h);
        }
    }
    mt_status rc = ensure_wave(h);
    if (rc != MT_OK) return rc;
    return nrc_alloc(h, *c);
}

mt_status mt_nrc_frame(mt_handle* h, float* d_accum, uint32_t accum_index, void* cuda_stream)
{
    mt_status rc = nrc_ready(h);
    if (rc != MT_OK) return rc;
    auto& N = h->nrc;
    const mt_nrc_config& nc = N.cfg;
    const mt_config& c = h->cfg;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);  // 0: the legacy default stream
    const WaveViews v = views(h);
    const uint64_t npix = static_cast<uint64_t>(c.width) * c.height;
    NrcShade base;
    base.rough_min = nc.rough_min;
    base.end_at = nc.end_at;
    for (int k = 0; k < 3; ++k) {
        base.lo[k] = h->world_lo[k];
        const float ext = h->world_hi[k] - h->world_lo[k];
        base.inv_ext[k] = ext > 1e-12f ? 1.0f / ext : 1.0f;
    }
    uint64_t launches = 0;
    // 1. full-length training paths from pixels spread over the image
    DevScene St = h->S;
    St.key0 ^= 0x85EBCA6Bu * static_cast<uint32_t>(N.frames + 1) + nc.seed;
    St.key1 ^= 0xC2B2AE35u;
    NrcShade T = base;
    T.mode = MT_NRC_TRAIN;
    T.rec = N.trec.p;
    T.samples = N.samples.p;
    T.sample_count = N.counters.p + 1;
    T.sample_cap = N.sample_cap;
    T.target_cap = nc.target_cap > 0.0f ? nc.target_cap / h->S.exposure : 0.0f;
    uint64_t mul = (0x9E3779B1ull + 2 * N.frames) % npix;
    if (mul == 0) mul = 1;
    while (gcd64(mul, npix) != 1) mul = (mul + 1) % npix ? (mul + 1) % npix : 1;
    const uint64_t add0 = (N.frames * 0x632BE5ABull) % npix;
    // the training (paths, targets, Adam steps) runs on the cache's own stream
    // with its own wavefront state, beside the cached render below
    const cudaStream_t ts = N.tstream;
    MT_CUDA(cudaEventRecord(N.ev_fork, st));
    MT_CUDA(cudaStreamWaitEvent(ts, N.ev_fork, 0));
    MT_CUDA(cudaMemsetAsync(N.counters.p + 1, 0, sizeof(uint32_t), ts));  // training samples
    MT_CUDA(cudaMemsetAsync(N.counters.p + 3, 0, sizeof(uint32_t), ts));  // summed step losses
    MT_CUDA(cudaMemsetAsync(N.counters.p + 2, 0, sizeof(uint32_t), st));  // the frame's queries
    PathState Pt;
    {
        const uint64_t B = N.train_chunk;
        float4* f = N.tstate.p;
        Pt.ro = f;
        Pt.rd = f + B;
        Pt.cur = f + 2 * B;
        Pt.tot = f + 3 * B;
        Pt.prev = f + 4 * B;
        Pt.emit = f + 5 * B;
        Pt.direct = f + 6 * B;
        Pt.indirect = f + 7 * B;
        Pt.sky = f + 8 * B;
        Pt.hitA = f + 9 * B;
        Pt.hitB = N.thit.p;
    }
    ShadowQueue SQt;
    SQt.o = N.tsq.p;
    SQt.d = N.tsq.p + N.train_chunk;
    SQt.c = N.tsq.p + 2ull * N.train_chunk;
    WaveBuffers Wt{};  // no sample planes: training paths add no image samples
    Wt.q[0] = N.tqueues.p;
    Wt.q[1] = N.tqueues.p + N.train_chunk;
    Wt.counts = N.tcounts.p;
    Wt.rays = N.trays.p;
    for (uint32_t c0 = 0; c0 < nc.train_paths; c0 += N.train_chunk) {
        const uint32_t n = std::min<uint32_t>(N.train_chunk, nc.train_paths - c0);
        BatchExtra X;
        X.nrc = &T;
        X.sample_base = 0;
        X.scatter_mul = static_cast<uint32_t>(mul);
        X.scatter_add = static_cast<uint32_t>((add0 + (static_cast<uint64_t>(c0) % npix) * mul) % npix);
        MT_CUDA(launch_batch(St, Pt, SQt, Wt, 0, n, static_cast<uint32_t>(npix), 0, ts, &launches, nullptr,
                             nullptr, &X));
    }
    // 2. Adam steps on random vertices of those paths, replayed as one CUDA
    //    graph (the launches are fixed; step numbers live on the device)
    if (nc.train_steps) {
        rc = nrc_steps_graph(h);
        if (rc != MT_OK) return rc;
        MT_CUDA(cudaGraphLaunch(N.steps_graph, ts));
        N.opt.step += nc.train_steps;
        launches += 3ull * nc.train_steps;
    }
    MT_CUDA(cudaEventRecord(N.ev_trained, ts));
    // 3. the cached render
    if (d_accum) {
        DevScene Sr = h->S;
        Sr.spp = nc.spp;
        WaveBuffers Wr = v.W;
        Wr.sr = N.planes.p;
        Wr.sg = N.planes.p + N.plane_capacity;
        Wr.sb = N.planes.p + 2 * N.plane_capacity;
        NrcShade Q = base;
        Q.mode = MT_NRC_QUERY;
        Q.rec = N.qrec.p;
        Q.count = N.counters.p;
        Q.net = N.infer.p;
        Q.total = N.counters.p + 2;
        Q.err = h->error_flag.p + 1;
        const uint64_t rows_per_band = N.plane_capacity / (static_cast<uint64_t>(c.width) * nc.spp);
        for (uint64_t r0 = 0; r0 < c.height; r0 += rows_per_band) {
            const uint64_t rows = std::min<uint64_t>(rows_per_band, c.height - r0);
            const uint32_t band_pix = static_cast<uint32_t>(rows * c.width);
            const uint32_t pix_base = static_cast<uint32_t>(r0 * c.width);
            const uint64_t paths = static_cast<uint64_t>(band_pix) * nc.spp;
            for (uint64_t g0 = 0; g0 < paths; g0 += h->batch) {
                const uint32_t n = static_cast<uint32_t>(std::min<uint64_t>(h->batch, paths - g0));
                MT_CUDA(cudaMemsetAsync(N.counters.p, 0, sizeof(uint32_t), st));
                BatchExtra X;
                X.nrc = &Q;
                X.sample_base = static_cast<uint32_t>(N.frames * nc.spp);
                X.query_after = N.ev_trained;
                MT_CUDA(launch_batch(Sr, v.P, v.SQ, Wr, g0, n, band_pix, pix_base, st, &launches, nullptr, nullptr,
                                     &X));
            }
            MT_CUDA(launch_resolve(Sr, Wr, band_pix, pix_base, N.frame.p, st, nullptr));
            ++launches;
        }
        MT_CUDA(launch_nrc_blend(d_accum, N.frame.p, npix * 3, accum_index, st));
        ++launches;
    }
    MT_CUDA(cudaStreamWaitEvent(st, N.ev_trained, 0));  // the frame's work ends on the caller's stream
    N.frames += 1;
    h->launches += launches;
    return MT_OK;
}

mt_status mt_nrc_get_stats(mt_handle* h, mt_nrc_stats* out)
{
    mt_status rc = nrc_ready(h);
    if (rc != MT_OK) return rc;
    if (!out) return set_err(MT_ERR_INVALID, "null argument");
    uint32_t c[4];
    int flag = 0;
    MT_CUDA(cudaDeviceSynchronize());
    MT_CUDA(cudaMemcpy(c, h->nrc.counters.p, sizeof(c), cudaMemcpyDeviceToHost));
    MT_CUDA(cudaMemcpy(&flag, h->error_flag.p + 1, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag & MT_ERRBIT_TIMEOUT) {
        // reported once: the word is cleared so the handle's later work is judged afresh
        MT_CUDA(cudaMemset(h->error_flag.p + 1, 0, sizeof(int)));
        return set_err(MT_ERR_TIMEOUT, "a bounded wait on the tensor cores ran out");
    }
    std::memset(out, 0, sizeof(*out));
    out->frames = h->nrc.frames;
    out->adam_steps = h->nrc.opt.step;
    out->train_samples = std::min(c[1], h->nrc.sample_cap);
    out->queries = c[2];
    float loss;
    std::memcpy(&loss, &c[3], sizeof(loss));
    out->train_loss = h->nrc.cfg.train_steps ? loss / static_cast<float>(h->nrc.cfg.train_steps) : 0.0f;
    return MT_OK;
}

mt_status mt_nrc_get_params(mt_handle* h, float* params)
{
    mt_status rc = nrc_ready(h);
    if (rc != MT_OK) return rc;
    if (!params) return set_err(MT_ERR_INVALID, "null argument");
    MT_CUDA(cudaDeviceSynchronize());
    MT_CUDA(cudaMemcpy(params, h->nrc.master.p, kNrcParams * sizeof(float), cudaMemcpyDeviceToHost));
    return MT_OK;
}

mt_status mt_nrc_set_params(mt_handle* h, const float* params)
{
    mt_status rc = nrc_ready(h);
    if (rc != MT_OK) return rc;
    if (!params) return set_err(MT_ERR_INVALID, "null argument");
    auto& N = h->nrc;
    MT_CUDA(cudaDeviceSynchronize());
    MT_CUDA(cudaMemcpy(N.master.p, params, kNrcParams * sizeof(float), cudaMemcpyHostToDevice));
    MT_CUDA(cudaMemset(N.m.p, 0, kNrcParams * sizeof(float)));
    MT_CUDA(cudaMemset(N.v.p, 0, kNrcParams * sizeof(float)));
    MT_CUDA(cudaMemset(N.step.p, 0, 2 * sizeof(uint32_t)));
    N.opt.step = 0;
    MT_CUDA(launch_nrc_publish(N.opt, h->stream));
    MT_CUDA(cudaStreamSynchronize(h->stream));
    return MT_OK;
}

mt_status mt_nrc_infer(mt_handle* h, const float* d_features, uint32_t n, float* d_rgb, void* cuda_stream)
{
    mt_status rc = nrc_ready(h);
    if (rc != MT_OK) return rc;
    if (n && (!d_features || !d_rgb)) return set_err(MT_ERR_INVALID, "null argument");
    if (reinterpret_cast<uintptr_t>(d_features) % 16)
        return set_err(MT_ERR_INVALID, "d_features must be 16-byte aligned (records are copied as float4)");
    MT_CUDA(launch_nrc_infer(h->nrc.infer.p, d_features, n, d_rgb, h->error_flag.p + 1,
                             static_cast<cudaStream_t>(cuda_stream)));
    h->launches += n ? 1 : 0;
    return MT_OK;
}

mt_status mt_nrc_train_step(mt_handle* h, const float* d_features, const float* d_targets, uint32_t n,
                            float* d_loss, float* d_grad, void* cuda_stream)
{
    mt_status rc = nrc_ready(h);
    if (rc != MT_OK) return rc;
    if (!d_features || !d_targets) return set_err(MT_ERR_INVALID, "null argument");
    if (reinterpret_cast<uintptr_t>(d_features) % 16)
        return set_err(MT_ERR_INVALID, "d_features must be 16-byte aligned (records are read as float4)");
    if (n == 0 || static_cast<uint64_t>(n) > 4ull * h->nrc.cfg.train_batch)
        return set_err(MT_ERR_INVALID, "n must be in [1, 4 * train_batch]");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    if (d_loss) MT_CUDA(cudaMemsetAsync(d_loss, 0, sizeof(float), st));
    NrcTrainArgs a{};
    a.feat = reinterpret_cast<const float4*>(d_features);
    a.fstride = 5;
    a.targets = d_targets;
    a.tstride = 3;
    a.count = nullptr;
    a.rows = n;
    MT_CUDA(launch_nrc_train_step(h->nrc.opt, a, d_loss, d_grad, st));
    h->launches += 3;
    return MT_OK;
}

mt_status mt_nrc_encode(const float* d_features, uint32_t n, float* d_encoded, void* cuda_stream)
{
    if (n && (!d_features || !d_encoded)) return set_err(MT_ERR_INVALID, "null argument");
    MT_CUDA(launch_nrc_encode(d_features, n, d_encoded, static_cast<cudaStream_t>(cuda_stream)));
    return MT_OK;
}

mt_status mt_update_materials(mt_handle* h, const mt_material_desc* materials, uint32_t n)
{
    if (check_handle(h) != MT_OK || (n && !materials)) return set_err(MT_ERR_INVALID, "null argument");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    if (n != h->host_mats.size()) return set_err(MT_ERR_INVALID, "the material count cannot change");
    std::vector<DevMaterial> mats(n);
    for (uint32_t i = 0; i < n; ++i) {
        mats[i] = dev_material(materials[i]);
        const DevMaterial& o = h->host_mats[i];
        if (mats[i].base_tex != o.base_tex || mats[i].mr_tex != o.mr_tex || mats[i].nrm_tex != o.nrm_tex ||
            mats[i].em_tex != o.em_tex)
            return set_err(MT_ERR_INVALID, "material " + std::to_string(i) + " changes a texture slot");
    }
    MT_CUDA(cudaStreamSynchronize(h->stream));
    MT_CUDA(cudaDeviceSynchronize());
    if (n) MT_CUDA(cudaMemcpy(h->materials.p, mats.data(), n * sizeof(DevMaterial), cudaMemcpyHostToDevice));
    h->host_mats = mats;
    return MT_OK;
}

mt_status mt_update_lights(mt_handle* h, const mt_light_desc* lights, uint32_t n)
{
    if (check_handle(h) != MT_OK || (n && !lights)) return set_err(MT_ERR_INVALID, "null argument");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    if (n != h->host_lights.size()) return set_err(MT_ERR_INVALID, "the light count cannot change");
    std::vector<DevLight> ls(n);
    for (uint32_t i = 0; i < n; ++i) {
        ls[i] = dev_light(lights[i]);
        if (ls[i].type != h->host_lights[i].type)
            return set_err(MT_ERR_INVALID, "light " + std::to_string(i) + " changes its type");
    }
    MT_CUDA(cudaDeviceSynchronize());
    if (n) MT_CUDA(cudaMemcpy(h->lights.p, ls.data(), n * sizeof(DevLight), cudaMemcpyHostToDevice));
    h->host_lights = ls;
    return MT_OK;
}

mt_status mt_update_texture(mt_handle* h, uint32_t index, const void* texels)
{
    if (check_handle(h) != MT_OK || !texels) return set_err(MT_ERR_INVALID, "null argument");
    if (h->running) return set_err(MT_ERR_STATE, "an asynchronous render is running");
    if (index >= h->tex8.size()) return set_err(MT_ERR_INVALID, "texture index out of range");
    MT_CUDA(cudaDeviceSynchronize());
    if (h->texf[index].p)
        MT_CUDA(cudaMemcpy(h->texf[index].p, texels, h->texf[index].n * sizeof(float), cudaMemcpyHostToDevice));
    else
        MT_CUDA(cudaMemcpy(h->tex8[index].p, texels, h->tex8[index].n, cudaMemcpyHostToDevice));
    return MT_OK;
}

}  // extern "C"
