// api.cu -- the extern "C" entry points of libsplat (include/splat.h).
#include <atomic>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "kernels.h"
#include "mesh.h"

using namespace splat;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
namespace {

thread_local std::string g_last_error;

splat_status_t fail(splat_status_t code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

splat_status_t cuda_fail(cudaError_t e, const char* what) {
    return fail(SPLAT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define SPLAT_CUDA(call, what)                      \
    do {                                            \
        cudaError_t e_ = (call);                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

int sm_count_current() {
    // read from any host thread: each device's count is written once
    static std::atomic<int> cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    if (dev >= 0 && dev < 64) {
        int c = cache[dev].load(std::memory_order_relaxed);
        if (c) return c;
    }
    int n = 152;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (dev >= 0 && dev < 64) cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

constexpr size_t kAlign = 256;
size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

size_t soa_bytes(int64_t cap) {
    return align_up((size_t)kPlanes * 4 * (size_t)cap) + 2 * align_up(4 * (size_t)cap) + align_up((size_t)cap);
}

RaySoA carve_soa(char*& p, int64_t cap) {
    RaySoA s;
    s.cap = cap;
    s.f = reinterpret_cast<float*>(p);
    p += align_up((size_t)kPlanes * 4 * (size_t)cap);
    s.ignore = reinterpret_cast<int32_t*>(p);
    p += align_up(4 * (size_t)cap);
    s.id = reinterpret_cast<uint32_t*>(p);
    p += align_up(4 * (size_t)cap);
    s.medium = reinterpret_cast<uint8_t*>(p);
    p += align_up((size_t)cap);
    return s;
}

// Bounce-loop scratch: two SoA ray buffers, hit indices, the packed-argmin
// array of split brute-force launches, counters and the kernel error word.
struct Work {
    RaySoA a, b, q;  // bounce ping-pong buffers and the splat queue
    int32_t* hit;
    uint64_t* tmp;
    int64_t* counts;  // counts[b] = active rays after bounce b (b <= 64); counts[kSplatCount] = queued
    void* order;      // ray-order sort scratch (ray_order_bytes(cap))
};
constexpr int kSplatCount = 96;
constexpr int kSplatSnap = 100;  // counts[kSplatSnap + b]: splat queue length after bounce b (b <= 8)
constexpr int kFetchBase = 128;  // counts[kFetchBase + b]: work counter of bounce b's hit launch (b <= 64)
constexpr size_t kCounterBytes = 2048;

size_t work_bytes(int64_t cap) {
    return 3 * soa_bytes(cap) + align_up(4 * (size_t)cap) + align_up(8 * (size_t)cap) + kCounterBytes +
           align_up(ray_order_bytes(cap)) + kAlign;
}

Work carve_work(void* ws, int64_t cap) {
    char* p = reinterpret_cast<char*>(align_up(reinterpret_cast<size_t>(ws)));
    Work w;
    w.a = carve_soa(p, cap);
    w.b = carve_soa(p, cap);
    w.q = carve_soa(p, cap);
    w.hit = reinterpret_cast<int32_t*>(p);
    p += align_up(4 * (size_t)cap);
    w.tmp = reinterpret_cast<uint64_t*>(p);
    p += align_up(8 * (size_t)cap);
    w.counts = reinterpret_cast<int64_t*>(p);
    p += kCounterBytes;
    w.order = p;
    return w;
}

// Traversal form of bounce b (1-based) under the SPLAT_TUNE_BVH_PACKET knob:
// 0 one ray per lane; 1 warp packets; 2, 3 per-warp choice by ray spread
// (loose, tight thresholds).
int32_t packet_for(int32_t b) { return packet_form(g_tune[SPLAT_TUNE_BVH_PACKET], b == 1); }

bool valid_material(const splat_material_t* m) {
    return m && m->kind >= SPLAT_MATERIAL_LINEAR_REF && m->kind <= SPLAT_MATERIAL_SELLMEIER;
}

}  // namespace

// ---------------------------------------------------------------------------
// launch profiling
// ---------------------------------------------------------------------------
struct splat_profile {
    int32_t max = 0;
    int32_t used = 0;
    std::vector<cudaEvent_t> ev;  // 2 per scope
    std::vector<int32_t> kind;
    std::vector<int64_t> kernels;  // kernels launched inside the scope
};

namespace {
thread_local splat_profile* g_prof = nullptr;

// Brackets one launcher call with events on its stream while a profile is
// attached to this thread.
struct ProfScope {
    int idx = -1;
    cudaStream_t s;
    int64_t k0;
    ProfScope(int kind, cudaStream_t st) : s(st), k0(g_launches) {
        splat_profile* p = g_prof;
        if (p && p->used < p->max) {
            idx = p->used++;
            p->kind[(size_t)idx] = kind;
            cudaEventRecord(p->ev[2 * (size_t)idx], s);
        }
    }
    ~ProfScope() {
        if (idx >= 0 && g_prof) {
            g_prof->kernels[(size_t)idx] = g_launches - k0;
            cudaEventRecord(g_prof->ev[2 * (size_t)idx + 1], s);
        }
    }
};
}  // namespace

// ---------------------------------------------------------------------------
// scene
// ---------------------------------------------------------------------------
struct splat_scene {
    int device = 0;
    int64_t n_tris = 0, first_diffuse = 0;
    splat_ftri_t* d_ftri = nullptr;
    TriHit* d_brute = nullptr;
    TriBox* d_boxes = nullptr;   // padded boxes of the brute-force records
    unsigned* d_scale = nullptr; // max |vertex coordinate| (float bits), sets the box padding
    int64_t n_recs = 0;
    BvhNode* d_nodes = nullptr;
    int64_t n_nodes = 0;
    TriHit* d_bvh = nullptr;
    int32_t* d_order = nullptr;
    int32_t* d_bvh_pos = nullptr;  // inverse of d_order (n_tris + 1 entries, by reference index)
    int32_t* d_links = nullptr;  // refit links of the two-child tree
    Bvh4Node* d_nodes4 = nullptr;
    int64_t n_nodes4 = 0;
    int32_t* d_links4 = nullptr;  // refit links of the four-wide tree
    unsigned* d_flags = nullptr;  // refit arrival counts
    int depth = 0, max_leaf = 0;
    int64_t leaves = 0;
    float pad_abs = 0.f, pad_rel = 0.f;
    float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    int32_t* d_err = nullptr;
    int64_t bytes = 0;
    // GPU rebuild (linear BVH): scratch and node capacities; once the tree
    // comes from the GPU the host level lists no longer match it, and updates
    // rebuild instead of refitting
    void* d_lbvh = nullptr;
    int64_t cap_nodes = 0, cap_nodes4 = 0;
    bool gpu_bvh = false;
};

static void scene_free(splat_scene* s) {
    if (!s) return;
    cudaFree(s->d_ftri);
    cudaFree(s->d_brute);
    cudaFree(s->d_boxes);
    cudaFree(s->d_scale);
    cudaFree(s->d_nodes);
    cudaFree(s->d_bvh);
    cudaFree(s->d_order);
    cudaFree(s->d_bvh_pos);
    cudaFree(s->d_links);
    cudaFree(s->d_nodes4);
    cudaFree(s->d_links4);
    cudaFree(s->d_flags);
    cudaFree(s->d_err);
    cudaFree(s->d_lbvh);
    delete s;
}

template <class T>
static cudaError_t dalloc(T** p, size_t bytes, int64_t& total) {
    total += (int64_t)bytes;
    return cudaMalloc(reinterpret_cast<void**>(p), bytes < 16 ? 16 : bytes);
}

static splat_status_t scene_pack(splat_scene* s, cudaStream_t st) {
    ProfScope ps(SPLAT_KERNEL_AUX, st);
    cudaError_t e = launch_pack_hits(s->d_ftri, s->n_tris, s->d_brute, s->d_boxes, s->d_scale, s->d_order, s->d_bvh,
                                     s->d_bvh_pos, st);
    if (e != cudaSuccess) return cuda_fail(e, "pack hit records");
    if (s->d_nodes && s->d_links) {
        e = launch_refit_tree(s->d_nodes, false, s->n_nodes, s->d_links, s->d_flags, s->d_bvh, s->d_ftri, s->d_scale,
                              s->pad_rel, st);
        if (e != cudaSuccess) return cuda_fail(e, "BVH refit");
    }
    if (s->d_nodes4 && s->d_links4) {
        e = launch_refit_tree(s->d_nodes4, true, s->n_nodes4, s->d_links4, s->d_flags, s->d_bvh, s->d_ftri, s->d_scale,
                              s->pad_rel, st);
        if (e != cudaSuccess) return cuda_fail(e, "BVH4 refit");
    }
    return SPLAT_OK;
}

namespace splat {
splat_status_t set_error(splat_status_t code, const std::string& msg) { return fail(code, msg); }
}  // namespace splat

extern "C" {

int32_t splat_abi_version(void) { return SPLAT_ABI_VERSION; }

const char* splat_last_error(void) { return g_last_error.c_str(); }

splat_status_t splat_device_info(int32_t* sm_count, char* name, int32_t name_len) {
    int dev = 0;
    SPLAT_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    cudaDeviceProp prop;
    SPLAT_CUDA(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (name && name_len > 0) {
        std::strncpy(name, prop.name, (size_t)name_len - 1);
        name[name_len - 1] = 0;
    }
    return SPLAT_OK;
}

splat_status_t splat_scene_create(const splat_ftri_t* host_tris, int64_t n_tris, int64_t first_diffuse,
                                  int32_t build_bvh_flag, void* stream, splat_scene_t** out) {
    if (!out) return fail(SPLAT_ERR_INVALID, "scene_create: out is null");
    *out = nullptr;
    if (!host_tris || n_tris < 1) return fail(SPLAT_ERR_INVALID, "scene_create: need at least the sentinel triangle");
    if (n_tris >= (int64_t(1) << 31)) return fail(SPLAT_ERR_INVALID, "scene_create: too many triangles");
    if (first_diffuse < 1) return fail(SPLAT_ERR_INVALID, "scene_create: first_diffuse must be >= 1");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    splat_scene* s = new (std::nothrow) splat_scene();
    if (!s) return fail(SPLAT_ERR_ALLOC, "scene_create: host allocation");
    cudaGetDevice(&s->device);
    s->n_tris = n_tris;
    s->first_diffuse = first_diffuse;
    s->n_recs = n_tris - 1;
    for (int a = 0; a < 3; ++a) {
        s->lo[a] = INFINITY;
        s->hi[a] = -INFINITY;
    }
    for (int64_t j = 1; j < n_tris; ++j)
        for (int v = 1; v < 4; ++v)
            for (int a = 0; a < 3; ++a) {
                s->lo[a] = std::min(s->lo[a], host_tris[j].v[v][a]);
                s->hi[a] = std::max(s->hi[a], host_tris[j].v[v][a]);
            }
    BvhHost bvh;
    if (build_bvh_flag) {
        std::string err;
        if (!build_bvh(host_tris, n_tris, bvh, err)) {
            delete s;
            return fail(SPLAT_ERR_INVALID, "scene_create: " + err);
        }
    }
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess && x != cudaSuccess) e = x;
    };
    chk(dalloc(&s->d_ftri, sizeof(splat_ftri_t) * (size_t)n_tris, s->bytes));
    chk(dalloc(&s->d_brute, sizeof(TriHit) * (size_t)s->n_recs, s->bytes));
    chk(dalloc(&s->d_boxes, sizeof(TriBox) * (size_t)s->n_recs, s->bytes));
    chk(dalloc(&s->d_scale, sizeof(unsigned), s->bytes));
    chk(dalloc(&s->d_err, sizeof(int32_t) * 4, s->bytes));
    if (build_bvh_flag && !bvh.nodes.empty()) {
        s->n_nodes = (int64_t)bvh.nodes.size();
        chk(dalloc(&s->d_nodes, sizeof(BvhNode) * bvh.nodes.size(), s->bytes));
        chk(dalloc(&s->d_bvh, sizeof(TriHit) * (size_t)s->n_recs, s->bytes));
        chk(dalloc(&s->d_order, sizeof(int32_t) * bvh.order.size(), s->bytes));
        chk(dalloc(&s->d_bvh_pos, sizeof(int32_t) * ((size_t)n_tris + 1), s->bytes));
        chk(dalloc(&s->d_links, sizeof(int32_t) * bvh.links.size(), s->bytes));
        s->n_nodes4 = (int64_t)bvh.nodes4.size();
        s->cap_nodes = s->n_nodes;
        s->cap_nodes4 = s->n_nodes4;
        chk(dalloc(&s->d_nodes4, sizeof(Bvh4Node) * bvh.nodes4.size(), s->bytes));
        chk(dalloc(&s->d_links4, sizeof(int32_t) * bvh.links4.size(), s->bytes));
        chk(dalloc(&s->d_flags, sizeof(unsigned) * std::max(bvh.nodes.size(), bvh.nodes4.size()), s->bytes));
        s->depth = bvh.depth;
        s->max_leaf = bvh.max_leaf;
        s->leaves = bvh.leaves;
        s->pad_abs = bvh.pad_abs;
        s->pad_rel = bvh.pad_rel;
    }
    if (e != cudaSuccess) {
        scene_free(s);
        return fail(SPLAT_ERR_ALLOC, std::string("scene_create: cudaMalloc: ") + cudaGetErrorString(e));
    }
    chk(cudaMemcpyAsync(s->d_ftri, host_tris, sizeof(splat_ftri_t) * (size_t)n_tris, cudaMemcpyHostToDevice, st));
    chk(cudaMemsetAsync(s->d_err, 0, sizeof(int32_t) * 4, st));
    if (s->d_nodes) {
        chk(cudaMemcpyAsync(s->d_nodes, bvh.nodes.data(), sizeof(BvhNode) * bvh.nodes.size(), cudaMemcpyHostToDevice,
                            st));
        chk(cudaMemcpyAsync(s->d_order, bvh.order.data(), sizeof(int32_t) * bvh.order.size(), cudaMemcpyHostToDevice,
                            st));
        chk(cudaMemcpyAsync(s->d_links, bvh.links.data(), sizeof(int32_t) * bvh.links.size(), cudaMemcpyHostToDevice,
                            st));
        chk(cudaMemcpyAsync(s->d_nodes4, bvh.nodes4.data(), sizeof(Bvh4Node) * bvh.nodes4.size(),
                            cudaMemcpyHostToDevice, st));
        chk(cudaMemcpyAsync(s->d_links4, bvh.links4.data(), sizeof(int32_t) * bvh.links4.size(),
                            cudaMemcpyHostToDevice, st));
    }
    if (e == cudaSuccess)
        chk(launch_pack_hits(s->d_ftri, n_tris, s->d_brute, s->d_boxes, s->d_scale, s->d_order, s->d_bvh,
                             s->d_bvh_pos, st));
    // host vectors above must outlive the async copies
    if (e == cudaSuccess) chk(cudaStreamSynchronize(st));
    if (e != cudaSuccess) {
        scene_free(s);
        return cuda_fail(e, "scene_create");
    }
    *out = s;
    return SPLAT_OK;
}

splat_status_t splat_scene_destroy(splat_scene_t* scene) {
    if (!scene) return fail(SPLAT_ERR_INVALID, "scene_destroy: null scene");
    scene_free(scene);
    return SPLAT_OK;
}

splat_status_t splat_scene_info(const splat_scene_t* s, splat_scene_info_t* info) {
    if (!s || !info) return fail(SPLAT_ERR_INVALID, "scene_info: null argument");
    std::memset(info, 0, sizeof(*info));
    info->n_tris = s->n_tris;
    info->first_diffuse = s->first_diffuse;
    info->bvh_nodes = s->n_nodes;
    info->bvh_leaves = s->leaves;
    info->bvh_depth = s->depth;
    info->bvh_max_leaf = s->max_leaf;
    info->device_bytes = s->bytes;
    for (int a = 0; a < 3; ++a) {
        info->bounds_lo[a] = s->lo[a];
        info->bounds_hi[a] = s->hi[a];
    }
    info->bvh_pad = s->pad_abs;
    return SPLAT_OK;
}

splat_status_t splat_scene_errors(splat_scene_t* s, int32_t reset, int32_t* out, void* stream) {
    if (!s || !out) return fail(SPLAT_ERR_INVALID, "scene_errors: null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int32_t err = 0;
    SPLAT_CUDA(cudaMemcpyAsync(&err, s->d_err, sizeof(err), cudaMemcpyDeviceToHost, st), "read error word");
    SPLAT_CUDA(cudaStreamSynchronize(st), "read error word");
    if (reset) SPLAT_CUDA(cudaMemsetAsync(s->d_err, 0, sizeof(int32_t), st), "clear error word");
    *out = err;
    return SPLAT_OK;
}

const splat_ftri_t* splat_scene_tris(const splat_scene_t* s) { return s ? s->d_ftri : nullptr; }

// BVH of the scene's current FTri data rebuilt on the GPU (linear BVH).
static splat_status_t scene_rebuild_gpu(splat_scene* s, cudaStream_t st) {
    const int64_t np = s->n_tris - 1;
    if (np < 1) return SPLAT_OK;
    const int64_t need = np > 1 ? np - 1 : 1;
    auto grow = [&](auto** p, int64_t& cap, int64_t want, size_t elem) -> cudaError_t {
        if (*p && cap >= want) return cudaSuccess;
        cudaFree(*p);
        *p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), elem * (size_t)want);
        if (e == cudaSuccess) {
            cap = want;
            s->bytes += (int64_t)(elem * (size_t)want);
        }
        return e;
    };
    SPLAT_CUDA(grow(&s->d_nodes, s->cap_nodes, need, sizeof(BvhNode)), "scene_rebuild: node array");
    SPLAT_CUDA(grow(&s->d_nodes4, s->cap_nodes4, need, sizeof(Bvh4Node)), "scene_rebuild: four-wide node array");
    if (!s->d_bvh) {
        int64_t cap = 0;
        SPLAT_CUDA(grow(&s->d_bvh, cap, np, sizeof(TriHit)), "scene_rebuild: hit records");
    }
    if (!s->d_order) {
        int64_t cap = 0;
        SPLAT_CUDA(grow(&s->d_order, cap, np, sizeof(int32_t)), "scene_rebuild: order");
    }
    if (!s->d_bvh_pos) {
        int64_t cap = 0;
        SPLAT_CUDA(grow(&s->d_bvh_pos, cap, s->n_tris + 1, sizeof(int32_t)), "scene_rebuild: order inverse");
    }
    if (!s->d_lbvh) {
        const size_t b = lbvh_scratch_bytes(np);
        SPLAT_CUDA(cudaMalloc(&s->d_lbvh, b), "scene_rebuild: scratch");
        s->bytes += (int64_t)b;
    }
    SPLAT_CUDA(launch_lbvh_build(s->d_ftri, s->n_tris, kLbvhLeaf, s->d_lbvh, s->d_nodes, s->d_nodes4, s->d_order,
                                 sm_count_current(), st),
               "scene_rebuild: build");
    SPLAT_CUDA(launch_pack_hits(s->d_ftri, s->n_tris, s->d_brute, s->d_boxes, s->d_scale, s->d_order, s->d_bvh,
                                s->d_bvh_pos, st),
               "scene_rebuild: pack");
    s->gpu_bvh = true;
    s->n_nodes = need;
    s->n_nodes4 = need;
    s->max_leaf = kLbvhLeaf;
    s->depth = 0;
    s->leaves = 0;
    return SPLAT_OK;
}

splat_status_t splat_scene_rebuild(splat_scene_t* s, const splat_ftri_t* d_tris, void* stream) {
    if (!s) return fail(SPLAT_ERR_INVALID, "scene_rebuild: null scene");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (d_tris && d_tris != s->d_ftri)
        SPLAT_CUDA(cudaMemcpyAsync(s->d_ftri, d_tris, sizeof(splat_ftri_t) * (size_t)s->n_tris,
                                   cudaMemcpyDeviceToDevice, st),
                   "scene_rebuild copy");
    ProfScope ps(SPLAT_KERNEL_AUX, st);
    return scene_rebuild_gpu(s, st);
}

splat_status_t splat_scene_update(splat_scene_t* s, const splat_ftri_t* d_tris, void* stream) {
    if (!s || !d_tris) return fail(SPLAT_ERR_INVALID, "scene_update: null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (s->gpu_bvh) return splat_scene_rebuild(s, d_tris, stream);
    if (d_tris != s->d_ftri)
        SPLAT_CUDA(cudaMemcpyAsync(s->d_ftri, d_tris, sizeof(splat_ftri_t) * (size_t)s->n_tris,
                                   cudaMemcpyDeviceToDevice, st),
                   "scene_update copy");
    return scene_pack(s, st);
}

// ---------------------------------------------------------------------------
// plugin boundary
// ---------------------------------------------------------------------------
static bool light_ok(const splat_rect_light_t* L, int64_t upscale) {
    return L && upscale >= 1 && L->res1 / upscale >= 1 && L->res2 / upscale >= 1;
}

splat_status_t splat_rays_from_light(const splat_rect_light_t* light, int64_t upscale,
                                     const splat_lambda_mode_t* lambda_mode, uint64_t seed, uint32_t light_index,
                                     splat_adray_t* d_rays, void* stream) {
    if (!light_ok(light, upscale) || !d_rays) return fail(SPLAT_ERR_INVALID, "rays_from_light: bad light or output");
    GenParams g;
    g.light = *light;
    g.upscale = upscale;
    g.lm = lambda_mode ? *lambda_mode : splat_lambda_mode_t{SPLAT_LAMBDA_FIXED, 1, 550.0f, 550.0f};
    if (g.lm.mode == SPLAT_LAMBDA_STRATIFIED && g.lm.n_strata < 1) return fail(SPLAT_ERR_INVALID, "n_strata < 1");
    g.seed = seed;
    g.light_index = light_index;
    g.ray_begin = 0;
    const int64_t n = (light->res1 / upscale) * (light->res2 / upscale);
    ProfScope ps(SPLAT_KERNEL_GENERATE, reinterpret_cast<cudaStream_t>(stream));
    SPLAT_CUDA(launch_generate_aos(g, n, d_rays, reinterpret_cast<cudaStream_t>(stream)), "rays_from_light");
    return SPLAT_OK;
}

splat_status_t splat_next_hit_brute(const splat_adray_t* d_rays, int64_t n_rays, const splat_ntri_t* d_n_tris,
                                    int64_t n_tris, uint64_t* d_tmp, int32_t* d_hit_idx, void* stream) {
    if (n_rays < 0 || n_tris < 0) return fail(SPLAT_ERR_INVALID, "next_hit_brute: negative size");
    if (n_rays == 0) return SPLAT_OK;
    if (!d_rays || !d_tmp || !d_hit_idx || (n_tris > 0 && !d_n_tris))
        return fail(SPLAT_ERR_INVALID, "next_hit_brute: null pointer");
    ProfScope ps(SPLAT_KERNEL_HIT_BRUTE, reinterpret_cast<cudaStream_t>(stream));
    SPLAT_CUDA(launch_hit_brute_ntris(d_rays, n_rays, d_n_tris, n_tris, d_tmp, d_hit_idx, sm_count_current(),
                                      reinterpret_cast<cudaStream_t>(stream)),
               "next_hit_brute");
    return SPLAT_OK;
}

splat_status_t splat_next_hit_brute_static(const splat_adray_t* d_rays, int64_t n_rays, const splat_ntri_t* d_n_tris,
                                           int64_t n_tris, int32_t* d_hit_idx, void* stream) {
    if (n_rays < 0 || n_tris < 0) return fail(SPLAT_ERR_INVALID, "next_hit_brute_static: negative size");
    if (n_rays > SPLAT_STATIC_HIT_MAX_RAYS)
        return fail(SPLAT_ERR_INVALID, "next_hit_brute_static: n_rays " + std::to_string(n_rays) +
                                           " exceeds the static scratch of " +
                                           std::to_string(SPLAT_STATIC_HIT_MAX_RAYS) + " rays");
    if (n_rays == 0) return SPLAT_OK;
    if (!d_rays || !d_hit_idx || (n_tris > 0 && !d_n_tris))
        return fail(SPLAT_ERR_INVALID, "next_hit_brute_static: null pointer");
    ProfScope ps(SPLAT_KERNEL_HIT_BRUTE, reinterpret_cast<cudaStream_t>(stream));
    SPLAT_CUDA(launch_hit_brute_ntris_static(d_rays, n_rays, d_n_tris, n_tris, d_hit_idx, sm_count_current(),
                                             reinterpret_cast<cudaStream_t>(stream)),
               "next_hit_brute_static");
    return SPLAT_OK;
}

static splat_status_t hit_any(const splat_scene_t* s, int32_t hitter, const RaySrc& src, int64_t cap,
                              int32_t* hit_idx, float* hit_t, uint64_t* tmp, cudaStream_t st) {
    cudaError_t e;
    const bool bvh = hitter == SPLAT_HITTER_BVH || hitter == SPLAT_HITTER_BVH2;
    ProfScope ps(bvh && s->d_nodes ? SPLAT_KERNEL_HIT_BVH : SPLAT_KERNEL_HIT_BRUTE, st);
    if (bvh) {
        if (!s->d_nodes) {
            if (s->n_recs > 0) return fail(SPLAT_ERR_INVALID, "BVH hitter on a scene created without BVH");
            e = launch_hit_brute(src, cap, s->d_brute, s->d_boxes, 0, hit_idx, hit_t, nullptr, s->d_err,
                                 sm_count_current(), st);
        } else if (hitter == SPLAT_HITTER_BVH) {
            e = launch_hit_bvh4(src, cap, Bvh4View{s->d_nodes4, s->d_bvh}, hit_idx, hit_t, s->d_err,
                                sm_count_current(), st);
        } else {
            e = launch_hit_bvh(src, cap, BvhView{s->d_nodes, s->d_bvh}, hit_idx, hit_t, s->d_err, sm_count_current(),
                               st);
        }
    } else if (hitter == SPLAT_HITTER_BRUTE) {
        e = launch_hit_brute(src, cap, s->d_brute, s->d_boxes, s->n_recs, hit_idx, hit_t, tmp, s->d_err,
                             sm_count_current(), st);
    } else {
        return fail(SPLAT_ERR_INVALID, "unknown hitter");
    }
    if (e != cudaSuccess) return cuda_fail(e, "hit kernel");
    return SPLAT_OK;
}

splat_status_t splat_next_hit(const splat_scene_t* scene, int32_t hitter, const splat_adray_t* d_rays, int64_t n_rays,
                              int32_t* d_hit_idx, float* d_hit_t, void* stream) {
    if (!scene || n_rays < 0) return fail(SPLAT_ERR_INVALID, "next_hit: bad scene or size");
    if (n_rays == 0) return SPLAT_OK;
    if (!d_rays || !d_hit_idx) return fail(SPLAT_ERR_INVALID, "next_hit: null pointer");
    RaySrc src{};
    src.aos = d_rays;
    src.n = n_rays;
    src.packet = packet_for(2);
    return hit_any(scene, hitter, src, n_rays, d_hit_idx, d_hit_t, nullptr, reinterpret_cast<cudaStream_t>(stream));
}

size_t splat_run_evolution_workspace_size(int64_t n_rays) { return n_rays <= 0 ? kAlign : work_bytes(n_rays); }

static SplatParams make_splat(const float* spectrum, int32_t n_lambda, int64_t upscale, void* map, int32_t accum,
                              int32_t frac_bits, int64_t w, int64_t h) {
    SplatParams sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.map = map;
    sp.accum = accum;
    sp.scale = std::ldexp(1.0f, frac_bits);
    sp.w = w;
    sp.h = h;
    sp.n_lambda = n_lambda;
    for (int i = 0; i < n_lambda; ++i) sp.spectrum[i] = spectrum[i];
    sp.n_delta = (int32_t)upscale;
    // upres(N), src/alg_types.jl:108
    for (int k = 1; k <= sp.n_delta; ++k)
        sp.deltas[k - 1] = ((float)k / (float)sp.n_delta - 0.5f) - (1.0f / (2.0f * (float)sp.n_delta));
    sp.n_samples = (n_lambda > 0 ? n_lambda : 1) * sp.n_delta * sp.n_delta;
    // splat kernel: one lane per (ray, plane)
    const int planes = n_lambda > 0 ? n_lambda : 1;
    int l2 = 0;
    while ((1 << l2) < planes && l2 < 5) ++l2;
    sp.lanes_log2 = l2;
    sp.chunks = (planes + (1 << l2) - 1) >> l2;
    sp.inv_nd = 1.0f / (float)sp.n_delta;
    sp.inv_nd2 = 1.0f / (float)(sp.n_delta * sp.n_delta);
    return sp;
}

static splat_status_t check_map(const float* spectrum, int32_t n_lambda, int64_t upscale, const void* map,
                                int32_t accum, int32_t frac_bits, int64_t w, int64_t h) {
    if (!map) return fail(SPLAT_ERR_INVALID, "light map is null");
    if (n_lambda < 0 || n_lambda > SPLAT_MAX_LAMBDA || (n_lambda > 0 && !spectrum))
        return fail(SPLAT_ERR_INVALID, "n_lambda must be 0..64 with a spectrum");
    if (upscale < 1 || upscale > 16) return fail(SPLAT_ERR_INVALID, "upscale must be 1..16");
    if (accum != SPLAT_ACCUM_F32 && accum != SPLAT_ACCUM_I32) return fail(SPLAT_ERR_INVALID, "unknown accumulation");
    if (frac_bits < 0 || frac_bits > 30) return fail(SPLAT_ERR_INVALID, "frac_bits must be 0..30");
    if (w < 1 || h < 1 || w > (1 << 24) || h > (1 << 24)) return fail(SPLAT_ERR_INVALID, "bad light map size");
    if (w * h * (int64_t)(n_lambda > 0 ? n_lambda : 1) >= (int64_t(1) << 31))
        return fail(SPLAT_ERR_INVALID, "light map larger than 2^31 texels");
    return SPLAT_OK;
}

splat_status_t splat_run_evolution(const splat_scene_t* scene, int32_t hitter, splat_adray_t* d_rays, int64_t n_rays,
                                   int32_t depth, const splat_material_t* material, float force_rand, uint64_t seed,
                                   uint32_t flags, int32_t* d_hit_idx, void* d_workspace, size_t workspace_bytes,
                                   void* stream) {
    if (!scene || n_rays < 0 || depth < 0 || depth > 64) return fail(SPLAT_ERR_INVALID, "run_evolution: bad arguments");
    if (!valid_material(material)) return fail(SPLAT_ERR_INVALID, "run_evolution: bad material");
    if (n_rays == 0) return SPLAT_OK;
    if (!d_rays || !d_hit_idx || !d_workspace) return fail(SPLAT_ERR_INVALID, "run_evolution: null pointer");
    if (workspace_bytes < work_bytes(n_rays)) return fail(SPLAT_ERR_WORKSPACE, "run_evolution: workspace too small");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Work w = carve_work(d_workspace, n_rays);
    SPLAT_CUDA(cudaMemsetAsync(w.counts, 0, kCounterBytes, st), "memset counters");
    {
        ProfScope ps(SPLAT_KERNEL_AUX, st);
        SPLAT_CUDA(launch_aos_to_soa(d_rays, n_rays, w.a, &w.counts[0], st), "aos_to_soa");
    }
    RaySoA cur = w.a, nxt = w.b;
    EvolveArgs ea;
    std::memset(&ea, 0, sizeof(ea));
    ea.tris = scene->d_ftri;
    ea.n_tris = scene->n_tris;
    ea.err = scene->d_err;
    ea.first_diffuse = scene->first_diffuse;
    ea.material = *material;
    ea.seed = seed;
    ea.force_rand = force_rand;
    ea.quirks = (flags & SPLAT_FLAG_REF_QUIRKS) ? 1 : 0;
    ea.aos = d_rays;
    for (int32_t b = 1; b <= depth; ++b) {
        RaySrc src{cur.f, cur.ignore, cur.cap, nullptr, &w.counts[b - 1], 0,
                   reinterpret_cast<unsigned long long*>(&w.counts[kFetchBase + b]), packet_for(b)};
        splat_status_t rc = hit_any(scene, hitter, src, n_rays, w.hit, nullptr, w.tmp, st);
        if (rc != SPLAT_OK) return rc;
        ea.in = cur;
        ea.out = nxt;
        ea.in_count = &w.counts[b - 1];
        ea.out_count = &w.counts[b];
        ea.hit_idx = w.hit;
        ea.bounce = (uint32_t)b;
        ea.last = 0;
        {
            ProfScope ps(SPLAT_KERNEL_EVOLVE, st);
            SPLAT_CUDA(launch_evolve_plugin(ea, n_rays, sm_count_current(), st), "evolve");
        }
        std::swap(cur, nxt);
    }
    {
        ProfScope ps(SPLAT_KERNEL_AUX, st);
        SPLAT_CUDA(launch_soa_to_aos(cur, &w.counts[depth], d_rays, kStatusActive, st), "soa_to_aos");
    }
    // realign: the hit of every ray's final state (src/tracer.jl:279-280)
    RaySrc all{};
    all.aos = d_rays;
    all.n = n_rays;
    return hit_any(scene, hitter, all, n_rays, d_hit_idx, nullptr, w.tmp, st);
}

splat_status_t splat_evolve(const splat_scene_t* scene, splat_adray_t* d_rays, int64_t n_rays,
                            const int32_t* d_hit_idx, const float* d_rndm, const splat_material_t* material,
                            float force_rand, uint64_t seed, uint32_t bounce, uint32_t flags, void* stream) {
    if (!scene || n_rays < 0) return fail(SPLAT_ERR_INVALID, "evolve: bad arguments");
    if (!valid_material(material)) return fail(SPLAT_ERR_INVALID, "evolve: bad material");
    if (n_rays == 0) return SPLAT_OK;
    if (!d_rays || !d_hit_idx) return fail(SPLAT_ERR_INVALID, "evolve: null pointer");
    EvolveArgs ea;
    std::memset(&ea, 0, sizeof(ea));
    ea.tris = scene->d_ftri;
    ea.n_tris = scene->n_tris;
    ea.err = scene->d_err;
    ea.first_diffuse = scene->first_diffuse;
    ea.material = *material;
    ea.seed = seed;
    ea.bounce = bounce;
    ea.force_rand = force_rand;
    ea.quirks = (flags & SPLAT_FLAG_REF_QUIRKS) ? 1 : 0;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    ProfScope ps(SPLAT_KERNEL_EVOLVE, st);
    SPLAT_CUDA(launch_evolve_aos(d_rays, n_rays, d_hit_idx, d_rndm, ea, sm_count_current(), st), "evolve");
    return SPLAT_OK;
}

static size_t partition_bytes(int64_t n_rays) {
    return kAlign + (size_t)(n_rays > 0 ? n_rays : 0) * sizeof(splat_adray_t);
}

size_t splat_partition_workspace_size(int64_t n_rays) { return partition_bytes(n_rays); }

splat_status_t splat_partition(splat_adray_t* d_rays, int64_t n_rays, int64_t* d_n_active, void* d_workspace,
                               size_t workspace_bytes, void* stream) {
    if (n_rays < 0 || !d_n_active || !d_workspace) return fail(SPLAT_ERR_INVALID, "partition: bad arguments");
    if (n_rays > 0 && !d_rays) return fail(SPLAT_ERR_INVALID, "partition: null rays");
    if (workspace_bytes < partition_bytes(n_rays)) return fail(SPLAT_ERR_WORKSPACE, "partition: workspace too small");
    if (reinterpret_cast<uintptr_t>(d_workspace) % 16) return fail(SPLAT_ERR_INVALID, "partition: workspace not 16-byte aligned");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int64_t* counts = reinterpret_cast<int64_t*>(d_workspace);
    splat_adray_t* swap = reinterpret_cast<splat_adray_t*>(static_cast<char*>(d_workspace) + kAlign);
    {
        ProfScope ps(SPLAT_KERNEL_AUX, st);
        SPLAT_CUDA(launch_partition(d_rays, n_rays, swap, counts, sm_count_current(), st), "partition");
    }
    SPLAT_CUDA(cudaMemcpyAsync(d_n_active, counts, sizeof(int64_t), cudaMemcpyDeviceToDevice, st), "partition count");
    return SPLAT_OK;
}

splat_status_t splat_continuum_light_map(const splat_scene_t* scene, splat_adray_t* d_rays, int64_t n_rays,
                                         const int32_t* d_hit_idx, const float* spectrum, int32_t n_lambda,
                                         int64_t upscale, void* d_tex, int32_t accum, int32_t frac_bits,
                                         int64_t map_w, int64_t map_h, void* stream) {
    if (!scene || n_rays < 0) return fail(SPLAT_ERR_INVALID, "continuum_light_map: bad arguments");
    splat_status_t rc = check_map(spectrum, n_lambda, upscale, d_tex, accum, frac_bits, map_w, map_h);
    if (rc != SPLAT_OK) return rc;
    if (n_rays == 0) return SPLAT_OK;
    if (!d_rays || !d_hit_idx) return fail(SPLAT_ERR_INVALID, "continuum_light_map: null pointer");
    SplatParams sp = make_splat(spectrum, n_lambda, upscale, d_tex, accum, frac_bits, map_w, map_h);
    ProfScope ps(SPLAT_KERNEL_EVOLVE, reinterpret_cast<cudaStream_t>(stream));
    SPLAT_CUDA(launch_light_map(d_rays, n_rays, d_hit_idx, scene->d_ftri, scene->n_tris, scene->d_err, sp,
                                sm_count_current(),
                                reinterpret_cast<cudaStream_t>(stream)),
               "light map");
    return SPLAT_OK;
}

// ---------------------------------------------------------------------------
// fused trace step
// ---------------------------------------------------------------------------


// A side stream per (device, caller stream) of the calling host thread, with
// fork / join events, for splats that run while later bounces trace.
namespace {
constexpr int kSideEvents = 10;
constexpr int kMaxTraceParts = 4;
constexpr int64_t kSplitMinRays = int64_t(1) << 17;  // smaller steps stay in one range
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t ev[kSideEvents] = {};
    cudaStream_t part[kMaxTraceParts - 1] = {};   // streams of the concurrent ray ranges
    cudaEvent_t part_ev[kMaxTraceParts] = {};     // fork, then one join per extra range
};

cudaError_t part_streams_ready(SideStream* x, int k) {
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < k; ++i)
        if (!x->part[i] && (e = cudaStreamCreateWithFlags(&x->part[i], cudaStreamNonBlocking)) != cudaSuccess) return e;
    for (int i = 0; i <= k; ++i)
        if (!x->part_ev[i] && (e = cudaEventCreateWithFlags(&x->part_ev[i], cudaEventDisableTiming)) != cudaSuccess)
            return e;
    return cudaSuccess;
}

// Workspace of a step over cnt rays run as `parts` concurrent ranges.
size_t trace_ws_bytes(int64_t cnt, int parts) {
    return parts <= 1 ? work_bytes(cnt) : (size_t)parts * work_bytes((cnt + parts - 1) / parts);
}
}  // namespace

// room for the step run as up to kMaxTraceParts concurrent ranges, plus the
// statistics block splat_trace_forward_host keeps at the end
constexpr size_t kHostStatsBytes = 256;

size_t splat_trace_workspace_size(int64_t n_rays) {
    if (n_rays <= 0) return kAlign;
    size_t m = 0;
    for (int p = 1; p <= kMaxTraceParts; ++p) m = std::max(m, trace_ws_bytes(n_rays, p));
    return m + kHostStatsBytes;
}

// At most kSideStreams per host thread: a caller that cycles through many
// short-lived streams gets the least recently used side stream destroyed
// (CUDA releases a stream and its events once their pending work is done).
constexpr size_t kSideStreams = 32;

static cudaError_t side_stream_for(cudaStream_t caller, SideStream** out) {
    thread_local std::map<std::pair<int, cudaStream_t>, std::pair<uint64_t, SideStream>> streams;
    thread_local uint64_t clock = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const std::pair<int, cudaStream_t> key{dev, caller};
    if (streams.find(key) == streams.end() && streams.size() >= kSideStreams) {
        auto lru = streams.begin();
        for (auto it = streams.begin(); it != streams.end(); ++it)
            if (it->second.first < lru->second.first) lru = it;
        SideStream& old = lru->second.second;
        for (cudaEvent_t ev : old.ev)
            if (ev) cudaEventDestroy(ev);
        for (cudaEvent_t ev : old.part_ev)
            if (ev) cudaEventDestroy(ev);
        for (cudaStream_t ps : old.part)
            if (ps) cudaStreamDestroy(ps);
        if (old.s) cudaStreamDestroy(old.s);
        streams.erase(lru);
    }
    auto& entry = streams[key];
    entry.first = ++clock;
    SideStream& x = entry.second;
    if (!x.s) {
        if ((e = cudaStreamCreateWithFlags(&x.s, cudaStreamNonBlocking)) != cudaSuccess) return e;
        for (cudaEvent_t& ev : x.ev)
            if ((e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) return e;
    }
    *out = &x;
    return cudaSuccess;
}

static int64_t grid_rays(const splat_trace_params_t* P) {
    return (P->light.res1 / P->upscale) * (P->light.res2 / P->upscale);
}

// The forward step over rays [rb, rb + cnt) of the grid in the work area w,
// on stream st: generate, depth x {hit, evolve (+ compaction, diffuse
// queue)}, the splat (segments on a side stream), the statistics.  The map
// and d_stats were cleared by the caller; statistics accumulate.
static splat_status_t trace_part(const splat_scene_t* scene, const splat_trace_params_t* P, void* d_map, Work w,
                                 int64_t rb, int64_t cnt, splat_trace_stats_t* d_stats, cudaStream_t st, int sm) {
    GenParams g;
    g.light = P->light;
    g.upscale = P->upscale;
    g.lm = P->lambda_mode;
    g.seed = P->seed;
    g.light_index = 0;
    g.ray_begin = rb;
    {
        ProfScope ps(SPLAT_KERNEL_GENERATE, st);
        SPLAT_CUDA(launch_generate_soa(g, cnt, w.a, &w.counts[0], st), "generate");
    }

    EvolveArgs ea;
    std::memset(&ea, 0, sizeof(ea));
    ea.tris = scene->d_ftri;
    ea.n_tris = scene->n_tris;
    ea.err = scene->d_err;
    ea.first_diffuse = scene->first_diffuse;
    ea.material = P->material;
    ea.seed = P->seed;
    ea.force_rand = P->force_rand;
    ea.quirks = (P->flags & SPLAT_FLAG_REF_QUIRKS) ? 1 : 0;
    const SplatParams sp =
        make_splat(P->spectrum, P->n_lambda, P->upscale, d_map, P->accum, P->frac_bits, P->map_w, P->map_h);
    ea.splat_q = w.q;
    ea.splat_count = &w.counts[kSplatCount];
    // Splat overlap: the queue segment of bounces (seg, b] is splatted on the
    // side stream from a snapshot of the queue length, while the main stream
    // traces bounce b + 1.  Integer maps are sums, so the segmentation does
    // not change them; float maps change only in summation order.
    const int overlap = P->depth > 1 ? g_tune[SPLAT_TUNE_SPLAT_OVERLAP].load() : 0;
    SideStream* side = nullptr;
    if (overlap) SPLAT_CUDA(side_stream_for(st, &side), "side stream");
    splat_status_t rc = SPLAT_OK;
    int64_t* snap = &w.counts[kSplatSnap];
    int seg = 0, n_ev = 0;
    RaySoA cur = w.a, nxt = w.b;
    const int order_bits = g_tune[SPLAT_TUNE_RAY_ORDER].load();
    for (int32_t b = 1; b <= P->depth; ++b) {
        RaySrc src{cur.f, cur.ignore, cur.cap, nullptr, &w.counts[b - 1], 0,
                   reinterpret_cast<unsigned long long*>(&w.counts[kFetchBase + b]), packet_for(b)};
        {
            // the first bounce's rays are the light grid's columns in order
            // (the range starts on a column): packet warps take 8 x 4 tiles
            // of it instead of 32 x 1 strips, and evolve takes them in the
            // same order, so its survivors leave as compact patches
            const int64_t gh = P->light.res1 / P->upscale;
            if (b == 1 && rb % gh == 0 && gh <= (int64_t)kGridTileMaxRows) src.tile_h = (int32_t)gh;
        }
        if (b >= 2 && order_bits > 0 && P->hitter == SPLAT_HITTER_BVH && scene->d_nodes4 && scene->d_bvh_pos) {
            // secondary rays in coherent order: (octant, position of the triangle they leave)
            ProfScope ps(SPLAT_KERNEL_AUX, st);
            SPLAT_CUDA(launch_ray_order(cur.f, cur.ignore, cur.cap, &w.counts[b - 1], scene->d_bvh_pos,
                                        scene->n_tris, order_bits, w.order, &src.perm, sm, st),
                       "ray order");
        }
        rc = hit_any(scene, P->hitter, src, cnt, w.hit, nullptr, w.tmp, st);
        if (rc != SPLAT_OK) return rc;
        ea.in = cur;
        ea.out = nxt;
        ea.in_count = &w.counts[b - 1];
        ea.out_count = &w.counts[b];
        ea.hit_idx = w.hit;
        ea.bounce = (uint32_t)b;
        ea.last = b == P->depth ? 1 : 0;
        ea.tile_h = src.tile_h;  // the first bounce's survivors leave in tile order
        {
            ProfScope ps(SPLAT_KERNEL_EVOLVE, st);
            SPLAT_CUDA(launch_evolve_trace(ea, cnt, sm, st), "evolve");
        }
        std::swap(cur, nxt);
        if (overlap && b < P->depth && (overlap == 2 || b == P->depth - 1)) {
            {
                ProfScope ps(SPLAT_KERNEL_AUX, st);
                SPLAT_CUDA(launch_copy_count(&w.counts[kSplatCount], &snap[b], st), "queue snapshot");
            }
            SPLAT_CUDA(cudaEventRecord(side->ev[n_ev], st), "fork");
            SPLAT_CUDA(cudaStreamWaitEvent(side->s, side->ev[n_ev++], 0), "fork");
            ProfScope ps(SPLAT_KERNEL_SPLAT, side->s);
            SPLAT_CUDA(launch_splat(w.q, &snap[seg], &snap[b], scene->d_ftri, sp, d_stats, sm, side->s), "splat");
            seg = b;
        }
    }
    {
        ProfScope ps(SPLAT_KERNEL_SPLAT, st);
        SPLAT_CUDA(launch_splat(w.q, seg ? &snap[seg] : nullptr, &w.counts[kSplatCount], scene->d_ftri, sp, d_stats,
                                sm, st),
                   "splat");
    }
    if (seg) {
        SPLAT_CUDA(cudaEventRecord(side->ev[n_ev], side->s), "join");
        SPLAT_CUDA(cudaStreamWaitEvent(st, side->ev[n_ev], 0), "join");
    }
    if (d_stats) {
        ProfScope ps(SPLAT_KERNEL_AUX, st);
        SPLAT_CUDA(launch_stats_finish(w.counts, P->depth, &w.counts[kSplatCount], d_stats, scene->d_err, st),
                   "stats");
    }
    return SPLAT_OK;
}


splat_status_t splat_trace_forward(const splat_scene_t* scene, const splat_trace_params_t* P, void* d_map,
                                   void* d_workspace, size_t workspace_bytes, splat_trace_stats_t* d_stats,
                                   void* stream) {
    if (!scene || !P) return fail(SPLAT_ERR_INVALID, "trace_forward: null scene or params");
    if (!light_ok(&P->light, P->upscale)) return fail(SPLAT_ERR_INVALID, "trace_forward: bad light / upscale");
    if (P->depth < 1 || P->depth > 8) return fail(SPLAT_ERR_INVALID, "trace_forward: depth must be 1..8");
    if (!valid_material(&P->material)) return fail(SPLAT_ERR_INVALID, "trace_forward: bad material");
    if (P->lambda_mode.mode == SPLAT_LAMBDA_STRATIFIED && P->lambda_mode.n_strata < 1)
        return fail(SPLAT_ERR_INVALID, "trace_forward: n_strata < 1");
    splat_status_t rc =
        check_map(P->spectrum, P->n_lambda, P->upscale, d_map, P->accum, P->frac_bits, P->map_w, P->map_h);
    if (rc != SPLAT_OK) return rc;
    if ((P->hitter == SPLAT_HITTER_BVH || P->hitter == SPLAT_HITTER_BVH2) && !scene->d_nodes && scene->n_recs > 0)
        return fail(SPLAT_ERR_INVALID, "trace_forward: BVH hitter on a scene without BVH");
    const int64_t n_grid = grid_rays(P);
    const int64_t rb = P->ray_begin < 0 ? 0 : P->ray_begin;
    const int64_t re = (P->ray_end <= 0 || P->ray_end > n_grid) ? n_grid : P->ray_end;
    if (n_grid >= (int64_t(1) << 32)) return fail(SPLAT_ERR_INVALID, "trace_forward: more than 2^32 rays");
    const int64_t cnt = re - rb;
    if (cnt <= 0) return fail(SPLAT_ERR_INVALID, "trace_forward: empty ray range");
    if (!d_workspace || workspace_bytes < work_bytes(cnt))
        return fail(SPLAT_ERR_WORKSPACE, "trace_forward: workspace smaller than splat_trace_workspace_size");
    // concurrent ray ranges (SPLAT_TUNE_TRACE_SPLIT), as many as the workspace holds
    int parts = cnt >= kSplitMinRays ? g_tune[SPLAT_TUNE_TRACE_SPLIT].load() : 1;
    while (parts > 1 && trace_ws_bytes(cnt, parts) > workspace_bytes) --parts;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int sm = sm_count_current();
    if (d_stats) SPLAT_CUDA(cudaMemsetAsync(d_stats, 0, sizeof(splat_trace_stats_t), st), "memset stats");
    const int64_t planes = P->n_lambda > 0 ? P->n_lambda : 1;
    if (P->zero_map) SPLAT_CUDA(cudaMemsetAsync(d_map, 0, (size_t)P->map_w * P->map_h * planes * 4, st), "clear map");
    if (parts == 1) {
        Work w = carve_work(d_workspace, cnt);
        SPLAT_CUDA(cudaMemsetAsync(w.counts, 0, kCounterBytes, st), "memset counters");
        return trace_part(scene, P, d_map, w, rb, cnt, d_stats, st, sm);
    }
    // the ranges are independent (ray ids are grid indices); each runs on its
    // own stream after the clears above and joins the caller's stream
    SideStream* side = nullptr;
    SPLAT_CUDA(side_stream_for(st, &side), "part streams");
    SPLAT_CUDA(part_streams_ready(side, parts - 1), "part streams");
    SPLAT_CUDA(cudaEventRecord(side->part_ev[0], st), "fork ranges");
    const int64_t each = (cnt + parts - 1) / parts;
    const size_t region = work_bytes(each);
    char* base = static_cast<char*>(d_workspace);
    for (int i = 0; i < parts; ++i) {
        const int64_t lo = rb + (int64_t)i * each;
        const int64_t n_i = std::min(each, rb + cnt - lo);
        cudaStream_t si = i == 0 ? st : side->part[i - 1];
        if (i > 0) SPLAT_CUDA(cudaStreamWaitEvent(si, side->part_ev[0], 0), "fork ranges");
        Work w = carve_work(base + (size_t)i * region, n_i);
        SPLAT_CUDA(cudaMemsetAsync(w.counts, 0, kCounterBytes, si), "memset counters");
        splat_status_t rc = trace_part(scene, P, d_map, w, lo, n_i, d_stats, si, sm);
        if (rc != SPLAT_OK) return rc;
    }
    for (int i = 1; i < parts; ++i) {
        SPLAT_CUDA(cudaEventRecord(side->part_ev[i], side->part[i - 1]), "join ranges");
        SPLAT_CUDA(cudaStreamWaitEvent(st, side->part_ev[i], 0), "join ranges");
    }
    return SPLAT_OK;
}

splat_status_t splat_trace_forward_host(splat_scene_t* scene, const splat_ftri_t* host_tris,
                                        const splat_trace_params_t* P, void* host_map, void* d_map, void* d_workspace,
                                        size_t workspace_bytes, splat_trace_stats_t* host_stats, void* stream) {
    if (!scene || !P || !host_map) return fail(SPLAT_ERR_INVALID, "trace_forward_host: null argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (host_tris) {
        SPLAT_CUDA(cudaMemcpyAsync(scene->d_ftri, host_tris, sizeof(splat_ftri_t) * (size_t)scene->n_tris,
                                   cudaMemcpyHostToDevice, st),
                   "upload triangles");
        splat_status_t rc = scene_pack(scene, st);
        if (rc != SPLAT_OK) return rc;
    }
    // the statistics go to the last kHostStatsBytes of the workspace
    if (workspace_bytes < kHostStatsBytes + kAlign)
        return fail(SPLAT_ERR_WORKSPACE, "trace_forward_host: workspace smaller than splat_trace_workspace_size");
    const size_t usable = (workspace_bytes - kHostStatsBytes) & ~size_t(15);
    splat_trace_stats_t* d_stats = reinterpret_cast<splat_trace_stats_t*>(static_cast<char*>(d_workspace) + usable);
    splat_status_t rc = splat_trace_forward(scene, P, d_map, d_workspace, usable, d_stats, stream);
    if (rc != SPLAT_OK) return rc;
    const int64_t planes = P->n_lambda > 0 ? P->n_lambda : 1;
    SPLAT_CUDA(cudaMemcpyAsync(host_map, d_map, (size_t)P->map_w * P->map_h * planes * 4, cudaMemcpyDeviceToHost, st),
               "download map");
    if (host_stats)
        SPLAT_CUDA(cudaMemcpyAsync(host_stats, d_stats, sizeof(*host_stats), cudaMemcpyDeviceToHost, st),
                   "download statistics");
    SPLAT_CUDA(cudaStreamSynchronize(st), "trace_forward_host sync");
    int32_t err = 0;
    SPLAT_CUDA(cudaMemcpy(&err, scene->d_err, sizeof(err), cudaMemcpyDeviceToHost), "read error word");
    if (err) return fail(SPLAT_ERR_DEVICE, "trace_forward_host: kernel error word " + std::to_string(err));
    return SPLAT_OK;
}

splat_status_t splat_hit_work(int64_t out[4], int32_t reset, void* stream) {
    if (!out) return fail(SPLAT_ERR_INVALID, "hit_work: null output");
    uint64_t w[4] = {0, 0, 0, 0};
    SPLAT_CUDA(read_hit_work(w, reset != 0, reinterpret_cast<cudaStream_t>(stream)), "hit_work");
    for (int i = 0; i < 4; ++i) out[i] = (int64_t)w[i];
    return SPLAT_OK;
}

splat_status_t splat_set_tuning(int32_t key, int32_t value) {
    if (key < 0 || key >= SPLAT_TUNE_KEYS) return fail(SPLAT_ERR_INVALID, "set_tuning: unknown key");
    if (key == SPLAT_TUNE_SPLAT_AGGREGATE) {
        if (value != 0 && value != 1) return fail(SPLAT_ERR_INVALID, "set_tuning: aggregate must be 0 or 1");
    } else if (key == SPLAT_TUNE_BVH_PACKET) {
        if (value < 0 || value > 5) return fail(SPLAT_ERR_INVALID, "set_tuning: packet mode must be 0..5");
    } else if (key == SPLAT_TUNE_SPLAT_OVERLAP) {
        if (value < 0 || value > 2) return fail(SPLAT_ERR_INVALID, "set_tuning: splat overlap must be 0..2");
    } else if (key == SPLAT_TUNE_BVH_REFILL) {
        if (value < 0 || value > 32) return fail(SPLAT_ERR_INVALID, "set_tuning: refill threshold must be 0..32");
    } else if (key == SPLAT_TUNE_TRACE_SPLIT) {
        if (value < 1 || value > kMaxTraceParts) return fail(SPLAT_ERR_INVALID, "set_tuning: split must be 1..4");
    } else if (key == SPLAT_TUNE_BATCH_PERSISTENT) {
        if (value < 0 || value > 8) return fail(SPLAT_ERR_INVALID, "set_tuning: persistent pass share must be 0..8");
    } else if (key == SPLAT_TUNE_COUNT_WORK) {
        if (value != 0 && value != 1) return fail(SPLAT_ERR_INVALID, "set_tuning: count work must be 0 or 1");
    } else if (key == SPLAT_TUNE_BRUTE_TILE) {
        if (value != 32 && value != 64 && value != 128)
            return fail(SPLAT_ERR_INVALID, "set_tuning: brute tile must be 32, 64 or 128");
    } else if (key == SPLAT_TUNE_RAY_ORDER) {
        if (value != 0 && (value < 4 || value > 22))
            return fail(SPLAT_ERR_INVALID, "set_tuning: ray order bits must be 0 or 4..22");
    } else if (key == SPLAT_TUNE_TEST_WAIT_STALL) {
        if (value < 0 || value > (1 << 20)) return fail(SPLAT_ERR_INVALID, "set_tuning: stall tile must be 0..2^20");
    } else if (value < 1 || value > 256) {
        return fail(SPLAT_ERR_INVALID, "set_tuning: value must be 1..256");
    }
    g_tune[key] = value;
    return SPLAT_OK;
}

int32_t splat_get_tuning(int32_t key) { return key < 0 || key >= SPLAT_TUNE_KEYS ? -1 : g_tune[key].load(); }

splat_status_t splat_profile_create(int32_t max_launches, splat_profile_t** out) {
    if (!out || max_launches < 1 || max_launches > (1 << 20)) return fail(SPLAT_ERR_INVALID, "profile_create: bad argument");
    splat_profile* p = new (std::nothrow) splat_profile();
    if (!p) return fail(SPLAT_ERR_ALLOC, "profile_create: host allocation");
    p->max = max_launches;
    p->ev.resize(2 * (size_t)max_launches);
    p->kind.assign((size_t)max_launches, 0);
    p->kernels.assign((size_t)max_launches, 0);
    for (auto& e : p->ev) {
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) {
            for (auto& x : p->ev)
                if (x) cudaEventDestroy(x);
            delete p;
            return cuda_fail(r, "profile_create: cudaEventCreate");
        }
    }
    *out = p;
    return SPLAT_OK;
}

splat_status_t splat_profile_attach(splat_profile_t* profile) {
    g_prof = profile;
    return SPLAT_OK;
}

splat_status_t splat_profile_reset(splat_profile_t* p) {
    if (!p) return fail(SPLAT_ERR_INVALID, "profile_reset: null profile");
    p->used = 0;
    return SPLAT_OK;
}

splat_status_t splat_profile_read(splat_profile_t* p, int32_t kind, int64_t* launches, double* total_ms) {
    if (!p || kind < 0 || kind > SPLAT_KERNEL_KINDS) return fail(SPLAT_ERR_INVALID, "profile_read: bad argument");
    int64_t n = 0;
    double ms = 0.0;
    for (int32_t i = 0; i < p->used; ++i) {
        if (kind != SPLAT_KERNEL_KINDS && p->kind[(size_t)i] != kind) continue;
        SPLAT_CUDA(cudaEventSynchronize(p->ev[2 * (size_t)i + 1]), "profile_read: sync");
        float t = 0.f;
        SPLAT_CUDA(cudaEventElapsedTime(&t, p->ev[2 * (size_t)i], p->ev[2 * (size_t)i + 1]), "profile_read: elapsed");
        ms += t;
        n += p->kernels[(size_t)i];
    }
    if (launches) *launches = n;
    if (total_ms) *total_ms = ms;
    return SPLAT_OK;
}

splat_status_t splat_profile_destroy(splat_profile_t* p) {
    if (!p) return fail(SPLAT_ERR_INVALID, "profile_destroy: null profile");
    if (g_prof == p) g_prof = nullptr;
    for (auto& e : p->ev) cudaEventDestroy(e);
    delete p;
    return SPLAT_OK;
}

// ---------------------------------------------------------------------------
// batch engine
// ---------------------------------------------------------------------------
}  // extern "C"

struct splat_batch {
    int device = 0;
    int32_t max_items = 0;
    int64_t cap = 0;
    size_t item_bytes = 0;
    char* d_mem = nullptr;
    size_t d_bytes = 0;
    void* d_items = nullptr;
    void* d_fresh = nullptr;
    RaySoA a{}, b{}, q{};
    int32_t* hit = nullptr;
    int64_t* counts = nullptr;  // [0], [1]: ping-pong active counts, [2]: splat queue
    int32_t* d_err = nullptr;
    char* h_stage[2] = {nullptr, nullptr};  // pinned copies of the item table
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    int stage_idx = 0;
    std::vector<char> h_items;
    std::vector<uint8_t> used;
    std::vector<int64_t> rays;
    std::vector<int32_t> start, depth;
    std::vector<uint8_t> brute;  // item runs the per-ray brute-force hitter
    std::vector<int32_t> mat_kind;  // item's material kind
    std::vector<void*> maps;
    std::vector<size_t> map_bytes;
    std::vector<uint8_t> zero_map;
    int32_t tick = 0;
    int parity = 0;
    bool dirty = true;
    // ray order (SPLAT_TUNE_RAY_ORDER > 0): keys, permutation, bucket counts,
    // scan sums; buckets of the uploaded item table
    uint32_t* ord_keys = nullptr;
    int32_t* ord_perm = nullptr;
    uint32_t* ord_cnt = nullptr;
    uint32_t* ord_sums = nullptr;
    int64_t order_buckets = 0;
    cudaGraphExec_t exec = nullptr;
    // captured graphs: the splat of tick t on a side stream beside tick t + 1
    // (queues alternate by tick parity; q2 is allocated at the first such capture)
    RaySoA q2{};
    void* q2_mem = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t traced_ev[2] = {nullptr, nullptr}, splat_ev[2] = {nullptr, nullptr};
    bool splat_pending[2] = {false, false};
    bool overlap = false;    // set while capturing with the overlap
    int32_t cap_t1 = 0;      // host tick after the captured ticks
    int cap_parity1 = 0;     // buffer parity after them
    int32_t cap_t0 = 0;      // host tick and parity the captured ticks start from
    int cap_parity0 = 0;
};

namespace {

// ray order of the batch: keys and permutation per pool ray, bucket counts
// and the scan's tile sums for 2^kBatchOrderBits buckets
size_t batch_order_bytes(int64_t cap) {
    const int64_t buckets = int64_t(1) << kBatchOrderBits;
    return 2 * align_up(4 * (size_t)cap) + align_up(4 * (size_t)buckets) + align_up(4 * order_sums_count(buckets));
}

size_t batch_bytes(int32_t max_items, int64_t cap) {
    return align_up(batch_item_bytes() * (size_t)max_items) + align_up(batch_fresh_bytes()) + 3 * soa_bytes(cap) +
           align_up(4 * (size_t)cap) + kCounterBytes + batch_order_bytes(cap) + kAlign;
}

void batch_free(splat_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    cudaFree(b->d_mem);
    if (b->q2_mem) cudaFree(b->q2_mem);
    for (int i = 0; i < 2; ++i) {
        if (b->traced_ev[i]) cudaEventDestroy(b->traced_ev[i]);
        if (b->splat_ev[i]) cudaEventDestroy(b->splat_ev[i]);
    }
    if (b->side) cudaStreamDestroy(b->side);
    for (int i = 0; i < 2; ++i) {
        if (b->h_stage[i]) cudaFreeHost(b->h_stage[i]);
        if (b->stage_ev[i]) cudaEventDestroy(b->stage_ev[i]);
    }
    delete b;
}

// Pool rays still needed by items whose last tick is at or after `tick`.
int64_t pool_in_use(const splat_batch* b) {
    int64_t r = 0;
    for (int32_t s = 0; s < b->max_items; ++s)
        if (b->used[(size_t)s] && b->start[(size_t)s] + b->depth[(size_t)s] - 1 >= b->tick) r += b->rays[(size_t)s];
    return r;
}

splat_status_t batch_upload(splat_batch* b, cudaStream_t st) {
    if (!b->dirty) return SPLAT_OK;
    const int i = b->stage_idx;
    b->stage_idx ^= 1;
    SPLAT_CUDA(cudaEventSynchronize(b->stage_ev[i]), "batch: stage reuse");
    b->order_buckets =
        batch_assign_order_keys(b->h_items.data(), b->used.data(), b->max_items, kBatchOrderBits);
    std::memcpy(b->h_stage[i], b->h_items.data(), b->h_items.size());
    SPLAT_CUDA(cudaMemcpyAsync(b->d_items, b->h_stage[i], b->h_items.size(), cudaMemcpyHostToDevice, st),
               "batch: upload items");
    SPLAT_CUDA(cudaEventRecord(b->stage_ev[i], st), "batch: stage event");
    b->dirty = false;
    return SPLAT_OK;
}

// Enqueues one tick (no table upload).
// The second queue, side stream and fork / join events of a capture with
// the splat overlap, made on first use.
cudaError_t batch_overlap_ready(splat_batch* b) {
    cudaError_t e = cudaSuccess;
    if (!b->q2_mem) {
        e = cudaMalloc(&b->q2_mem, soa_bytes(b->cap) + kAlign);
        if (e != cudaSuccess) return e;
        char* p = reinterpret_cast<char*>(align_up(reinterpret_cast<size_t>(b->q2_mem)));
        b->q2 = carve_soa(p, b->cap);
    }
    if (!b->side && (e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking)) != cudaSuccess) return e;
    for (int i = 0; i < 2; ++i) {
        if (!b->traced_ev[i] && (e = cudaEventCreateWithFlags(&b->traced_ev[i], cudaEventDisableTiming)) != cudaSuccess)
            return e;
        if (!b->splat_ev[i] && (e = cudaEventCreateWithFlags(&b->splat_ev[i], cudaEventDisableTiming)) != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

splat_status_t batch_enqueue_tick(splat_batch* b, cudaStream_t st, int32_t* done_slots, int32_t max_done,
                                  int32_t* n_done) {
    int64_t fresh_rays = 0, cap_rays = 0;
    int32_t nd = 0;
    bool any_brute = false;
    int32_t kind = -2;  // material kind shared by every item in flight; -1 mixed
    for (int32_t s = 0; s < b->max_items; ++s) {
        if (!b->used[(size_t)s]) continue;
        const int32_t st0 = b->start[(size_t)s], last = st0 + b->depth[(size_t)s] - 1;
        if (b->tick < st0 || b->tick > last) continue;
        cap_rays += b->rays[(size_t)s];
        any_brute = any_brute || b->brute[(size_t)s];
        kind = kind == -2 || kind == b->mat_kind[(size_t)s] ? b->mat_kind[(size_t)s] : -1;
        if (b->tick == st0) {
            fresh_rays += b->rays[(size_t)s];
            if (b->zero_map[(size_t)s])
                SPLAT_CUDA(cudaMemsetAsync(b->maps[(size_t)s], 0, b->map_bytes[(size_t)s], st), "batch: clear map");
        }
        if (b->tick == last) {
            if (done_slots && nd < max_done) done_slots[nd] = s;
            ++nd;
        }
    }
    if (n_done) *n_done = nd;
    int64_t* cur_count = &b->counts[b->parity];
    int64_t* next_count = &b->counts[b->parity ^ 1];
    // with the overlap, tick t splats queue (t & 1) on the side stream; the
    // main stream reuses that queue two ticks later, after that splat
    const int qp = b->overlap ? (b->tick & 1) : 0;
    RaySoA queue = qp ? b->q2 : b->q;
    int64_t* queue_count = qp ? &b->counts[5] : &b->counts[2];
    if (b->overlap && b->splat_pending[qp]) {
        SPLAT_CUDA(cudaStreamWaitEvent(st, b->splat_ev[qp], 0), "batch: wait for the queue's splat");
        b->splat_pending[qp] = false;
    }
    SPLAT_CUDA(cudaMemsetAsync(next_count, 0, sizeof(int64_t), st), "batch: reset count");
    SPLAT_CUDA(cudaMemsetAsync(queue_count, 0, sizeof(int64_t), st), "batch: reset queue");
    SPLAT_CUDA(cudaMemsetAsync(&b->counts[3], 0, sizeof(int64_t), st), "batch: reset work counter");
    if (cap_rays > 0) {
        ProfScope ps(SPLAT_KERNEL_BATCH, st);
        BatchTickArgs a;
        a.items = b->d_items;
        a.n_slots = b->max_items;
        a.tick = b->tick;
        a.fresh = b->d_fresh;
        a.cur = b->parity ? b->b : b->a;
        a.next = b->parity ? b->a : b->b;
        a.queue = queue;
        a.cur_count = cur_count;
        a.next_count = next_count;
        a.queue_count = queue_count;
        a.fresh_rays = fresh_rays;
        a.cap_rays = cap_rays;
        a.hit_idx = b->hit;
        a.err = b->d_err;
        a.sm_count = sm_count_current();
        a.any_brute = any_brute;
        a.material_kind = kind < 0 ? -1 : kind;
        a.fetch = reinterpret_cast<unsigned long long*>(&b->counts[3]);
        const bool order = g_tune[SPLAT_TUNE_RAY_ORDER] > 0 && b->order_buckets > 0;
        a.order_buckets = order ? b->order_buckets : 0;
        a.order_keys = b->ord_keys;
        a.order_cnt = b->ord_cnt;
        a.order_sums = b->ord_sums;
        a.order_perm = b->ord_perm;
        if (b->overlap) {
            SPLAT_CUDA(launch_batch_trace(a, st), "batch tick");
            SPLAT_CUDA(cudaEventRecord(b->traced_ev[qp], st), "batch: fork");
            SPLAT_CUDA(cudaStreamWaitEvent(b->side, b->traced_ev[qp], 0), "batch: fork");
            SPLAT_CUDA(launch_batch_splat(a, b->side), "batch splat");
            SPLAT_CUDA(cudaEventRecord(b->splat_ev[qp], b->side), "batch: join");
            b->splat_pending[qp] = true;
        } else {
            SPLAT_CUDA(launch_batch_tick(a, st), "batch tick");
        }
        b->parity ^= 1;
    }
    b->tick += 1;
    return SPLAT_OK;
}

// Counters of a persistent pass in the batch's counter block (int64 slots).
constexpr int kPassCount = 16, kPassQCount = 26, kPassQMark = 28, kPassFetch = 40, kPassSplatFetch = 50,
              kPassBar = 60, kPassEnd = 64;

// Every tick from b->tick to `last` as one persistent launch over 1/share of
// the GPU (items all start at b->tick); the host bookkeeping advances as the
// tick-by-tick path would.
cudaError_t batch_enqueue_pass(splat_batch* b, cudaStream_t st, int32_t last, int share) {
    const int32_t t0 = b->tick;
    int32_t kind = -2;
    for (int32_t s = 0; s < b->max_items; ++s) {
        if (!b->used[(size_t)s] || b->start[(size_t)s] + b->depth[(size_t)s] - 1 < t0) continue;
        kind = kind == -2 || kind == b->mat_kind[(size_t)s] ? b->mat_kind[(size_t)s] : -1;
        if (b->start[(size_t)s] == t0 && b->zero_map[(size_t)s]) {
            cudaError_t e = cudaMemsetAsync(b->maps[(size_t)s], 0, b->map_bytes[(size_t)s], st);
            if (e != cudaSuccess) return e;
        }
    }
    cudaError_t e = cudaMemsetAsync(&b->counts[kPassCount], 0, sizeof(int64_t) * (kPassEnd - kPassCount), st);
    if (e != cudaSuccess) return e;
    BatchPassArgs a;
    a.items = b->d_items;
    a.fresh = b->d_fresh;
    a.n_slots = b->max_items;
    a.t0 = t0;
    a.n_ticks = last - t0 + 1;
    a.material_kind = kind < 0 ? -1 : kind;
    a.a = b->parity ? b->b : b->a;
    a.b = b->parity ? b->a : b->b;
    a.queue = b->q;
    a.count = &b->counts[kPassCount];
    a.qcount = &b->counts[kPassQCount];
    a.qmark = &b->counts[kPassQMark];
    a.fetch = reinterpret_cast<unsigned long long*>(&b->counts[kPassFetch]);
    a.splat_fetch = reinterpret_cast<unsigned long long*>(&b->counts[kPassSplatFetch]);
    a.bar = reinterpret_cast<unsigned*>(&b->counts[kPassBar]);
    a.hit_idx = b->hit;
    a.err = b->d_err;
    a.packet_mode = g_tune[SPLAT_TUNE_BVH_PACKET];
    {
        ProfScope ps(SPLAT_KERNEL_BATCH, st);
        e = launch_batch_pass(a, share, sm_count_current(), st);
        if (e != cudaSuccess) return e;
    }
    b->tick = last + 1;
    b->parity ^= a.n_ticks & 1;
    return cudaSuccess;
}

}  // namespace

extern "C" {

size_t splat_batch_device_bytes(int32_t max_items, int64_t max_pool_rays) {
    return max_items < 1 || max_pool_rays < 1 ? 0 : batch_bytes(max_items, max_pool_rays);
}

splat_status_t splat_batch_create(int32_t max_items, int64_t max_pool_rays, splat_batch_t** out) {
    if (!out) return fail(SPLAT_ERR_INVALID, "batch_create: out is null");
    *out = nullptr;
    if (max_items < 1 || max_items > 256) return fail(SPLAT_ERR_INVALID, "batch_create: max_items must be 1..256");
    if (max_pool_rays < 1 || max_pool_rays > (int64_t(1) << 31))
        return fail(SPLAT_ERR_INVALID, "batch_create: max_pool_rays must be 1..2^31");
    splat_batch* b = new (std::nothrow) splat_batch();
    if (!b) return fail(SPLAT_ERR_ALLOC, "batch_create: host allocation");
    cudaGetDevice(&b->device);
    b->max_items = max_items;
    b->cap = max_pool_rays;
    b->item_bytes = batch_item_bytes();
    b->d_bytes = batch_bytes(max_items, max_pool_rays);
    cudaError_t e = cudaMalloc(&b->d_mem, b->d_bytes);
    if (e != cudaSuccess) {
        delete b;
        return fail(SPLAT_ERR_ALLOC, std::string("batch_create: cudaMalloc: ") + cudaGetErrorString(e));
    }
    char* p = reinterpret_cast<char*>(align_up(reinterpret_cast<size_t>(b->d_mem)));
    b->d_items = p;
    p += align_up(b->item_bytes * (size_t)max_items);
    b->d_fresh = p;
    p += align_up(batch_fresh_bytes());
    b->a = carve_soa(p, max_pool_rays);
    b->b = carve_soa(p, max_pool_rays);
    b->q = carve_soa(p, max_pool_rays);
    b->hit = reinterpret_cast<int32_t*>(p);
    p += align_up(4 * (size_t)max_pool_rays);
    b->counts = reinterpret_cast<int64_t*>(p);
    b->d_err = reinterpret_cast<int32_t*>(p + 512);
    p += kCounterBytes;
    b->ord_keys = reinterpret_cast<uint32_t*>(p);
    p += align_up(4 * (size_t)max_pool_rays);
    b->ord_perm = reinterpret_cast<int32_t*>(p);
    p += align_up(4 * (size_t)max_pool_rays);
    b->ord_cnt = reinterpret_cast<uint32_t*>(p);
    p += align_up(4 * (size_t)(int64_t(1) << kBatchOrderBits));
    b->ord_sums = reinterpret_cast<uint32_t*>(p);
    const size_t table = b->item_bytes * (size_t)max_items;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaMallocHost(&b->h_stage[i], table);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->stage_ev[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaMemset(b->counts, 0, kCounterBytes);
    if (e != cudaSuccess) {
        batch_free(b);
        return fail(SPLAT_ERR_ALLOC, std::string("batch_create: ") + cudaGetErrorString(e));
    }
    b->h_items.assign(table, 0);
    for (int32_t s = 0; s < max_items; ++s) batch_clear_item(b->h_items.data() + b->item_bytes * (size_t)s);
    b->used.assign((size_t)max_items, 0);
    b->rays.assign((size_t)max_items, 0);
    b->start.assign((size_t)max_items, -1);
    b->depth.assign((size_t)max_items, 0);
    b->brute.assign((size_t)max_items, 0);
    b->mat_kind.assign((size_t)max_items, -1);
    b->maps.assign((size_t)max_items, nullptr);
    b->map_bytes.assign((size_t)max_items, 0);
    b->zero_map.assign((size_t)max_items, 0);
    *out = b;
    return SPLAT_OK;
}

splat_status_t splat_batch_destroy(splat_batch_t* b) {
    if (!b) return fail(SPLAT_ERR_INVALID, "batch_destroy: null batch");
    cudaDeviceSynchronize();
    batch_free(b);
    return SPLAT_OK;
}

splat_status_t splat_batch_admit(splat_batch_t* b, const splat_scene_t* scene, const splat_trace_params_t* P,
                                 void* d_map, int32_t* slot_out) {
    if (!b || !scene || !P || !slot_out) return fail(SPLAT_ERR_INVALID, "batch_admit: null argument");
    *slot_out = -1;
    if (!light_ok(&P->light, P->upscale)) return fail(SPLAT_ERR_INVALID, "batch_admit: bad light / upscale");
    if (P->depth < 1 || P->depth > 8) return fail(SPLAT_ERR_INVALID, "batch_admit: depth must be 1..8");
    if (!valid_material(&P->material)) return fail(SPLAT_ERR_INVALID, "batch_admit: bad material");
    if (P->lambda_mode.mode == SPLAT_LAMBDA_STRATIFIED && P->lambda_mode.n_strata < 1)
        return fail(SPLAT_ERR_INVALID, "batch_admit: n_strata < 1");
    splat_status_t rc =
        check_map(P->spectrum, P->n_lambda, P->upscale, d_map, P->accum, P->frac_bits, P->map_w, P->map_h);
    if (rc != SPLAT_OK) return rc;
    const bool bvh = P->hitter == SPLAT_HITTER_BVH || P->hitter == SPLAT_HITTER_BVH2;
    if (bvh && !scene->d_nodes4 && scene->n_recs > 0)
        return fail(SPLAT_ERR_INVALID, "batch_admit: BVH hitter on a scene without BVH");
    const int64_t n_grid = grid_rays(P);
    const int64_t rb = P->ray_begin < 0 ? 0 : P->ray_begin;
    const int64_t re = (P->ray_end <= 0 || P->ray_end > n_grid) ? n_grid : P->ray_end;
    const int64_t n = re - rb;
    if (n <= 0) return fail(SPLAT_ERR_INVALID, "batch_admit: empty ray range");
    if (n > (int64_t(1) << 24)) return fail(SPLAT_ERR_INVALID, "batch_admit: more than 2^24 rays in one item");
    if (n_grid >= (int64_t(1) << 32)) return fail(SPLAT_ERR_INVALID, "batch_admit: more than 2^32 grid rays");
    int32_t slot = -1;
    for (int32_t s = 0; s < b->max_items; ++s)
        if (!b->used[(size_t)s]) {
            slot = s;
            break;
        }
    if (slot < 0) return fail(SPLAT_ERR_WORKSPACE, "batch_admit: no free slot");
    if (pool_in_use(b) + n > b->cap) return fail(SPLAT_ERR_WORKSPACE, "batch_admit: ray pool full");
    GenParams g;
    g.light = P->light;
    g.upscale = P->upscale;
    g.lm = P->lambda_mode;
    g.seed = P->seed;
    g.light_index = 0;
    g.ray_begin = rb;
    BatchSceneRef sc{scene->d_ftri, scene->d_brute, scene->d_boxes, scene->d_nodes4, scene->d_bvh, scene->n_recs,
                     scene->n_tris, scene->first_diffuse, scene->d_bvh_pos};
    const SplatParams sp =
        make_splat(P->spectrum, P->n_lambda, P->upscale, d_map, P->accum, P->frac_bits, P->map_w, P->map_h);
    batch_fill_item(b->h_items.data() + b->item_bytes * (size_t)slot, sc, g, n, P->depth,
                    bvh ? SPLAT_HITTER_BVH : SPLAT_HITTER_BRUTE, b->tick, (P->flags & SPLAT_FLAG_REF_QUIRKS) ? 1 : 0,
                    P->force_rand, P->material, sp);
    b->used[(size_t)slot] = 1;
    b->rays[(size_t)slot] = n;
    b->start[(size_t)slot] = b->tick;
    b->depth[(size_t)slot] = P->depth;
    b->brute[(size_t)slot] = (!bvh || !scene->d_nodes4) ? 1 : 0;
    b->mat_kind[(size_t)slot] = P->material.kind;
    b->maps[(size_t)slot] = d_map;
    b->map_bytes[(size_t)slot] = (size_t)P->map_w * P->map_h * (P->n_lambda > 0 ? P->n_lambda : 1) * 4;
    b->zero_map[(size_t)slot] = P->zero_map ? 1 : 0;
    b->dirty = true;
    *slot_out = slot;
    return SPLAT_OK;
}

splat_status_t splat_batch_tick(splat_batch_t* b, void* stream, int32_t* done_slots, int32_t max_done,
                                int32_t* n_done) {
    if (!b) return fail(SPLAT_ERR_INVALID, "batch_tick: null batch");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    splat_status_t rc = batch_upload(b, st);
    if (rc != SPLAT_OK) return rc;
    return batch_enqueue_tick(b, st, done_slots, max_done, n_done);
}

splat_status_t splat_batch_release(splat_batch_t* b, int32_t slot) {
    if (!b || slot < 0 || slot >= b->max_items || !b->used[(size_t)slot])
        return fail(SPLAT_ERR_INVALID, "batch_release: bad slot");
    if (b->start[(size_t)slot] + b->depth[(size_t)slot] - 1 >= b->tick)
        return fail(SPLAT_ERR_INVALID, "batch_release: item still in flight");
    b->used[(size_t)slot] = 0;
    b->start[(size_t)slot] = -1;
    batch_clear_item(b->h_items.data() + b->item_bytes * (size_t)slot);
    b->dirty = true;
    return SPLAT_OK;
}

splat_status_t splat_batch_status(const splat_batch_t* b, int32_t* in_flight, int64_t* pool_rays, int32_t* tick) {
    if (!b) return fail(SPLAT_ERR_INVALID, "batch_status: null batch");
    int32_t f = 0;
    for (int32_t s = 0; s < b->max_items; ++s)
        if (b->used[(size_t)s] && b->start[(size_t)s] + b->depth[(size_t)s] - 1 >= b->tick) ++f;
    if (in_flight) *in_flight = f;
    if (pool_rays) *pool_rays = pool_in_use(b);
    if (tick) *tick = b->tick;
    return SPLAT_OK;
}

splat_status_t splat_batch_capture(splat_batch_t* b, void* stream, int32_t* n_ticks) {
    if (!b) return fail(SPLAT_ERR_INVALID, "batch_capture: null batch");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // capturing again the item set a replay has just run (nothing admitted
    // since): start from the previous capture's first tick again, so the
    // same frames are captured with the launch shapes now set
    if (b->exec && b->tick == b->cap_t1) {
        bool fresh = false;
        for (int32_t s = 0; s < b->max_items; ++s)
            if (b->used[(size_t)s] && b->start[(size_t)s] >= b->cap_t1) fresh = true;
        if (!fresh) {
            b->tick = b->cap_t0;
            b->parity = b->cap_parity0;
        }
    }
    int32_t last = b->tick - 1;
    for (int32_t s = 0; s < b->max_items; ++s) {
        if (!b->used[(size_t)s] || b->start[(size_t)s] + b->depth[(size_t)s] - 1 < b->tick) continue;
        if (b->start[(size_t)s] != b->tick)
            return fail(SPLAT_ERR_INVALID, "batch_capture: an item is already in flight");
        last = std::max(last, b->start[(size_t)s] + b->depth[(size_t)s] - 1);
    }
    if (last < b->tick) return fail(SPLAT_ERR_INVALID, "batch_capture: no admitted item");
    if (st == nullptr || st == cudaStreamLegacy || st == cudaStreamPerThread)
        return fail(SPLAT_ERR_INVALID, "batch_capture: needs a created (non-default) stream");
    splat_status_t rc = batch_upload(b, st);
    if (rc != SPLAT_OK) return rc;
    SPLAT_CUDA(cudaStreamSynchronize(st), "batch_capture: sync");
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    const int32_t t0 = b->tick;
    const int p0 = b->parity;
    cudaGraph_t graph = nullptr;
    b->overlap = g_tune[SPLAT_TUNE_SPLAT_OVERLAP] > 0 && batch_overlap_ready(b) == cudaSuccess;
    b->splat_pending[0] = b->splat_pending[1] = false;
    const int persistent = g_tune[SPLAT_TUNE_BATCH_PERSISTENT].load();
    if (persistent > 0 && last - t0 + 1 > kMaxPassTicks)
        return fail(SPLAT_ERR_INVALID, "batch_capture: a persistent pass holds at most 8 ticks");
    if (persistent > 0) b->overlap = false;
    SPLAT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "batch_capture: begin");
    cudaError_t e = cudaMemsetAsync(&b->counts[p0], 0, sizeof(int64_t), st);
    rc = SPLAT_OK;
    if (persistent > 0) {
        if (e == cudaSuccess) e = batch_enqueue_pass(b, st, last, persistent);
    } else {
        while (e == cudaSuccess && rc == SPLAT_OK && b->tick <= last) rc = batch_enqueue_tick(b, st, nullptr, 0, nullptr);
    }
    for (int p = 0; p < 2 && e == cudaSuccess; ++p)
        if (b->overlap && b->splat_pending[p]) {
            e = cudaStreamWaitEvent(st, b->splat_ev[p], 0);  // join the side stream before the capture ends
            b->splat_pending[p] = false;
        }
    b->overlap = false;
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    if (e != cudaSuccess) return cuda_fail(e, "batch_capture: memset");
    if (rc != SPLAT_OK) return rc;
    if (e2 != cudaSuccess) return cuda_fail(e2, "batch_capture: end");
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "batch_capture: instantiate");
    if (n_ticks) *n_ticks = b->tick - t0;
    // the captured ticks have not run yet: each replay runs them
    b->cap_t1 = b->tick;
    b->cap_parity1 = b->parity;
    b->cap_t0 = t0;
    b->cap_parity0 = p0;
    b->tick = t0;
    b->parity = p0;
    return SPLAT_OK;
}

splat_status_t splat_batch_replay(splat_batch_t* b, const uint64_t* seeds, int32_t n_seeds, void* stream) {
    if (!b || !b->exec) return fail(SPLAT_ERR_INVALID, "batch_replay: nothing captured");
    if (n_seeds < 0 || n_seeds > b->max_items || (n_seeds > 0 && !seeds))
        return fail(SPLAT_ERR_INVALID, "batch_replay: bad seeds");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    for (int32_t s = 0; s < n_seeds; ++s) {
        batch_set_seed(b->h_items.data() + b->item_bytes * (size_t)s, seeds[s]);
        b->dirty = true;
    }
    splat_status_t rc = batch_upload(b, st);
    if (rc != SPLAT_OK) return rc;
    ProfScope ps(SPLAT_KERNEL_BATCH, st);
    SPLAT_CUDA(cudaGraphLaunch(b->exec, st), "batch_replay: launch");
    if (b->tick < b->cap_t1) {
        b->tick = b->cap_t1;
        b->parity = b->cap_parity1;
    }
    return SPLAT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// camera pass
// ---------------------------------------------------------------------------
namespace {

// Retina response curves of src/rgb_spectrum.jl:32-91 (the reference's
// `piecewise` knots, nm -> response): the table has to be the same for the
// shading to match.  piecewise() interpolates linearly on the segment whose
// left knot is the last one <= lambda (first / last segment outside the
// knots), as (y1 - y0) / (x1 - x0) * (lambda - x1) + y1 in double with the
// difference lambda - x1 taken in the argument's own type.
struct Knot {
    int x;
    double y;
};
const Knot kRetinaRed[] = {{399, 0},         {400, 0.0647036}, {420, 0.147492}, {438, 0.195683}, {460, 0.162951},
                           {466, 0},         {534, 0},         {538, 0.243127}, {571, 0.798209}, {593, 0.980253},
                           {602, 0.999977},  {610, 0.98481},   {660, 0.375838}, {680, 0.210109}, {700, 0.11005}};
const Knot kRetinaGreen[] = {{399, 0},        {462, 0},        {467, 0.165356}, {474, 0.280228}, {502, 0.587139},
                             {521, 0.829692}, {534, 0.924245}, {551, 0.910167}, {572, 0.777366}, {600, 0.372516},
                             {609, 0.158767}, {612, 0},        {700, 0}};
const Knot kRetinaBlue[] = {{399, 0},         {413, 0.23889},  {418, 0.291473}, {437, 0.437376}, {456, 0.590128},
                            {463, 0.72815},   {476, 0.581812}, {494, 0.452254}, {515, 0.407615}, {528, 0.299756},
                            {536, 0},         {608, 0},        {611, 0.0407256}, {614, 0.154091}, {620, 0.220637},
                            {635, 0.225269},  {667, 0.116114}, {700, 0.0424846}};

template <int N>
int segment_of(const Knot (&k)[N], double lam) {
    int s = 0;
    while (s + 2 < N && !(lam < (double)k[s + 1].x)) ++s;
    return s;
}

// Float32 argument (a spectrum wavelength): lambda - x1 in float.
template <int N>
double piecewise_f(const Knot (&k)[N], float lam) {
    const int s = segment_of(k, (double)lam);
    const double slope = (k[s + 1].y - k[s].y) / (double)(k[s + 1].x - k[s].x);
    const float d = lam - (float)k[s + 1].x;
    return slope * (double)d + k[s + 1].y;
}

// Integer argument (the normalisers' 400:700 sweep): lambda - x1 exact.
template <int N>
double piecewise_i(const Knot (&k)[N], int lam) {
    const int s = segment_of(k, (double)lam);
    const double slope = (k[s + 1].y - k[s].y) / (double)(k[s + 1].x - k[s].x);
    return slope * (double)(lam - k[s + 1].x) + k[s + 1].y;
}

// sum(f(x) for x = 400:700): a left fold.
template <int N>
double retina_norm(const Knot (&k)[N]) {
    double s = piecewise_i(k, 400);
    for (int x = 401; x <= 700; ++x) s = s + piecewise_i(k, x);
    return s;
}

}  // namespace

struct splat_shader {
    int device = 0;
    int64_t map_w = 0, map_h = 0, sky_w = 0, sky_h = 0;
    int32_t planes = 0;
    cudaArray_t map_arr = nullptr, sky_arr = nullptr;
    cudaTextureObject_t map_tex = 0, sky_tex = 0;
    cudaSurfaceObject_t map_surf = 0;
};

namespace {

void shader_free(splat_shader* s) {
    if (!s) return;
    if (s->map_tex) cudaDestroyTextureObject(s->map_tex);
    if (s->sky_tex) cudaDestroyTextureObject(s->sky_tex);
    if (s->map_surf) cudaDestroySurfaceObject(s->map_surf);
    if (s->map_arr) cudaFreeArray(s->map_arr);
    if (s->sky_arr) cudaFreeArray(s->sky_arr);
    delete s;
}

// CuTexture(CuTextureArray(a); interpolation = LinearInterpolation()):
// float elements, linear filter, clamp addressing, unnormalised coordinates.
cudaError_t make_texture(cudaArray_t arr, cudaTextureObject_t* tex) {
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    return cudaCreateTextureObject(tex, &rd, &td, nullptr);
}

cudaError_t copy_to_array(const void* src, int64_t w, int64_t h, int64_t d, cudaArray_t arr, cudaStream_t st) {
    cudaMemcpy3DParms p;
    std::memset(&p, 0, sizeof(p));
    p.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), (size_t)w * 4, (size_t)w, (size_t)h);
    p.dstArray = arr;
    p.extent = make_cudaExtent((size_t)w, (size_t)h, (size_t)d);
    p.kind = cudaMemcpyDeviceToDevice;
    return cudaMemcpy3DAsync(&p, st);
}

bool camera_ok(const splat_camera_t* c) {
    if (!c) return false;
    const float* v[5] = {c->pos, c->look_at, c->dir, c->up, c->right};
    for (auto p : v)
        for (int i = 0; i < 3; ++i)
            if (!std::isfinite(p[i])) return false;
    return std::isfinite(c->fov_half_sin) && c->fov_half_sin > 0.0f;
}

CameraParams camera_params(const splat_camera_t* cam, int64_t h, int64_t w, float lambda, uint64_t seed) {
    CameraParams c;
    std::memset(&c, 0, sizeof(c));
    c.cam = *cam;
    c.h = h;
    c.w = w;
    c.seed = seed;
    c.lambda = lambda;
    c.cos45 = 1.0 / std::sqrt(2.0);
    return c;
}

ShadeParams shade_params(const splat_shader* sh, const float* spectrum, const float* retina, int32_t n_lambda,
                         int64_t upscale, int64_t height, float* rgb, int32_t retina_stride) {
    ShadeParams p;
    std::memset(&p, 0, sizeof(p));
    p.map_tex = sh->map_tex;
    p.sky_tex = sh->sky_tex;
    p.map_w = sh->map_w;
    p.map_h = sh->map_h;
    p.sky_w = sh->sky_w;
    p.sky_h = sh->sky_h;
    p.has_sky = sh->sky_arr ? 1 : 0;
    p.n_lambda = n_lambda;
    p.nd = (int32_t)upscale;
    p.cam_h = height / upscale;
    p.height = height;
    p.rgb = rgb;
    // upres(N), src/alg_types.jl:108
    for (int k = 1; k <= p.nd; ++k)
        p.deltas[k - 1] = ((float)k / (float)p.nd - 0.5f) - (1.0f / (2.0f * (float)p.nd));
    for (int i = 0; i < n_lambda; ++i) {
        p.spectrum[i] = spectrum[i];
        for (int c = 0; c < 3; ++c) p.retina[c][i] = retina[(size_t)c * retina_stride + i];
    }
    return p;
}

splat_status_t check_image(int64_t height, int64_t width, int64_t upscale) {
    if (upscale < 1 || upscale > 16) return fail(SPLAT_ERR_INVALID, "upscale must be 1..16");
    if (height < upscale || width < upscale || height % upscale || width % upscale)
        return fail(SPLAT_ERR_INVALID, "image size must be a positive multiple of upscale");
    if ((height / upscale) * (width / upscale) >= (int64_t(1) << 32))
        return fail(SPLAT_ERR_INVALID, "more than 2^32 camera rays");
    return SPLAT_OK;
}

}  // namespace

splat_status_t splat_camera_look_at(const float pos[3], const float look_at[3], const float true_up[3], double fov,
                                    splat_camera_t* out) {
    if (!pos || !look_at || !true_up || !out) return fail(SPLAT_ERR_INVALID, "camera_look_at: null pointer");
    if (!(fov > 0.0) || !(fov < 2.0 * M_PI)) return fail(SPLAT_ERR_INVALID, "camera_look_at: fov must be in (0, 2 pi)");
    auto sub = [](const float* a, const float* b, float* o) {
        for (int i = 0; i < 3; ++i) o[i] = a[i] - b[i];
    };
    auto cross = [](const float* a, const float* b, float* o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    auto normalize = [](float* v) {
        const float inv = 1.0f / std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
        for (int i = 0; i < 3; ++i) v[i] = v[i] * inv;
    };
    splat_camera_t c;
    std::memset(&c, 0, sizeof(c));
    for (int i = 0; i < 3; ++i) {
        c.pos[i] = pos[i];
        c.look_at[i] = look_at[i];
    }
    sub(look_at, pos, c.dir);
    normalize(c.dir);
    cross(c.dir, true_up, c.right);
    normalize(c.right);
    cross(c.right, c.dir, c.up);
    normalize(c.up);
    c.fov_half_sin = (float)std::sin(fov / 2.0);
    if (!camera_ok(&c)) return fail(SPLAT_ERR_INVALID, "camera_look_at: degenerate camera (up parallel to view?)");
    *out = c;
    return SPLAT_OK;
}

splat_status_t splat_camera_rays(const splat_camera_t* camera, int64_t height, int64_t width, float lambda,
                                 uint64_t seed, splat_adray_t* d_rays, void* stream) {
    if (!camera_ok(camera)) return fail(SPLAT_ERR_INVALID, "camera_rays: bad camera");
    if (height < 1 || width < 1 || height * width >= (int64_t(1) << 32))
        return fail(SPLAT_ERR_INVALID, "camera_rays: bad grid size");
    if (!d_rays) return fail(SPLAT_ERR_INVALID, "camera_rays: null output");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    ProfScope ps(SPLAT_KERNEL_SHADE, st);
    SPLAT_CUDA(launch_camera_aos(camera_params(camera, height, width, lambda, seed), height * width, d_rays,
                                 sm_count_current(), st),
               "camera rays");
    return SPLAT_OK;
}

splat_status_t splat_retina_factors(const float* spectrum, int32_t n_lambda, float* out) {
    if (n_lambda < 0 || (n_lambda > 0 && (!spectrum || !out))) return fail(SPLAT_ERR_INVALID, "retina_factors: bad arguments");
    const double r0 = retina_norm(kRetinaRed), g0 = retina_norm(kRetinaGreen), b0 = retina_norm(kRetinaBlue);
    for (int32_t i = 0; i < n_lambda; ++i) {
        out[i] = (float)(piecewise_f(kRetinaRed, spectrum[i]) / r0);
        out[n_lambda + i] = (float)(piecewise_f(kRetinaGreen, spectrum[i]) / g0);
        out[2 * n_lambda + i] = (float)(piecewise_f(kRetinaBlue, spectrum[i]) / b0);
    }
    return SPLAT_OK;
}

splat_status_t splat_shader_create(int64_t map_w, int64_t map_h, int32_t n_planes, int64_t sky_w, int64_t sky_h,
                                   splat_shader_t** out) {
    if (!out) return fail(SPLAT_ERR_INVALID, "shader_create: null output");
    *out = nullptr;
    cudaDeviceProp prop;
    int dev = 0;
    SPLAT_CUDA(cudaGetDevice(&dev), "shader_create: device");
    SPLAT_CUDA(cudaGetDeviceProperties(&prop, dev), "shader_create: properties");
    const int64_t lim = prop.maxTexture3D[0];
    if (map_w < 1 || map_h < 1 || n_planes < 1 || n_planes > SPLAT_MAX_LAMBDA || map_w > lim ||
        map_h > prop.maxTexture3D[1])
        return fail(SPLAT_ERR_INVALID, "shader_create: light map size outside the 3-D texture limits");
    if (sky_w < 0 || sky_h < 0 || (sky_w > 0) != (sky_h > 0) || sky_w > lim || sky_h > prop.maxTexture3D[1])
        return fail(SPLAT_ERR_INVALID, "shader_create: bad skydome size");
    splat_shader* s = new (std::nothrow) splat_shader();
    if (!s) return fail(SPLAT_ERR_ALLOC, "shader_create: host allocation");
    s->device = dev;
    s->map_w = map_w;
    s->map_h = map_h;
    s->planes = n_planes;
    s->sky_w = sky_w;
    s->sky_h = sky_h;
    const cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
    cudaError_t e = cudaMalloc3DArray(&s->map_arr, &fd, make_cudaExtent((size_t)map_w, (size_t)map_h, (size_t)n_planes),
                                      cudaArraySurfaceLoadStore);
    if (e == cudaSuccess) e = make_texture(s->map_arr, &s->map_tex);
    if (e == cudaSuccess) {
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = s->map_arr;
        e = cudaCreateSurfaceObject(&s->map_surf, &rd);
    }
    if (e == cudaSuccess && sky_w > 0) {
        e = cudaMalloc3DArray(&s->sky_arr, &fd, make_cudaExtent((size_t)sky_w, (size_t)sky_h, 3), 0);
        if (e == cudaSuccess) e = make_texture(s->sky_arr, &s->sky_tex);
    }
    if (e != cudaSuccess) {
        shader_free(s);
        return cuda_fail(e, "shader_create: texture arrays");
    }
    *out = s;
    return SPLAT_OK;
}

splat_status_t splat_shader_destroy(splat_shader_t* shader) {
    shader_free(shader);
    return SPLAT_OK;
}

splat_status_t splat_shader_set_light_map(splat_shader_t* sh, const void* d_map, int32_t accum, int32_t frac_bits,
                                          void* stream) {
    if (!sh || !d_map) return fail(SPLAT_ERR_INVALID, "shader_set_light_map: null argument");
    if (frac_bits < 0 || frac_bits > 30) return fail(SPLAT_ERR_INVALID, "shader_set_light_map: frac_bits must be 0..30");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    ProfScope ps(SPLAT_KERNEL_SHADE, st);
    if (accum == SPLAT_ACCUM_F32) {
        SPLAT_CUDA(copy_to_array(d_map, sh->map_w, sh->map_h, sh->planes, sh->map_arr, st), "light map -> array");
    } else if (accum == SPLAT_ACCUM_I32) {
        SPLAT_CUDA(launch_map_to_array(reinterpret_cast<const int32_t*>(d_map), sh->map_w, sh->map_h, sh->planes,
                                       std::ldexp(1.0f, -frac_bits), sh->map_surf, sm_count_current(), st),
                   "light map -> array");
    } else {
        return fail(SPLAT_ERR_INVALID, "shader_set_light_map: unknown accumulation");
    }
    return SPLAT_OK;
}

splat_status_t splat_shader_set_skydome(splat_shader_t* sh, const float* d_sky, void* stream) {
    if (!sh || !d_sky) return fail(SPLAT_ERR_INVALID, "shader_set_skydome: null argument");
    if (!sh->sky_arr) return fail(SPLAT_ERR_INVALID, "shader_set_skydome: shader created without a skydome");
    SPLAT_CUDA(copy_to_array(d_sky, sh->sky_w, sh->sky_h, 3, sh->sky_arr, reinterpret_cast<cudaStream_t>(stream)),
               "skydome -> array");
    return SPLAT_OK;
}

splat_status_t splat_continuum_shade(const splat_scene_t* scene, const splat_shader_t* shader, splat_adray_t* d_rays,
                                     int64_t n_rays, const int32_t* d_hit_idx, const float* spectrum,
                                     const float* retina, int32_t n_lambda, int64_t upscale, int64_t height,
                                     int64_t width, float* d_rgb, void* stream) {
    if (!scene || !shader) return fail(SPLAT_ERR_INVALID, "continuum_shade: null scene or shader");
    splat_status_t rc = check_image(height, width, upscale);
    if (rc != SPLAT_OK) return rc;
    if (n_rays != (height / upscale) * (width / upscale))
        return fail(SPLAT_ERR_INVALID, "continuum_shade: n_rays must be (height / upscale) * (width / upscale)");
    if (n_lambda < 1 || n_lambda > shader->planes || !spectrum || !retina)
        return fail(SPLAT_ERR_INVALID, "continuum_shade: spectrum must have 1..planes wavelengths");
    if (!d_rays || !d_hit_idx || !d_rgb) return fail(SPLAT_ERR_INVALID, "continuum_shade: null pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const ShadeParams p = shade_params(shader, spectrum, retina, n_lambda, upscale, height, d_rgb, n_lambda);
    ProfScope ps(SPLAT_KERNEL_SHADE, st);
    SPLAT_CUDA(launch_shade_aos(d_rays, n_rays, d_hit_idx, scene->d_ftri, scene->n_tris, scene->d_err, p,
                                sm_count_current(), st),
               "continuum_shade");
    return SPLAT_OK;
}

size_t splat_render_workspace_size(int64_t n_camera_rays) {
    return n_camera_rays <= 0 ? kAlign : work_bytes(n_camera_rays) + soa_bytes(n_camera_rays) + kAlign;
}

splat_status_t splat_render_camera(const splat_scene_t* scene, const splat_shader_t* shader,
                                   const splat_render_params_t* P, float* d_rgb, void* d_workspace,
                                   size_t workspace_bytes, void* stream) {
    return splat_render_camera_after(scene, shader, P, d_rgb, d_workspace, workspace_bytes, stream, nullptr);
}

splat_status_t splat_render_camera_after(const splat_scene_t* scene, const splat_shader_t* shader,
                                         const splat_render_params_t* P, float* d_rgb, void* d_workspace,
                                         size_t workspace_bytes, void* stream, void* map_ready) {
    if (!scene || !shader || !P) return fail(SPLAT_ERR_INVALID, "render_camera: null argument");
    if (!camera_ok(&P->camera)) return fail(SPLAT_ERR_INVALID, "render_camera: bad camera");
    splat_status_t rc = check_image(P->height, P->width, P->upscale);
    if (rc != SPLAT_OK) return rc;
    if (P->depth < 1 || P->depth > 8) return fail(SPLAT_ERR_INVALID, "render_camera: depth must be 1..8");
    if (!valid_material(&P->material)) return fail(SPLAT_ERR_INVALID, "render_camera: bad material");
    if (P->n_lambda < 1 || P->n_lambda > shader->planes)
        return fail(SPLAT_ERR_INVALID, "render_camera: n_lambda must be 1..planes of the shader's map");
    if ((P->hitter == SPLAT_HITTER_BVH || P->hitter == SPLAT_HITTER_BVH2) && !scene->d_nodes && scene->n_recs > 0)
        return fail(SPLAT_ERR_INVALID, "render_camera: BVH hitter on a scene without BVH");
    if (!d_rgb) return fail(SPLAT_ERR_INVALID, "render_camera: null image");
    const int64_t ch = P->height / P->upscale, cw = P->width / P->upscale;
    const int64_t cnt = ch * cw;
    if (!d_workspace || workspace_bytes < splat_render_workspace_size(cnt))
        return fail(SPLAT_ERR_WORKSPACE, "render_camera: workspace smaller than splat_render_workspace_size");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int sm = sm_count_current();
    Work w = carve_work(d_workspace, cnt);
    char* p = static_cast<char*>(w.order) + align_up(ray_order_bytes(cnt));
    p = reinterpret_cast<char*>(align_up(reinterpret_cast<size_t>(p)));
    const RaySoA sky = carve_soa(p, cnt);
    int64_t* sky_count = &w.counts[kSplatCount + 1];
    SPLAT_CUDA(cudaMemsetAsync(w.counts, 0, kCounterBytes, st), "memset counters");
    SPLAT_CUDA(cudaMemsetAsync(d_rgb, 0, (size_t)P->height * P->width * 3 * sizeof(float), st), "clear image");
    {
        ProfScope ps(SPLAT_KERNEL_SHADE, st);
        SPLAT_CUDA(launch_camera_soa(camera_params(&P->camera, ch, cw, P->lambda, P->seed), cnt, w.a, &w.counts[0],
                                     sm, st),
                   "camera rays");
    }
    EvolveArgs ea;
    std::memset(&ea, 0, sizeof(ea));
    ea.tris = scene->d_ftri;
    ea.n_tris = scene->n_tris;
    ea.err = scene->d_err;
    ea.first_diffuse = scene->first_diffuse;
    ea.material = P->material;
    ea.seed = P->seed;
    ea.force_rand = P->force_rand;
    ea.quirks = (P->flags & SPLAT_FLAG_REF_QUIRKS) ? 1 : 0;
    ea.splat_q = w.q;
    ea.splat_count = &w.counts[kSplatCount];
    ea.sky_q = sky;
    ea.sky_count = sky_count;
    RaySoA cur = w.a, nxt = w.b;
    for (int32_t b = 1; b <= P->depth; ++b) {
        RaySrc src{cur.f, cur.ignore, cur.cap, nullptr, &w.counts[b - 1], 0,
                   reinterpret_cast<unsigned long long*>(&w.counts[kFetchBase + b]), packet_for(b)};
        // camera rays are the sub-sample grid's columns in order: first-bounce
        // packets take 8 x 4 tiles of it
        if (b == 1 && ch <= (int64_t)kGridTileMaxRows) src.tile_h = (int32_t)ch;
        rc = hit_any(scene, P->hitter, src, cnt, w.hit, nullptr, w.tmp, st);
        if (rc != SPLAT_OK) return rc;
        ea.in = cur;
        ea.out = nxt;
        ea.in_count = &w.counts[b - 1];
        ea.out_count = &w.counts[b];
        ea.hit_idx = w.hit;
        ea.bounce = (uint32_t)b;
        ea.last = b == P->depth ? 1 : 0;
        ea.tile_h = src.tile_h;
        {
            ProfScope ps(SPLAT_KERNEL_EVOLVE, st);
            SPLAT_CUDA(launch_evolve_camera(ea, cnt, sm, st), "evolve");
        }
        std::swap(cur, nxt);
    }
    const ShadeParams sp =
        shade_params(shader, P->spectrum, &P->retina[0][0], P->n_lambda, P->upscale, P->height, d_rgb, SPLAT_MAX_LAMBDA);
    if (map_ready) SPLAT_CUDA(cudaStreamWaitEvent(st, reinterpret_cast<cudaEvent_t>(map_ready), 0), "wait for the map");
    ProfScope ps(SPLAT_KERNEL_SHADE, st);
    SPLAT_CUDA(launch_shade_queues(w.q, &w.counts[kSplatCount], sky, sky_count, scene->d_ftri, sp, cnt, sm, st),
               "shade");
    return SPLAT_OK;
}

splat_status_t splat_image_accumulate(float* d_out, const float* d_rgb, int64_t n, int32_t iteration, void* stream) {
    if (n < 0 || iteration < 1) return fail(SPLAT_ERR_INVALID, "image_accumulate: bad size or iteration");
    if (n == 0) return SPLAT_OK;
    if (!d_out || !d_rgb) return fail(SPLAT_ERR_INVALID, "image_accumulate: null pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    ProfScope ps(SPLAT_KERNEL_SHADE, st);
    SPLAT_CUDA(launch_image_accumulate(d_out, d_rgb, n, iteration, sm_count_current(), st), "image_accumulate");
    return SPLAT_OK;
}

splat_status_t splat_obj_to_ftri(const char* path, splat_ftri_t* out, int64_t capacity, int64_t* n_tris) {
    if (!path || !n_tris) return fail(SPLAT_ERR_INVALID, "obj_to_ftri: null argument");
    std::vector<splat_ftri_t> tris;
    std::string err;
    if (!obj_to_ftri(path, tris, err)) return fail(SPLAT_ERR_INVALID, "obj_to_ftri: " + err);
    *n_tris = (int64_t)tris.size();
    if (!out) return SPLAT_OK;
    if (capacity < (int64_t)tris.size()) return fail(SPLAT_ERR_WORKSPACE, "obj_to_ftri: capacity below the count");
    std::memcpy(out, tris.data(), tris.size() * sizeof(splat_ftri_t));
    return SPLAT_OK;
}
