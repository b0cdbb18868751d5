// kernels.h -- host-side launchers shared by the translation units.
#pragma once

#include <atomic>
#include <string>

#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace splat {

// Kernels launched by this thread (for launch profiling).
extern thread_local int64_t g_launches;
// Launch-shape knobs, indexed by SPLAT_TUNE_*.
extern std::atomic<int32_t> g_tune[SPLAT_TUNE_KEYS];  // process-wide launch knobs (splat_set_tuning)

// Where a hit kernel reads its rays: the structure-of-arrays bounce state
// (count on the device) or the reference's AoS ADRay array.
struct RaySrc {
    const float* f;          // SoA planes (nullptr for AoS)
    const int32_t* ignore;
    int64_t cap;
    const splat_adray_t* aos;  // AoS rays (nullptr for SoA)
    const int64_t* d_count;    // active count on the device (SoA)
    int64_t n;                 // ray count when d_count is null
    unsigned long long* fetch; // zeroed work counter: warps take rays 32 at a time (nullptr: grid-stride)
    int32_t packet;            // four-wide BVH: packet_form of the launch (0 one ray per lane)
    const int32_t* perm;       // BVH hitters: the k-th ray traced is ray perm[k] (nullptr: ray k); results
                               // go to the ray's own index
    int32_t tile_h;            // packet kernels, no perm: rays are a light grid of tile_h rows in column-major
                               // order; warps take 8 x 4 tiles of it (0: in order)
};

// Which traversal a warp of four-wide BVH rays takes, from
// SPLAT_TUNE_BVH_PACKET and whether the rays are on their first bounce:
// 0 one ray per lane, 1 a packet, 2 / 3 a packet when the warp's rays are
// coherent by the loose / tight thresholds of packet_coherent (hitcore.cuh).
__host__ __device__ inline int packet_form(int mode, bool first_bounce) {
    switch (mode) {
        case 1: return first_bounce ? 1 : 0;
        case 2: return 1;
        case 3: return first_bounce ? 1 : 2;
        case 4: return first_bounce ? 1 : 3;
        case 5: return 2;
        default: return 0;
    }
}

// Flattened BVH2 node (Aila & Laine 2009 layout): the boxes of both children
// and their references.  ref >= 0: inner node index; ref < 0: leaf,
// ~ref = first << 4 | (count - 1) in the BVH-ordered hit-record array.
struct __align__(16) BvhNode {
    float4 x;  // c0.lo.x, c0.hi.x, c1.lo.x, c1.hi.x
    float4 y;
    float4 z;
    int4 c;    // ref0, ref1, 0, 0
};
static_assert(sizeof(BvhNode) == 64, "BvhNode layout");

// Four-wide node collapsed from the binary tree: child i's box in
// component i of the six float4s.  Slots i >= meta.x are empty boxes
// (lo = +inf, hi = -inf), which no ray enters, so traversal needs no count.
struct __align__(16) Bvh4Node {
    float4 lox, hix, loy, hiy, loz, hiz;
    int4 c;      // child refs (as BvhNode)
    int4 meta;   // x: number of children (2..4)
};
static_assert(sizeof(Bvh4Node) == 128, "Bvh4Node layout");

struct Bvh4View {
    const Bvh4Node* nodes;
    const TriHit* tris;  // BVH order (shared with the binary tree)
};

constexpr int kLeafMax = 16;
constexpr int kBvhStack = 64;

struct BvhView {
    const BvhNode* nodes;
    const TriHit* tris;  // BVH order
};

// brute force over prepacked hit records (reference indices 2..T in order),
// each behind its padded box
cudaError_t launch_hit_brute(const RaySrc& rays, int64_t cap, const TriHit* recs, const TriBox* boxes, int64_t n_recs,
                             int32_t* hit_idx, float* hit_t, uint64_t* tmp, int32_t* err, int sm_count,
                             cudaStream_t s);
// brute force over the reference's n_tris array (Tuple{Int32,Tri})
cudaError_t launch_hit_brute_ntris(const splat_adray_t* rays, int64_t n_rays, const splat_ntri_t* ntris,
                                   int64_t n_tris, uint64_t* tmp, int32_t* hit_idx, int sm_count, cudaStream_t s);
// splat_next_hit_brute_static: the same hitter with its scratch in a
// file-scope device array (no allocation); n_rays <= kStaticHitMaxRays
constexpr int64_t kStaticHitMaxRays = SPLAT_STATIC_HIT_MAX_RAYS;
cudaError_t launch_hit_brute_ntris_static(const splat_adray_t* rays, int64_t n_rays, const splat_ntri_t* ntris,
                                          int64_t n_tris, int32_t* hit_idx, int sm_count, cudaStream_t s);
cudaError_t launch_hit_bvh(const RaySrc& rays, int64_t cap, const BvhView& bvh, int32_t* hit_idx, float* hit_t,
                           int32_t* err, int sm_count, cudaStream_t s);
cudaError_t launch_hit_bvh4(const RaySrc& rays, int64_t cap, const Bvh4View& bvh, int32_t* hit_idx, float* hit_t,
                            int32_t* err, int sm_count, cudaStream_t s);
// traversal work counted while SPLAT_TUNE_COUNT_WORK is set (nodes, triangle
// pre-tests, full triangle tests, rays); synchronises s; reset clears them
cudaError_t read_hit_work(uint64_t out[4], bool reset, cudaStream_t s);
// grid of a work-counter traversal launch (one resident wave)
int resident_grid(const void* kernel, int64_t cap, int sm_count, int threads, int max_per_sm);
// one-launch bottom-up refit of a two-child (wide = false) or four-wide tree;
// links: parent per node, then number of inner children per node
cudaError_t launch_refit_tree(void* nodes, bool wide, int64_t n_nodes, const int32_t* links, unsigned* flags,
                              const TriHit* bvh_recs, const splat_ftri_t* ftri, const unsigned* scale, float pad_rel,
                              cudaStream_t s);


// GPU BVH rebuild (lbvh.cu): linear BVH over Morton-sorted centroids, written
// as two-child and four-wide nodes with leaves of at most leaf_max triangles
constexpr int kLbvhLeaf = 4;
size_t lbvh_scratch_bytes(int64_t n_prims);
cudaError_t launch_lbvh_build(const splat_ftri_t* ftri, int64_t n_tris, int leaf_max, void* scratch,
                              BvhNode* nodes2, Bvh4Node* nodes4, int32_t* order, int sm_count, cudaStream_t s);

// Coherent ray order (lbvh.cu): a permutation of the d_count active rays of
// a SoA bounce buffer, grouped by (direction octant, BVH-order position of
// the triangle the ray leaves) with a counting sort over a key of key_bits
// (4..22) bits (the position's low bits dropped to fit).  Rays that leave
// neighbouring triangles in similar directions then share warps, so the
// traversal's lanes take similar paths.  bvh_pos[i]: BVH record position of
// reference index i (0 for indices outside 1..n_tris).  *perm_out points
// into scratch.
size_t ray_order_bytes(int64_t cap);
cudaError_t launch_ray_order(const float* soa_f, const int32_t* ignore, int64_t cap, const int64_t* d_count,
                             const int32_t* bvh_pos, int64_t n_tris, int key_bits, void* scratch,
                             const int32_t** perm_out, int sm_count, cudaStream_t s);

// The bucket offsets of that counting sort for keys counted elsewhere: cnt
// holds each bucket's size (buckets entries) and is scanned in place into
// offsets (sums: order_sums_count(buckets) words of scratch).
size_t order_sums_count(int64_t buckets);
cudaError_t launch_order_scan(uint32_t* cnt, int64_t buckets, uint32_t* sums, cudaStream_t s);

// scene packing / refit.  scale: device word holding max |vertex coordinate|
// (float bits), from which every padded box takes pad_abs = 1e-4 max(1, scale).
// bvh_pos (optional, n_tris + 1 entries): the inverse of bvh_order.
cudaError_t launch_pack_hits(const splat_ftri_t* ftri, int64_t n_tris, TriHit* brute_recs, TriBox* brute_boxes,
                             unsigned* scale, const int32_t* bvh_order, TriHit* bvh_recs, int32_t* bvh_pos,
                             cudaStream_t s);


// generation and conversion
struct GenParams {
    splat_rect_light_t light;
    int64_t upscale;
    splat_lambda_mode_t lm;
    uint64_t seed;
    uint32_t light_index;
    int64_t ray_begin;
};
cudaError_t launch_generate_soa(const GenParams& g, int64_t n, RaySoA out, int64_t* d_count, cudaStream_t s);
cudaError_t launch_generate_aos(const GenParams& g, int64_t n, splat_adray_t* out, cudaStream_t s);
cudaError_t launch_aos_to_soa(const splat_adray_t* in, int64_t n, RaySoA out, int64_t* d_count, cudaStream_t s);
cudaError_t launch_soa_to_aos(RaySoA in, const int64_t* d_count, splat_adray_t* out, int status, cudaStream_t s);

// evolve (+ compaction, + fused splat in trace mode)
struct SplatParams {
    void* map;
    int32_t accum;  // SPLAT_ACCUM_*
    float scale;    // 2^frac_bits
    int64_t w, h;
    int32_t n_lambda;  // 0: own wavelength
    int32_t n_delta;
    int32_t n_samples;   // planes x n_delta^2 per ray
    int32_t lanes_log2;  // lanes per ray in the splat kernel = 1 << lanes_log2 (<= 32)
    int32_t chunks;      // sample chunks per lane
    float inv_nd, inv_nd2;  // 1 / n_delta, 1 / n_delta^2 (index decode)
    float spectrum[SPLAT_MAX_LAMBDA];
    float deltas[16];
};

struct EvolveArgs {
    RaySoA in, out;
    const int64_t* in_count;
    int64_t* out_count;
    const int32_t* hit_idx;
    const splat_ftri_t* tris;
    int64_t n_tris;         // hit indices outside 1..n_tris are reported and treated as misses
    int32_t* err;           // error word (bit 4: bad hit index)
    int64_t first_diffuse;
    splat_material_t material;
    uint64_t seed;
    uint32_t bounce;
    float force_rand;
    int32_t quirks;
    int32_t last;           // trace mode: last bounce, no optics
    splat_adray_t* aos;     // plugin mode: retired rays written back here
    RaySoA splat_q;         // trace mode: final-evolved diffuse rays (ignore = hit triangle)
    int64_t* splat_count;
    RaySoA sky_q;           // camera mode: rays that escaped, unchanged
    int64_t* sky_count;
    int32_t tile_h;         // > 0: the input is a light grid of tile_h rows in column order, taken in its
                            // 8 x 4 tiles (grid_tile_ray), so the survivors leave in tile order
};
cudaError_t launch_evolve_trace(const EvolveArgs& a, int64_t cap, int sm_count, cudaStream_t s);
// trace mode plus the escaped rays queued for the skydome (camera pass)
cudaError_t launch_evolve_camera(const EvolveArgs& a, int64_t cap, int sm_count, cudaStream_t s);
cudaError_t launch_evolve_plugin(const EvolveArgs& a, int64_t cap, int sm_count, cudaStream_t s);
// one evolve_ray broadcast on AoS rays (rndm: per-ray draws or null)
cudaError_t launch_evolve_aos(splat_adray_t* rays, int64_t n, const int32_t* hit_idx, const float* rndm,
                              const EvolveArgs& a, int sm_count, cudaStream_t s);
// partition!: ACTIVE rays first via swap; counts[0] = their number (3 int64)
cudaError_t launch_partition(splat_adray_t* rays, int64_t n, splat_adray_t* swap, int64_t* counts, int sm_count,
                             cudaStream_t s);
cudaError_t launch_light_map(splat_adray_t* rays, int64_t n, const int32_t* hit_idx, const splat_ftri_t* tris,
                             int64_t n_tris, int32_t* err, const SplatParams& sp, int sm_count, cudaStream_t s);
// camera pass (shade.cu)
struct CameraParams {
    splat_camera_t cam;
    int64_t h, w;      // camera grid (image / upscale)
    uint64_t seed;
    float lambda;
    double cos45;      // 1 / sqrt(2), the reference's _COS_45 (src/geo.jl:13)
};
struct ShadeParams {
    cudaTextureObject_t map_tex, sky_tex;
    int64_t map_w, map_h, sky_w, sky_h;
    int32_t has_sky;
    int32_t n_lambda;
    int32_t nd;          // upscale: nd x nd sub-samples (pixels) per camera ray
    int64_t cam_h;       // camera grid rows
    int64_t height;      // image rows
    float* rgb;          // image, column-major RGB float triples
    float deltas[16];    // upres(nd)
    float spectrum[SPLAT_MAX_LAMBDA];
    float retina[3][SPLAT_MAX_LAMBDA];
};
cudaError_t launch_camera_soa(const CameraParams& c, int64_t n, RaySoA out, int64_t* count, int sm_count,
                              cudaStream_t s);
cudaError_t launch_camera_aos(const CameraParams& c, int64_t n, splat_adray_t* out, int sm_count, cudaStream_t s);
cudaError_t launch_shade_queues(const RaySoA& dq, const int64_t* d_count, const RaySoA& sq, const int64_t* s_count,
                                const splat_ftri_t* tris, const ShadeParams& p, int64_t cap, int sm_count,
                                cudaStream_t s);
cudaError_t launch_shade_aos(splat_adray_t* rays, int64_t n, const int32_t* hit_idx, const splat_ftri_t* tris,
                             int64_t n_tris, int32_t* err, const ShadeParams& p, int sm_count, cudaStream_t s);
cudaError_t launch_image_accumulate(float* out, const float* rgb, int64_t n, int32_t k, int sm_count,
                                    cudaStream_t s);
cudaError_t launch_map_to_array(const int32_t* map, int64_t w, int64_t h, int64_t planes, float inv_scale,
                                cudaSurfaceObject_t surf, int sm_count, cudaStream_t s);

// light-map splat of the queued diffuse rays [*d_begin, *d_count) (d_begin
// null: from 0)
cudaError_t launch_splat(const RaySoA& q, const int64_t* d_begin, const int64_t* d_count, const splat_ftri_t* tris,
                         const SplatParams& sp, splat_trace_stats_t* stats, int sm_count, cudaStream_t s);
// *dst = *src in stream order (a queue-length snapshot)
cudaError_t launch_copy_count(const int64_t* src, int64_t* dst, cudaStream_t s);
cudaError_t launch_stats_finish(const int64_t* counts, int depth, const int64_t* splat_count,
                                splat_trace_stats_t* stats, const int32_t* err, cudaStream_t s);
cudaError_t launch_unpack_hits(const uint64_t* tmp, int64_t n, const int64_t* d_count, int32_t* hit_idx,
                               float* hit_t, cudaStream_t s);

// ---------------------------------------------------------------------------
// batch engine (batch.cu)
// ---------------------------------------------------------------------------
struct BatchSceneRef {
    const splat_ftri_t* ftri;
    const TriHit* brute;
    const TriBox* brute_boxes;
    const Bvh4Node* nodes4;
    const TriHit* bvh_tris;
    int64_t n_recs, n_tris, first_diffuse;
    const int32_t* bvh_pos;  // BVH record position of each reference index (nullptr: none)
};

// Ray order of the batch engine: bucket keys over every item of the table,
// (item's key base + BVH position of the triangle left >> pos_shift) x 8 +
// direction octant, at most 2^kBatchOrderBits buckets.
constexpr int kBatchOrderBits = 24;

struct BatchTickArgs {
    void* items;  // device item table
    int n_slots;
    int tick;
    void* fresh;  // device FreshList
    RaySoA cur, next, queue;
    int64_t* cur_count;
    int64_t* next_count;
    int64_t* queue_count;
    int64_t fresh_rays;  // rays generated this tick (known on the host)
    int64_t cap_rays;    // bound on the rays active this tick
    int32_t* hit_idx;
    int32_t* err;
    int sm_count;
    bool any_brute;      // some item in flight uses the brute-force hitter (or has no BVH)
    int material_kind;   // material kind shared by every item in flight, -1 when mixed
    unsigned long long* fetch;  // zeroed work counter of this tick's hit kernel
    // ray order before the hit kernel (order_buckets > 0): keys and perm of
    // cap_rays entries, bucket counts (order_buckets) and their scan's sums
    int64_t order_buckets;
    uint32_t* order_keys;
    uint32_t* order_cnt;
    uint32_t* order_sums;
    int32_t* order_perm;
};

cudaError_t launch_batch_tick(const BatchTickArgs& a, cudaStream_t s);

// A whole pass (ticks t0 .. t0 + n_ticks - 1 of items that all start at t0)
// as one persistent cooperative launch over 1/share of the GPU's resident
// blocks; every counter below is zeroed by the caller before the launch.
constexpr int kMaxPassTicks = 8;
struct BatchPassArgs {
    void* items;
    void* fresh;
    int n_slots, t0, n_ticks;
    int material_kind;   // shared by every item, -1 when mixed
    RaySoA a, b, queue;  // a: the first tick's rays
    int64_t* count;      // count[i]: rays entering tick t0 + i (n_ticks + 1 slots)
    int64_t* qcount;     // queue entries so far
    int64_t* qmark;      // qmark[i]: queue length before tick i's evolve (n_ticks slots)
    unsigned long long* fetch;        // per-tick traversal work counters (n_ticks)
    unsigned long long* splat_fetch;  // per-tick splat work counters (n_ticks)
    unsigned* bar;       // grid-wait arrivals
    int32_t* hit_idx;
    int32_t* err;
    int packet_mode;     // SPLAT_TUNE_BVH_PACKET when the pass was launched
};
cudaError_t launch_batch_pass(const BatchPassArgs& a, int share, int sm_count, cudaStream_t s);
// the two halves of a tick: reserve, generate, hit, evolve; and the splat of the tick's queue
cudaError_t launch_batch_trace(const BatchTickArgs& a, cudaStream_t s);
cudaError_t launch_batch_splat(const BatchTickArgs& a, cudaStream_t s);
// sets splat_last_error() of the calling thread and returns code (api.cu)
splat_status_t set_error(splat_status_t code, const std::string& msg);
size_t batch_item_bytes();
size_t batch_fresh_bytes();
void batch_fill_item(void* dst, const BatchSceneRef& sc, const GenParams& gen, int64_t n_rays, int32_t depth,
                     int32_t hitter, int32_t start_tick, int32_t quirks, float force_rand,
                     const splat_material_t& material, const SplatParams& sp);
void batch_clear_item(void* dst);
// Assigns every used item of a host item table its ray-order key base (items
// in slot order, each (n_tris >> shift) + 1 positions, one shift for all,
// the smallest that fits 8 x positions in 2^max_bits buckets); returns the
// number of buckets.
int64_t batch_assign_order_keys(void* items, const uint8_t* used, int32_t n_slots, int max_bits);
void batch_set_seed(void* dst, uint64_t seed);

}  // namespace splat
