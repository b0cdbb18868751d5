// batch.cu -- many frames of many scenes traced together.
//
// An item is one frame: a resident scene plus one splat_trace_params_t and
// its light map.  Items live in a device table; their rays share one
// structure-of-arrays pool whose ray ids carry the item slot (slot << 24 |
// local ray index).  One tick advances every in-flight item by one bounce:
//
//   reserve   one thread per item slot; block scans over the slots give
//             each item starting this tick its offset in the ray pool, after
//             the survivors of the previous tick
//   generate  rays_from_light of those items (src/ray_generators.jl:64-97)
//   order     (optional, SPLAT_TUNE_RAY_ORDER) a counting sort of the rays
//             by (item, BVH position of the triangle left, direction
//             octant), so that a warp's rays share an item and a path
//   hit       its item's four-wide BVH (a warp of one item's coherent rays
//             as a packet) or a per-ray brute loop
//   evolve    per ray, evolve_ray with its item's material, seed and bounce
//             (src/tracer.jl:181-201); compaction and the diffuse-ray queue
//             as in the single-scene step
//   splat     per queued ray (all its planes), into its item's light map
//
// Items therefore join and leave at bounce granularity: a request that
// arrives while others are in flight starts at the next tick and overlaps
// with them on the device (continuous batching).  Every draw is keyed by the
// item's seed and the ray's grid index, and int32 maps accumulate exactly, so
// an item's map is the same alone, in any mix, and through
// splat_trace_forward.  A fixed set of admitted items can be captured once
// into a CUDA graph and replayed (the batched form).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "hitcore.cuh"
#include "optics.cuh"

namespace splat {

constexpr int kSlotShift = 24;
constexpr uint32_t kLocalMask = (1u << kSlotShift) - 1u;
constexpr int kMaxBatchItems = 256;

struct BatchItem {
    const splat_ftri_t* ftri;
    const TriHit* brute;
    const TriBox* brute_boxes;
    const Bvh4Node* nodes4;
    const TriHit* bvh_tris;
    int64_t n_recs, n_tris, first_diffuse;
    int32_t hitter;      // SPLAT_HITTER_BRUTE or SPLAT_HITTER_BVH
    int32_t depth;
    int32_t start_tick;  // tick of the first bounce; < 0: slot unused
    int32_t quirks;
    float force_rand;
    int32_t _pad0;
    GenParams gen;
    int64_t n_rays;
    splat_material_t material;
    SplatParams sp;
    const int32_t* bvh_pos;  // ray order: BVH position of each reference index
    int64_t key_base;        // ray order: the item's first bucket position
    int32_t pos_shift;       // ray order: low position bits dropped
    int32_t grid_rows;       // first tick: rows of the item's light grid when its rays start on a column
                             // (its fresh rays are taken in 8 x 4 tiles), else 0
};

struct FreshList {
    int32_t n;
    int32_t _pad;
    int64_t total;
    int32_t slot[kMaxBatchItems];
    int64_t prefix[kMaxBatchItems + 1];
    int64_t offset[kMaxBatchItems];
};

// Phase bodies of a tick, shared by the per-tick kernels and the persistent
// pass kernel: each takes its block index and block count.

// The items starting this tick, in slot order, get consecutive pool ranges
// after the survivors: one thread per slot, block-wide exclusive scans of
// (starts, rays).  One block of kMaxBatchItems threads.
__device__ __forceinline__ void reserve_phase(const BatchItem* items, int n_slots, int tick, int64_t* cur_count,
                                              FreshList* fresh) {
    __shared__ int s_wcount[kMaxBatchItems / 32];
    __shared__ long long s_wrays[kMaxBatchItems / 32];
    const int s = threadIdx.x;
    const int lane = s & 31, wid = s >> 5;
    const bool starts = s < n_slots && items[s].start_tick == tick;
    const long long nr = starts ? (long long)items[s].n_rays : 0;
    const unsigned m = __ballot_sync(0xffffffffu, starts);
    long long incl = nr;  // inclusive scan of the rays within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) {
        s_wcount[wid] = __popc(m);
        s_wrays[wid] = incl;
    }
    const int64_t base = *cur_count;
    __syncthreads();
    int cbase = 0;
    long long rbase = 0;
    for (int w = 0; w < wid; ++w) {
        cbase += s_wcount[w];
        rbase += s_wrays[w];
    }
    if (starts) {
        const int f = cbase + __popc(m & ((1u << lane) - 1u));
        const long long run = rbase + incl - nr;
        fresh->slot[f] = s;
        fresh->prefix[f] = run;
        fresh->offset[f] = base + run;
    }
    __syncthreads();  // every thread has read *cur_count
    if (s == kMaxBatchItems - 1) {
        const int n_fresh = cbase + __popc(m);
        const long long total = rbase + incl;
        fresh->prefix[n_fresh] = total;
        fresh->n = n_fresh;
        fresh->total = total;
        *cur_count = base + total;
    }
}

__global__ void __launch_bounds__(kMaxBatchItems) batch_reserve_kernel(const BatchItem* items, int n_slots, int tick,
                                                                       int64_t* cur_count, FreshList* fresh) {
    reserve_phase(items, n_slots, tick, cur_count, fresh);
}

// The pool position a kernel of this tick takes as its kk-th: fresh rays of
// an item on its first tick in 8 x 4 tiles of the item's light grid
// (grid_tile_ray: a bijection of the item's range), so that a warp's
// first-bounce rays are a compact patch and evolve's survivors leave as
// such; every other position as it is.  Hit and evolve use the same map.
__device__ __forceinline__ int64_t fresh_tiled(const FreshList* __restrict__ fresh,
                                               const BatchItem* __restrict__ items, int64_t kk) {
    const int nf = fresh->n;
    if (nf == 0 || kk < fresh->offset[0]) return kk;
    int lo = 0, hi = nf - 1;
    while (lo < hi) {  // last f with offset[f] <= kk
        const int mid = (lo + hi + 1) >> 1;
        if (fresh->offset[mid] <= kk) lo = mid;
        else hi = mid - 1;
    }
    const int64_t local = kk - fresh->offset[lo];
    const int64_t nr = fresh->prefix[lo + 1] - fresh->prefix[lo];
    const int32_t h = items[fresh->slot[lo]].grid_rows;
    if (h <= 0 || local >= nr) return kk;
    return fresh->offset[lo] + (int64_t)grid_tile_ray((uint32_t)local, (uint32_t)h, (uint32_t)nr);
}

__device__ __forceinline__ void generate_phase(const BatchItem* __restrict__ items,
                                               const FreshList* __restrict__ fresh, RaySoA out, int64_t bid,
                                               int64_t nblk) {
    const int64_t total = fresh->total;
    const int nf = fresh->n;
    for (int64_t g = bid * blockDim.x + threadIdx.x; g < total; g += nblk * blockDim.x) {
        int lo = 0, hi = nf - 1;
        while (lo < hi) {  // last f with prefix[f] <= g
            const int mid = (lo + hi + 1) >> 1;
            if (fresh->prefix[mid] <= g) lo = mid;
            else hi = mid - 1;
        }
        const int slot = fresh->slot[lo];
        const int64_t local = g - fresh->prefix[lo];
        const BatchItem& it = items[slot];
        const RayState r = gen_ray(it.gen, it.gen.ray_begin + local);
        store_ray(out, fresh->offset[lo] + local, r, ((uint32_t)slot << kSlotShift) | (uint32_t)local);
    }
}

__global__ void batch_generate_kernel(const BatchItem* __restrict__ items, const FreshList* __restrict__ fresh,
                                      RaySoA out) {
    generate_phase(items, fresh, out, blockIdx.x, gridDim.x);
}

// A warp whose 32 rays all belong to one BVH item may walk them as a packet
// (bvh4_closest_packet on pstack, the warp's kPacketStack entries of shared
// memory), by packet_form of packet_mode and of whether the item is on its
// first bounce this tick; every other warp traces one ray per lane.
// perm (optional): the rays in ray order, perm[j] the pool index of the j-th.
template <bool ANY_BRUTE>
__device__ __forceinline__ void hit_phase(RaySoA in, const int64_t* __restrict__ count,
                                          const BatchItem* __restrict__ items, int32_t* hit_idx, int32_t* err,
                                          unsigned long long* fetch, int tick, int packet_mode, int2* pstack,
                                          const int32_t* __restrict__ perm = nullptr,
                                          const FreshList* __restrict__ fresh = nullptr) {
    const int64_t n = *count;
    const int lane = threadIdx.x & 31;
    int2 stack[kBvhStack];
    RaySrc src{};
    src.f = in.f;
    src.ignore = in.ignore;
    src.cap = in.cap;
    for_each_warp_batch(n, fetch, [&](int64_t base) {
        const bool valid = base + lane < n;
        const int64_t kk = valid ? base + lane : base;  // idle lanes repeat lane 0's ray
        int64_t k = kk;
        if (perm) {
            k = (int64_t)perm[kk];
            if ((uint64_t)k >= (uint64_t)n) {  // never: perm is a permutation of 0 .. n - 1
                atomicOr(err, 4);
                k = kk;
            }
        } else if (fresh) {
            k = fresh_tiled(fresh, items, kk);
        }
        const HitRay r = load_hit_ray<false>(src, k);
        const uint32_t slot = in.id[k] >> kSlotShift;
        const BatchItem& it = items[slot];
        const bool bvh = !ANY_BRUTE || (it.hitter == SPLAT_HITTER_BVH && it.nodes4);
        const uint32_t slot0 = __shfl_sync(0xffffffffu, slot, 0);
        bool packet = false;
        if (packet_mode > 0 && __all_sync(0xffffffffu, bvh & (slot == slot0))) {
            const int form = packet_form(packet_mode, tick == it.start_tick);  // warp-uniform: one item
            packet = form == 1 || (form >= 2 && packet_coherent(r, form, bvh4_extent(it.nodes4)));
        }
        float best;
        int32_t bi;
        if (packet) {
            bvh4_closest_packet(r, valid, Bvh4View{it.nodes4, it.bvh_tris}, pstack, err, best, bi);
        } else if (valid) {
            if (bvh)
                bvh4_closest(r, Bvh4View{it.nodes4, it.bvh_tris}, stack, err, best, bi);
            else
                brute_closest(r, it.brute, it.brute_boxes, it.n_recs, best, bi);
        }
        if (valid) hit_idx[k] = bi;
    });
}

constexpr int kBatchHitThreads = 128;

// ORDER: the rays are read through the ray-order permutation perm (where an
// item's fresh rays sit in one bucket per octant, in placement order);
// otherwise in pool order with each item's first-tick rays in 8 x 4 tiles of
// its light grid (fresh_tiled).  Separate instantiations, so the form
// without perm keeps its register count.
template <bool ANY_BRUTE, bool ORDER>
__global__ void __launch_bounds__(kBatchHitThreads, 8) batch_hit_kernel(RaySoA in, const int64_t* __restrict__ count,
                                                                        const BatchItem* __restrict__ items,
                                                                        int32_t* hit_idx, int32_t* err,
                                                                        unsigned long long* fetch, int tick,
                                                                        int packet_mode,
                                                                        const int32_t* __restrict__ perm,
                                                                        const FreshList* __restrict__ fresh) {
    __shared__ int2 s_pstack[kBatchHitThreads / 32][kPacketStack];
    hit_phase<ANY_BRUTE>(in, count, items, hit_idx, err, fetch, tick, packet_mode, s_pstack[threadIdx.x >> 5],
                         ORDER ? perm : nullptr, ORDER ? nullptr : fresh);
}

// Ray-order keys of the tick's active rays and the size of every bucket
// (one atomic per group of equal keys in a warp).  A ray's key is its
// item's base plus the BVH position of the triangle it leaves (0 for a
// fresh ray), shifted, times 8, plus its direction octant; items without a
// BVH have one position.
__global__ void batch_order_count_kernel(RaySoA in, const int64_t* __restrict__ count, int64_t cap_rays,
                                         const BatchItem* __restrict__ items, uint32_t* __restrict__ keys,
                                         uint32_t* __restrict__ cnt) {
    const int64_t n = min(min(in.cap, cap_rays), *count);  // the rays the placement kernel places
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride) {
        const int64_t k = base + lane;
        const bool valid = k < n;
        uint32_t key = 0xffffffffu;
        if (valid) {
            const BatchItem& it = items[in.id[k] >> kSlotShift];
            const int32_t ig = in.ignore[k];
            const uint32_t pos = (it.bvh_pos && ig >= 1 && (int64_t)ig <= it.n_tris)
                                     ? (uint32_t)it.bvh_pos[ig] >> it.pos_shift : 0u;
            const uint32_t cls = (in.f[3 * in.cap + k] < 0.0f ? 1u : 0u) | (in.f[4 * in.cap + k] < 0.0f ? 2u : 0u) |
                                 (in.f[5 * in.cap + k] < 0.0f ? 4u : 0u);
            key = ((uint32_t)it.key_base + pos) * 8u + cls;
            keys[k] = key;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&cnt[key], (uint32_t)__popc(peers));
    }
}

// Slots of the ray order: every ray takes the next slot of its bucket, one
// atomic per group of equal keys in a warp.  Threads take the pool in the
// order the unordered hit kernel would (an item's fresh rays in tiles), and
// one block per 256 rays starts in index order, so a bucket's rays keep
// nearly that order.
__global__ void batch_order_place_kernel(const uint32_t* __restrict__ keys, const int64_t* __restrict__ count,
                                         int64_t cap_rays, int64_t pool_cap, uint32_t* __restrict__ off,
                                         int32_t* __restrict__ perm, const BatchItem* __restrict__ items,
                                         const FreshList* __restrict__ fresh) {
    const int64_t n = min(min(pool_cap, cap_rays), *count);
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride) {
        const bool valid = base + lane < n;
        const int64_t k = valid ? fresh_tiled(fresh, items, base + lane) : 0;
        const uint32_t key = valid ? keys[k] : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        uint32_t slot = 0;
        if (valid && lane == leader) slot = atomicAdd(&off[key], (uint32_t)__popc(peers));
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (valid) perm[slot + (uint32_t)__popc(peers & below)] = (int32_t)k;
    }
}

constexpr int kBatchThreads = 256;

// MK >= 0: every item in flight has this material kind (compile-time, so
// only its optics is inlined); -1: per item.  Whole blocks of kBatchThreads.
template <int MK>
__device__ __forceinline__ void evolve_phase(RaySoA in, RaySoA out, RaySoA queue, const int64_t* __restrict__ in_count,
                                             int64_t* out_count, int64_t* queue_count,
                                             const BatchItem* __restrict__ items, int tick,
                                             const int32_t* __restrict__ hit_idx, int32_t* err, int64_t bid,
                                             int64_t nblk, const FreshList* __restrict__ fresh = nullptr) {
    // double-buffered by iteration parity, as in evolve_kernel
    __shared__ int s_keep2[2][kBatchThreads / 32], s_dif2[2][kBatchThreads / 32];
    __shared__ unsigned long long s_kbase2[2], s_dbase2[2];
    const int64_t n = *in_count;
    const int lane = lane_id();
    const int wid = threadIdx.x >> 5;
    int par = 0;
    for (int64_t base = bid * kBatchThreads; base < n; base += nblk * kBatchThreads, par ^= 1) {
        int* s_keep = s_keep2[par];
        int* s_dif = s_dif2[par];
        unsigned long long& s_kbase = s_kbase2[par];
        unsigned long long& s_dbase = s_dbase2[par];
        int64_t k = base + threadIdx.x;
        bool keep = false, dif = false;
        RayState o;
        uint32_t id = 0;
        if (k < n) {
            if (fresh) k = fresh_tiled(fresh, items, k);
            const RayState r = load_ray(in, k);
            id = in.id[k];
            const BatchItem& it = items[id >> kSlotShift];
            const uint32_t bounce = (uint32_t)(tick - it.start_tick + 1);
            EvolveView v{it.ftri, it.n_tris, err, it.first_diffuse, it.material, it.gen.seed, bounce,
                         it.force_rand, it.quirks != 0, (int)bounce >= it.depth};
            if (MK >= 0) v.material.kind = MK;
            int32_t ih;
            const uint32_t grid_id = (uint32_t)(it.gen.ray_begin + (id & kLocalMask));
            const int fate = evolve_one<true>(r, hit_idx[k], grid_id, v, o, ih);
            keep = fate == kFateKeep;
            dif = fate == kFateDiffuse;
        }
        const unsigned kb = __ballot_sync(0xffffffffu, keep);
        const unsigned db = __ballot_sync(0xffffffffu, dif);
        if (lane == 0) {
            s_keep[wid] = __popc(kb);
            s_dif[wid] = __popc(db);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int tk = 0, td = 0;
            for (int w = 0; w < kBatchThreads / 32; ++w) {
                const int a = s_keep[w], b = s_dif[w];
                s_keep[w] = tk;
                s_dif[w] = td;
                tk += a;
                td += b;
            }
            s_kbase = tk ? atomicAdd(reinterpret_cast<unsigned long long*>(out_count), (unsigned long long)tk) : 0ull;
            s_dbase = td ? atomicAdd(reinterpret_cast<unsigned long long*>(queue_count), (unsigned long long)td) : 0ull;
        }
        __syncthreads();
        const unsigned below = (1u << lane) - 1u;
        if (keep) store_ray(out, (int64_t)s_kbase + s_keep[wid] + __popc(kb & below), o, id);
        else if (dif) store_ray(queue, (int64_t)s_dbase + s_dif[wid] + __popc(db & below), o, id);
    }
}

template <int MK>
__global__ void __launch_bounds__(kBatchThreads) batch_evolve_kernel(RaySoA in, RaySoA out, RaySoA queue,
                                                                     const int64_t* __restrict__ in_count,
                                                                     int64_t* out_count, int64_t* queue_count,
                                                                     const BatchItem* __restrict__ items, int tick,
                                                                     const int32_t* __restrict__ hit_idx,
                                                                     int32_t* err,
                                                                     const FreshList* __restrict__ fresh) {
    evolve_phase<MK>(in, out, queue, in_count, out_count, queue_count, items, tick, hit_idx, err, blockIdx.x,
                     gridDim.x, fresh);
}

// One lane per queued ray, walking all of its planes: rays of one item are
// adjacent in the queue, so a warp's lanes usually share an item and its
// plane count, and no lane idles on frames with few planes.
__device__ __forceinline__ void splat_one(RaySoA q, int64_t k, const BatchItem* __restrict__ items) {
    const RayState r = load_ray(q, k);
    const BatchItem& it = items[q.id[k] >> kSlotShift];
    const SplatView sp = splat_view(it.sp);
    const int planes = sp.n_lambda > 0 ? sp.n_lambda : 1;
    const Tri T = load_tri(it.ftri, r.ignore);
    const TriUV quv = tri_uv(T);
    for (int il = 0; il < planes; ++il) (void)splat_ray_plane(sp, r, T, quv, il);
}

__global__ void __launch_bounds__(256, 2) batch_splat_kernel(RaySoA q, const int64_t* __restrict__ count,
                                                             const BatchItem* __restrict__ items) {
    const int64_t n = *count;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        splat_one(q, k, items);
}

// The same through the block's shared texel table keyed by texel address
// (rays of one block may splat into different items' maps): plane by plane
// up to the block's largest plane count.
__global__ void __launch_bounds__(256, 2) batch_splat_agg_kernel(RaySoA q, const int64_t* __restrict__ count,
                                                                 const BatchItem* __restrict__ items) {
    __shared__ unsigned long long s_key[kAggSlots];
    __shared__ int32_t s_val[kAggSlots];
    __shared__ int s_planes;
    const int64_t n = *count;
    addr_table_clear(s_key, s_val);
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = base + threadIdx.x;
        const bool live = k < n;
        if (threadIdx.x == 0) s_planes = 0;
        __syncthreads();
        RayState r;
        Tri T;
        TriUV quv;
        const BatchItem* it = nullptr;
        int planes = 0;
        if (live) {
            r = load_ray(q, k);
            it = &items[q.id[k] >> kSlotShift];
            planes = it->sp.n_lambda > 0 ? it->sp.n_lambda : 1;
            T = load_tri(it->ftri, r.ignore);
            quv = tri_uv(T);
            atomicMax(&s_planes, planes);
        }
        __syncthreads();
        const int block_planes = s_planes;
        for (int il = 0; il < block_planes; ++il) {
            if (il < planes) (void)splat_ray_plane(it->sp, r, T, quv, il, AddrTableSink{it->sp, s_key, s_val});
            __syncthreads();
            addr_table_flush(s_key, s_val);
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// persistent pass: every tick of a captured pass in one cooperative launch
// ---------------------------------------------------------------------------
// All items start at the pass's first tick.  Per tick: reserve (block 0) |
// generate | this tick's traversal, then the previous tick's splat segment
// (warps take 32 rays at a time from work counters, so the blocks done with
// the traversal splat while its last rays are traced) | evolve, with a
// bounded grid-wide wait between the phases.  The splat queue fills over the
// whole pass (a ray is queued at most once, so the pool's capacity holds
// it); tick i's segment is [qmark[i], qmark[i + 1]).
constexpr uint32_t kGridWaitLimit = 1u << 22;  // polls of >= 256 ns: over a second

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide wait: every block arrives, then waits until `target` arrivals,
// at most kGridWaitLimit polls; gives up with error bit 64 (no trap, no
// unbounded spin).  The fences make every block's writes before the wait
// visible to every block after it.
__device__ __forceinline__ bool grid_wait(unsigned* bar, unsigned target, int32_t* err) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        int ok = 1;
        for (uint32_t it = 0; ld_acquire(bar) < target; ++it) {
            if (it >= kGridWaitLimit) {
                atomicOr(err, 64);
                ok = 0;
                break;
            }
            __nanosleep(256);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <int MK>
__global__ void __launch_bounds__(kBatchThreads, 2) batch_pass_kernel(BatchPassArgs P) {
    const BatchItem* items = reinterpret_cast<const BatchItem*>(P.items);
    FreshList* fresh = reinterpret_cast<FreshList*>(P.fresh);
    __shared__ int2 s_pstack[kBatchThreads / 32][kPacketStack];
    const unsigned nblk = gridDim.x;
    unsigned waits = 0;
    for (int i = 0; i < P.n_ticks; ++i) {
        const int tick = P.t0 + i;
        const RaySoA cur = (i & 1) ? P.b : P.a, nxt = (i & 1) ? P.a : P.b;
        if (blockIdx.x == 0) {
            reserve_phase(items, P.n_slots, tick, &P.count[i], fresh);
            if (threadIdx.x == 0) P.qmark[i] = *P.qcount;  // the queue before this tick's evolve
        }
        if (!grid_wait(P.bar, ++waits * nblk, P.err)) return;
        generate_phase(items, fresh, cur, blockIdx.x, nblk);
        if (!grid_wait(P.bar, ++waits * nblk, P.err)) return;
        hit_phase<true>(cur, &P.count[i], items, P.hit_idx, P.err, &P.fetch[i], tick, P.packet_mode,
                        s_pstack[threadIdx.x >> 5]);
        if (i > 0) {
            const int64_t q0 = P.qmark[i - 1], q1 = P.qmark[i];
            for_each_ray(q1 - q0, &P.splat_fetch[i - 1], [&](int64_t k) { splat_one(P.queue, q0 + k, items); });
        }
        if (!grid_wait(P.bar, ++waits * nblk, P.err)) return;
        evolve_phase<MK>(cur, nxt, P.queue, &P.count[i], &P.count[i + 1], P.qcount, items, tick, P.hit_idx, P.err,
                         blockIdx.x, nblk);
        if (!grid_wait(P.bar, ++waits * nblk, P.err)) return;
    }
    const int64_t q0 = P.qmark[P.n_ticks - 1], q1 = *P.qcount;
    for_each_ray(q1 - q0, &P.splat_fetch[P.n_ticks - 1], [&](int64_t k) { splat_one(P.queue, q0 + k, items); });
}

template <int MK>
static cudaError_t launch_pass_mk(const BatchPassArgs& a, int share, int sm_count, cudaStream_t s) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_pass_kernel<MK>, kBatchThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int grid = per_sm * sm_count / (share < 1 ? 1 : share);
    if (grid < 1) grid = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, batch_pass_kernel<MK>, a);
    ++g_launches;
    return e;
}

cudaError_t launch_batch_pass(const BatchPassArgs& a, int share, int sm_count, cudaStream_t s) {
    if (a.n_ticks < 1 || a.n_ticks > kMaxPassTicks) return cudaErrorInvalidValue;
    switch (a.material_kind) {
        case SPLAT_MATERIAL_LINEAR_REF: return launch_pass_mk<SPLAT_MATERIAL_LINEAR_REF>(a, share, sm_count, s);
        case SPLAT_MATERIAL_CAUCHY: return launch_pass_mk<SPLAT_MATERIAL_CAUCHY>(a, share, sm_count, s);
        case SPLAT_MATERIAL_SELLMEIER: return launch_pass_mk<SPLAT_MATERIAL_SELLMEIER>(a, share, sm_count, s);
        default: return launch_pass_mk<-1>(a, share, sm_count, s);
    }
}

static int grid_cap(int64_t n, int threads, int sm_count, int per_sm) {
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count * per_sm;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_batch_tick(const BatchTickArgs& a, cudaStream_t s) {
    cudaError_t e = launch_batch_trace(a, s);
    if (e != cudaSuccess) return e;
    return launch_batch_splat(a, s);
}

cudaError_t launch_batch_trace(const BatchTickArgs& a, cudaStream_t s) {
    const BatchItem* items = reinterpret_cast<const BatchItem*>(a.items);
    FreshList* fresh = reinterpret_cast<FreshList*>(a.fresh);
    batch_reserve_kernel<<<1, kMaxBatchItems, 0, s>>>(items, a.n_slots, a.tick, a.cur_count, fresh);
    ++g_launches;
    if (a.fresh_rays > 0) {
        batch_generate_kernel<<<grid_cap(a.fresh_rays, 256, a.sm_count, 8), 256, 0, s>>>(items, fresh, a.cur);
        ++g_launches;
    }
    if (a.cap_rays > 0) {
        const int mode = g_tune[SPLAT_TUNE_BVH_PACKET];
        const int32_t* perm = nullptr;
        if (a.order_buckets > 0 && a.order_perm) {
            cudaError_t e = cudaMemsetAsync(a.order_cnt, 0, sizeof(uint32_t) * (size_t)a.order_buckets, s);
            if (e != cudaSuccess) return e;
            batch_order_count_kernel<<<grid_cap(a.cap_rays, 256, a.sm_count, 8), 256, 0, s>>>(
                a.cur, a.cur_count, a.cap_rays, items, a.order_keys, a.order_cnt);
            ++g_launches;
            if ((e = launch_order_scan(a.order_cnt, a.order_buckets, a.order_sums, s)) != cudaSuccess) return e;
            batch_order_place_kernel<<<(unsigned)((a.cap_rays + 255) / 256), 256, 0, s>>>(
                a.order_keys, a.cur_count, a.cap_rays, a.cur.cap, a.order_cnt, a.order_perm, items, fresh);
            ++g_launches;
            perm = a.order_perm;
        }
        auto hit = [&](auto kernel) {
            const int grid = resident_grid(reinterpret_cast<const void*>(kernel), a.cap_rays, a.sm_count,
                                           kBatchHitThreads, g_tune[SPLAT_TUNE_BVH_BLOCKS_PER_SM]);
            kernel<<<grid, kBatchHitThreads, 0, s>>>(a.cur, a.cur_count, items, a.hit_idx, a.err, a.fetch, a.tick,
                                                      mode, perm, fresh);
        };
        if (a.any_brute)
            perm ? hit(batch_hit_kernel<true, true>) : hit(batch_hit_kernel<true, false>);
        else
            perm ? hit(batch_hit_kernel<false, true>) : hit(batch_hit_kernel<false, false>);
        ++g_launches;
        const int eg = grid_cap(a.cap_rays, kBatchThreads, a.sm_count, g_tune[SPLAT_TUNE_EVOLVE_BLOCKS_PER_SM]);
#define SPLAT_BATCH_EVOLVE(MK)                                                                            \
    batch_evolve_kernel<MK><<<eg, kBatchThreads, 0, s>>>(a.cur, a.next, a.queue, a.cur_count, a.next_count, \
                                                         a.queue_count, items, a.tick, a.hit_idx, a.err, fresh)
        switch (a.material_kind) {
            case SPLAT_MATERIAL_LINEAR_REF: SPLAT_BATCH_EVOLVE(SPLAT_MATERIAL_LINEAR_REF); break;
            case SPLAT_MATERIAL_CAUCHY: SPLAT_BATCH_EVOLVE(SPLAT_MATERIAL_CAUCHY); break;
            case SPLAT_MATERIAL_SELLMEIER: SPLAT_BATCH_EVOLVE(SPLAT_MATERIAL_SELLMEIER); break;
            default: SPLAT_BATCH_EVOLVE(-1); break;
        }
#undef SPLAT_BATCH_EVOLVE
        ++g_launches;
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_splat(const BatchTickArgs& a, cudaStream_t s) {
    if (a.cap_rays <= 0) return cudaSuccess;
    const BatchItem* items = reinterpret_cast<const BatchItem*>(a.items);
    const int sg = grid_cap(a.cap_rays, 256, a.sm_count, g_tune[SPLAT_TUNE_SPLAT_BLOCKS_PER_SM]);
    if (g_tune[SPLAT_TUNE_SPLAT_AGGREGATE])
        batch_splat_agg_kernel<<<sg, 256, 0, s>>>(a.queue, a.queue_count, items);
    else
        batch_splat_kernel<<<sg, 256, 0, s>>>(a.queue, a.queue_count, items);
    ++g_launches;
    return cudaGetLastError();
}

size_t batch_item_bytes() { return sizeof(BatchItem); }
size_t batch_fresh_bytes() { return sizeof(FreshList); }

void batch_fill_item(void* dst, const BatchSceneRef& sc, const GenParams& gen, int64_t n_rays, int32_t depth,
                     int32_t hitter, int32_t start_tick, int32_t quirks, float force_rand,
                     const splat_material_t& material, const SplatParams& sp) {
    BatchItem it;
    std::memset(&it, 0, sizeof(it));
    it.ftri = sc.ftri;
    it.brute = sc.brute;
    it.brute_boxes = sc.brute_boxes;
    it.nodes4 = sc.nodes4;
    it.bvh_tris = sc.bvh_tris;
    it.n_recs = sc.n_recs;
    it.n_tris = sc.n_tris;
    it.first_diffuse = sc.first_diffuse;
    it.hitter = hitter;
    it.depth = depth;
    it.start_tick = start_tick;
    it.quirks = quirks;
    it.force_rand = force_rand;
    it.gen = gen;
    it.n_rays = n_rays;
    it.material = material;
    it.sp = sp;
    it.bvh_pos = sc.nodes4 ? sc.bvh_pos : nullptr;
    const int64_t rows = gen.light.res1 / gen.upscale;
    it.grid_rows = (rows >= 1 && rows <= (int64_t)kGridTileMaxRows && gen.ray_begin % rows == 0) ? (int32_t)rows : 0;
    std::memcpy(dst, &it, sizeof(it));
}

int64_t batch_assign_order_keys(void* items, const uint8_t* used, int32_t n_slots, int max_bits) {
    BatchItem* it = reinterpret_cast<BatchItem*>(items);
    const int64_t limit = (int64_t(1) << max_bits) / 8;  // positions that fit
    for (int shift = 0; shift < 31; ++shift) {
        int64_t total = 0;
        for (int32_t s = 0; s < n_slots; ++s)
            if (used[s]) total += (it[s].bvh_pos ? (it[s].n_tris >> shift) : 0) + 1;
        if (total > limit) continue;
        int64_t base = 0;
        for (int32_t s = 0; s < n_slots; ++s) {
            if (!used[s]) continue;
            it[s].key_base = base;
            it[s].pos_shift = shift;
            base += (it[s].bvh_pos ? (it[s].n_tris >> shift) : 0) + 1;
        }
        return total * 8;
    }
    return 0;
}

void batch_clear_item(void* dst) {
    BatchItem it;
    std::memset(&it, 0, sizeof(it));
    it.start_tick = -1;
    std::memcpy(dst, &it, sizeof(it));
}

void batch_set_seed(void* dst, uint64_t seed) { reinterpret_cast<BatchItem*>(dst)->gen.seed = seed; }

}  // namespace splat
