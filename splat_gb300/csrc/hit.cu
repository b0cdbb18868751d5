// hit.cu -- nearest-hit kernels.
//
// Semantics (src/hitters.jl:24-30, src/tracer.jl:45-59): for every ray, the
// lexicographic minimum of (t, index) over the triangles with
// in_triangle(o + d t) && t > 0 && index != ignore_tri; (Inf, 1) when none.
// All kernels evaluate the reference's test with the same binary32
// operations, so t and the index are bit-identical to the CPU restatement.
//
// * hit_brute_kernel: all pairs.  Hit records are staged through shared
//   memory by TMA bulk copies (cp.async.bulk + mbarrier, 4-stage ring, no
//   multicast); each thread keeps RPT rays in registers and their running
//   argmin.  Triangle ranges split over blockIdx.y merge with a packed 64-bit
//   atomicMin (src/atomic_argmin.jl).
// * hit_bvh_kernel: one thread per ray walks the flattened BVH2 with a short
//   per-thread stack; boxes are padded so every triangle whose test can
//   succeed is visited, and the same lexicographic rule makes the result
//   identical to brute force.
#include <cstdio>
#include <mutex>
#include <unordered_map>

#include "hitcore.cuh"

namespace splat {

thread_local int64_t g_launches = 0;
std::atomic<int32_t> g_tune[SPLAT_TUNE_KEYS] = {4, 16, 8, 8, 0, 1, 2, 0, 2, 0, 0, 64, 0, 0};

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + bulk copy (sm_90+ async proxy)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after kWaitLimit polls (each poll may suspend the
// thread for a hardware-chosen time), so a lost copy cannot hang the GPU.
constexpr uint32_t kWaitLimit = 1u << 24;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t limit = kWaitLimit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}
// Polls of the stalled wait that SPLAT_TUNE_TEST_WAIT_STALL injects.
constexpr uint32_t kStallPolls = 64;

// ---------------------------------------------------------------------------
// brute force, TMA-staged tiles
// ---------------------------------------------------------------------------
constexpr int kBruteThreads = 256;
constexpr int kTile = 64;  // records per tile of the n_tris drop-in kernel
constexpr int kStages = 4;

// TILE: hit records per stage of the ring (SPLAT_TUNE_BRUTE_TILE: 32, 64 or
// 128); the ring holds kStages x TILE x 112 bytes of shared memory.
template <int RPT, bool AOS, int TILE>
__global__ void __launch_bounds__(kBruteThreads) hit_brute_kernel(RaySrc src, const TriHit* __restrict__ recs,
                                                                  const TriBox* __restrict__ boxes,
                                                                  int64_t n_recs, int64_t per_split,
                                                                  int32_t* __restrict__ hit_idx,
                                                                  float* __restrict__ hit_t,
                                                                  unsigned long long* __restrict__ tmp,
                                                                  int32_t* err, int stall_tile) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TriHit* tiles = reinterpret_cast<TriHit*>(smem_raw);
    TriBox* btiles = reinterpret_cast<TriBox*>(smem_raw + (size_t)kStages * TILE * sizeof(TriHit));
    __shared__ __align__(8) uint64_t bars[kStages];
    // stall_tile >= 0 (test only): the wait for that tile polls `stall`, a
    // barrier that no copy and no thread ever completes, kStallPolls times,
    // so the block takes the failure path below with its copies in flight
    __shared__ __align__(8) uint64_t stall;

    const int64_t n = src.d_count ? *src.d_count : src.n;
    const int64_t ray0 = (int64_t)blockIdx.x * kBruteThreads * RPT;
    if (ray0 >= n) return;
    const int64_t tb = (int64_t)blockIdx.y * per_split;
    const int64_t te = min(n_recs, tb + per_split);
    if (tb >= te) return;
    const int n_tiles = (int)((te - tb + TILE - 1) / TILE);

    HitRay ray[RPT];
    float best[RPT];
    int32_t bi[RPT];
    float inv[RPT][3], oinv[RPT][3];  // slab-test terms of the padded-box pre-test
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const int64_t k = ray0 + threadIdx.x + (int64_t)r * kBruteThreads;
        if (k < n) {
            ray[r] = load_hit_ray<AOS>(src, k);
        } else {
            ray[r] = HitRay{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
        }
        best[r] = __int_as_float(0x7f800000);
        bi[r] = 1;
        inv[r][0] = safe_inv(ray[r].dx);
        inv[r][1] = safe_inv(ray[r].dy);
        inv[r][2] = safe_inv(ray[r].dz);
        oinv[r][0] = ray[r].ox * inv[r][0];
        oinv[r][1] = ray[r].oy * inv[r][1];
        oinv[r][2] = ray[r].oz * inv[r][2];
    }

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
        mbar_init(&stall, 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto issue = [&](int kt) {
        const int s = kt % kStages;
        const int64_t first = tb + (int64_t)kt * TILE;
        const uint32_t cnt = (uint32_t)min((int64_t)TILE, te - first);
        const uint32_t bytes = cnt * (uint32_t)sizeof(TriHit), bbytes = cnt * (uint32_t)sizeof(TriBox);
        mbar_arrive_expect_tx(&bars[s], bytes + bbytes);
        bulk_g2s(tiles + s * TILE, recs + first, bytes, &bars[s]);
        bulk_g2s(btiles + s * TILE, boxes + first, bbytes, &bars[s]);
    };
    if (threadIdx.x == 0) {
        for (int kt = 0; kt < min(kStages, n_tiles); ++kt) issue(kt);
    }

    int consumed = 0;
    bool failed = false;
    for (int kt = 0; kt < n_tiles; ++kt) {
        const int s = kt % kStages;
        const uint32_t ph = (uint32_t)(kt / kStages) & 1u;
        const bool ok = kt == stall_tile ? mbar_wait_bounded(&stall, 0u, kStallPolls) : mbar_wait_bounded(&bars[s], ph);
        if (__syncthreads_or(!ok)) {
            failed = true;
            break;
        }
        const int cnt = (int)min((int64_t)TILE, te - (tb + (int64_t)kt * TILE));
        const TriHit* tile = tiles + s * TILE;
        const TriBox* btile = btiles + s * TILE;
#pragma unroll 2
        for (int j = 0; j < cnt; ++j) {
            const float4 lo = btile[j].lo, hi = btile[j].hi;
#pragma unroll
            for (int r = 0; r < RPT; ++r) {
                // the padded box first (the BVH leaves' test): a ray that misses it
                // cannot be accepted by the triangle's test
                const float a0 = fmaf(lo.x, inv[r][0], -oinv[r][0]), b0 = fmaf(hi.x, inv[r][0], -oinv[r][0]);
                const float a1 = fmaf(lo.y, inv[r][1], -oinv[r][1]), b1 = fmaf(hi.y, inv[r][1], -oinv[r][1]);
                const float a2 = fmaf(lo.z, inv[r][2], -oinv[r][2]), b2 = fmaf(hi.z, inv[r][2], -oinv[r][2]);
                const float tmin = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fminf(a2, b2));
                const float tmax = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fmaxf(a2, b2));
                if (!((tmin <= tmax) & (tmax >= 0.0f) & (tmin <= best[r]))) continue;
                const float4 q0 = tile[j].n_nv;
                float num, den;
                if (!tri_candidate(q0, ray[r], best[r], num, den)) continue;
                const float4 q1 = tile[j].a_idx;
                const int32_t idx = __float_as_int(q1.w);
                bool inside;
                const float t = tri_t_from(num, den, q1, tile[j].e0, tile[j].e1, tile[j].inv, ray[r], inside);
                if (inside & (t > 0.0f) & (idx != ray[r].ig) & (t < best[r])) {
                    best[r] = t;
                    bi[r] = idx;
                }
            }
        }
        consumed = kt + 1;
        __syncthreads();
        if (threadIdx.x == 0 && kt + kStages < n_tiles) {
            fence_proxy_async();
            issue(kt + kStages);
        }
    }
    if (failed) {
        if (threadIdx.x == 0) {
            atomicOr(err, 1);
            // drain this block's copies still in flight (bounded) before exit:
            // tiles consumed .. consumed + kStages - 1 were issued
            const int issued = min(n_tiles, consumed + kStages);
            for (int kt = consumed; kt < issued; ++kt)
                (void)mbar_wait_bounded(&bars[kt % kStages], (uint32_t)(kt / kStages) & 1u);
        }
        return;
    }

#pragma unroll
    for (int r = 0; r < RPT; ++r) {
        const int64_t k = ray0 + threadIdx.x + (int64_t)r * kBruteThreads;
        if (k >= n) continue;
        if (tmp) {
            if (bi[r] != 1) atomicMin(tmp + k, (unsigned long long)pack_argmin(best[r], (uint32_t)bi[r]));
        } else {
            hit_idx[k] = bi[r];
            if (hit_t) hit_t[k] = best[r];
        }
    }
}

__global__ void fill_u64_kernel(unsigned long long* p, int64_t n, const int64_t* d_count, unsigned long long v) {
    const int64_t m = d_count ? *d_count : n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x)
        p[k] = v;
}

__global__ void unpack_hits_kernel(const unsigned long long* tmp, int64_t n, const int64_t* d_count,
                                   int32_t* hit_idx, float* hit_t) {
    const int64_t m = d_count ? *d_count : n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t v = tmp[k];
        hit_idx[k] = (int32_t)(uint32_t)(v & 0xffffffffull);
        if (hit_t) hit_t[k] = monotonic_f32((uint32_t)(v >> 32));
    }
}

__global__ void miss_kernel(int64_t n, const int64_t* d_count, int32_t* hit_idx, float* hit_t) {
    const int64_t m = d_count ? *d_count : n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
        hit_idx[k] = 1;
        if (hit_t) hit_t[k] = __int_as_float(0x7f800000);
    }
}

static int grid_for(int64_t n, int threads, int sm_count, int per_sm) {
    int64_t b = (n + threads - 1) / threads;
    int64_t cap = (int64_t)sm_count * per_sm;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_unpack_hits(const uint64_t* tmp, int64_t n, const int64_t* d_count, int32_t* hit_idx,
                               float* hit_t, cudaStream_t s) {
    unpack_hits_kernel<<<grid_for(n, 256, 152, 8), 256, 0, s>>>((const unsigned long long*)tmp, n, d_count, hit_idx,
                                                                hit_t);
    ++g_launches;
    return cudaGetLastError();
}

constexpr int kRPT = 2;

template <int TILE>
static void launch_brute_tiles(dim3 grid, cudaStream_t s, const RaySrc& rays, const TriHit* recs, const TriBox* boxes,
                               int64_t n_recs, int64_t per_split, int32_t* hit_idx, float* hit_t,
                               unsigned long long* tmp, int32_t* err, int stall_tile) {
    const size_t smem = (size_t)kStages * TILE * (sizeof(TriHit) + sizeof(TriBox));
    static bool configured = false;  // rings above 48 KB need the opt-in
    if (!configured) {
        cudaFuncSetAttribute(hit_brute_kernel<kRPT, true, TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(hit_brute_kernel<kRPT, false, TILE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        configured = true;
    }
    if (rays.aos)
        hit_brute_kernel<kRPT, true, TILE><<<grid, kBruteThreads, smem, s>>>(rays, recs, boxes, n_recs, per_split,
                                                                             hit_idx, hit_t, tmp, err, stall_tile);
    else
        hit_brute_kernel<kRPT, false, TILE><<<grid, kBruteThreads, smem, s>>>(rays, recs, boxes, n_recs, per_split,
                                                                              hit_idx, hit_t, tmp, err, stall_tile);
}

cudaError_t launch_hit_brute(const RaySrc& rays, int64_t cap, const TriHit* recs, const TriBox* boxes, int64_t n_recs,
                             int32_t* hit_idx, float* hit_t, uint64_t* tmp, int32_t* err, int sm_count,
                             cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    const int tile = g_tune[SPLAT_TUNE_BRUTE_TILE].load();
    const int64_t rays_per_block = (int64_t)kBruteThreads * kRPT;
    const int64_t ray_blocks = (cap + rays_per_block - 1) / rays_per_block;
    // split the triangle range so the grid covers the GPU a few times over
    int64_t splits = ((int64_t)sm_count * g_tune[SPLAT_TUNE_BRUTE_BLOCKS_PER_SM] + ray_blocks - 1) / ray_blocks;
    const int64_t max_splits = (n_recs + 4 * tile - 1) / (4 * tile);
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    if (splits > 65535) splits = 65535;
    if (tmp == nullptr) splits = 1;
    int64_t per_split = (n_recs + splits - 1) / splits;
    per_split = ((per_split + tile - 1) / tile) * tile;
    splits = (n_recs + per_split - 1) / per_split;
    if (splits < 1) splits = 1;
    const bool use_tmp = splits > 1;
    const int stall_tile = g_tune[SPLAT_TUNE_TEST_WAIT_STALL] - 1;
    if (use_tmp) {
        fill_u64_kernel<<<grid_for(cap, 256, sm_count, 8), 256, 0, s>>>((unsigned long long*)tmp, cap, rays.d_count,
                                                                        (unsigned long long)kNoHit);
        ++g_launches;
    }
    dim3 grid((unsigned)ray_blocks, (unsigned)splits);
    if (n_recs > 0) {
        unsigned long long* t = use_tmp ? (unsigned long long*)tmp : nullptr;
        if (tile == 32)
            launch_brute_tiles<32>(grid, s, rays, recs, boxes, n_recs, per_split, hit_idx, hit_t, t, err, stall_tile);
        else if (tile == 128)
            launch_brute_tiles<128>(grid, s, rays, recs, boxes, n_recs, per_split, hit_idx, hit_t, t, err, stall_tile);
        else
            launch_brute_tiles<64>(grid, s, rays, recs, boxes, n_recs, per_split, hit_idx, hit_t, t, err, stall_tile);
        ++g_launches;
    } else {
        // no triangles: every ray misses
        miss_kernel<<<grid_for(cap, 256, sm_count, 8), 256, 0, s>>>(cap, rays.d_count, hit_idx, hit_t);
        ++g_launches;
        return cudaGetLastError();
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (use_tmp) return launch_unpack_hits(tmp, cap, rays.d_count, hit_idx, hit_t, s);
    return cudaSuccess;
}

// ---------------------------------------------------------------------------
// brute force over the reference's n_tris array (next_hit_kernel6 drop-in)
// ---------------------------------------------------------------------------
__device__ __forceinline__ TriHit pack_one(int32_t idx, F3 n, F3 a, F3 b, F3 c) {
    TriHit h;
    F3 v0 = c - a, v1 = b - a;
    float dot00 = dot(v0, v0), dot01 = dot(v0, v1), dot11 = dot(v1, v1);
    float invDenom = 1.0f / (dot00 * dot11 - dot01 * dot01);
    h.n_nv = make_float4(n.x, n.y, n.z, dot(n, a));
    h.a_idx = make_float4(a.x, a.y, a.z, __int_as_float(idx));
    h.e0 = make_float4(v0.x, v0.y, v0.z, dot00);
    h.e1 = make_float4(v1.x, v1.y, v1.z, dot11);
    h.inv = make_float4(dot01, invDenom, 0.f, 0.f);
    return h;
}

__global__ void __launch_bounds__(kBruteThreads) hit_ntris_kernel(const splat_adray_t* __restrict__ rays,
                                                                   int64_t n_rays, const splat_ntri_t* __restrict__ nt,
                                                                   int64_t n_tris, int64_t per_split,
                                                                   unsigned long long* __restrict__ tmp) {
    __shared__ TriHit tile[kTile];
    RaySrc src{};
    src.aos = rays;
    src.n = n_rays;
    const int64_t ray0 = (int64_t)blockIdx.x * kBruteThreads * kRPT;
    const int64_t tb = (int64_t)blockIdx.y * per_split;
    const int64_t te = min(n_tris, tb + per_split);
    if (tb >= te) return;
    HitRay ray[kRPT];
    float best[kRPT];
    int32_t bi[kRPT];
#pragma unroll
    for (int r = 0; r < kRPT; ++r) {
        const int64_t k = ray0 + threadIdx.x + (int64_t)r * kBruteThreads;
        ray[r] = k < n_rays ? load_hit_ray<true>(src, k) : HitRay{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
        best[r] = __int_as_float(0x7f800000);
        bi[r] = 1;
    }
    for (int64_t base = tb; base < te; base += kTile) {
        const int cnt = (int)min((int64_t)kTile, te - base);
        if (threadIdx.x < cnt) {
            const splat_ntri_t& q = nt[base + threadIdx.x];
            tile[threadIdx.x] = pack_one(q.idx, f3(q.v[0]), f3(q.v[1]), f3(q.v[2]), f3(q.v[3]));
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const float4 q0 = tile[j].n_nv, q1 = tile[j].a_idx, q2 = tile[j].e0, q3 = tile[j].e1, q4 = tile[j].inv;
            const int32_t idx = __float_as_int(q1.w);
#pragma unroll
            for (int r = 0; r < kRPT; ++r) {
                bool inside;
                const float t = tri_t(q0, q1, q2, q3, q4, ray[r], inside);
                // next_hit_kernel6 (src/hitters.jl:183) has no i != 1 test: the
                // sentinel's t is NaN and fails t > 0.
                if (inside & (t > 0.0f) & (idx != ray[r].ig) & (t < best[r])) {
                    best[r] = t;
                    bi[r] = idx;
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < kRPT; ++r) {
        const int64_t k = ray0 + threadIdx.x + (int64_t)r * kBruteThreads;
        if (k < n_rays && bi[r] != 1) atomicMin(tmp + k, (unsigned long long)pack_argmin(best[r], (uint32_t)bi[r]));
    }
}

cudaError_t launch_hit_brute_ntris(const splat_adray_t* rays, int64_t n_rays, const splat_ntri_t* ntris,
                                   int64_t n_tris, uint64_t* tmp, int32_t* hit_idx, int sm_count, cudaStream_t s) {
    if (n_rays <= 0) return cudaSuccess;
    fill_u64_kernel<<<grid_for(n_rays, 256, sm_count, 8), 256, 0, s>>>((unsigned long long*)tmp, n_rays, nullptr,
                                                                       (unsigned long long)kNoHit);
    ++g_launches;
    const int64_t rays_per_block = (int64_t)kBruteThreads * kRPT;
    const int64_t ray_blocks = (n_rays + rays_per_block - 1) / rays_per_block;
    int64_t splits = ((int64_t)sm_count * 4 + ray_blocks - 1) / ray_blocks;
    const int64_t max_splits = (n_tris + 4 * kTile - 1) / (4 * kTile);
    if (splits > max_splits) splits = max_splits;
    if (splits < 1) splits = 1;
    if (splits > 65535) splits = 65535;
    int64_t per_split = (n_tris + splits - 1) / splits;
    per_split = ((per_split + kTile - 1) / kTile) * kTile;
    if (per_split < kTile) per_split = kTile;
    splits = (n_tris + per_split - 1) / per_split;
    if (n_tris > 0) {
        dim3 grid((unsigned)ray_blocks, (unsigned)splits);
        hit_ntris_kernel<<<grid, kBruteThreads, 0, s>>>(rays, n_rays, ntris, n_tris, per_split,
                                                         (unsigned long long*)tmp);
        ++g_launches;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_unpack_hits(tmp, n_rays, nullptr, hit_idx, nullptr, s);
}

// ---------------------------------------------------------------------------
// brute force over n_tris with library-held scratch (no allocation)
// ---------------------------------------------------------------------------
// The packed (t, index) words of splat_next_hit_brute_static live here rather
// than in caller memory.  Every GPU that loads the library holds this array
// until the process exits; all calls share it.
static __device__ __align__(256) unsigned long long g_static_hit_tmp[kStaticHitMaxRays];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {nullptr};

// Device address of g_static_hit_tmp on the current device, looked up once
// per device (host code only has a host-side stand-in for the symbol).
cudaError_t static_hit_scratch(unsigned long long** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (g_static_ptr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_hit_tmp);
        if (e != cudaSuccess) return e;
        g_static_ptr[dev] = p;
    }
    *out = reinterpret_cast<unsigned long long*>(g_static_ptr[dev]);
    return cudaSuccess;
}
}  // namespace

cudaError_t launch_hit_brute_ntris_static(const splat_adray_t* rays, int64_t n_rays, const splat_ntri_t* ntris,
                                          int64_t n_tris, int32_t* hit_idx, int sm_count, cudaStream_t s) {
    unsigned long long* tmp = nullptr;
    cudaError_t e = static_hit_scratch(&tmp);
    if (e != cudaSuccess) return e;
    // launch_hit_brute_ntris first resets the n_rays words it uses to (Inf, 1)
    return launch_hit_brute_ntris(rays, n_rays, ntris, n_tris, reinterpret_cast<uint64_t*>(tmp), hit_idx, sm_count,
                                  s);
}

// ---------------------------------------------------------------------------
// BVH traversal
// ---------------------------------------------------------------------------
constexpr int kBvhThreads = 128;

// Grid of a work-counter launch: as many blocks as stay resident together
// (capped by a blocks-per-SM knob and by the work), so the launch is one
// wave that drains the counter.
int resident_grid(const void* kernel, int64_t cap, int sm_count, int threads, int max_per_sm) {
    static std::mutex mu;
    static std::unordered_map<const void*, int> occ;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = occ.find(kernel);
        if (it == occ.end()) {
            int nb = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, 0) != cudaSuccess || nb < 1)
                nb = 4;
            it = occ.emplace(kernel, nb).first;
        }
        per_sm = it->second;
    }
    if (per_sm > max_per_sm) per_sm = max_per_sm;
    return grid_for(cap, threads, sm_count, per_sm);
}

template <bool AOS>
__global__ void __launch_bounds__(kBvhThreads) hit_bvh_kernel(RaySrc src, BvhView bvh, int32_t* __restrict__ hit_idx,
                                                              float* __restrict__ hit_t, int32_t* err) {
    const int64_t n = src.d_count ? *src.d_count : src.n;
    int2 stack[kBvhStack];  // (ref, entry distance bits)
    for_each_ray(n, src.fetch, [&](int64_t kk) {
        const int64_t k = src.perm ? (int64_t)src.perm[kk] : kk;
        const HitRay r = load_hit_ray<AOS>(src, k);
        const float ix = safe_inv(r.dx), iy = safe_inv(r.dy), iz = safe_inv(r.dz);
        const float oix = r.ox * ix, oiy = r.oy * iy, oiz = r.oz * iz;
        float best = __int_as_float(0x7f800000);
        int32_t bi = 1;
        int sp = 0;
        int ref = 0;
        while (true) {
            if (ref >= 0) {
                const BvhNode* nd = bvh.nodes + ref;
                const float4 bx = __ldg(&nd->x);
                const float4 by = __ldg(&nd->y);
                const float4 bz = __ldg(&nd->z);
                const int4 c = __ldg(&nd->c);
                const float a0 = fmaf(bx.x, ix, -oix), b0 = fmaf(bx.y, ix, -oix);
                const float a1 = fmaf(by.x, iy, -oiy), b1 = fmaf(by.y, iy, -oiy);
                const float a2 = fmaf(bz.x, iz, -oiz), b2 = fmaf(bz.y, iz, -oiz);
                const float tmin0 = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fminf(a2, b2));
                const float tmax0 = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fmaxf(a2, b2));
                const float e0 = fmaf(bx.z, ix, -oix), f0 = fmaf(bx.w, ix, -oix);
                const float e1 = fmaf(by.z, iy, -oiy), f1 = fmaf(by.w, iy, -oiy);
                const float e2 = fmaf(bz.z, iz, -oiz), f2 = fmaf(bz.w, iz, -oiz);
                const float tmin1 = fmaxf(fmaxf(fminf(e0, f0), fminf(e1, f1)), fminf(e2, f2));
                const float tmax1 = fminf(fminf(fmaxf(e0, f0), fmaxf(e1, f1)), fmaxf(e2, f2));
                const bool h0 = (tmin0 <= tmax0) & (tmax0 >= 0.0f) & (tmin0 <= best);
                const bool h1 = (tmin1 <= tmax1) & (tmax1 >= 0.0f) & (tmin1 <= best);
                if (h0 && h1) {
                    int near_ref = c.x, far_ref = c.y;
                    float far_t = tmin1;
                    if (tmin1 < tmin0) {
                        near_ref = c.y;
                        far_ref = c.x;
                        far_t = tmin0;
                    }
                    if (sp < kBvhStack) {
                        stack[sp++] = make_int2(far_ref, __float_as_int(far_t));
                    } else {
                        atomicOr(err, 2);
                    }
                    ref = near_ref;
                    continue;
                }
                if (h0) {
                    ref = c.x;
                    continue;
                }
                if (h1) {
                    ref = c.y;
                    continue;
                }
            } else {
                const int enc = ~ref;
                const int first = enc >> 4;
                const int count = (enc & 15) + 1;
                for (int j = 0; j < count; ++j) {
                    const TriHit* h = bvh.tris + first + j;
                    float num, den;
                    if (!tri_candidate(__ldg(&h->n_nv), r, best, num, den)) continue;
                    const float4 q1 = __ldg(&h->a_idx);
                    const int32_t idx = __float_as_int(q1.w);
                    bool inside;
                    const float t = tri_t_from(num, den, q1, __ldg(&h->e0), __ldg(&h->e1), __ldg(&h->inv), r, inside);
                    if (inside & (t > 0.0f) & (idx != r.ig) & ((t < best) | ((t == best) & (idx < bi)))) {
                        best = t;
                        bi = idx;
                    }
                }
            }
            bool found = false;
            while (sp > 0) {
                const int2 e = stack[--sp];
                if (__int_as_float(e.y) <= best) {
                    ref = e.x;
                    found = true;
                    break;
                }
            }
            if (!found) break;
        }
        hit_idx[k] = bi;
        if (hit_t) hit_t[k] = best;
    });
}

cudaError_t launch_hit_bvh(const RaySrc& rays, int64_t cap, const BvhView& bvh, int32_t* hit_idx, float* hit_t,
                           int32_t* err, int sm_count, cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    const int grid = rays.fetch ? resident_grid(reinterpret_cast<const void*>(hit_bvh_kernel<false>), cap, sm_count,
                                                kBvhThreads, g_tune[SPLAT_TUNE_BVH_BLOCKS_PER_SM])
                                : grid_for(cap, kBvhThreads, sm_count, g_tune[SPLAT_TUNE_BVH_BLOCKS_PER_SM]);
    if (rays.aos)
        hit_bvh_kernel<true><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err);
    else
        hit_bvh_kernel<false><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err);
    ++g_launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// four-wide BVH traversal
// ---------------------------------------------------------------------------
// One thread per ray.  A node fetch (128 bytes) tests four child boxes; the
// hit children are sorted by entry distance, the nearest is visited next and
// the others are pushed farthest first together with their entry distance,
// so a popped entry that lies beyond the current best hit is skipped.
// Traversal work of the counting kernels (SPLAT_TUNE_COUNT_WORK): nodes
// visited, triangle pre-tests, full triangle tests, rays traced.  Every GPU
// that loads the library holds these four words; splat_hit_work reads and
// clears them.
__device__ unsigned long long g_hit_work[4];

__device__ __forceinline__ void flush_work(const WorkCount& wc, uint32_t rays) {
    unsigned long long v[4] = {wc.nodes, wc.pre, wc.full, rays};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        for (int o = 16; o; o >>= 1) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
        if ((threadIdx.x & 31) == 0 && v[i]) atomicAdd(&g_hit_work[i], v[i]);
    }
}

template <bool AOS, bool COUNT>
__global__ void __launch_bounds__(kBvhThreads) hit_bvh4_kernel(RaySrc src, Bvh4View bvh,
                                                               int32_t* __restrict__ hit_idx,
                                                               float* __restrict__ hit_t, int32_t* err) {
    const int64_t n = src.d_count ? *src.d_count : src.n;
    int2 stack[kBvhStack];
    WorkCount wc{0u, 0u, 0u};
    uint32_t rays = 0;
    for_each_ray(n, src.fetch, [&](int64_t kk) {
        const int64_t k = src.perm ? (int64_t)src.perm[kk] : kk;
        const HitRay r = load_hit_ray<AOS>(src, k);
        float best;
        int32_t bi;
        bvh4_closest(r, bvh, stack, err, best, bi, COUNT ? &wc : nullptr);
        if (COUNT) ++rays;
        hit_idx[k] = bi;
        if (hit_t) hit_t[k] = best;
    });
    if (COUNT) flush_work(wc, rays);
}


// The per-ray form with finished lanes refilled from the work counter.
template <bool AOS>
__global__ void __launch_bounds__(kBvhThreads) hit_bvh4_refill_kernel(RaySrc src, Bvh4View bvh,
                                                                      int32_t* __restrict__ hit_idx,
                                                                      float* __restrict__ hit_t, int32_t* err,
                                                                      int refill_min) {
    const int64_t n = src.d_count ? *src.d_count : src.n;
    auto ray_of = [&](int64_t k) { return src.perm ? (int64_t)src.perm[k] : k; };
    bvh4_refill_loop(
        n, src.fetch, refill_min, err, [&](int64_t k) { return load_hit_ray<AOS>(src, ray_of(k)); },
        [&](int64_t) { return bvh; },
        [&](int64_t k, float best, int32_t bi) {
            const int64_t kk = ray_of(k);
            hit_idx[kk] = bi;
            if (hit_t) hit_t[kk] = best;
        });
}

// Packet form: each warp traverses its 32 rays together (bvh4_closest_packet)
// on a shared-memory stack.  ADAPT: per warp, packets only when its rays are
// coherent by packet_coherent's thresholds of `form` (2 loose, 3 tight);
// otherwise one ray per lane.  Rays are taken through src.perm when set, or,
// with src.tile_h set (a first bounce: the light grid's columns in order),
// in 8 x 4 tiles of the grid (grid_tile_ray), so a warp holds a compact
// patch of rays.
template <bool AOS, bool ADAPT, bool COUNT = false>
__global__ void __launch_bounds__(kBvhThreads) hit_bvh4_packet_kernel(RaySrc src, Bvh4View bvh,
                                                                      int32_t* __restrict__ hit_idx,
                                                                      float* __restrict__ hit_t, int32_t* err,
                                                                      int form) {
    WorkCount wc{0u, 0u, 0u};
    uint32_t rays = 0;
    __shared__ int2 s_stack[kBvhThreads / 32][kPacketStack];
    int2* stack = s_stack[threadIdx.x >> 5];
    const int64_t n = src.d_count ? *src.d_count : src.n;
    const int lane = threadIdx.x & 31;
    const float extent = ADAPT ? bvh4_extent(bvh.nodes) : 0.0f;
    int2 lane_stack[ADAPT ? kBvhStack : 1];
    for_each_warp_batch(n, src.fetch, [&](int64_t base) {
        const bool valid = base + lane < n;
        const int64_t kk = valid ? base + lane : base;
        int64_t k = src.perm ? (int64_t)src.perm[kk] : kk;
        if (!src.perm && src.tile_h > 0 && n < (int64_t(1) << 32))  // 8 x 4 tiles of the grid
            k = (int64_t)grid_tile_ray((uint32_t)kk, (uint32_t)src.tile_h, (uint32_t)n);
        const HitRay r = load_hit_ray<AOS>(src, k);
        float best;
        int32_t bi;
        const bool packet = !ADAPT || packet_coherent(r, form, extent);
        if (packet) {
            bvh4_closest_packet(r, valid, bvh, stack, err, best, bi, COUNT ? &wc : nullptr);
        } else if (ADAPT && valid) {
            bvh4_closest(r, bvh, lane_stack, err, best, bi, COUNT ? &wc : nullptr);
        }
        if (valid) {
            if (COUNT) ++rays;
            hit_idx[k] = bi;
            if (hit_t) hit_t[k] = best;
        }
    });
    if (COUNT) flush_work(wc, rays);
}

// The traversal kernels use no shared memory: give the whole L1/shared
// array to L1, where the upper BVH levels and hot hit records live.
template <class K>
static void prefer_l1(K kernel) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
}

template <bool COUNT>
static void launch_bvh4_form(const RaySrc& rays, int64_t cap, const Bvh4View& bvh, int32_t* hit_idx, float* hit_t,
                             int32_t* err, int sm_count, cudaStream_t s) {
    const int knob = g_tune[SPLAT_TUNE_BVH_BLOCKS_PER_SM];
    auto grid_of = [&](const void* k) {
        return rays.fetch ? resident_grid(k, cap, sm_count, kBvhThreads, knob) : grid_for(cap, kBvhThreads, sm_count, knob);
    };
    if (rays.packet) {
        // packet_form: 1 every warp; 2, 3 per warp by ray spread (loose, tight)
        const int form = rays.packet;
        if (form == 1) {
            const int grid = grid_of(reinterpret_cast<const void*>(hit_bvh4_packet_kernel<false, false, COUNT>));
            if (rays.aos)
                hit_bvh4_packet_kernel<true, false, COUNT><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err,
                                                                                       form);
            else
                hit_bvh4_packet_kernel<false, false, COUNT><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t,
                                                                                        err, form);
        } else {
            const int grid = grid_of(reinterpret_cast<const void*>(hit_bvh4_packet_kernel<false, true, COUNT>));
            if (rays.aos)
                hit_bvh4_packet_kernel<true, true, COUNT><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err,
                                                                                      form);
            else
                hit_bvh4_packet_kernel<false, true, COUNT><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err,
                                                                                       form);
        }
        return;
    }
    if (!COUNT && rays.fetch && g_tune[SPLAT_TUNE_BVH_REFILL] > 0) {
        const int grid = resident_grid(reinterpret_cast<const void*>(hit_bvh4_refill_kernel<false>), cap, sm_count,
                                       kBvhThreads, knob);
        const int m = g_tune[SPLAT_TUNE_BVH_REFILL];
        if (rays.aos)
            hit_bvh4_refill_kernel<true><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err, m);
        else
            hit_bvh4_refill_kernel<false><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err, m);
        return;
    }
    const int grid = grid_of(reinterpret_cast<const void*>(hit_bvh4_kernel<false, COUNT>));
    if (rays.aos)
        hit_bvh4_kernel<true, COUNT><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err);
    else
        hit_bvh4_kernel<false, COUNT><<<grid, kBvhThreads, 0, s>>>(rays, bvh, hit_idx, hit_t, err);
}

cudaError_t launch_hit_bvh4(const RaySrc& rays, int64_t cap, const Bvh4View& bvh, int32_t* hit_idx, float* hit_t,
                            int32_t* err, int sm_count, cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    static bool configured = false;
    if (!configured) {
        prefer_l1(hit_bvh4_kernel<true, false>);
        prefer_l1(hit_bvh4_kernel<false, false>);
        prefer_l1(hit_bvh4_kernel<true, true>);
        prefer_l1(hit_bvh4_kernel<false, true>);
        prefer_l1(hit_bvh4_refill_kernel<true>);
        prefer_l1(hit_bvh4_refill_kernel<false>);
        prefer_l1(hit_bvh_kernel<true>);
        prefer_l1(hit_bvh_kernel<false>);
        configured = true;
    }
    if (g_tune[SPLAT_TUNE_COUNT_WORK])
        launch_bvh4_form<true>(rays, cap, bvh, hit_idx, hit_t, err, sm_count, s);
    else
        launch_bvh4_form<false>(rays, cap, bvh, hit_idx, hit_t, err, sm_count, s);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t read_hit_work(uint64_t out[4], bool reset, cudaStream_t s) {
    cudaError_t e = cudaMemcpyFromSymbolAsync(out, g_hit_work, 4 * sizeof(unsigned long long), 0,
                                              cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    if (reset) {
        static const unsigned long long zero[4] = {0ull, 0ull, 0ull, 0ull};
        if ((e = cudaMemcpyToSymbolAsync(g_hit_work, zero, sizeof(zero), 0, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return e;
        e = cudaStreamSynchronize(s);
    }
    return e;
}

// ---------------------------------------------------------------------------
// scene packing and BVH refit
// ---------------------------------------------------------------------------
// max |vertex coordinate| of the hit triangles (float bits; NaN skipped).
__global__ void scene_scale_kernel(const splat_ftri_t* __restrict__ ftri, int64_t n_tris, unsigned* scale) {
    unsigned m = 0u;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j + 1 < n_tris;
         j += (int64_t)gridDim.x * blockDim.x) {
        const float* p = ftri[j + 1].v[1];
        for (int v = 0; v < 9; ++v) {
            const float x = fabsf(p[v]);
            if (x == x) m = max(m, __float_as_uint(x));
        }
    }
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(scale, m);
}

__device__ __forceinline__ void padded_box(const float* p, float pad_abs, float pad_rel, float lo[3], float hi[3]) {
    float tl[3], th[3];
    for (int a = 0; a < 3; ++a) {
        tl[a] = fminf(fminf(p[a], p[3 + a]), p[6 + a]);
        th[a] = fmaxf(fmaxf(p[a], p[3 + a]), p[6 + a]);
    }
    const float dx = th[0] - tl[0], dy = th[1] - tl[1], dz = th[2] - tl[2];
    const float pad = pad_abs + pad_rel * sqrtf(dx * dx + dy * dy + dz * dz);
    for (int a = 0; a < 3; ++a) {
        lo[a] = tl[a] - pad;
        hi[a] = th[a] + pad;
    }
}

__global__ void pack_hits_kernel(const splat_ftri_t* __restrict__ ftri, int64_t n_tris, TriHit* brute, TriBox* boxes,
                                 const unsigned* __restrict__ scale, const int32_t* __restrict__ bvh_order,
                                 TriHit* bvh, int32_t* bvh_pos) {
    const float pad_abs = pad_abs_of_scale(__uint_as_float(*scale));
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j + 1 < n_tris;
         j += (int64_t)gridDim.x * blockDim.x) {
        // brute record j <- reference index j + 2 (the sentinel is never hit)
        const float* p = ftri[j + 1].v[0];
        brute[j] = pack_one((int32_t)(j + 2), f3(p), f3(p + 3), f3(p + 6), f3(p + 9));
        float lo[3], hi[3];
        padded_box(p + 3, pad_abs, 1.0e-3f, lo, hi);
        boxes[j] = TriBox{make_float4(lo[0], lo[1], lo[2], 0.0f), make_float4(hi[0], hi[1], hi[2], 0.0f)};
        if (bvh) {
            const int32_t idx = bvh_order[j];
            const float* q = ftri[idx - 1].v[0];
            bvh[j] = pack_one(idx, f3(q), f3(q + 3), f3(q + 6), f3(q + 9));
            if (bvh_pos) bvh_pos[idx] = (int32_t)j;
        }
    }
    if (bvh_pos && blockIdx.x == 0 && threadIdx.x == 0) {
        bvh_pos[0] = 0;
        bvh_pos[1] = 0;  // the sentinel
    }
}

cudaError_t launch_pack_hits(const splat_ftri_t* ftri, int64_t n_tris, TriHit* brute_recs, TriBox* brute_boxes,
                             unsigned* scale, const int32_t* bvh_order, TriHit* bvh_recs, int32_t* bvh_pos,
                             cudaStream_t s) {
    if (n_tris <= 1) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scale, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    scene_scale_kernel<<<grid_for(n_tris, 256, 152, 8), 256, 0, s>>>(ftri, n_tris, scale);
    pack_hits_kernel<<<grid_for(n_tris, 256, 152, 8), 256, 0, s>>>(ftri, n_tris, brute_recs, brute_boxes, scale,
                                                                    bvh_order, bvh_recs, bvh_order ? bvh_pos : nullptr);
    g_launches += 2;
    return cudaGetLastError();
}

__device__ __forceinline__ void leaf_box(int ref, const TriHit* recs, const splat_ftri_t* ftri, float pad_abs,
                                         float pad_rel, float lo[3], float hi[3]) {
    const int enc = ~ref;
    const int first = enc >> 4, count = (enc & 15) + 1;
    for (int j = 0; j < count; ++j) {
        const int32_t idx = __float_as_int(recs[first + j].a_idx.w);
        const float* p = ftri[idx - 1].v[1];
        float tl[3], th[3];
        for (int a = 0; a < 3; ++a) {
            tl[a] = fminf(fminf(p[a], p[3 + a]), p[6 + a]);
            th[a] = fmaxf(fmaxf(p[a], p[3 + a]), p[6 + a]);
        }
        const float dx = th[0] - tl[0], dy = th[1] - tl[1], dz = th[2] - tl[2];
        const float pad = pad_abs + pad_rel * sqrtf(dx * dx + dy * dy + dz * dz);
        for (int a = 0; a < 3; ++a) {
            lo[a] = fminf(lo[a], tl[a] - pad);
            hi[a] = fmaxf(hi[a], th[a] + pad);
        }
    }
}

// One-launch refit: the threads of the nodes whose children are all leaves
// start; each node's box union is written by the last of its inner children
// to finish (atomic arrival count against its number of inner children), so
// the tree is refit bottom-up without a launch per level.  links[q] =
// parent of node q (-1: root), links[n + q] = its number of inner children.
// Child nodes written by other threads are read through L2 (__ldcg).
__device__ __forceinline__ float4 ldcg4(const float4* p) { return __ldcg(p); }

__device__ __forceinline__ void refit2_node(BvhNode* nodes, int q, const TriHit* recs, const splat_ftri_t* ftri,
                                            float pad_abs, float pad_rel) {
    const int4 c = nodes[q].c;
    float l[2][3], h[2][3];
    const int refs[2] = {c.x, c.y};
    for (int i = 0; i < 2; ++i) {
        for (int a = 0; a < 3; ++a) {
            l[i][a] = __int_as_float(0x7f800000);
            h[i][a] = -__int_as_float(0x7f800000);
        }
        if (refs[i] >= 0) {
            const float4 x = ldcg4(&nodes[refs[i]].x), y = ldcg4(&nodes[refs[i]].y), z = ldcg4(&nodes[refs[i]].z);
            l[i][0] = fminf(x.x, x.z);
            h[i][0] = fmaxf(x.y, x.w);
            l[i][1] = fminf(y.x, y.z);
            h[i][1] = fmaxf(y.y, y.w);
            l[i][2] = fminf(z.x, z.z);
            h[i][2] = fmaxf(z.y, z.w);
        } else {
            leaf_box(refs[i], recs, ftri, pad_abs, pad_rel, l[i], h[i]);
        }
    }
    nodes[q].x = make_float4(l[0][0], h[0][0], l[1][0], h[1][0]);
    nodes[q].y = make_float4(l[0][1], h[0][1], l[1][1], h[1][1]);
    nodes[q].z = make_float4(l[0][2], h[0][2], l[1][2], h[1][2]);
}

__device__ __forceinline__ void refit4_node(Bvh4Node* nodes, int q, const TriHit* recs, const splat_ftri_t* ftri,
                                            float pad_abs, float pad_rel) {
    const int nc = nodes[q].meta.x;
    const int4 c = nodes[q].c;
    const int refs[4] = {c.x, c.y, c.z, c.w};
    float lo[3][4], hi[3][4];
    for (int i = 0; i < 4; ++i) {
        float l[3] = {__int_as_float(0x7f800000), __int_as_float(0x7f800000), __int_as_float(0x7f800000)};
        float h[3] = {-l[0], -l[0], -l[0]};
        if (i < nc) {
            if (refs[i] >= 0) {
                const Bvh4Node* ch = nodes + refs[i];
                const float4 lx = ldcg4(&ch->lox), hx = ldcg4(&ch->hix), ly = ldcg4(&ch->loy), hy = ldcg4(&ch->hiy);
                const float4 lz = ldcg4(&ch->loz), hz = ldcg4(&ch->hiz);
                const int cn = __ldcg(&ch->meta.x);
                for (int j = 0; j < cn; ++j) {
                    l[0] = fminf(l[0], comp(lx, j));
                    h[0] = fmaxf(h[0], comp(hx, j));
                    l[1] = fminf(l[1], comp(ly, j));
                    h[1] = fmaxf(h[1], comp(hy, j));
                    l[2] = fminf(l[2], comp(lz, j));
                    h[2] = fmaxf(h[2], comp(hz, j));
                }
            } else {
                leaf_box(refs[i], recs, ftri, pad_abs, pad_rel, l, h);
            }
        }
        for (int a = 0; a < 3; ++a) {
            lo[a][i] = l[a];
            hi[a][i] = h[a];
        }
    }
    Bvh4Node& nd = nodes[q];
    nd.lox = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
    nd.hix = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
    nd.loy = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
    nd.hiy = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
    nd.loz = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
    nd.hiz = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
}

template <bool WIDE>
__global__ void refit_tree_kernel(void* nodes_v, int64_t n_nodes, const int32_t* __restrict__ links, unsigned* flags,
                                  const TriHit* __restrict__ recs, const splat_ftri_t* __restrict__ ftri,
                                  const unsigned* __restrict__ scale, float pad_rel) {
    const float pad_abs = pad_abs_of_scale(__uint_as_float(*scale));
    for (int64_t q0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q0 < n_nodes;
         q0 += (int64_t)gridDim.x * blockDim.x) {
        if (links[n_nodes + q0] != 0) continue;  // has inner children: reached by its last child
        int q = (int)q0;
        for (int64_t guard = 0; guard < n_nodes; ++guard) {
            if (WIDE) refit4_node(reinterpret_cast<Bvh4Node*>(nodes_v), q, recs, ftri, pad_abs, pad_rel);
            else refit2_node(reinterpret_cast<BvhNode*>(nodes_v), q, recs, ftri, pad_abs, pad_rel);
            const int p = links[q];
            if (p < 0) break;
            __threadfence();
            if ((int)atomicAdd(&flags[p], 1u) + 1 < links[n_nodes + p]) break;
            __threadfence();
            q = p;
        }
    }
}

cudaError_t launch_refit_tree(void* nodes, bool wide, int64_t n_nodes, const int32_t* links, unsigned* flags,
                              const TriHit* bvh_recs, const splat_ftri_t* ftri, const unsigned* scale, float pad_rel,
                              cudaStream_t s) {
    if (n_nodes <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(flags, 0, sizeof(unsigned) * (size_t)n_nodes, s);
    if (e != cudaSuccess) return e;
    if (wide)
        refit_tree_kernel<true><<<grid_for(n_nodes, 128, 152, 8), 128, 0, s>>>(nodes, n_nodes, links, flags, bvh_recs,
                                                                             ftri, scale, pad_rel);
    else
        refit_tree_kernel<false><<<grid_for(n_nodes, 128, 152, 8), 128, 0, s>>>(nodes, n_nodes, links, flags, bvh_recs,
                                                                              ftri, scale, pad_rel);
    ++g_launches;
    return cudaGetLastError();
}

}  // namespace splat
