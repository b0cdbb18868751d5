// evolve.cu -- evolve_ray over the active rays of one bounce, with the ray
// compaction (warp ballot + block scan, one atomic per block) fused in.  In
// trace mode the diffuse rays' final_evolution is fused in as well and the
// result is compacted into a splat queue; one splat launch per frame then
// spreads (ray, sample) pairs over full warps.
//
// Reference: evolve_ray src/tracer.jl:181-201, partition! src/partition.jl
// (semantics: the active rays, in any order, and their count),
// final_evolution src/ray_imagers.jl:4-37, atomic_spectrum_kernel2
// src/ray_imagers.jl:78-113.  Each ray's Fresnel draw is keyed by its id, so
// results do not depend on the order compaction leaves the rays in.
//
// Splat: one thread per (queued ray, sample); a ray's n_lambda x N x N
// samples are consecutive, so a warp's lanes share (broadcast-load) one or a
// few rays.  Fixed-point maps add round(intensity * 2^frac_bits) with warp-aggregated
// integer atomics (lanes on the same texel are summed by match_any +
// reduce_add first), which makes the map independent of ray order and
// bit-exact run to run.  Float maps use plain float atomics, as the
// reference does.
#include "kernels.h"
#include "optics.cuh"

namespace splat {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kEvolveThreads = 256;

__device__ __forceinline__ F3 shfl3(F3 v, int src) {
    return {__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src), __shfl_sync(kFull, v.z, src)};
}

__device__ __forceinline__ RayState shfl_ray(const RayState& r, int src) {
    RayState q;
    q.pos = shfl3(r.pos, src);
    q.dir = shfl3(r.dir, src);
    q.dpl = shfl3(r.dpl, src);
    q.dpx = shfl3(r.dpx, src);
    q.dpy = shfl3(r.dpy, src);
    q.ddl = shfl3(r.ddl, src);
    q.ddx = shfl3(r.ddx, src);
    q.ddy = shfl3(r.ddy, src);
    q.lam = __shfl_sync(kFull, r.lam, src);
    q.x = __shfl_sync(kFull, r.x, src);
    q.y = __shfl_sync(kFull, r.y, src);
    q.ignore = __shfl_sync(kFull, r.ignore, src);
    q.medium = __shfl_sync(kFull, r.medium, src);
    return q;
}

// Sample s of a ray: s = ix + nd (iy + nd il), the CartesianIndices order of
// atomic_spectrum_kernel2's threads.
__device__ __forceinline__ bool sample_of(const SplatParams& sp, const RayState& q, const Tri& T, int s,
                                          int64_t& off, float& inten) {
    const int nd = sp.n_delta;
    const int ix = s % nd;
    const int iy = (s / nd) % nd;
    const int il = s / (nd * nd);
    const float lam = sp.n_lambda > 0 ? sp.spectrum[il] : q.lam;
    const float xs = q.x + sp.deltas[ix];
    const float ys = q.y + sp.deltas[iy];
    int64_t oij;
    if (!splat_sample(q, T, lam, xs, ys, sp.w, sp.h, oij, inten)) return false;
    off = oij + (int64_t)il * sp.w * sp.h;
    return true;
}

// All 32 lanes call; lanes with ok add their sample.
__device__ __forceinline__ void accumulate_warp(const SplatParams& sp, bool ok, int64_t off, float inten) {
    if (sp.accum == SPLAT_ACCUM_I32) {
        const unsigned act = __ballot_sync(kFull, ok);
        if (ok) {
            const int v = __float2int_rn(inten * sp.scale);
            const unsigned m = __match_any_sync(act, (unsigned long long)off);
            const int sum = __reduce_add_sync(m, v);
            if (lane_id() == __ffs(m) - 1) atomicAdd(reinterpret_cast<int*>(sp.map) + off, sum);
        }
    } else if (ok) {
        atomicAdd(reinterpret_cast<float*>(sp.map) + off, inten);
    }
}

__device__ __forceinline__ void accumulate_one(const SplatParams& sp, int64_t off, float inten) {
    if (sp.accum == SPLAT_ACCUM_I32)
        atomicAdd(reinterpret_cast<int*>(sp.map) + off, __float2int_rn(inten * sp.scale));
    else
        atomicAdd(reinterpret_cast<float*>(sp.map) + off, inten);
}

// Splat the diffuse rays held by the lanes of this warp (all lanes call).
// Returns the number of samples this lane accumulated.
__device__ __forceinline__ int splat_warp(const SplatParams& sp, const splat_ftri_t* tris, bool dif,
                                          const RayState& fe, int32_t ti) {
    const int S = (sp.n_lambda > 0 ? sp.n_lambda : 1) * sp.n_delta * sp.n_delta;
    int done = 0;
    if (S >= 8) {
        unsigned dm = __ballot_sync(kFull, dif);
        while (dm) {
            const int src = __ffs(dm) - 1;
            dm &= dm - 1;
            const RayState q = shfl_ray(fe, src);
            const int32_t qi = __shfl_sync(kFull, ti, src);
            const Tri T = load_tri(tris, qi);
            for (int s0 = 0; s0 < S; s0 += 32) {
                const int s = s0 + lane_id();
                bool ok = false;
                int64_t off = 0;
                float inten = 0.f;
                if (s < S) ok = sample_of(sp, q, T, s, off, inten);
                accumulate_warp(sp, ok, off, inten);
                done += ok ? 1 : 0;
            }
        }
    } else if (dif) {
        const Tri T = load_tri(tris, ti);
        for (int s = 0; s < S; ++s) {
            int64_t off;
            float inten;
            if (sample_of(sp, fe, T, s, off, inten)) {
                accumulate_one(sp, off, inten);
                ++done;
            }
        }
    }
    return done;
}

__device__ __forceinline__ void add_stats(splat_trace_stats_t* st, int diffuse, int samples) {
    if (!st) return;
    const int d = __reduce_add_sync(kFull, diffuse);
    const int s = __reduce_add_sync(kFull, samples);
    if (lane_id() == 0) {
        if (d) atomicAdd(reinterpret_cast<unsigned long long*>(&st->diffuse), (unsigned long long)d);
        if (s) atomicAdd(reinterpret_cast<unsigned long long*>(&st->samples), (unsigned long long)s);
    }
}

// TRACE: diffuse rays are final-evolved and splatted here, misses dropped, the
// last bounce skips the optics.  PLUGIN: retired rays are written back to the
// caller's AoS array with their status, as run_evolution! leaves them.
// MODE 0: plugin (retired rays written back to the caller's AoS array);
// 1: trace (diffuse rays final-evolved into the splat queue, escaped rays
// dropped); 2: camera (as trace, escaped rays queued unchanged for the sky).
// MK >= 0: the material kind, fixed at compile time so that only that
// material's optics is inlined (smaller code, no per-evaluation switch).
template <int MODE, int MK>
__global__ void __launch_bounds__(kEvolveThreads) evolve_kernel(EvolveArgs A) {
    constexpr bool TRACE = MODE != 0;
    constexpr bool SKY = MODE == 2;
    // double-buffered by iteration parity: iteration i + 2 writes a buffer
    // only after every thread has passed both barriers of iteration i + 1,
    // so no third barrier is needed at the end of an iteration
    __shared__ int s_warp2[2][kEvolveThreads / 32];
    __shared__ int s_wdif2[2][kEvolveThreads / 32];
    __shared__ int s_wsky2[2][kEvolveThreads / 32];
    __shared__ unsigned long long s_base2[2], s_dbase2[2], s_sbase2[2];
    const int64_t n = *A.in_count;
    const int lane = lane_id();
    const int wid = threadIdx.x >> 5;
    const bool quirks = A.quirks != 0;
    int par = 0;
    for (int64_t base = (int64_t)blockIdx.x * kEvolveThreads; base < n;
         base += (int64_t)gridDim.x * kEvolveThreads, par ^= 1) {
        int* s_warp = s_warp2[par];
        int* s_wdif = s_wdif2[par];
        int* s_wsky = s_wsky2[par];
        unsigned long long& s_base = s_base2[par];
        unsigned long long& s_dbase = s_dbase2[par];
        unsigned long long& s_sbase = s_sbase2[par];
        int64_t k = base + threadIdx.x;
        bool keep = false, dif = false, sky = false;
        RayState r, o;
        uint32_t id = 0;
        int32_t ih = 1;
        if (k < n) {
            if (A.tile_h > 0 && n < (int64_t(1) << 32))
                k = (int64_t)grid_tile_ray((uint32_t)k, (uint32_t)A.tile_h, (uint32_t)n);
            r = load_ray(A.in, k);
            id = A.in.id[k];
            EvolveView v{A.tris, A.n_tris, A.err, A.first_diffuse, A.material, A.seed, A.bounce,
                         A.force_rand, quirks, A.last != 0};
            if (MK >= 0) v.material.kind = MK;
            const int fate = evolve_one<TRACE>(r, A.hit_idx[k], id, v, o, ih);
            keep = fate == kFateKeep;
            dif = fate == kFateDiffuse;
            sky = SKY && fate == kFateInfinity;
            if (!TRACE && fate == kFateDiffuse) ray_to_aos(A.aos[id], r, kStatusDiffuse);
            if (!TRACE && fate == kFateInfinity) ray_to_aos(A.aos[id], r, kStatusInfinity);
        }
        // compaction of the survivors (and, tracing, of the diffuse rays into
        // the splat queue and of the escaped ones into the sky queue): ballot
        // -> block scan -> one atomic per block and queue
        const unsigned kb = __ballot_sync(kFull, keep);
        const unsigned db = TRACE ? __ballot_sync(kFull, dif) : 0u;
        const unsigned sb = SKY ? __ballot_sync(kFull, sky) : 0u;
        if (lane == 0) {
            s_warp[wid] = __popc(kb);
            s_wdif[wid] = __popc(db);
            s_wsky[wid] = __popc(sb);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0, dtot = 0, stot = 0;
            for (int w = 0; w < kEvolveThreads / 32; ++w) {
                const int c = s_warp[w], d = s_wdif[w], e = s_wsky[w];
                s_warp[w] = tot;
                s_wdif[w] = dtot;
                s_wsky[w] = stot;
                tot += c;
                dtot += d;
                stot += e;
            }
            s_base = tot ? atomicAdd(reinterpret_cast<unsigned long long*>(A.out_count), (unsigned long long)tot) : 0ull;
            s_dbase = dtot ? atomicAdd(reinterpret_cast<unsigned long long*>(A.splat_count), (unsigned long long)dtot)
                           : 0ull;
            if (SKY)
                s_sbase = stot ? atomicAdd(reinterpret_cast<unsigned long long*>(A.sky_count), (unsigned long long)stot)
                               : 0ull;
        }
        __syncthreads();
        const unsigned below = (1u << lane) - 1u;
        if (keep) {
            store_ray(A.out, (int64_t)s_base + s_warp[wid] + __popc(kb & below), o, id);
        } else if (TRACE && dif) {
            store_ray(A.splat_q, (int64_t)s_dbase + s_wdif[wid] + __popc(db & below), o, id);
        } else if (SKY && sky) {
            store_ray(A.sky_q, (int64_t)s_sbase + s_wsky[wid] + __popc(sb & below), r, id);
        }
    }
}

static int evolve_grid(int64_t cap, int sm_count) {
    int64_t b = (cap + kEvolveThreads - 1) / kEvolveThreads;
    const int64_t lim = (int64_t)sm_count * g_tune[SPLAT_TUNE_EVOLVE_BLOCKS_PER_SM];
    if (b > lim) b = lim;
    return (int)(b < 1 ? 1 : b);
}

template <int MODE>
static cudaError_t launch_evolve_mode(const EvolveArgs& a, int64_t cap, int sm_count, cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    const int grid = evolve_grid(cap, sm_count);
    switch (a.material.kind) {
        case SPLAT_MATERIAL_LINEAR_REF: evolve_kernel<MODE, SPLAT_MATERIAL_LINEAR_REF><<<grid, kEvolveThreads, 0, s>>>(a); break;
        case SPLAT_MATERIAL_CAUCHY: evolve_kernel<MODE, SPLAT_MATERIAL_CAUCHY><<<grid, kEvolveThreads, 0, s>>>(a); break;
        case SPLAT_MATERIAL_SELLMEIER: evolve_kernel<MODE, SPLAT_MATERIAL_SELLMEIER><<<grid, kEvolveThreads, 0, s>>>(a); break;
        default: evolve_kernel<MODE, -1><<<grid, kEvolveThreads, 0, s>>>(a); break;
    }
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t launch_evolve_trace(const EvolveArgs& a, int64_t cap, int sm_count, cudaStream_t s) {
    return launch_evolve_mode<1>(a, cap, sm_count, s);
}

cudaError_t launch_evolve_camera(const EvolveArgs& a, int64_t cap, int sm_count, cudaStream_t s) {
    return launch_evolve_mode<2>(a, cap, sm_count, s);
}

cudaError_t launch_evolve_plugin(const EvolveArgs& a, int64_t cap, int sm_count, cudaStream_t s) {
    return launch_evolve_mode<0>(a, cap, sm_count, s);
}

// evolve_ray broadcast (src/tracer.jl:181-201: `rays .= evolve_ray.(rays,
// hit_idx, tri_view, rndm, first_diffuse)`) on the caller's AoS rays: every
// ACTIVE ray evolves in place with its hit index and its Fresnel draw
// rndm[k] (the reference's rand! output; without an array, Philox(seed) at
// (k, 0, 1, bounce), or force_rand when >= 0); a ray that hits a diffuse
// triangle or nothing only changes status; other rays are untouched.
__global__ void __launch_bounds__(kEvolveThreads) evolve_aos_kernel(splat_adray_t* rays, int64_t n,
                                                                    const int32_t* __restrict__ hit_idx,
                                                                    const float* __restrict__ rndm, EvolveArgs A) {
    const bool quirks = A.quirks != 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        splat_adray_t& a = rays[k];
        if (a.status != kStatusActive) continue;
        const RayState r = ray_from_aos(a);
        const EvolveView v{A.tris, A.n_tris, A.err, A.first_diffuse, A.material, A.seed, A.bounce,
                           rndm ? rndm[k] : A.force_rand, quirks, false};
        RayState o;
        int32_t ih;
        const int fate = evolve_one<false>(r, hit_idx[k], (uint32_t)k, v, o, ih);
        if (fate == kFateKeep) ray_to_aos(a, o, kStatusActive);
        else if (fate == kFateDiffuse) a.status = (uint8_t)kStatusDiffuse;
        else if (fate == kFateInfinity) a.status = (uint8_t)kStatusInfinity;
    }
}

cudaError_t launch_evolve_aos(splat_adray_t* rays, int64_t n, const int32_t* hit_idx, const float* rndm,
                              const EvolveArgs& a, int sm_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    evolve_aos_kernel<<<evolve_grid(n, sm_count), kEvolveThreads, 0, s>>>(rays, n, hit_idx, rndm, a);
    ++g_launches;
    return cudaGetLastError();
}

// partition! (src/partition.jl:10-132): the ACTIVE rays first, in no
// particular order (the reference's blocks claim offsets atomically too).
// counts[0] = number of ACTIVE rays (the result); counts[1], counts[2] =
// active and other rays placed so far.
__global__ void partition_count_kernel(const splat_adray_t* __restrict__ rays, int64_t n, int64_t* counts) {
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = base + threadIdx.x;
        const unsigned m = __ballot_sync(kFull, k < n && rays[k].status == kStatusActive);
        if (lane_id() == 0 && m) atomicAdd(reinterpret_cast<unsigned long long*>(&counts[0]), (unsigned long long)__popc(m));
    }
}

__global__ void partition_scatter_kernel(const splat_adray_t* __restrict__ rays, int64_t n, int64_t* counts,
                                         splat_adray_t* __restrict__ out) {
    const int64_t n_active = counts[0];
    unsigned long long* placed_active = reinterpret_cast<unsigned long long*>(&counts[1]);
    unsigned long long* placed_other = reinterpret_cast<unsigned long long*>(&counts[2]);
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = base + threadIdx.x;
        const bool valid = k < n;
        const bool act = valid && rays[k].status == kStatusActive;
        const unsigned ma = __ballot_sync(kFull, act), mi = __ballot_sync(kFull, valid && !act);
        const unsigned below = (1u << lane_id()) - 1u;
        unsigned long long ba = 0, bi = 0;
        if (lane_id() == 0) {
            if (ma) ba = atomicAdd(placed_active, (unsigned long long)__popc(ma));
            if (mi) bi = atomicAdd(placed_other, (unsigned long long)__popc(mi));
        }
        ba = __shfl_sync(kFull, ba, 0);
        bi = __shfl_sync(kFull, bi, 0);
        if (act) out[(int64_t)ba + __popc(ma & below)] = rays[k];
        else if (valid) out[n_active + (int64_t)bi + __popc(mi & below)] = rays[k];
    }
}

cudaError_t launch_partition(splat_adray_t* rays, int64_t n, splat_adray_t* swap, int64_t* counts, int sm_count,
                             cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(counts, 0, 3 * sizeof(int64_t), s);
    if (e != cudaSuccess || n <= 0) return e;
    partition_count_kernel<<<evolve_grid(n, sm_count), kEvolveThreads, 0, s>>>(rays, n, counts);
    partition_scatter_kernel<<<evolve_grid(n, sm_count), kEvolveThreads, 0, s>>>(rays, n, counts, swap);
    g_launches += 2;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaMemcpyAsync(rays, swap, sizeof(splat_adray_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
}

// continuum_light_map2! on the caller's AoS rays: final_evolution in place,
// then the splat.
__global__ void __launch_bounds__(kEvolveThreads) light_map_kernel(splat_adray_t* rays, int64_t n,
                                                                   const int32_t* __restrict__ hit_idx,
                                                                   const splat_ftri_t* __restrict__ tris,
                                                                   int64_t n_tris, int32_t* err, SplatParams sp) {
    for (int64_t base = (int64_t)blockIdx.x * kEvolveThreads; base < n; base += (int64_t)gridDim.x * kEvolveThreads) {
        const int64_t k = base + threadIdx.x;
        bool dif = false;
        RayState o;
        int32_t ih = 1;
        if (k < n && rays[k].status == kStatusDiffuse) {
            const int32_t i = hit_idx[k];
            if (i >= 1 && i <= n_tris) {
                const RayState r = ray_from_aos(rays[k]);
                const Tri T = load_tri(tris, i);
                HitDerivs h;
                ih = get_hit_ad(r, i, T, h);
                final_evolution(r, h, ih, o);
                ray_to_aos(rays[k], o, kStatusDiffuse);
                dif = true;
            } else {
                atomicOr(err, 16);
            }
        }
        (void)splat_warp(sp, tris, dif, o, ih);
    }
}

cudaError_t launch_light_map(splat_adray_t* rays, int64_t n, const int32_t* hit_idx, const splat_ftri_t* tris,
                             int64_t n_tris, int32_t* err, const SplatParams& sp, int sm_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    light_map_kernel<<<evolve_grid(n, sm_count), kEvolveThreads, 0, s>>>(rays, n, hit_idx, tris, n_tris, err, sp);
    ++g_launches;
    return cudaGetLastError();
}

// Queued diffuse rays -> light map, one lane per ray walking all its planes
// (each plane's N x N sub-samples in the reference's order, x offset
// fastest; runs of samples on the same texel add in a register before one
// atomic).  Integer maps are bit-exact; float maps change only the order of
// additions, which float atomics never fix anyway.
__global__ void __launch_bounds__(256, 3) splat_kernel(RaySoA q, const int64_t* __restrict__ d_begin,
                                                       const int64_t* __restrict__ d_count,
                                                       const splat_ftri_t* __restrict__ tris, SplatParams sp,
                                                       splat_trace_stats_t* st) {
    const int64_t k0 = d_begin ? *d_begin : 0;
    const int64_t n = *d_count;
    const int planes = sp.n_lambda > 0 ? sp.n_lambda : 1;
    int done = 0;
    for (int64_t k = k0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const RayState r = load_ray(q, k);
        const Tri T = load_tri(tris, r.ignore);
        const TriUV quv = tri_uv(T);
        for (int il = 0; il < planes; ++il) done += splat_ray_plane(sp, r, T, quv, il);
    }
    add_stats(st, 0, done);
}

// The same splat through the block's shared texel table: the block takes
// 256 queued rays at a time and, plane by plane, sums their samples per
// texel before one map atomic per distinct texel.
__global__ void __launch_bounds__(256, 2) splat_agg_kernel(RaySoA q, const int64_t* __restrict__ d_begin,
                                                           const int64_t* __restrict__ d_count,
                                                           const splat_ftri_t* __restrict__ tris, SplatParams sp,
                                                           splat_trace_stats_t* st) {
    __shared__ int32_t s_key[kAggSlots], s_val[kAggSlots];
    const int64_t k0 = d_begin ? *d_begin : 0;
    const int64_t n = *d_count;
    const int planes = sp.n_lambda > 0 ? sp.n_lambda : 1;
    const TableSink sink{sp, s_key, s_val};
    table_clear(s_key, s_val);
    __syncthreads();
    int done = 0;
    for (int64_t base = k0 + (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = base + threadIdx.x;
        const bool live = k < n;
        RayState r;
        Tri T;
        TriUV quv;
        if (live) {
            r = load_ray(q, k);
            T = load_tri(tris, r.ignore);
            quv = tri_uv(T);
        }
        for (int il = 0; il < planes; ++il) {
            if (live) done += splat_ray_plane(sp, r, T, quv, il, sink);
            __syncthreads();
            table_flush(sp, s_key, s_val);
            __syncthreads();
        }
    }
    add_stats(st, 0, done);
}

cudaError_t launch_splat(const RaySoA& q, const int64_t* d_begin, const int64_t* d_count, const splat_ftri_t* tris,
                         const SplatParams& sp, splat_trace_stats_t* stats, int sm_count, cudaStream_t s) {
    if (q.cap <= 0) return cudaSuccess;
    int64_t b = (q.cap + 255) / 256;
    const int64_t lim = (int64_t)sm_count * g_tune[SPLAT_TUNE_SPLAT_BLOCKS_PER_SM];
    if (b > lim) b = lim;
    if (g_tune[SPLAT_TUNE_SPLAT_AGGREGATE])
        splat_agg_kernel<<<(int)(b < 1 ? 1 : b), 256, 0, s>>>(q, d_begin, d_count, tris, sp, stats);
    else
        splat_kernel<<<(int)(b < 1 ? 1 : b), 256, 0, s>>>(q, d_begin, d_count, tris, sp, stats);
    ++g_launches;
    return cudaGetLastError();
}

__global__ void copy_count_kernel(const int64_t* src, int64_t* dst) { *dst = *src; }

cudaError_t launch_copy_count(const int64_t* src, int64_t* dst, cudaStream_t s) {
    copy_count_kernel<<<1, 1, 0, s>>>(src, dst);
    ++g_launches;
    return cudaGetLastError();
}

__global__ void stats_finish_kernel(const int64_t* counts, int depth, const int64_t* splat_count,
                                    splat_trace_stats_t* st, const int32_t* err) {
    // accumulates: a step run as several ray ranges adds each range's counts
    // into statistics cleared once
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        for (int b = 0; b < depth && b < 8; ++b)
            atomicAdd(reinterpret_cast<unsigned long long*>(&st->rays_per_bounce[b]), (unsigned long long)counts[b]);
        if (splat_count) atomicAdd(reinterpret_cast<unsigned long long*>(&st->diffuse), (unsigned long long)*splat_count);
        if (err) atomicOr(reinterpret_cast<unsigned long long*>(&st->error), (unsigned long long)(uint32_t)*err);
    }
}

cudaError_t launch_stats_finish(const int64_t* counts, int depth, const int64_t* splat_count,
                                splat_trace_stats_t* stats, const int32_t* err, cudaStream_t s) {
    stats_finish_kernel<<<1, 32, 0, s>>>(counts, depth, splat_count, stats, err);
    ++g_launches;
    return cudaGetLastError();
}

__global__ void generate_soa_kernel(GenParams g, int64_t n, RaySoA out, int64_t* d_count) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && d_count) *d_count = n;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t kid = g.ray_begin + k;
        store_ray(out, k, gen_ray(g, kid), (uint32_t)kid);
    }
}

__global__ void generate_aos_kernel(GenParams g, int64_t n, splat_adray_t* out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const RayState r = gen_ray(g, g.ray_begin + k);
        splat_adray_t a;
        memset(&a, 0, sizeof(a));
        ray_to_aos(a, r, kStatusActive);
        a.dest = 0;
        out[k] = a;
    }
}

cudaError_t launch_generate_soa(const GenParams& g, int64_t n, RaySoA out, int64_t* d_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    generate_soa_kernel<<<evolve_grid(n, 152), 256, 0, s>>>(g, n, out, d_count);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t launch_generate_aos(const GenParams& g, int64_t n, splat_adray_t* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    generate_aos_kernel<<<evolve_grid(n, 152), 256, 0, s>>>(g, n, out);
    ++g_launches;
    return cudaGetLastError();
}

// active AoS rays -> SoA (id = slot), compacted with one atomic per warp
__global__ void aos_to_soa_kernel(const splat_adray_t* in, int64_t n, RaySoA out, int64_t* d_count) {
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = base + threadIdx.x;
        const bool act = k < n && in[k].status == kStatusActive;
        const unsigned b = __ballot_sync(kFull, act);
        unsigned long long wbase = 0;
        if (lane_id() == 0 && b)
            wbase = atomicAdd(reinterpret_cast<unsigned long long*>(d_count), (unsigned long long)__popc(b));
        wbase = __shfl_sync(kFull, wbase, 0);
        if (act) {
            const int64_t pos = (int64_t)wbase + __popc(b & ((1u << lane_id()) - 1u));
            store_ray(out, pos, ray_from_aos(in[k]), (uint32_t)k);
        }
    }
}

__global__ void soa_to_aos_kernel(RaySoA in, const int64_t* d_count, splat_adray_t* out, int status) {
    const int64_t n = *d_count;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        ray_to_aos(out[in.id[k]], load_ray(in, k), status);
}

cudaError_t launch_aos_to_soa(const splat_adray_t* in, int64_t n, RaySoA out, int64_t* d_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    aos_to_soa_kernel<<<evolve_grid(n, 152), 256, 0, s>>>(in, n, out, d_count);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(RaySoA in, const int64_t* d_count, splat_adray_t* out, int status, cudaStream_t s) {
    if (in.cap <= 0) return cudaSuccess;
    soa_to_aos_kernel<<<evolve_grid(in.cap, 152), 256, 0, s>>>(in, d_count, out, status);
    ++g_launches;
    return cudaGetLastError();
}

}  // namespace splat
