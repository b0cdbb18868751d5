// hitcore.cuh -- per-ray pieces of the hitters, shared by the single-scene
// kernels (hit.cu) and the multi-scene batch kernels (batch.cu).
#pragma once

#include <climits>

#include "kernels.h"

namespace splat {

// ---------------------------------------------------------------------------
// ray loading
// ---------------------------------------------------------------------------
struct HitRay {
    float ox, oy, oz, dx, dy, dz;
    int32_t ig;
};

template <bool AOS>
__device__ __forceinline__ HitRay load_hit_ray(const RaySrc& s, int64_t k) {
    HitRay r;
    if (AOS) {
        const splat_adray_t& a = s.aos[k];
        r.ox = a.pos[0];
        r.oy = a.pos[1];
        r.oz = a.pos[2];
        r.dx = a.dir[0];
        r.dy = a.dir[1];
        r.dz = a.dir[2];
        r.ig = (int32_t)a.ignore_tri;
    } else {
        const float* f = s.f;
        const int64_t c = s.cap;
        r.ox = f[k];
        r.oy = f[c + k];
        r.oz = f[2 * c + k];
        r.dx = f[3 * c + k];
        r.dy = f[4 * c + k];
        r.dz = f[5 * c + k];
        r.ig = s.ignore[k];
    }
    return r;
}

// Traversal work of one thread, counted only by the counting instantiations
// of the four-wide kernels (SPLAT_TUNE_COUNT_WORK): nodes visited, triangle
// pre-tests, full triangle tests.  Kernels that do not count pass nullptr,
// which removes the counting code.
struct WorkCount {
    uint32_t nodes, pre, full;
};

// Plane terms of distance_to_plane (src/geo.jl:433-435) and a conservative
// pre-test: an accepted hit has t = num / den > 0 (so num, den are non-zero
// with one sign) and t <= best; |num| > |den| best (1 + 2^-20), evaluated in
// binary32, implies fl(num / den) > best whatever the roundings.  Triangles
// failing the pre-test could never be accepted, so skipping them leaves the
// result bit-identical.
__device__ __forceinline__ bool tri_candidate(const float4& q0, const HitRay& r, float best, float& num, float& den) {
    num = q0.w - ((q0.x * r.ox + q0.y * r.oy) + q0.z * r.oz);
    den = (q0.x * r.dx + q0.y * r.dy) + q0.z * r.dz;
    const bool same_sign = ((num > 0.0f) & (den > 0.0f)) | ((num < 0.0f) & (den < 0.0f));
    return same_sign & !(fabsf(num) > (fabsf(den) * best) * (1.0f + 0x1p-20f));
}

// The rest of the reference's test on one hoisted record (src/geo.jl:433-466).
__device__ __forceinline__ float tri_t_from(float num, float den, const float4& q1, const float4& q2,
                                            const float4& q3, const float4& q4, const HitRay& r, bool& inside) {
    float t = num / den;
    float px = r.ox + r.dx * t;
    float py = r.oy + r.dy * t;
    float pz = r.oz + r.dz * t;
    float v2x = px - q1.x, v2y = py - q1.y, v2z = pz - q1.z;
    float d02 = (q2.x * v2x + q2.y * v2y) + q2.z * v2z;
    float d12 = (q3.x * v2x + q3.y * v2y) + q3.z * v2z;
    float u = (q3.w * d02 - q4.x * d12) * q4.y;
    float v = (q2.w * d12 - q4.x * d02) * q4.y;
    inside = (u >= 0.0f) & (v >= 0.0f) & (u + v < 1.0f);
    return t;
}

// The reference's test on one hoisted record (src/geo.jl:433-466).
__device__ __forceinline__ float tri_t(const float4& q0, const float4& q1, const float4& q2, const float4& q3,
                                       const float4& q4, const HitRay& r, bool& inside) {
    float num = q0.w - ((q0.x * r.ox + q0.y * r.oy) + q0.z * r.oz);
    float den = (q0.x * r.dx + q0.y * r.dy) + q0.z * r.dz;
    float t = num / den;
    float px = r.ox + r.dx * t;
    float py = r.oy + r.dy * t;
    float pz = r.oz + r.dz * t;
    float v2x = px - q1.x, v2y = py - q1.y, v2z = pz - q1.z;
    float d02 = (q2.x * v2x + q2.y * v2y) + q2.z * v2z;
    float d12 = (q3.x * v2x + q3.y * v2y) + q3.z * v2z;
    float u = (q3.w * d02 - q4.x * d12) * q4.y;
    float v = (q2.w * d12 - q4.x * d02) * q4.y;
    inside = (u >= 0.0f) & (v >= 0.0f) & (u + v < 1.0f);
    return t;
}

__device__ __forceinline__ float safe_inv(float d) {
    return 1.0f / (fabsf(d) > 1.0e-30f ? d : copysignf(1.0e-30f, d));
}

__device__ __forceinline__ float comp(const float4& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// Three-input min / max (one instruction each on sm_100 and later; the same
// IEEE minNum / maxNum rule as the nested two-input forms).
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Entry and exit distances of a ray through the four child boxes of a
// node.  The slab planes are picked by the signs of the inverse direction
// (ix < 0: the near x plane is hi, else lo), through the addresses of the
// node's per-axis float4s, so the test needs no per-axis min / max: each
// distance is the one min(a, b) / max(a, b) of the two planes would pick,
// bit for bit (lo <= hi for every real child; the empty slots, lo = +inf and
// hi = -inf, come out with t0 = +inf > tmax = -inf whatever the ray, as the
// inverse direction is finite and non-zero, and are never entered).  t0 is the entry distance clamped at the origin, max(tmin, 0):
// for non-NaN values (tmin <= tmax and tmax >= 0) is t0 <= tmax, and, as
// every accepted hit has t > 0, tmin <= best is t0 <= best, so a child is
// entered exactly when the unclamped test enters it.
__device__ __forceinline__ void node4_slabs(const Bvh4Node* nd, float ix, float iy, float iz, float oix, float oiy,
                                            float oiz, float t0[4], float tmax[4]) {
    const float4* q = reinterpret_cast<const float4*>(nd);  // lox, hix, loy, hiy, loz, hiz
    const int sx = ix < 0.0f ? 1 : 0, sy = iy < 0.0f ? 1 : 0, sz = iz < 0.0f ? 1 : 0;
    const float4 nx = __ldg(q + sx), fx = __ldg(q + 1 - sx);
    const float4 ny = __ldg(q + 2 + sy), fy = __ldg(q + 3 - sy);
    const float4 nz = __ldg(q + 4 + sz), fz = __ldg(q + 5 - sz);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        t0[i] = max3f(fmaf(comp(nx, i), ix, -oix), fmaf(comp(ny, i), iy, -oiy),
                      fmaxf(fmaf(comp(nz, i), iz, -oiz), 0.0f));
        tmax[i] = min3f(fmaf(comp(fx, i), ix, -oix), fmaf(comp(fy, i), iy, -oiy), fmaf(comp(fz, i), iz, -oiz));
    }
}

#define SPLAT_CSWAP(ka, ra, kb, rb)       \
    if (kb < ka) {                         \
        const float tk = ka;               \
        ka = kb;                           \
        kb = tk;                           \
        const int tr = ra;                 \
        ra = rb;                           \
        rb = tr;                           \
    }

// Closest hit of one ray in a four-wide BVH.  A node fetch (128 bytes)
// tests four child boxes; hit children are sorted by entry distance, the
// nearest is visited next and the others are pushed farthest first with
// their entry distance, so a popped entry beyond the current best hit is
// skipped.  stack holds kBvhStack entries of (ref, entry distance bits), so
// a push or a pop is one 8-byte local access.
__device__ __forceinline__ void bvh4_closest(const HitRay& r, const Bvh4View& bvh, int2* stack, int32_t* err,
                                             float& best_out, int32_t& bi_out, WorkCount* wc = nullptr) {
    const float kInf = __int_as_float(0x7f800000);
    const float kMax = 3.402823466e38f;
    const float ix = safe_inv(r.dx), iy = safe_inv(r.dy), iz = safe_inv(r.dz);
    const float oix = r.ox * ix, oiy = r.oy * iy, oiz = r.oz * iz;
    float best = kInf;
    int32_t bi = 1;
    int sp = 0;
    int ref = 0;
    while (true) {
        if (ref >= 0) {
            const Bvh4Node* nd = bvh.nodes + ref;
            if (wc) ++wc->nodes;
            const int4 c = __ldg(&nd->c);
            float tmin[4], tmax[4], key[4];
            node4_slabs(nd, ix, iy, iz, oix, oiy, oiz, tmin, tmax);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const bool h = (tmin[i] <= tmax[i]) & (tmin[i] <= best);  // tmin: clamped at 0; empty slots fail
                key[i] = h ? fminf(tmin[i], kMax) : kInf;
            }
            float k0 = key[0], k1 = key[1], k2 = key[2], k3 = key[3];
            int r0 = c.x, r1 = c.y, r2 = c.z, r3 = c.w;
            SPLAT_CSWAP(k0, r0, k1, r1);
            SPLAT_CSWAP(k2, r2, k3, r3);
            SPLAT_CSWAP(k0, r0, k2, r2);
            SPLAT_CSWAP(k1, r1, k3, r3);
            SPLAT_CSWAP(k1, r1, k2, r2);
            if (k0 < kInf) {
                if (sp + 3 <= kBvhStack) {
                    if (k3 < kInf) stack[sp++] = make_int2(r3, __float_as_int(k3));
                    if (k2 < kInf) stack[sp++] = make_int2(r2, __float_as_int(k2));
                    if (k1 < kInf) stack[sp++] = make_int2(r1, __float_as_int(k1));
                } else {
                    atomicOr(err, 2);
                }
                ref = r0;
                continue;
            }
        } else {
            const int enc = ~ref;
            const int first = enc >> 4;
            const int count = (enc & 15) + 1;
            for (int j = 0; j < count; ++j) {
                const TriHit* h = bvh.tris + first + j;
                float num, den;
                if (wc) ++wc->pre;
                if (!tri_candidate(__ldg(&h->n_nv), r, best, num, den)) continue;
                if (wc) ++wc->full;
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
    best_out = best;
    bi_out = bi;
}
// Per-lane ray replacement over a work counter (the "dynamic fetch" of
// Aila and Laine, "Understanding the efficiency of ray traversal on GPUs",
// HPG 2009): every lane walks its own ray through the four-wide BVH exactly
// as bvh4_closest does, one node or leaf per loop iteration, and when at
// least refill_min lanes of the warp have finished, the warp takes that many
// new rays from the counter in one atomic.  A warp no longer waits for its
// slowest ray before the others start new work.  load(k) returns ray k,
// view(k) the BVH it is traced in, store(k, t, index) takes its result.
// Every node and leaf of a ray is entered at most once; kBvhVisitCap bounds
// a ray's loop all the same (error bit 8).
constexpr int kBvhVisitCap = 1 << 22;

template <class Load, class View, class Store>
__device__ __forceinline__ void bvh4_refill_loop(int64_t n, unsigned long long* fetch, int refill_min, int32_t* err,
                                                 const Load& load, const View& view, const Store& store) {
    constexpr int kDone = INT_MIN;  // no leaf reference is INT_MIN (at most 2^27 triangles)
    const float kInf = __int_as_float(0x7f800000);
    const float kMax = 3.402823466e38f;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    int2 stack[kBvhStack];
    HitRay r{};
    Bvh4View bvh{};
    float ix = 0.f, iy = 0.f, iz = 0.f, oix = 0.f, oiy = 0.f, oiz = 0.f, best = kInf;
    int32_t bi = 1;
    int sp = 0, node = kDone, visits = 0;
    int64_t k = 0;
    bool more = true;  // warp-uniform: the counter may still hold rays
    while (true) {
        const unsigned idle = __ballot_sync(0xffffffffu, node == kDone);
        const int n_idle = __popc(idle);
        if (more && (n_idle >= refill_min || idle == 0xffffffffu)) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(fetch, (unsigned long long)n_idle);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base + (unsigned long long)n_idle >= (unsigned long long)n) more = false;
            if (node == kDone) {
                const unsigned long long kk = base + (unsigned long long)__popc(idle & below);
                if (kk < (unsigned long long)n) {
                    k = (int64_t)kk;
                    r = load(k);
                    bvh = view(k);
                    ix = safe_inv(r.dx);
                    iy = safe_inv(r.dy);
                    iz = safe_inv(r.dz);
                    oix = r.ox * ix;
                    oiy = r.oy * iy;
                    oiz = r.oz * iz;
                    best = kInf;
                    bi = 1;
                    sp = 0;
                    node = 0;
                    visits = 0;
                }
            }
        }
        if (!more && __all_sync(0xffffffffu, node == kDone)) break;
        if (node == kDone) continue;
        if (++visits > kBvhVisitCap) {
            atomicOr(err, 8);
            sp = 0;
        } else if (node >= 0) {
            const Bvh4Node* nd = bvh.nodes + node;
            const int4 c = __ldg(&nd->c);
            float tmin[4], tmax[4], key[4];
            node4_slabs(nd, ix, iy, iz, oix, oiy, oiz, tmin, tmax);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const bool h = (tmin[i] <= tmax[i]) & (tmin[i] <= best);  // tmin: clamped at 0; empty slots fail
                key[i] = h ? fminf(tmin[i], kMax) : kInf;
            }
            float k0 = key[0], k1 = key[1], k2 = key[2], k3 = key[3];
            int r0 = c.x, r1 = c.y, r2 = c.z, r3 = c.w;
            SPLAT_CSWAP(k0, r0, k1, r1);
            SPLAT_CSWAP(k2, r2, k3, r3);
            SPLAT_CSWAP(k0, r0, k2, r2);
            SPLAT_CSWAP(k1, r1, k3, r3);
            SPLAT_CSWAP(k1, r1, k2, r2);
            if (k0 < kInf) {
                if (sp + 3 <= kBvhStack) {
                    if (k3 < kInf) stack[sp++] = make_int2(r3, __float_as_int(k3));
                    if (k2 < kInf) stack[sp++] = make_int2(r2, __float_as_int(k2));
                    if (k1 < kInf) stack[sp++] = make_int2(r1, __float_as_int(k1));
                } else {
                    atomicOr(err, 2);
                }
                node = r0;
                continue;
            }
        } else {
            const int enc = ~node;
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
        node = kDone;
        while (sp > 0) {
            const int2 e = stack[--sp];
            if (__int_as_float(e.y) <= best) {
                node = e.x;
                break;
            }
        }
        if (node == kDone) store(k, best, bi);
    }
}

#undef SPLAT_CSWAP

// Packet traversal of a four-wide BVH: the 32 rays of a warp walk one
// shared stack.  A child is entered when any lane's ray enters its box at or
// before that lane's best hit; children are visited in the order of the
// warp's smallest entry distance (a __reduce_min over order-preserving
// codes), so every decision is warp-uniform and the node loads are
// broadcasts.  Every lane tests every triangle of a visited leaf against its
// own ray.  Each lane still ends with the lexicographic (t, index) minimum
// over every triangle whose padded box its ray enters at or before its best
// hit, so the result equals the per-ray traversal and brute force.  For
// coherent rays (a light's primary rays, refraction through smooth glass)
// the union of the lanes' paths is little more than one ray's path, and the
// warp runs it with all lanes busy.  A pushed child keeps the warp's
// smallest entry distance; it is popped only while that distance is at or
// before the largest best hit of the warp's lanes (the per-ray form's pop
// test, taken over the warp: a lane entered the child at or after that
// distance, and a lane whose best hit is nearer cannot need it).  stack:
// kPacketStack (ref, entry distance bits) pairs shared by the warp; every
// lane writes every entry (same value), so no warp barrier.
constexpr int kPacketStack = 128;

__device__ __forceinline__ void bvh4_closest_packet(const HitRay& r, bool valid, const Bvh4View& bvh, int2* stack,
                                                    int32_t* err, float& best_out, int32_t& bi_out,
                                                    WorkCount* wc = nullptr) {
    const float kInf = __int_as_float(0x7f800000);
    const float ix = safe_inv(r.dx), iy = safe_inv(r.dy), iz = safe_inv(r.dz);
    const float oix = r.ox * ix, oiy = r.oy * iy, oiz = r.oz * iz;
    float best = kInf;
    float reach = kInf;  // the largest best hit over the warp's valid lanes
    int32_t bi = 1;
    int sp = 0;
    int ref = 0;
    while (true) {
        if (ref >= 0) {
            const Bvh4Node* nd = bvh.nodes + ref;
            if (wc && valid) ++wc->nodes;
            const int4 c = __ldg(&nd->c);
            float tmin[4], tmax[4];
            node4_slabs(nd, ix, iy, iz, oix, oiy, oiz, tmin, tmax);
            unsigned u[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                // tmin is clamped at 0 (node4_slabs): non-negative floats order as
                // their bits, so its bits are the sort key (a -0 from the max sorts
                // last: order only, never which children are entered)
                const float t0 = tmin[i];
                const bool h = valid & (t0 <= tmax[i]) & (t0 <= best);  // empty slots fail
                u[i] = __reduce_min_sync(0xffffffffu, h ? __float_as_uint(t0) : 0xffffffffu);
            }
            unsigned k0 = u[0], k1 = u[1], k2 = u[2], k3 = u[3];
            int r0 = c.x, r1 = c.y, r2 = c.z, r3 = c.w;
#define SPLAT_USWAP(ka, ra, kb, rb)          \
    if (kb < ka) {                           \
        const unsigned tk = ka;              \
        ka = kb;                             \
        kb = tk;                             \
        const int tr = ra;                   \
        ra = rb;                             \
        rb = tr;                             \
    }
            SPLAT_USWAP(k0, r0, k1, r1);
            SPLAT_USWAP(k2, r2, k3, r3);
            SPLAT_USWAP(k0, r0, k2, r2);
            SPLAT_USWAP(k1, r1, k3, r3);
            SPLAT_USWAP(k1, r1, k2, r2);
#undef SPLAT_USWAP
            if (k0 != 0xffffffffu) {
                if (sp + 3 <= kPacketStack) {
                    if (k3 != 0xffffffffu) stack[sp++] = make_int2(r3, (int)k3);
                    if (k2 != 0xffffffffu) stack[sp++] = make_int2(r2, (int)k2);
                    if (k1 != 0xffffffffu) stack[sp++] = make_int2(r1, (int)k1);
                } else if (threadIdx.x % 32 == 0) {
                    atomicOr(err, 2);
                }
                ref = r0;
                continue;
            }
        } else {
            const int enc = ~ref;
            const int first = enc >> 4;
            const int count = (enc & 15) + 1;
            for (int j = 0; j < count; ++j) {
                const TriHit* h = bvh.tris + first + j;
                float num, den;
                if (wc && valid) ++wc->pre;
                const bool cand = valid && tri_candidate(__ldg(&h->n_nv), r, best, num, den);
                if (!cand) continue;
                if (wc) ++wc->full;
                const float4 q1 = __ldg(&h->a_idx);
                const int32_t idx = __float_as_int(q1.w);
                bool inside;
                const float t = tri_t_from(num, den, q1, __ldg(&h->e0), __ldg(&h->e1), __ldg(&h->inv), r, inside);
                if (inside & (t > 0.0f) & (idx != r.ig) & ((t < best) | ((t == best) & (idx < bi)))) {
                    best = t;
                    bi = idx;
                }
            }
            // best >= 0 (or +inf), so its bits order as the floats
            reach = __uint_as_float(__reduce_max_sync(0xffffffffu, valid ? __float_as_uint(best) : 0u));
        }
        bool found = false;
        while (sp > 0) {
            const int2 e = stack[--sp];
            if (__int_as_float(e.y) <= reach) {  // a -0 entry compares as 0
                ref = e.x;
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    best_out = best;
    bi_out = bi;
}

// Spread of a warp's rays, max over axes of (max - min) of a coordinate.
__device__ __forceinline__ float warp_spread(float a, float b, float c) {
    float m = 0.0f;
    const float v[3] = {a, b, c};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float lo = v[i], hi = v[i];
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        m = fmaxf(m, hi - lo);
    }
    return m;
}

// Largest extent of the scene: the root's child boxes, max over axes.
__device__ __forceinline__ float bvh4_extent(const Bvh4Node* nodes) {
    const Bvh4Node& root = nodes[0];
    const float4 lx = __ldg(&root.lox), hx = __ldg(&root.hix), ly = __ldg(&root.loy), hy = __ldg(&root.hiy);
    const float4 lz = __ldg(&root.loz), hz = __ldg(&root.hiz);
    const int nc = __ldg(&root.meta.x);
    float lo[3] = {lx.x, ly.x, lz.x}, hi[3] = {hx.x, hy.x, hz.x};
    for (int i = 1; i < nc; ++i) {
        lo[0] = fminf(lo[0], comp(lx, i));
        lo[1] = fminf(lo[1], comp(ly, i));
        lo[2] = fminf(lo[2], comp(lz, i));
        hi[0] = fmaxf(hi[0], comp(hx, i));
        hi[1] = fmaxf(hi[1], comp(hy, i));
        hi[2] = fmaxf(hi[2], comp(hz, i));
    }
    return fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
}

// Packet forms 2 / 3: the warp's rays are nearly parallel (direction spread
// <= 0.3 / 0.1) and close together (origin spread <= 0.05 / 0.01 x the
// scene's extent).  All 32 lanes call.
__device__ __forceinline__ bool packet_coherent(const HitRay& r, int form, float extent) {
    const float dir_spread = form == 2 ? 0.3f : 0.1f, org_spread = form == 2 ? 0.05f : 0.01f;
    const float ds = warp_spread(r.dx, r.dy, r.dz), os = warp_spread(r.ox, r.oy, r.oz);
    return ds <= dir_spread && os <= org_spread * extent;
}

// Closest hit of one ray over hit records in reference-index order (the
// per-ray form of the brute-force hitter; strict < keeps the smaller index),
// each record behind its padded box as in the tiled kernel.
__device__ __forceinline__ void brute_closest(const HitRay& r, const TriHit* recs, const TriBox* boxes,
                                              int64_t n_recs, float& best_out, int32_t& bi_out) {
    float best = __int_as_float(0x7f800000);
    int32_t bi = 1;
    const float ix = safe_inv(r.dx), iy = safe_inv(r.dy), iz = safe_inv(r.dz);
    const float oix = r.ox * ix, oiy = r.oy * iy, oiz = r.oz * iz;
    for (int64_t j = 0; j < n_recs; ++j) {
        const float4 lo = __ldg(&boxes[j].lo), hi = __ldg(&boxes[j].hi);
        const float a0 = fmaf(lo.x, ix, -oix), b0 = fmaf(hi.x, ix, -oix);
        const float a1 = fmaf(lo.y, iy, -oiy), b1 = fmaf(hi.y, iy, -oiy);
        const float a2 = fmaf(lo.z, iz, -oiz), b2 = fmaf(hi.z, iz, -oiz);
        const float tmin = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fminf(a2, b2));
        const float tmax = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fmaxf(a2, b2));
        if (!((tmin <= tmax) & (tmax >= 0.0f) & (tmin <= best))) continue;
        const TriHit* h = recs + j;
        float num, den;
        if (!tri_candidate(__ldg(&h->n_nv), r, best, num, den)) continue;
        const float4 q1 = __ldg(&h->a_idx);
        const int32_t idx = __float_as_int(q1.w);
        bool inside;
        const float t = tri_t_from(num, den, q1, __ldg(&h->e0), __ldg(&h->e1), __ldg(&h->inv), r, inside);
        if (inside & (t > 0.0f) & (idx != r.ig) & (t < best)) {
            best = t;
            bi = idx;
        }
    }
    best_out = best;
    bi_out = bi;
}

}  // namespace splat
