// common.cuh -- records, exact binary32 vector math, dual numbers, Philox.
//
// Every translation unit of the trace path is compiled with -fmad=false and
// IEEE division / square root, so each operation below rounds once, in the
// reference's source order (a + b + c is the left fold, dot(a, b) is
// (a1 b1 + a2 b2) + a3 b3, cross is StaticArrays' component formula,
// normalize(v) = v * (1 / norm(v))).  That is what makes hit indices, hit
// distances and fixed-point light maps bit-identical to the CPU restatement
// of the reference.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#include "../../include/splat.h"

namespace splat {

constexpr int kStatusDiffuse = 0;
constexpr int kStatusActive = 1;
constexpr int kStatusInfinity = 2;

// ----------------------------------------------------------------------------
// vectors over float or dual scalars
// ----------------------------------------------------------------------------

// Dual number with one partial: ForwardDiff's Dual{T,Float32,1} restated
// (dual.jl / partials.jl).  Plain float operands are constants of the
// closure being differentiated and contribute no partial.
struct D {
    float v, d;
};

__host__ __device__ __forceinline__ D operator+(D a, D b) { return {a.v + b.v, a.d + b.d}; }
__host__ __device__ __forceinline__ D operator+(D a, float b) { return {a.v + b, a.d}; }
__host__ __device__ __forceinline__ D operator+(float a, D b) { return {a + b.v, b.d}; }
__host__ __device__ __forceinline__ D operator-(D a, D b) { return {a.v - b.v, a.d - b.d}; }
__host__ __device__ __forceinline__ D operator-(D a, float b) { return {a.v - b, a.d}; }
__host__ __device__ __forceinline__ D operator-(float a, D b) { return {a - b.v, -b.d}; }
__host__ __device__ __forceinline__ D operator*(D a, D b) { return {a.v * b.v, b.v * a.d + a.v * b.d}; }
__host__ __device__ __forceinline__ D operator*(float a, D b) { return {a * b.v, a * b.d}; }
__host__ __device__ __forceinline__ D operator*(D a, float b) { return {a.v * b, a.d * b}; }
__host__ __device__ __forceinline__ D operator/(D a, D b) {
    return {a.v / b.v, (1.0f / b.v) * a.d + (-(a.v / (b.v * b.v))) * b.d};
}
__host__ __device__ __forceinline__ D operator/(D a, float b) { return {a.v / b, a.d / b}; }
__host__ __device__ __forceinline__ D operator/(float a, D b) {
    float q = a / b.v;
    return {q, -(q / b.v) * b.d};
}
__host__ __device__ __forceinline__ D dsqrt(D a) {
    float s = sqrtf(a.v);
    return {s, (1.0f / (2.0f * s)) * a.d};
}
__host__ __device__ __forceinline__ float dsqrt(float a) { return sqrtf(a); }
__host__ __device__ __forceinline__ float val(float a) { return a; }
__host__ __device__ __forceinline__ float val(D a) { return a.v; }
__host__ __device__ __forceinline__ float par(D a) { return a.d; }

template <class T>
struct V3 {
    T x, y, z;
};

using F3 = V3<float>;
using D3 = V3<D>;

template <class A, class B>
__host__ __device__ __forceinline__ auto operator+(V3<A> a, V3<B> b) -> V3<decltype(a.x + b.x)> {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <class A, class B>
__host__ __device__ __forceinline__ auto operator-(V3<A> a, V3<B> b) -> V3<decltype(a.x - b.x)> {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
// vector * scalar, each component a_i * s
template <class A, class S>
__host__ __device__ __forceinline__ auto operator*(V3<A> a, S s) -> V3<decltype(a.x * s)> {
    return {a.x * s, a.y * s, a.z * s};
}
template <class A, class B>
__host__ __device__ __forceinline__ auto dot(V3<A> a, V3<B> b) -> decltype(a.x * b.x) {
    return (a.x * b.x + a.y * b.y) + a.z * b.z;
}
template <class A, class B>
__host__ __device__ __forceinline__ auto cross(V3<A> a, V3<B> b) -> V3<decltype(a.x * b.x)> {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class A>
__host__ __device__ __forceinline__ A norm(V3<A> a) {
    return dsqrt((a.x * a.x + a.y * a.y) + a.z * a.z);
}
template <class A>
__host__ __device__ __forceinline__ V3<A> normalize(V3<A> a) {
    A inv = 1.0f / norm(a);
    return {a.x * inv, a.y * inv, a.z * inv};
}
template <class A>
__host__ __device__ __forceinline__ F3 vval(V3<A> a) {
    return {val(a.x), val(a.y), val(a.z)};
}
__host__ __device__ __forceinline__ F3 vpar(D3 a) { return {a.x.d, a.y.d, a.z.d}; }

// ----------------------------------------------------------------------------
// records
// ----------------------------------------------------------------------------

// Hit-test record of one triangle: the per-triangle invariants of the
// reference's distance_to_plane / in_triangle (src/geo.jl:433-466) hoisted
// out of the ray loop with the same binary32 operations, so the per-ray test
// reproduces the reference bit for bit.  80 bytes, 16-byte aligned.
struct __align__(16) TriHit {
    float4 n_nv;   // plane normal n (as stored in the FTri), nv = dot(n, v1)
    float4 a_idx;  // v1, reference index (int bits)
    float4 e0;     // c - a, dot00
    float4 e1;     // b - a, dot11
    float4 inv;    // dot01, invDenom, 0, 0
};
static_assert(sizeof(TriHit) == 80, "TriHit layout");

// Padded vertex box of a triangle (lo.xyz, hi.xyz; w unused): the box the
// BVH's leaves use, pad = pad_abs + pad_rel |box diagonal|.  A ray that
// misses it cannot be accepted by the triangle's test.
struct __align__(16) TriBox {
    float4 lo, hi;
};
static_assert(sizeof(TriBox) == 32, "TriBox layout");

__host__ __device__ __forceinline__ float pad_abs_of_scale(float max_abs_coord) {
    return 1.0e-4f * (max_abs_coord > 1.0f ? max_abs_coord : 1.0f);
}

__host__ __device__ __forceinline__ F3 f3(const float* p) { return {p[0], p[1], p[2]}; }

// FTri as loaded into registers (src/geo.jl:18).
struct Tri {
    F3 n, a, b, c, na, nb, nc, ta, tb, tc;
};

__device__ __forceinline__ Tri load_tri(const splat_ftri_t* tris, int32_t idx1) {
    const float* p = tris[idx1 - 1].v[0];
    Tri t;
    t.n = {__ldg(p + 0), __ldg(p + 1), __ldg(p + 2)};
    t.a = {__ldg(p + 3), __ldg(p + 4), __ldg(p + 5)};
    t.b = {__ldg(p + 6), __ldg(p + 7), __ldg(p + 8)};
    t.c = {__ldg(p + 9), __ldg(p + 10), __ldg(p + 11)};
    t.na = {__ldg(p + 12), __ldg(p + 13), __ldg(p + 14)};
    t.nb = {__ldg(p + 15), __ldg(p + 16), __ldg(p + 17)};
    t.nc = {__ldg(p + 18), __ldg(p + 19), __ldg(p + 20)};
    t.ta = {__ldg(p + 21), __ldg(p + 22), __ldg(p + 23)};
    t.tb = {__ldg(p + 24), __ldg(p + 25), __ldg(p + 26)};
    t.tc = {__ldg(p + 27), __ldg(p + 28), __ldg(p + 29)};
    return t;
}

// Structure-of-arrays ray state for the bounce loop.  Float planes:
// 0-2 pos, 3-5 dir, 6-8 dp/dlambda, 9-11 dp/dx, 12-14 dp/dy,
// 15-17 dd/dlambda, 18-20 dd/dx, 21-23 dd/dy, 24 lambda, 25 x, 26 y.
constexpr int kPlanes = 27;
struct RaySoA {
    float* f;          // kPlanes x cap
    int32_t* ignore;   // reference index of the triangle the ray left
    uint32_t* id;      // ray id (generation index or AoS slot)
    uint8_t* medium;   // in_medium
    int64_t cap;
};

struct RayState {
    F3 pos, dir, dpl, dpx, dpy, ddl, ddx, ddy;
    float lam, x, y;
    int32_t ignore;
    int32_t medium;
};

__device__ __forceinline__ F3 ld3(const float* f, int64_t cap, int plane, int64_t k) {
    return {f[plane * cap + k], f[(plane + 1) * cap + k], f[(plane + 2) * cap + k]};
}
__device__ __forceinline__ void st3(float* f, int64_t cap, int plane, int64_t k, F3 v) {
    f[plane * cap + k] = v.x;
    f[(plane + 1) * cap + k] = v.y;
    f[(plane + 2) * cap + k] = v.z;
}

__device__ __forceinline__ RayState load_ray(const RaySoA& s, int64_t k) {
    RayState r;
    const float* f = s.f;
    int64_t c = s.cap;
    r.pos = ld3(f, c, 0, k);
    r.dir = ld3(f, c, 3, k);
    r.dpl = ld3(f, c, 6, k);
    r.dpx = ld3(f, c, 9, k);
    r.dpy = ld3(f, c, 12, k);
    r.ddl = ld3(f, c, 15, k);
    r.ddx = ld3(f, c, 18, k);
    r.ddy = ld3(f, c, 21, k);
    r.lam = f[24 * c + k];
    r.x = f[25 * c + k];
    r.y = f[26 * c + k];
    r.ignore = s.ignore[k];
    r.medium = s.medium[k];
    return r;
}

__device__ __forceinline__ void store_ray(const RaySoA& s, int64_t k, const RayState& r, uint32_t id) {
    float* f = s.f;
    int64_t c = s.cap;
    st3(f, c, 0, k, r.pos);
    st3(f, c, 3, k, r.dir);
    st3(f, c, 6, k, r.dpl);
    st3(f, c, 9, k, r.dpx);
    st3(f, c, 12, k, r.dpy);
    st3(f, c, 15, k, r.ddl);
    st3(f, c, 18, k, r.ddx);
    st3(f, c, 21, k, r.ddy);
    f[24 * c + k] = r.lam;
    f[25 * c + k] = r.x;
    f[26 * c + k] = r.y;
    s.ignore[k] = r.ignore;
    s.medium[k] = (uint8_t)r.medium;
    s.id[k] = id;
}

__device__ __forceinline__ RayState ray_from_aos(const splat_adray_t& a) {
    RayState r;
    r.pos = f3(a.pos);
    r.dpl = f3(a.dp_dl);
    r.dpx = f3(a.dp_dx);
    r.dpy = f3(a.dp_dy);
    r.dir = f3(a.dir);
    r.ddl = f3(a.dd_dl);
    r.ddx = f3(a.dd_dx);
    r.ddy = f3(a.dd_dy);
    r.lam = a.lambda;
    r.x = a.x;
    r.y = a.y;
    r.ignore = (int32_t)a.ignore_tri;
    r.medium = a.in_medium;
    return r;
}

__device__ __forceinline__ void ray_to_aos(splat_adray_t& a, const RayState& r, int status) {
    auto put = [](float* d, F3 v) {
        d[0] = v.x;
        d[1] = v.y;
        d[2] = v.z;
    };
    put(a.pos, r.pos);
    put(a.dp_dl, r.dpl);
    put(a.dp_dx, r.dpx);
    put(a.dp_dy, r.dpy);
    put(a.dir, r.dir);
    put(a.dd_dl, r.ddl);
    put(a.dd_dx, r.ddx);
    put(a.dd_dy, r.ddy);
    a.in_medium = (uint8_t)r.medium;
    a.ignore_tri = r.ignore;
    a.lambda = r.lam;
    a.x = r.x;
    a.y = r.y;
    a.status = (uint8_t)status;
}

// ----------------------------------------------------------------------------
// packed argmin, src/atomic_argmin.jl:5-30
// ----------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t monotonic_u32(float f) {
#ifdef __CUDA_ARCH__
    uint32_t u = __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
#endif
    return u > (1u << 31) ? ~u : (u | (1u << 31));
}
__host__ __device__ __forceinline__ uint64_t pack_argmin(float t, uint32_t idx) {
    return ((uint64_t)monotonic_u32(t) << 32) | (uint64_t)idx;
}
__host__ __device__ __forceinline__ float monotonic_f32(uint32_t i) {
    uint32_t u = (i >> 31) == 0 ? ~i : (i ^ (1u << 31));
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
constexpr uint64_t kNoHit = 0xFF80000000000001ull;  // pack_argmin(Inf, 1)

// ----------------------------------------------------------------------------
// first-bounce tiling of a light grid
// ----------------------------------------------------------------------------
// A grid of h rows is generated column by column (ray j at row j % h, column
// j / h).  grid_tile_ray(p) is the ray a traversal takes as its p-th: the
// positions are grouped by kGridTileCols columns; inside a group the first
// 8 floor(h / 8) rows come as 8 x 4 tiles of 32 consecutive positions, four
// tiles side by side per tile row (so 256 consecutive positions are a
// 16 x 16 patch), and the rows below them after, column by column; columns
// past the last full group keep their order.  A warp of 32 consecutive
// positions then holds a compact patch of the grid instead of a 32 x 1
// strip.  The map is a bijection of 0 .. n - 1; 32-bit arithmetic, for
// n < 2^32 and h <= kGridTileMaxRows (callers check).
constexpr uint32_t kGridTileMaxRows = 1u << 26;
constexpr uint32_t kGridTileCols = 16;  // columns per group: 4 tiles side by side

__host__ __device__ __forceinline__ uint32_t grid_tile_ray(uint32_t p, uint32_t h, uint32_t n) {
    const uint32_t span = kGridTileCols * h, g = p / span;
    if (g >= n / span) return p;
    const uint32_t h8 = h & ~7u, off = p - g * span;
    if (off < kGridTileCols * h8) {
        const uint32_t t = off >> 5, tr = t / (kGridTileCols / 4u), tc = t - tr * (kGridTileCols / 4u);
        return (g * kGridTileCols + tc * 4u + ((off & 31u) >> 3)) * h + tr * 8u + (off & 7u);
    }
    const uint32_t o2 = off - kGridTileCols * h8, rem = h - h8;
    return (g * kGridTileCols + o2 / rem) * h + h8 + o2 % rem;
}

// ----------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11) and the draws of the trace step
// ----------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        uint4 n;
        n.x = (uint32_t)(p1 >> 32) ^ c.y ^ k0;
        n.y = (uint32_t)p1;
        n.z = (uint32_t)(p0 >> 32) ^ c.w ^ k1;
        n.w = (uint32_t)p0;
        c = n;
    }
    return c;
}
__host__ __device__ __forceinline__ float uniform24(uint32_t bits) { return (float)(bits >> 8) * 0x1p-24f; }

// Fresnel draw of ray `id` at bounce `b` (1-based): counter (id, 0, 1, b).
__device__ __forceinline__ float fresnel_draw(uint64_t seed, uint32_t id, uint32_t b) {
    uint4 o = philox(make_uint4(id, 0u, 1u, b), (uint32_t)seed, (uint32_t)(seed >> 32));
    return uniform24(o.x);
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// The rays [0, n) a thread traces.  With a work counter, each warp takes 32
// consecutive rays at a time until the counter passes n (dynamic balance: a
// warp whose rays finish early takes more, and the launch ends when the work
// does); without one, a static grid-stride loop.
template <class F>
__device__ __forceinline__ void for_each_ray(int64_t n, unsigned long long* fetch, F&& body) {
    if (fetch) {
        const int lane = threadIdx.x & 31;
        while (true) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(fetch, 32ull);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= (unsigned long long)n) break;
            const int64_t k = (int64_t)base + lane;
            if (k < n) body(k);
        }
    } else {
        for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
            body(k);
    }
}

// Warp-uniform batches of 32 consecutive rays [base, base + 32) (lanes past
// n idle inside the body): from a work counter, or a static grid-stride over
// warps.  Every lane of the warp runs the body, so it may use warp votes.
template <class F>
__device__ __forceinline__ void for_each_warp_batch(int64_t n, unsigned long long* fetch, F&& body) {
    const int lane = threadIdx.x & 31;
    if (fetch) {
        while (true) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(fetch, 32ull);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= (unsigned long long)n) break;
            body((int64_t)base);
        }
    } else {
        const int64_t stride = (int64_t)gridDim.x * blockDim.x;
        for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride)
            body(base);
    }
}


}  // namespace splat
