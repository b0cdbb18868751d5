// optics.cuh -- evolve_ray, final_evolution and the light-map sample on one
// ray, as device functions.
//
// The primal computation follows the reference expression by expression
// (src/tracer.jl:61-201, src/ray_imagers.jl:4-113, src/geo.jl:170-561),
// including its zero-offset expansions (pos + dp/dlambda * 0 + ...), whose
// NaN / signed-zero behaviour the reference's results depend on.
//
// Derivatives: every ForwardDiff.derivative(f, a) of the reference becomes
// one evaluation of f with the differentiated argument a dual (struct D) and
// everything else plain float.  The operand types therefore mirror the
// reference closures exactly (a normal held at r.lambda stays a float, air()
// of a dual wavelength is a dual with zero partial), which is what makes the
// partials -- and through them the fixed-point light map -- reproducible.
#pragma once

#include "kernels.h"

namespace splat {

// ----------------------------------------------------------------------------
// materials, src/material.jl:1-13
// ----------------------------------------------------------------------------
template <class L>
__device__ __forceinline__ L glass(const splat_material_t& m, L lam) {
    if (m.kind == SPLAT_MATERIAL_CAUCHY) {
        L lu = lam * 1.0e-3f;
        return m.a + m.b / (lu * lu);
    }
    if (m.kind == SPLAT_MATERIAL_SELLMEIER) {
        L lu = lam * 1.0e-3f;
        L l2 = lu * lu;
        L t0 = (m.sb[0] * l2) / (l2 - m.sc[0]);
        L t1 = (m.sb[1] * l2) / (l2 - m.sc[1]);
        L t2 = (m.sb[2] * l2) / (l2 - m.sc[2]);
        L acc = 1.0f + t0;
        acc = acc + t1;
        acc = acc + t2;
        return dsqrt(acc);
    }
    const float l1 = 400.0f, l2 = 700.0f, g1 = 1.3f, g2 = 1.4f;
    const float slope = (g2 - g1) / (l2 - l1);
    return slope * (lam - l1) + g1;
}
__device__ __forceinline__ float air(float) { return 1.0f; }
__device__ __forceinline__ D air(D) { return {1.0f, 0.0f}; }

// ----------------------------------------------------------------------------
// expansions, src/geo.jl:398-410 and src/tracer.jl:109-116
// ----------------------------------------------------------------------------
template <class L, class X, class Y>
__device__ __forceinline__ auto p_expansion(const RayState& r, L lam, X x, Y y) {
    auto dl = lam - r.lam;
    auto dx = x - r.x;
    auto dy = y - r.y;
    auto a0 = r.pos + r.dpl * dl;
    auto a1 = a0 + r.dpx * dx;
    return a1 + r.dpy * dy;
}

template <class L, class X, class Y>
__device__ __forceinline__ auto d_expansion(const RayState& r, L lam, X x, Y y) {
    auto dl = lam - r.lam;
    auto dx = x - r.x;
    auto dy = y - r.y;
    auto a0 = r.dir + r.ddl * dl;
    auto a1 = a0 + r.ddx * dx;
    return a1 + r.ddy * dy;
}

struct HitDerivs {
    float t, dtl, dtx, dty;
};

template <class L, class X, class Y>
__device__ __forceinline__ auto next_p(const RayState& r, const HitDerivs& h, L lam, X x, Y y) {
    auto dl = lam - r.lam;
    auto dx = x - r.x;
    auto dy = y - r.y;
    auto s0 = h.t + h.dtl * dl;
    auto s1 = s0 + h.dtx * dx;
    auto s = s1 + h.dty * dy;
    return p_expansion(r, lam, x, y) + d_expansion(r, lam, x, y) * s;
}

// distance_to_plane(r, T, lambda, x, y), src/geo.jl:441-443
template <class L, class X, class Y>
__device__ __forceinline__ auto distance_to_plane_d(const RayState& r, const Tri& T, L lam, X x, Y y) {
    auto o = p_expansion(r, lam, x, y);
    auto d = d_expansion(r, lam, x, y);
    auto num = dot(T.n, T.a) - dot(T.n, o);
    return num / dot(T.n, d);
}

// src/geo.jl:446-466 (Blackpawn)
__device__ __forceinline__ bool in_triangle(F3 p, F3 a, F3 b, F3 c) {
    F3 v0 = c - a;
    F3 v1 = b - a;
    F3 v2 = p - a;
    float dot00 = dot(v0, v0);
    float dot01 = dot(v0, v1);
    float dot02 = dot(v0, v2);
    float dot11 = dot(v1, v1);
    float dot12 = dot(v1, v2);
    float invDenom = 1.0f / (dot00 * dot11 - dot01 * dot01);
    float u = (dot11 * dot02 - dot01 * dot12) * invDenom;
    float v = (dot00 * dot12 - dot01 * dot02) * invDenom;
    return (u >= 0.0f) && (v >= 0.0f) && (u + v < 1.0f);
}

// get_hit(::Tuple{Int32,Tri}, ::ADRay), src/tracer.jl:61-81.  Returns the
// index (1 on a miss) and t with its three partials (Inf on a miss).
__device__ __forceinline__ int32_t get_hit_ad(const RayState& r, int32_t i, const Tri& T, HitDerivs& h) {
    float t0 = (dot(T.n, T.a) - dot(T.n, r.pos)) / dot(T.n, r.dir);
    F3 p0 = r.pos + r.dir * t0;
    if (in_triangle(p0, T.a, T.b, T.c) && t0 > 0.0f && r.ignore != i) {
        h.t = t0;
        h.dtl = distance_to_plane_d(r, T, D{r.lam, 1.0f}, r.x, r.y).d;
        h.dtx = distance_to_plane_d(r, T, r.lam, D{r.x, 1.0f}, r.y).d;
        h.dty = distance_to_plane_d(r, T, r.lam, r.x, D{r.y, 1.0f}).d;
        return i;
    }
    h.t = h.dtl = h.dtx = h.dty = __int_as_float(0x7f800000);
    return 1;
}

// reverse_uv, src/geo.jl:232-258
template <class P>
__device__ __forceinline__ void reverse_uv(V3<P> pos, const Tri& T, P& u, P& v) {
    F3 v0v1 = T.b - T.a;
    F3 v0v2 = T.c - T.a;
    F3 N = cross(v0v1, v0v2);
    float denom = dot(N, N);
    F3 edge1 = T.c - T.b;
    auto C1 = cross(edge1, pos - T.b);
    P uu = dot(N, C1);
    F3 edge2 = T.a - T.c;
    auto C2 = cross(edge2, pos - T.c);
    P vv = dot(N, C2);
    u = uu / denom;
    v = vv / denom;
}

// optical_normal(::STri, pos), src/geo.jl:202-212
template <class P>
__device__ __forceinline__ V3<P> optical_normal(const Tri& T, V3<P> pos) {
    P u, v;
    reverse_uv(pos, T, u, v);
    P w = (1.0f - u) - v;
    auto n = (T.na * u + T.nb * v) + T.nc * w;
    return normalize(n);
}

template <class L, class X, class Y>
__device__ __forceinline__ auto N_at(const RayState& r, const HitDerivs& h, const Tri& T, L lam, X x, Y y) {
    return optical_normal(T, next_p(r, h, lam, x, y));
}

// refract, src/geo.jl:548-561 (the sign convention of c1 as written)
template <class A, class B, class C1, class C2>
__device__ __forceinline__ auto refract(V3<A> v, V3<B> normal, C1 n1, C2 n2) {
    V3<B> n = normalize(normal);
    if (val(dot(v, n)) > 0.0f) n = n * -1.0f;
    auto c1 = dot(normalize(v), n);
    auto s1 = dsqrt(1.0f - c1 * c1);
    auto s2 = (n1 / n2) * s1;
    auto c2 = dsqrt(1.0f - s2 * s2);
    auto k = (n1 / n2) * c1 - c2;
    return normalize(v * (n1 / n2) + n * k);
}

// reflect, src/geo.jl:481-486
template <class A, class B>
__device__ __forceinline__ auto reflect(V3<A> v, V3<B> normal) {
    V3<B> n = normalize(normal);
    auto dd = dot(n, v);
    auto ax = (n.x * dd) * 2.0f;
    auto ay = (n.y * dd) * 2.0f;
    auto az = (n.z * dd) * 2.0f;
    return V3<decltype(v.x - ax)>{v.x - ax, v.y - ay, v.z - az};
}

// can_refract, src/geo.jl:528-542 (1 - 1f-9 rounds to 1f0)
__device__ __forceinline__ bool can_refract(F3 v, F3 normal, float n1, float n2) {
    F3 n = normalize(normal);
    if (dot(n, v) > 0.0f) n = n * -1.0f;
    float c1 = dot(normalize(v), n);
    const float one_m_eps = 1.0f - 1.0e-9f;
    if (c1 * c1 > one_m_eps) return false;
    float s1 = sqrtf(1.0f - c1 * c1);
    float s2 = (n1 / n2) * s1;
    return fabsf(s2) < one_m_eps;
}

// reflectance, src/geo.jl:488-502
__device__ __forceinline__ float reflectance(F3 v, F3 normal, float n1, float n2) {
    F3 n = normalize(normal);
    if (dot(n, v) < 0.0f) n = n * -1.0f;
    float c1 = dot(normalize(v), n);
    float s1 = sqrtf(1.0f - c1 * c1);
    float r = n1 / n2;
    float s2 = sqrtf(1.0f - (r * r) * (s1 * s1));
    float hh = (n1 + n2) / 2.0f;
    float q = (hh * c1 - hh * s2) / (n1 * c1 + n2 * s2);
    return q * q;
}

// handle_optics, src/tracer.jl:118-179.  Writes the evolved ray into `o`.
__device__ __forceinline__ void handle_optics(const RayState& r, const HitDerivs& h, int32_t i, const Tri& T,
                                              const splat_material_t& mat, float rndm, bool quirks,
                                              RayState& o) {
    const float Lc = r.lam, Xc = r.x, Yc = r.y;
    const D Ld{r.lam, 1.0f}, Xd{r.x, 1.0f}, Yd{r.y, 1.0f};
    // the reference differentiates the direction in y at y = r.x
    const D Yq = quirks ? D{r.x, 1.0f} : Yd;

    F3 N0 = N_at(r, h, T, Lc, Xc, Yc);
    const bool in_med = r.medium != 0;
    float n1c = in_med ? glass(mat, Lc) : air(Lc);
    float n2c = in_med ? air(Lc) : glass(mat, Lc);
    bool refracts = can_refract(r.dir, N0, n1c, n2c) && rndm > reflectance(r.dir, N0, n1c, n2c);

    o.pos = next_p(r, h, Lc, Xc, Yc);
    o.dpl = vpar(next_p(r, h, Ld, Xc, Yc));
    o.dpx = vpar(next_p(r, h, Lc, Xd, Yc));
    o.dpy = vpar(next_p(r, h, Lc, Xc, Yd));

    // Each direction partial is the refraction or the reflection of the same
    // dual direction about the same dual normal: both are evaluated once,
    // before the lanes of a warp part on `refracts`, so a warp whose rays
    // take both ways runs only the short refract / reflect tails twice.
    o.dir = refracts ? refract(r.dir, N0, n1c, n2c) : reflect(r.dir, N0);
    {
        const auto dv = d_expansion(r, Ld, Xc, Yc);
        if (refracts && quirks) {
            const D n1d = in_med ? glass(mat, Ld) : air(Ld);
            const D n2d = in_med ? air(Ld) : glass(mat, Ld);
            o.ddl = vpar(refract(dv, N0, n1d, n2d));
        } else {
            const auto nv = N_at(r, h, T, Ld, Xc, Yc);
            if (refracts) {
                const D n1d = in_med ? glass(mat, Ld) : air(Ld);
                const D n2d = in_med ? air(Ld) : glass(mat, Ld);
                o.ddl = vpar(refract(dv, nv, n1d, n2d));
            } else {
                o.ddl = vpar(reflect(dv, nv));
            }
        }
    }
    {
        const auto dv = d_expansion(r, Lc, Xd, Yc);
        const auto nv = N_at(r, h, T, Lc, Xd, Yc);
        o.ddx = refracts ? vpar(refract(dv, nv, n1c, n2c)) : vpar(reflect(dv, nv));
    }
    {
        const auto dv = d_expansion(r, Lc, Xc, Yq);
        const auto nv = N_at(r, h, T, Lc, Xc, Yq);
        o.ddy = refracts ? vpar(refract(dv, nv, n1c, n2c)) : vpar(reflect(dv, nv));
    }
    o.medium = refracts ? (in_med ? 0 : 1) : r.medium;
    o.lam = r.lam;
    o.x = r.x;
    o.y = r.y;
    o.ignore = i;
}

// Per-ray parameters of one evolve (one scene, one bounce).
struct EvolveView {
    const splat_ftri_t* tris;
    int64_t n_tris;
    int32_t* err;
    int64_t first_diffuse;
    splat_material_t material;
    uint64_t seed;
    uint32_t bounce;
    float force_rand;
    bool quirks;
    bool last;  // trace mode: the last bounce, survivors are dropped
};

constexpr int kFateDrop = 0;      // trace mode: a survivor of the last bounce
constexpr int kFateKeep = 1;      // evolved, active in the next bounce (o)
constexpr int kFateDiffuse = 2;   // hit a diffuse triangle (trace mode: o is final-evolved)
constexpr int kFateInfinity = 3;  // missed everything; the ray is unchanged

__device__ __forceinline__ void final_evolution(const RayState& r, const HitDerivs& h, int32_t i, RayState& o);

// evolve_ray (src/tracer.jl:181-201) of one active ray whose hit index is
// i; rng_id keys its Fresnel draw.  Hit indices outside 1..n_tris are
// reported in the error word and treated as misses.
template <bool TRACE>
__device__ __forceinline__ int evolve_one(const RayState& r, int32_t i, uint32_t rng_id, const EvolveView& v,
                                          RayState& o, int32_t& ih) {
    if (i < 1 || i > v.n_tris) {
        atomicOr(v.err, 16);
        i = 1;
    }
    const Tri T = load_tri(v.tris, i);
    HitDerivs h;
    ih = get_hit_ad(r, i, T, h);
    if (ih >= v.first_diffuse) {
        if (TRACE) final_evolution(r, h, ih, o);
        return kFateDiffuse;
    }
    if (isinf(h.t)) return kFateInfinity;
    if (TRACE && v.last) return kFateDrop;
    const float u = v.force_rand >= 0.0f ? v.force_rand : fresnel_draw(v.seed, rng_id, v.bounce);
    handle_optics(r, h, ih, T, v.material, u, v.quirks, o);
    return kFateKeep;
}

// final_evolution(r, i, t, ...), src/ray_imagers.jl:4-22: position moved onto
// the hit with its partials; direction and its partials kept.
__device__ __forceinline__ void final_evolution(const RayState& r, const HitDerivs& h, int32_t i, RayState& o) {
    const float Lc = r.lam, Xc = r.x, Yc = r.y;
    o = r;
    o.pos = next_p(r, h, Lc, Xc, Yc);
    o.dpl = vpar(next_p(r, h, D{r.lam, 1.0f}, Xc, Yc));
    o.dpx = vpar(next_p(r, h, Lc, D{r.x, 1.0f}, Yc));
    o.dpy = vpar(next_p(r, h, Lc, Xc, D{r.y, 1.0f}));
    o.ignore = i;
}

// Triangle-only terms of reverse_uv (src/geo.jl:236-252), hoisted out of a
// ray's samples: identical values, computed once.
struct TriUV {
    F3 N, e1, e2;  // cross(b - a, c - a), c - b, a - c
    float denom;   // dot(N, N)
};
__device__ __forceinline__ TriUV tri_uv(const Tri& T) {
    TriUV q;
    q.N = cross(T.b - T.a, T.c - T.a);
    q.denom = dot(q.N, q.N);
    q.e1 = T.c - T.b;
    q.e2 = T.a - T.c;
    return q;
}

// splat_sample with the hoisted triangle terms.
__device__ __forceinline__ bool splat_sample_uv(const RayState& r, const Tri& T, const TriUV& q, float lam, float xs,
                                                float ys, int64_t W, int64_t H, int64_t& off_ij, float& intensity) {
    F3 pos = p_expansion(r, lam, xs, ys);
    F3 dir = d_expansion(r, lam, xs, ys);
    const float bu = dot(q.N, cross(q.e1, pos - T.b)) / q.denom;
    const float bv = dot(q.N, cross(q.e2, pos - T.c)) / q.denom;
    float bw = (1.0f - bu) - bv;
    float U = (T.ta.x * bu + T.tb.x * bv) + T.tc.x * bw;
    float Vt = (T.ta.y * bu + T.tb.y * bv) + T.tc.y * bw;
    if (isnan(U) || isnan(Vt) || isinf(U) || isinf(Vt)) return false;
    float ci = ceilf(U * (float)W), cj = ceilf(Vt * (float)H);
    ci = fminf(fmaxf(ci, 1.0f), (float)W);
    cj = fminf(fmaxf(cj, 1.0f), (float)H);
    off_ij = ((int64_t)ci - 1) + ((int64_t)cj - 1) * W;
    F3 n = (T.na * bu + T.nb * bv) + T.nc * bw;
    intensity = fabsf(dot(normalize(n), normalize(dir)));
    return true;
}

// One sample of atomic_spectrum_kernel2 (src/ray_imagers.jl:78-113):
// expand -> tex_uv -> texel -> cosine_shading.  False when uv is not finite.
__device__ __forceinline__ bool splat_sample(const RayState& r, const Tri& T, float lam, float xs, float ys,
                                             int64_t W, int64_t H, int64_t& off_ij, float& intensity) {
    F3 pos = p_expansion(r, lam, xs, ys);
    F3 dir = d_expansion(r, lam, xs, ys);
    float bu, bv;
    reverse_uv(pos, T, bu, bv);
    float bw = (1.0f - bu) - bv;
    float U = (T.ta.x * bu + T.tb.x * bv) + T.tc.x * bw;
    float Vt = (T.ta.y * bu + T.tb.y * bv) + T.tc.y * bw;
    if (isnan(U) || isnan(Vt) || isinf(U) || isinf(Vt)) return false;
    float ci = ceilf(U * (float)W), cj = ceilf(Vt * (float)H);
    ci = fminf(fmaxf(ci, 1.0f), (float)W);
    cj = fminf(fmaxf(cj, 1.0f), (float)H);
    off_ij = ((int64_t)ci - 1) + ((int64_t)cj - 1) * W;
    F3 n = (T.na * bu + T.nb * bv) + T.nc * bw;
    intensity = fabsf(dot(normalize(n), normalize(dir)));
    return true;
}

// ---------------------------------------------------------------------------
// ray generation, src/ray_generators.jl:64-97
// ---------------------------------------------------------------------------
__device__ __forceinline__ float gen_lambda(const splat_lambda_mode_t& lm, uint32_t k, float u) {
    if (lm.mode == SPLAT_LAMBDA_UNIFORM) return lm.lambda0 + (lm.lambda1 - lm.lambda0) * u;
    if (lm.mode == SPLAT_LAMBDA_STRATIFIED) {
        const float width = (lm.lambda1 - lm.lambda0) / (float)lm.n_strata;
        return lm.lambda0 + ((float)(k % (uint32_t)lm.n_strata) + u) * width;
    }
    return lm.lambda0;
}

__device__ __forceinline__ RayState gen_ray(const GenParams& g, int64_t kid) {
    const int64_t h = g.light.res1 / g.upscale, w = g.light.res2 / g.upscale;
    const int64_t row = kid % h + 1, col = kid / h + 1;
    const uint4 rnd = philox(make_uint4((uint32_t)kid, g.light_index, 0u, 0u), (uint32_t)g.seed,
                             (uint32_t)(g.seed >> 32));
    const float ddx = uniform24(rnd.x), ddy = uniform24(rnd.y);
    const float xf = (float)row + ddx, yf = (float)col + ddy;
    const float h2 = (float)(h / 2), w2 = (float)(w / 2);
    const F3 C = f3(g.light.center), d1 = f3(g.light.dim1), d2 = f3(g.light.dim2);
    const float sx = xf - h2, sy = yf - w2;
    const F3 A = {(d1.x * sx) / h2, (d1.y * sx) / h2, (d1.z * sx) / h2};
    const F3 B = {(d2.x * sy) / w2, (d2.y * sy) / w2, (d2.z * sy) / w2};
    RayState r;
    r.pos = (C + A) + B;
    r.dpl = {0.f, 0.f, 0.f};
    r.dpx = {d1.x / h2, d1.y / h2, d1.z / h2};
    r.dpy = {d2.x / w2, d2.y / w2, d2.z / w2};
    r.dir = f3(g.light.dir);
    r.ddl = {0.f, 0.f, 0.f};
    r.ddx = {0.f, 0.f, 0.f};
    r.ddy = {0.f, 0.f, 0.f};
    r.lam = gen_lambda(g.lm, (uint32_t)kid, uniform24(rnd.z));
    r.x = xf;
    r.y = yf;
    r.ignore = 1;
    r.medium = 0;
    return r;
}


// ---------------------------------------------------------------------------
// light-map splat of one (ray, plane)
// ---------------------------------------------------------------------------
// The scalars of a SplatParams held in registers, its arrays read in place
// (the batch engine's per-item parameters live in global memory).
struct SplatView {
    void* map;
    int32_t accum;
    float scale;
    int64_t w, h;
    int32_t n_lambda, n_delta;
    const float* spectrum;
    const float* deltas;
};
__device__ __forceinline__ SplatView splat_view(const SplatParams& sp) {
    return SplatView{sp.map, sp.accum, sp.scale, sp.w, sp.h, sp.n_lambda, sp.n_delta, sp.spectrum, sp.deltas};
}

template <class P>
__device__ __forceinline__ void flush_texel(const P& sp, int32_t off, int32_t vi, float vf) {
    if (off < 0) return;
    if (sp.accum == SPLAT_ACCUM_I32)
        atomicAdd(reinterpret_cast<int*>(sp.map) + off, vi);
    else
        atomicAdd(reinterpret_cast<float*>(sp.map) + off, vf);
}

// Sends a texel's partial sum straight to the map.
template <class P>
struct DirectSink {
    const P& sp;
    __device__ __forceinline__ void operator()(int32_t off, int32_t vi, float vf) const { flush_texel(sp, off, vi, vf); }
};

// Block-level texel aggregation.  Samples of the rays a block holds are
// summed per texel in a shared open-addressing table (texel offset -> partial
// sum) and the table is flushed with one map atomic per distinct texel.  Rays
// that are neighbours in the queue land on neighbouring texels, so this folds
// many map atomics (and the L2 serialisation on hot caustic texels) into
// shared-memory ones.  int32 sums wrap exactly like the map's own atomics, so
// fixed-point maps are bit-identical to direct accumulation; float maps
// differ by summation order only.  A sample that finds no slot within
// kAggProbes goes straight to the map.
constexpr int kAggLog2 = 11;
constexpr int kAggSlots = 1 << kAggLog2;
constexpr int kAggProbes = 16;

struct TableSink {
    const SplatParams& sp;
    int32_t* keys;  // shared, -1 = empty
    int32_t* vals;  // shared, int32 sum or float bits
    __device__ __forceinline__ void operator()(int32_t off, int32_t vi, float vf) const {
        if (off < 0) return;
        uint32_t h = ((uint32_t)off * 2654435761u) >> (32 - kAggLog2);
        for (int p = 0; p < kAggProbes; ++p) {
            const int32_t k = atomicCAS(&keys[h], -1, off);
            if (k == -1 || k == off) {
                if (sp.accum == SPLAT_ACCUM_I32) atomicAdd(&vals[h], vi);
                else atomicAdd(reinterpret_cast<float*>(&vals[h]), vf);
                return;
            }
            h = (h + 1) & (kAggSlots - 1);
        }
        flush_texel(sp, off, vi, vf);
    }
};

// The table of a block whose rays splat into different maps (the batch
// engine): keyed by the texel's address, its low bit set for float maps.
struct AddrTableSink {
    const SplatParams& sp;
    unsigned long long* keys;  // shared, 0 = empty
    int32_t* vals;
    __device__ __forceinline__ void operator()(int32_t off, int32_t vi, float vf) const {
        if (off < 0) return;
        const bool f32 = sp.accum != SPLAT_ACCUM_I32;
        const unsigned long long key =
            (unsigned long long)(reinterpret_cast<uintptr_t>(sp.map) + 4ull * (uint32_t)off) | (f32 ? 1ull : 0ull);
        uint32_t h = (uint32_t)(((key >> 2) * 0x9E3779B97F4A7C15ull) >> (64 - kAggLog2));
        for (int p = 0; p < kAggProbes; ++p) {
            const unsigned long long k = atomicCAS(&keys[h], 0ull, key);
            if (k == 0ull || k == key) {
                if (!f32) atomicAdd(&vals[h], vi);
                else atomicAdd(reinterpret_cast<float*>(&vals[h]), vf);
                return;
            }
            h = (h + 1) & (kAggSlots - 1);
        }
        flush_texel(sp, off, vi, vf);
    }
};

__device__ __forceinline__ void addr_table_clear(unsigned long long* keys, int32_t* vals) {
    for (int i = threadIdx.x; i < kAggSlots; i += blockDim.x) {
        keys[i] = 0ull;
        vals[i] = 0;
    }
}

__device__ __forceinline__ void addr_table_flush(unsigned long long* keys, int32_t* vals) {
    for (int i = threadIdx.x; i < kAggSlots; i += blockDim.x) {
        const unsigned long long k = keys[i];
        if (k != 0ull) {
            const int32_t v = vals[i];
            if (k & 1ull) atomicAdd(reinterpret_cast<float*>(k & ~3ull), __int_as_float(v));
            else atomicAdd(reinterpret_cast<int*>(k), v);
            keys[i] = 0ull;
            vals[i] = 0;
        }
    }
}

__device__ __forceinline__ void table_clear(int32_t* keys, int32_t* vals) {
    for (int i = threadIdx.x; i < kAggSlots; i += blockDim.x) {
        keys[i] = -1;
        vals[i] = 0;
    }
}

// Every thread of the block calls this between two __syncthreads().
__device__ __forceinline__ void table_flush(const SplatParams& sp, int32_t* keys, int32_t* vals) {
    for (int i = threadIdx.x; i < kAggSlots; i += blockDim.x) {
        const int32_t k = keys[i];
        if (k >= 0) {
            const int32_t v = vals[i];
            flush_texel(sp, k, v, __int_as_float(v));
            keys[i] = -1;
            vals[i] = 0;
        }
    }
}

// The N x N sub-samples of one (ray, plane), x offset fastest; returns the
// number of samples accumulated.  Consecutive samples on one texel are summed
// in registers before they reach the sink.  ND > 0: N known at compile time
// (the sample loops unroll and the samples' arithmetic interleaves); 0: N =
// sp.n_delta.
template <int ND, class P, class Sink>
__device__ __forceinline__ int splat_ray_plane_n(const P& sp, const RayState& r, const Tri& T, const TriUV& quv,
                                                 int il, const Sink& sink) {
    const int nd = ND > 0 ? ND : sp.n_delta;
    const int32_t W = (int32_t)sp.w, H = (int32_t)sp.h;
    const float Wf = (float)W, Hf = (float)H;
    int done = 0;
    const float lam = sp.n_lambda > 0 ? sp.spectrum[il] : r.lam;
    const float dl = lam - r.lam;
    const F3 pe = r.pos + r.dpl * dl;
    const F3 de = r.dir + r.ddl * dl;
    const int32_t plane_off = il * W * H;
    int32_t run_off = -1, run_i = 0;
    float run_f = 0.f;
#pragma unroll
    for (int iy = 0; iy < nd; ++iy) {
        const float dy = (r.y + sp.deltas[iy]) - r.y;
#pragma unroll
        for (int ix = 0; ix < nd; ++ix) {
            const float dx = (r.x + sp.deltas[ix]) - r.x;
            const F3 pos = (pe + r.dpx * dx) + r.dpy * dy;
            const F3 dir = (de + r.ddx * dx) + r.ddy * dy;
            const float bu = dot(quv.N, cross(quv.e1, pos - T.b)) / quv.denom;
            const float bv = dot(quv.N, cross(quv.e2, pos - T.c)) / quv.denom;
            const float bw = (1.0f - bu) - bv;
            const float U = (T.ta.x * bu + T.tb.x * bv) + T.tc.x * bw;
            const float V = (T.ta.y * bu + T.tb.y * bv) + T.tc.y * bw;
            if (isnan(U) || isnan(V) || isinf(U) || isinf(V)) continue;
            const float ci = fminf(fmaxf(ceilf(U * Wf), 1.0f), Wf);
            const float cj = fminf(fmaxf(ceilf(V * Hf), 1.0f), Hf);
            const int32_t off = plane_off + ((int32_t)ci - 1) + ((int32_t)cj - 1) * W;
            const F3 nn = (T.na * bu + T.nb * bv) + T.nc * bw;
            const float inten = fabsf(dot(normalize(nn), normalize(dir)));
            ++done;
            const int32_t vi = __float2int_rn(inten * sp.scale);
            if (off == run_off) {
                run_i += vi;
                run_f += inten;
            } else {
                sink(run_off, run_i, run_f);
                run_off = off;
                run_i = vi;
                run_f = inten;
            }
        }
    }
    sink(run_off, run_i, run_f);
    return done;
}

template <class P, class Sink>
__device__ __forceinline__ int splat_ray_plane(const P& sp, const RayState& r, const Tri& T, const TriUV& quv, int il,
                                               const Sink& sink) {
    if (sp.n_delta == 2) return splat_ray_plane_n<2>(sp, r, T, quv, il, sink);
    if (sp.n_delta == 1) return splat_ray_plane_n<1>(sp, r, T, quv, il, sink);
    return splat_ray_plane_n<0>(sp, r, T, quv, il, sink);
}

template <class P>
__device__ __forceinline__ int splat_ray_plane(const P& sp, const RayState& r, const Tri& T, const TriUV& quv, int il) {
    return splat_ray_plane(sp, r, T, quv, il, DirectSink<P>{sp});
}

}  // namespace splat
