/*
 * oracle.c -- CPU restatement of SPLAT's forward trace step.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Built with -O2 -ffp-contract=off
 * and no fast-math so every binary32 operation is rounded once, in the order
 * the reference writes it.  Reductions written in the reference as a + b + c
 * are left folds ((a + b) + c), as Julia's n-ary + is.  dot(a, b) is
 * (a1 b1 + a2 b2) + a3 b3 and cross is StaticArrays' component formula.
 * norm(v) = sqrt((x x + y y) + z z); normalize(v) = v * (1 / norm(v)) (the
 * multiply-by-inverse of LinearAlgebra.__normalize!).
 *
 * Dual numbers (ForwardDiff restated).  A dual is either a constant (the
 * closure does not depend on the differentiated argument) or a value with one
 * partial.  Rules, with p the partial:
 *   a +- b        p = pa +- pb      (constant operands contribute nothing)
 *   a * b         p = vb pa + va pb (constant * dual: va pb)
 *   a / b         dual/const: pa / vb; const/dual: -((va/vb)/vb) pb;
 *                 dual/dual:  (1/vb) pa + (-(va/(vb vb))) pb
 *   sqrt(a)       p = (1 / (2 sqrt(va))) pa
 * These are ForwardDiff's Dual rules (dual.jl, partials.jl _div_partials /
 * _mul_partials) as the reference's hot path uses them.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

int o_version(void) { return 1; }

/* ------------------------------------------------------------------------ */
/* Philox4x32-10, Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as  */
/* easy as 1, 2, 3", SC'11.  Round: (hi, lo) = M * x (32x32 -> 64),         */
/* keys bumped by the Weyl constants between rounds.                        */
/* ------------------------------------------------------------------------ */
void o_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* 24 high bits -> [0, 1), exact in binary32. */
float o_uniform(uint32_t bits) { return (float)(bits >> 8) * 0x1p-24f; }

static void draw4(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t out[4]) {
    uint32_t ctr[4] = {c0, c1, c2, c3};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    o_philox4x32_10(ctr, key, out);
}

float o_fresnel_draw(uint64_t seed, uint32_t ray_id, uint32_t bounce) {
    uint32_t o[4];
    draw4(seed, ray_id, 0u, 1u, bounce, o);
    return o_uniform(o[0]);
}

/* ------------------------------------------------------------------------ */
/* Packed argmin, src/atomic_argmin.jl:5-30                                  */
/* ------------------------------------------------------------------------ */
uint32_t o_monotonic_u32(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u > (1u << 31) ? ~u : (u | (1u << 31));
}

float o_monotonic_f32(uint32_t i) {
    uint32_t flipped = (i >> 31) << 31;
    uint32_t u = flipped == 0 ? ~i : (i ^ (1u << 31));
    float f;
    memcpy(&f, &u, 4);
    return f;
}

uint64_t o_pack_argmin(float t, uint32_t idx) { return ((uint64_t)o_monotonic_u32(t) << 32) | (uint64_t)idx; }

uint32_t o_retrieve_arg(uint64_t k) { return (uint32_t)(k ^ ((k >> 32) << 32)); }

/* ------------------------------------------------------------------------ */
/* Plain binary32 vector helpers (StaticArrays semantics)                    */
/* ------------------------------------------------------------------------ */
typedef struct { float x, y, z; } v3;

static inline v3 V(const float a[3]) { v3 r = {a[0], a[1], a[2]}; return r; }
static inline v3 vadd(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 vmul(v3 a, float s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static inline float vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static inline float vnorm(v3 a) { return sqrtf((a.x * a.x + a.y * a.y) + a.z * a.z); }
static inline v3 vnormalize(v3 a) { return vmul(a, 1.0f / vnorm(a)); }
static inline void vstore(float o[3], v3 a) { o[0] = a.x; o[1] = a.y; o[2] = a.z; }

/* ------------------------------------------------------------------------ */
/* Dual numbers (one partial), ForwardDiff restated                         */
/* ------------------------------------------------------------------------ */
typedef struct { float v, d; int c; } dual;
typedef struct { dual x, y, z; } dv3;

static inline dual DC(float v) { dual r = {v, 0.0f, 1}; return r; }
static inline dual DV(float v, float d) { dual r = {v, d, 0}; return r; }

static inline dual d_add(dual a, dual b) {
    float v = a.v + b.v;
    if (a.c && b.c) return DC(v);
    if (a.c) return DV(v, b.d);
    if (b.c) return DV(v, a.d);
    return DV(v, a.d + b.d);
}
static inline dual d_sub(dual a, dual b) {
    float v = a.v - b.v;
    if (a.c && b.c) return DC(v);
    if (a.c) return DV(v, -b.d);
    if (b.c) return DV(v, a.d);
    return DV(v, a.d - b.d);
}
static inline dual d_mul(dual a, dual b) {
    float v = a.v * b.v;
    if (a.c && b.c) return DC(v);
    if (a.c) return DV(v, a.v * b.d);
    if (b.c) return DV(v, a.d * b.v);
    return DV(v, b.v * a.d + a.v * b.d);
}
static inline dual d_div(dual a, dual b) {
    float v = a.v / b.v;
    if (a.c && b.c) return DC(v);
    if (b.c) return DV(v, a.d / b.v);
    if (a.c) return DV(v, -(v / b.v) * b.d);
    return DV(v, (1.0f / b.v) * a.d + (-(a.v / (b.v * b.v))) * b.d);
}
static inline dual d_sqrt(dual a) {
    float s = sqrtf(a.v);
    if (a.c) return DC(s);
    return DV(s, (1.0f / (2.0f * s)) * a.d);
}

static inline dv3 dvc(const float a[3]) { dv3 r = {DC(a[0]), DC(a[1]), DC(a[2])}; return r; }
static inline dv3 dvcv(v3 a) { dv3 r = {DC(a.x), DC(a.y), DC(a.z)}; return r; }
static inline v3 dval(dv3 a) { v3 r = {a.x.v, a.y.v, a.z.v}; return r; }
static inline v3 dpar(dv3 a) { v3 r = {a.x.d, a.y.d, a.z.d}; return r; }
static inline dv3 dv_add(dv3 a, dv3 b) { dv3 r = {d_add(a.x, b.x), d_add(a.y, b.y), d_add(a.z, b.z)}; return r; }
static inline dv3 dv_sub(dv3 a, dv3 b) { dv3 r = {d_sub(a.x, b.x), d_sub(a.y, b.y), d_sub(a.z, b.z)}; return r; }
static inline dv3 dv_scale(dv3 a, dual s) { dv3 r = {d_mul(a.x, s), d_mul(a.y, s), d_mul(a.z, s)}; return r; }
static inline dual dv_dot(dv3 a, dv3 b) { return d_add(d_add(d_mul(a.x, b.x), d_mul(a.y, b.y)), d_mul(a.z, b.z)); }
static inline dv3 dv_cross(dv3 a, dv3 b) {
    dv3 r = {d_sub(d_mul(a.y, b.z), d_mul(a.z, b.y)), d_sub(d_mul(a.z, b.x), d_mul(a.x, b.z)),
             d_sub(d_mul(a.x, b.y), d_mul(a.y, b.x))};
    return r;
}
static inline dual dv_norm(dv3 a) {
    return d_sqrt(d_add(d_add(d_mul(a.x, a.x), d_mul(a.y, a.y)), d_mul(a.z, a.z)));
}
static inline dv3 dv_normalize(dv3 a) {
    dual inv = d_div(DC(1.0f), dv_norm(a));
    dv3 r = {d_mul(a.x, inv), d_mul(a.y, inv), d_mul(a.z, inv)};
    return r;
}

/* ------------------------------------------------------------------------ */
/* Geometry and optics, src/geo.jl                                          */
/* ------------------------------------------------------------------------ */

/* src/geo.jl:433-435 (the @fastmath there changes no operation order). */
float o_distance_to_plane(const float o[3], const float d[3], const float pp[3], const float n[3]) {
    v3 N = V(n);
    return (vdot(N, V(pp)) - vdot(N, V(o))) / vdot(N, V(d));
}

/* src/geo.jl:446-466, Blackpawn barycentric test. */
static int in_triangle_v(v3 p, v3 a, v3 b, v3 c) {
    v3 v0 = vsub(c, a);
    v3 v1 = vsub(b, a);
    v3 v2 = vsub(p, a);
    float dot00 = vdot(v0, v0);
    float dot01 = vdot(v0, v1);
    float dot02 = vdot(v0, v2);
    float dot11 = vdot(v1, v1);
    float dot12 = vdot(v1, v2);
    float invDenom = 1.0f / (dot00 * dot11 - dot01 * dot01);
    float u = (dot11 * dot02 - dot01 * dot12) * invDenom;
    float v = (dot00 * dot12 - dot01 * dot02) * invDenom;
    return (u >= 0.0f) && (v >= 0.0f) && (u + v < 1.0f);
}

int o_in_triangle(const float p[3], const float a[3], const float b[3], const float c[3]) {
    return in_triangle_v(V(p), V(a), V(b), V(c));
}

/* src/geo.jl:481-486 */
static v3 reflect_v(v3 v, v3 normal) {
    v3 n = vnormalize(normal);
    float dd = vdot(n, v);
    v3 r = {v.x - (n.x * dd) * 2.0f, v.y - (n.y * dd) * 2.0f, v.z - (n.z * dd) * 2.0f};
    return r;
}
void o_reflect(const float v[3], const float n[3], float out[3]) { vstore(out, reflect_v(V(v), V(n))); }

/* src/geo.jl:548-561 (sign convention of c1 kept as written). */
static v3 refract_v(v3 v, v3 normal, float n1, float n2) {
    v3 n = vnormalize(normal);
    if (vdot(v, n) > 0.0f) n = vmul(n, -1.0f);
    float c1 = vdot(vnormalize(v), n);
    float s1 = sqrtf(1.0f - c1 * c1);
    float s2 = (n1 / n2) * s1;
    float c2 = sqrtf(1.0f - s2 * s2);
    return vnormalize(vadd(vmul(v, n1 / n2), vmul(n, (n1 / n2) * c1 - c2)));
}
void o_refract(const float v[3], const float n[3], float n1, float n2, float out[3]) {
    vstore(out, refract_v(V(v), V(n), n1, n2));
}

/* src/geo.jl:528-542.  eps = 1f-9 makes 1 - eps == 1f0 in binary32. */
static int can_refract_v(v3 v, v3 normal, float n1, float n2) {
    v3 n = vnormalize(normal);
    if (vdot(n, v) > 0.0f) n = vmul(n, -1.0f);
    float c1 = vdot(vnormalize(v), n);
    const float one_m_eps = 1.0f - 1.0e-9f;
    if (c1 * c1 > one_m_eps) return 0;
    float s1 = sqrtf(1.0f - c1 * c1);
    float s2 = (n1 / n2) * s1;
    return fabsf(s2) < one_m_eps;
}
int o_can_refract(const float v[3], const float n[3], float n1, float n2) {
    return can_refract_v(V(v), V(n), n1, n2);
}

/* src/geo.jl:488-502, average of s and p polarisations. */
static float reflectance_v(v3 v, v3 normal, float n1, float n2) {
    v3 n = vnormalize(normal);
    if (vdot(n, v) < 0.0f) n = vmul(n, -1.0f);
    float c1 = vdot(vnormalize(v), n);
    float s1 = sqrtf(1.0f - c1 * c1);
    float r = n1 / n2;
    float s2 = sqrtf(1.0f - (r * r) * (s1 * s1));
    float h = (n1 + n2) / 2.0f;
    float q = (h * c1 - h * s2) / (n1 * c1 + n2 * s2);
    return q * q;
}
float o_reflectance(const float v[3], const float n[3], float n1, float n2) {
    return reflectance_v(V(v), V(n), n1, n2);
}

/* src/alg_types.jl:108: (1:N) ./ N .- 0.5 .- 1 / (2N), binary32. */
void o_upres(int n, float* out) {
    for (int k = 1; k <= n; ++k) out[k - 1] = ((float)k / (float)n - 0.5f) - (1.0f / (2.0f * (float)n));
}

/* Glass index.  kind 0: src/material.jl:1-9 (m (lambda - 400) + 1.3 with
 * m = (1.4 - 1.3) / (700 - 400) in binary32).  kind 1: Cauchy
 * a + b / (lu lu), lu = lambda * 1e-3.  kind 2: Sellmeier
 * sqrt(((1 + b1 l2/(l2 - c1)) + b2 l2/(l2 - c2)) + b3 l2/(l2 - c3)). */
static dual glass_d(const o_material* m, dual lam) {
    if (m->kind == 1) {
        dual lu = d_mul(lam, DC(1.0e-3f));
        return d_add(DC(m->a), d_div(DC(m->b), d_mul(lu, lu)));
    }
    if (m->kind == 2) {
        dual lu = d_mul(lam, DC(1.0e-3f));
        dual l2 = d_mul(lu, lu);
        dual acc = DC(1.0f);
        for (int i = 0; i < 3; ++i) acc = d_add(acc, d_div(d_mul(DC(m->sb[i]), l2), d_sub(l2, DC(m->sc[i]))));
        return d_sqrt(acc);
    }
    const float l1 = 400.0f, l2 = 700.0f, g1 = 1.3f, g2 = 1.4f;
    float slope = (g2 - g1) / (l2 - l1);
    return d_add(d_mul(DC(slope), d_sub(lam, DC(l1))), DC(g1));
}
float o_glass(const o_material* m, float lambda) { return glass_d(m, DC(lambda)).v; }

/* air(lambda) = one(T): a dual with zero partial when lambda is a dual. */
static dual air_d(dual lam) { return lam.c ? DC(1.0f) : DV(1.0f, 0.0f); }

/* ------------------------------------------------------------------------ */
/* Ray generation, src/ray_generators.jl:64-97                               */
/* ------------------------------------------------------------------------ */
static float gen_lambda(const o_lambda_mode* lm, uint32_t k, float u) {
    if (lm == NULL) return 550.0f;
    if (lm->mode == 1) return lm->lambda0 + (lm->lambda1 - lm->lambda0) * u;
    if (lm->mode == 2) {
        float width = (lm->lambda1 - lm->lambda0) / (float)lm->n_strata;
        return lm->lambda0 + ((float)(k % (uint32_t)lm->n_strata) + u) * width;
    }
    return lm->lambda0;
}

static void gen_ray(const o_rect_light* L, int64_t upscale, const o_lambda_mode* lm, uint64_t seed,
                    uint32_t light_index, int64_t k, o_adray* r) {
    int64_t h = L->res1 / upscale, w = L->res2 / upscale;
    int64_t row = k % h + 1, col = k / h + 1;
    uint32_t rnd[4];
    draw4(seed, (uint32_t)k, light_index, 0u, 0u, rnd);
    float ddx = o_uniform(rnd[0]);
    float ddy = o_uniform(rnd[1]);
    float xf = (float)row + ddx;
    float yf = (float)col + ddy;
    float h2 = (float)(h / 2), w2 = (float)(w / 2);
    v3 C = V(L->center), d1 = V(L->dim1), d2 = V(L->dim2);
    float sx = xf - h2, sy = yf - w2;
    v3 A = {(d1.x * sx) / h2, (d1.y * sx) / h2, (d1.z * sx) / h2};
    v3 B = {(d2.x * sy) / w2, (d2.y * sy) / w2, (d2.z * sy) / w2};
    memset(r, 0, sizeof(*r));
    vstore(r->pos, vadd(vadd(C, A), B));
    v3 dpx = {d1.x / h2, d1.y / h2, d1.z / h2};
    v3 dpy = {d2.x / w2, d2.y / w2, d2.z / w2};
    vstore(r->dp_dx, dpx);
    vstore(r->dp_dy, dpy);
    memcpy(r->dir, L->dir, sizeof(r->dir));
    r->in_medium = 0;
    r->ignore_tri = 1;
    r->dest = 0;
    r->lambda = gen_lambda(lm, (uint32_t)k, o_uniform(rnd[2]));
    r->x = xf;
    r->y = yf;
    r->status = O_STATUS_ACTIVE;
}

void o_rays_from_light(const o_rect_light* L, int64_t upscale, const o_lambda_mode* lm, uint64_t seed,
                       uint32_t light_index, o_adray* out) {
    int64_t n = (L->res1 / upscale) * (L->res2 / upscale);
    for (int64_t k = 0; k < n; ++k) gen_ray(L, upscale, lm, seed, light_index, k, &out[k]);
}

/* ------------------------------------------------------------------------ */
/* Nearest hit, src/tracer.jl:45-59 + src/hitters.jl:24-30                   */
/* ------------------------------------------------------------------------ */
static void nearest_hit(const o_adray* r, const o_ftri* tris, int64_t n_tris, int32_t* idx, float* tt) {
    float best = INFINITY;
    int32_t bi = 1;
    v3 o = V(r->pos), d = V(r->dir);
    for (int64_t j = 0; j < n_tris; ++j) {
        const o_ftri* T = &tris[j];
        int32_t i = (int32_t)(j + 1);
        v3 n = V(T->v[0]), a = V(T->v[1]);
        float t = (vdot(n, a) - vdot(n, o)) / vdot(n, d);
        v3 p = vadd(o, vmul(d, t));
        if (in_triangle_v(p, a, V(T->v[2]), V(T->v[3])) && t > 0.0f && r->ignore_tri != i) {
            /* lexicographic (t, i) minimum; j ascends so strict < keeps the smaller index */
            if (t < best) {
                best = t;
                bi = i;
            }
        }
    }
    *idx = bi;
    *tt = best;
}

void o_next_hit(const o_adray* rays, int64_t n_rays, const o_ftri* tris, int64_t n_tris, int32_t* hit_idx,
                float* hit_t, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t k = 0; k < n_rays; ++k) {
        float t;
        int32_t i;
        nearest_hit(&rays[k], tris, n_tris, &i, &t);
        hit_idx[k] = i;
        if (hit_t) hit_t[k] = t;
    }
    (void)nthreads;
}

/* ------------------------------------------------------------------------ */
/* Expansions and evolve, src/geo.jl:398-410, src/tracer.jl:61-201           */
/* ------------------------------------------------------------------------ */
static dv3 p_expansion(const o_adray* r, dual lam, dual x, dual y) {
    dual dl = d_sub(lam, DC(r->lambda)), dx = d_sub(x, DC(r->x)), dy = d_sub(y, DC(r->y));
    dv3 acc = dvc(r->pos);
    acc = dv_add(acc, dv_scale(dvc(r->dp_dl), dl));
    acc = dv_add(acc, dv_scale(dvc(r->dp_dx), dx));
    acc = dv_add(acc, dv_scale(dvc(r->dp_dy), dy));
    return acc;
}

static dv3 d_expansion(const o_adray* r, dual lam, dual x, dual y) {
    dual dl = d_sub(lam, DC(r->lambda)), dx = d_sub(x, DC(r->x)), dy = d_sub(y, DC(r->y));
    dv3 acc = dvc(r->dir);
    acc = dv_add(acc, dv_scale(dvc(r->dd_dl), dl));
    acc = dv_add(acc, dv_scale(dvc(r->dd_dx), dx));
    acc = dv_add(acc, dv_scale(dvc(r->dd_dy), dy));
    return acc;
}

/* src/tracer.jl:109-116 */
static dv3 next_p(const o_adray* r, float t, float dtl, float dtx, float dty, dual lam, dual x, dual y) {
    dual dl = d_sub(lam, DC(r->lambda)), dx = d_sub(x, DC(r->x)), dy = d_sub(y, DC(r->y));
    dual s = d_add(d_add(d_add(DC(t), d_mul(DC(dtl), dl)), d_mul(DC(dtx), dx)), d_mul(DC(dty), dy));
    return dv_add(p_expansion(r, lam, x, y), dv_scale(d_expansion(r, lam, x, y), s));
}

/* src/geo.jl:441-443 in dual form */
static dual distance_to_plane_d(const o_adray* r, const o_ftri* T, dual lam, dual x, dual y) {
    dv3 o = p_expansion(r, lam, x, y), d = d_expansion(r, lam, x, y);
    dv3 n = dvc(T->v[0]);
    dual num = d_sub(DC(vdot(V(T->v[0]), V(T->v[1]))), dv_dot(n, o));
    return d_div(num, dv_dot(n, d));
}

/* src/geo.jl:232-258 in dual form */
static void reverse_uv_d(dv3 P, const o_ftri* T, dual* u, dual* v) {
    v3 a = V(T->v[1]), b = V(T->v[2]), c = V(T->v[3]);
    v3 v0v1 = vsub(b, a), v0v2 = vsub(c, a);
    v3 N = vcross(v0v1, v0v2);
    float denom = vdot(N, N);
    v3 edge1 = vsub(c, b);
    dv3 C = dv_cross(dvcv(edge1), dv_sub(P, dvcv(b)));
    dual uu = dv_dot(dvcv(N), C);
    v3 edge2 = vsub(a, c);
    C = dv_cross(dvcv(edge2), dv_sub(P, dvcv(c)));
    dual vv = dv_dot(dvcv(N), C);
    *u = d_div(uu, DC(denom));
    *v = d_div(vv, DC(denom));
}

/* src/geo.jl:202-212 */
static dv3 optical_normal_d(const o_ftri* T, dv3 P) {
    dual u, v;
    reverse_uv_d(P, T, &u, &v);
    dual w = d_sub(d_sub(DC(1.0f), u), v);
    dv3 na = dvc(T->v[4]), nb = dvc(T->v[5]), nc = dvc(T->v[6]);
    dv3 n = dv_add(dv_add(dv_scale(na, u), dv_scale(nb, v)), dv_scale(nc, w));
    return dv_normalize(n);
}

static dv3 N_at(const o_adray* r, const o_ftri* T, float t, float dtl, float dtx, float dty, dual lam, dual x,
                dual y) {
    return optical_normal_d(T, next_p(r, t, dtl, dtx, dty, lam, x, y));
}

static dv3 refract_d(dv3 v, dv3 normal, dual n1, dual n2) {
    dv3 n = dv_normalize(normal);
    if (dv_dot(v, n).v > 0.0f) n = dv_scale(n, DC(-1.0f));
    dual c1 = dv_dot(dv_normalize(v), n);
    dual s1 = d_sqrt(d_sub(DC(1.0f), d_mul(c1, c1)));
    dual s2 = d_mul(d_div(n1, n2), s1);
    dual c2 = d_sqrt(d_sub(DC(1.0f), d_mul(s2, s2)));
    dual k = d_sub(d_mul(d_div(n1, n2), c1), c2);
    return dv_normalize(dv_add(dv_scale(v, d_div(n1, n2)), dv_scale(n, k)));
}

static dv3 reflect_d(dv3 v, dv3 normal) {
    dv3 n = dv_normalize(normal);
    dual dd = dv_dot(n, v);
    dv3 r = {d_sub(v.x, d_mul(d_mul(n.x, dd), DC(2.0f))), d_sub(v.y, d_mul(d_mul(n.y, dd), DC(2.0f))),
             d_sub(v.z, d_mul(d_mul(n.z, dd), DC(2.0f)))};
    return r;
}

/* get_hit(::Tuple{Int32,Tri}, ::ADRay), src/tracer.jl:61-81.  Returns the
 * (possibly reset) index; t and partials are Inf on a miss. */
static int32_t get_hit_ad(const o_adray* r, int32_t i, const o_ftri* T, float* t, float* dtl, float* dtx,
                          float* dty) {
    v3 o = V(r->pos), d = V(r->dir);
    float t0 = o_distance_to_plane(r->pos, r->dir, T->v[1], T->v[0]);
    v3 p0 = vadd(o, vmul(d, t0));
    if (in_triangle_v(p0, V(T->v[1]), V(T->v[2]), V(T->v[3])) && t0 > 0.0f && r->ignore_tri != i) {
        *t = t0;
        *dtl = distance_to_plane_d(r, T, DV(r->lambda, 1.0f), DC(r->x), DC(r->y)).d;
        *dtx = distance_to_plane_d(r, T, DC(r->lambda), DV(r->x, 1.0f), DC(r->y)).d;
        *dty = distance_to_plane_d(r, T, DC(r->lambda), DC(r->x), DV(r->y, 1.0f)).d;
        return i;
    }
    *t = *dtl = *dtx = *dty = INFINITY;
    return 1;
}

/* src/tracer.jl:118-179 */
static void handle_optics(o_adray* r, float t, float dtl, float dtx, float dty, int32_t i, const o_ftri* T,
                          int in_medium, const o_material* mat, float rndm, int quirks) {
    const o_adray r0 = *r;
    const o_adray* R = &r0;
    dual Lc = DC(R->lambda), Xc = DC(R->x), Yc = DC(R->y);
    dual Ld = DV(R->lambda, 1.0f), Xd = DV(R->x, 1.0f), Yd = DV(R->y, 1.0f);
    /* the y partial of the direction is taken at y = r.x in the reference */
    dual Yq = quirks ? DV(R->x, 1.0f) : Yd;

    v3 N0 = dval(N_at(R, T, t, dtl, dtx, dty, Lc, Xc, Yc));
    dual n1c = in_medium ? glass_d(mat, Lc) : air_d(Lc);
    dual n2c = in_medium ? air_d(Lc) : glass_d(mat, Lc);
    v3 dir = V(R->dir);
    int refracts = can_refract_v(dir, N0, n1c.v, n2c.v) && rndm > reflectance_v(dir, N0, n1c.v, n2c.v);

    dv3 P = next_p(R, t, dtl, dtx, dty, Lc, Xc, Yc);
    vstore(r->pos, dval(P));
    vstore(r->dp_dl, dpar(next_p(R, t, dtl, dtx, dty, Ld, Xc, Yc)));
    vstore(r->dp_dx, dpar(next_p(R, t, dtl, dtx, dty, Lc, Xd, Yc)));
    vstore(r->dp_dy, dpar(next_p(R, t, dtl, dtx, dty, Lc, Xc, Yd)));

    if (refracts) {
        vstore(r->dir, dval(refract_d(dvcv(dir), dvcv(N0), n1c, n2c)));
        dual n1d = in_medium ? glass_d(mat, Ld) : air_d(Ld);
        dual n2d = in_medium ? air_d(Ld) : glass_d(mat, Ld);
        dv3 Nl = quirks ? dvcv(N0) : N_at(R, T, t, dtl, dtx, dty, Ld, Xc, Yc);
        vstore(r->dd_dl, dpar(refract_d(d_expansion(R, Ld, Xc, Yc), Nl, n1d, n2d)));
        vstore(r->dd_dx, dpar(refract_d(d_expansion(R, Lc, Xd, Yc), N_at(R, T, t, dtl, dtx, dty, Lc, Xd, Yc),
                                        n1c, n2c)));
        vstore(r->dd_dy, dpar(refract_d(d_expansion(R, Lc, Xc, Yq), N_at(R, T, t, dtl, dtx, dty, Lc, Xc, Yq),
                                        n1c, n2c)));
        r->in_medium = (uint8_t)!R->in_medium;
    } else {
        vstore(r->dir, dval(reflect_d(dvcv(dir), dvcv(N0))));
        vstore(r->dd_dl, dpar(reflect_d(d_expansion(R, Ld, Xc, Yc), N_at(R, T, t, dtl, dtx, dty, Ld, Xc, Yc))));
        vstore(r->dd_dx, dpar(reflect_d(d_expansion(R, Lc, Xd, Yc), N_at(R, T, t, dtl, dtx, dty, Lc, Xd, Yc))));
        vstore(r->dd_dy, dpar(reflect_d(d_expansion(R, Lc, Xc, Yq), N_at(R, T, t, dtl, dtx, dty, Lc, Xc, Yq))));
        r->in_medium = R->in_medium;
    }
    r->ignore_tri = i;
    r->status = O_STATUS_ACTIVE;
}

/* src/tracer.jl:181-201 */
static void evolve_one(o_adray* r, int32_t i, const o_ftri* tris, float rndm, int64_t first_diffuse,
                       const o_material* mat, int quirks) {
    if (r->status != O_STATUS_ACTIVE) return;
    const o_ftri* T = &tris[i - 1];
    float t, dtl, dtx, dty;
    int32_t ih = get_hit_ad(r, i, T, &t, &dtl, &dtx, &dty);
    if (ih >= first_diffuse) {
        r->status = O_STATUS_DIFFUSE;
        return;
    }
    if (isinf(t)) {
        r->status = O_STATUS_INFINITY;
        return;
    }
    handle_optics(r, t, dtl, dtx, dty, ih, T, r->in_medium, mat, rndm, quirks);
}

void o_evolve(o_adray* rays, int64_t n_rays, const int32_t* hit_idx, const o_ftri* tris, const float* rndm,
              int64_t first_diffuse, const o_material* mat, int ref_quirks, int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t k = 0; k < n_rays; ++k)
        evolve_one(&rays[k], hit_idx[k], tris, rndm[k], first_diffuse, mat, ref_quirks);
    (void)nthreads;
}

/* ------------------------------------------------------------------------ */
/* run_evolution!, src/tracer.jl:205-230                                     */
/* ------------------------------------------------------------------------ */
static void run_evolution_ids(o_adray* rays, const uint32_t* ids, int64_t n_rays, const o_ftri* tris,
                              int64_t n_tris, int32_t depth, int64_t first_diffuse, const o_material* mat,
                              float force_rand, uint64_t seed, int quirks, int32_t* hit_idx, int64_t* per_bounce,
                              int nthreads) {
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
    for (int64_t k = 0; k < n_rays; ++k) hit_idx[k] = 1;
    for (int32_t it = 1; it <= depth; ++it) {
        int64_t active = 0;
        /* Retired rays keep their state, so their next_hit! result is unchanged;
         * only active rays need a new hit. */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads) reduction(+ : active)
#endif
        for (int64_t k = 0; k < n_rays; ++k) {
            o_adray* r = &rays[k];
            if (r->status != O_STATUS_ACTIVE) continue;
            active += 1;
            float t;
            int32_t i;
            nearest_hit(r, tris, n_tris, &i, &t);
            hit_idx[k] = i;
            float u = force_rand >= 0.0f ? force_rand : o_fresnel_draw(seed, ids ? ids[k] : (uint32_t)k, (uint32_t)it);
            evolve_one(r, i, tris, u, first_diffuse, mat, quirks);
        }
        if (per_bounce && it <= 6) per_bounce[it - 1] = active;
    }
    /* realign: rays still active get the hit of their final state */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 8) num_threads(nthreads)
#endif
    for (int64_t k = 0; k < n_rays; ++k) {
        if (rays[k].status != O_STATUS_ACTIVE) continue;
        float t;
        nearest_hit(&rays[k], tris, n_tris, &hit_idx[k], &t);
    }
    (void)nthreads;
}

void o_run_evolution(o_adray* rays, int64_t n_rays, const o_ftri* tris, int64_t n_tris, int32_t depth,
                     int64_t first_diffuse, const o_material* mat, float force_rand, uint64_t seed, int ref_quirks,
                     int32_t* hit_idx, int nthreads) {
    run_evolution_ids(rays, NULL, n_rays, tris, n_tris, depth, first_diffuse, mat, force_rand, seed, ref_quirks,
                      hit_idx, NULL, nthreads);
}

/* ------------------------------------------------------------------------ */
/* Light map, src/ray_imagers.jl:4-37, 78-113                                */
/* ------------------------------------------------------------------------ */

/* final_evolution(r, i, T), src/ray_imagers.jl:4-37 */
static void final_evolution(o_adray* r, int32_t i, const o_ftri* T) {
    if (r->status != O_STATUS_DIFFUSE) return;
    float t, dtl, dtx, dty;
    int32_t ih = get_hit_ad(r, i, T, &t, &dtl, &dtx, &dty);
    const o_adray r0 = *r;
    const o_adray* R = &r0;
    dual Lc = DC(R->lambda), Xc = DC(R->x), Yc = DC(R->y);
    vstore(r->pos, dval(next_p(R, t, dtl, dtx, dty, Lc, Xc, Yc)));
    vstore(r->dp_dl, dpar(next_p(R, t, dtl, dtx, dty, DV(R->lambda, 1.0f), Xc, Yc)));
    vstore(r->dp_dx, dpar(next_p(R, t, dtl, dtx, dty, Lc, DV(R->x, 1.0f), Yc)));
    vstore(r->dp_dy, dpar(next_p(R, t, dtl, dtx, dty, Lc, Xc, DV(R->y, 1.0f))));
    r->ignore_tri = ih;
    r->status = O_STATUS_DIFFUSE;
}

/* reverse_uv / tex_uv / cosine_shading on plain values, src/geo.jl:214-286 */
static void reverse_uv_f(v3 P, const o_ftri* T, float* u, float* v) {
    v3 a = V(T->v[1]), b = V(T->v[2]), c = V(T->v[3]);
    v3 N = vcross(vsub(b, a), vsub(c, a));
    float denom = vdot(N, N);
    float uu = vdot(N, vcross(vsub(c, b), vsub(P, b)));
    float vv = vdot(N, vcross(vsub(a, c), vsub(P, c)));
    *u = uu / denom;
    *v = vv / denom;
}

/* One splat sample: expand -> tex_uv -> cosine_shading.  Returns 0 when the
 * uv is not finite (the sample is dropped), else texel (i, j) 1-based. */
static int splat_sample(const o_adray* r, const o_ftri* T, float lam, float xs, float ys, int64_t W, int64_t H,
                        int64_t* ti, int64_t* tj, float* intensity) {
    v3 pos = dval(p_expansion(r, DC(lam), DC(xs), DC(ys)));
    v3 dir = dval(d_expansion(r, DC(lam), DC(xs), DC(ys)));
    float bu, bv;
    reverse_uv_f(pos, T, &bu, &bv);
    float bw = (1.0f - bu) - bv;
    float U = (T->v[7][0] * bu + T->v[8][0] * bv) + T->v[9][0] * bw;
    float Vt = (T->v[7][1] * bu + T->v[8][1] * bv) + T->v[9][1] * bw;
    if (isnan(U) || isnan(Vt) || isinf(U) || isinf(Vt)) return 0;
    float ci = ceilf(U * (float)W), cj = ceilf(Vt * (float)H);
    if (ci < 1.0f) ci = 1.0f;
    if (ci > (float)W) ci = (float)W;
    if (cj < 1.0f) cj = 1.0f;
    if (cj > (float)H) cj = (float)H;
    *ti = (int64_t)ci;
    *tj = (int64_t)cj;
    v3 na = V(T->v[4]), nb = V(T->v[5]), nc = V(T->v[6]);
    v3 n = vadd(vadd(vmul(na, bu), vmul(nb, bv)), vmul(nc, bw));
    *intensity = fabsf(vdot(vnormalize(n), vnormalize(dir)));
    return 1;
}

static int64_t splat_ray(const o_adray* r, const o_ftri* T, const float* spectrum, int32_t n_lambda,
                         const float* deltas, int32_t nd, float* tex_f32, int32_t* tex_i32, int32_t frac_bits,
                         int64_t W, int64_t H) {
    int64_t n_ok = 0;
    int32_t nl = n_lambda > 0 ? n_lambda : 1;
    float scale = ldexpf(1.0f, frac_bits);
    for (int32_t il = 0; il < nl; ++il) {
        float lam = n_lambda > 0 ? spectrum[il] : r->lambda;
        for (int32_t iy = 0; iy < nd; ++iy) {
            for (int32_t ix = 0; ix < nd; ++ix) {
                float xs = r->x + deltas[ix], ys = r->y + deltas[iy];
                int64_t i, j;
                float inten;
                if (!splat_sample(r, T, lam, xs, ys, W, H, &i, &j, &inten)) continue;
                int64_t off = (i - 1) + (j - 1) * W + (int64_t)il * W * H;
                if (tex_f32) tex_f32[off] += inten;
                if (tex_i32) tex_i32[off] += (int32_t)lrintf(inten * scale);
                n_ok += 1;
            }
        }
    }
    return n_ok;
}

void o_continuum_light_map(o_adray* rays, int64_t n_rays, const int32_t* hit_idx, const o_ftri* tris,
                           const float* spectrum, int32_t n_lambda, int32_t upscale, float* tex_f32, int32_t* tex_i32,
                           int32_t frac_bits, int64_t width, int64_t height) {
    float deltas[64];
    int32_t nd = upscale < 1 ? 1 : (upscale > 64 ? 64 : upscale);
    o_upres(nd, deltas);
    for (int64_t k = 0; k < n_rays; ++k) {
        const o_ftri* T = &tris[hit_idx[k] - 1];
        final_evolution(&rays[k], hit_idx[k], T);
    }
    for (int64_t k = 0; k < n_rays; ++k) {
        if (rays[k].status != O_STATUS_DIFFUSE) continue;
        const o_ftri* T = &tris[hit_idx[k] - 1];
        splat_ray(&rays[k], T, spectrum, n_lambda, deltas, nd, tex_f32, tex_i32, frac_bits, width, height);
    }
}

/* ------------------------------------------------------------------------ */
/* Forward half of trace!, src/tracer.jl:317-342                             */
/* ------------------------------------------------------------------------ */
void o_trace_forward(const o_rect_light* light, int64_t upscale, const o_lambda_mode* lm, uint64_t seed,
                     const o_ftri* tris, int64_t n_tris, int64_t first_diffuse, int32_t depth, const o_material* mat,
                     float force_rand, int ref_quirks, const float* spectrum, int32_t n_lambda, float* tex_f32,
                     int32_t* tex_i32, int32_t frac_bits, int64_t width, int64_t height, int64_t ray_begin,
                     int64_t ray_end, o_adray* rays_out, int64_t* stats, int nthreads) {
    int64_t n = ray_end - ray_begin;
    if (n <= 0) return;
    o_adray* rays = rays_out ? rays_out : (o_adray*)malloc((size_t)n * sizeof(o_adray));
    uint32_t* ids = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    int32_t* hit = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    for (int64_t k = 0; k < n; ++k) {
        gen_ray(light, upscale, lm, seed, 0u, ray_begin + k, &rays[k]);
        ids[k] = (uint32_t)(ray_begin + k);
    }
    int64_t per_bounce[6] = {0, 0, 0, 0, 0, 0};
    run_evolution_ids(rays, ids, n, tris, n_tris, depth, first_diffuse, mat, force_rand, seed, ref_quirks, hit,
                      per_bounce, nthreads);
    float deltas[64];
    int32_t nd = upscale < 1 ? 1 : (upscale > 64 ? 64 : (int32_t)upscale);
    o_upres(nd, deltas);
    int64_t n_diffuse = 0, n_samples = 0;
    for (int64_t k = 0; k < n; ++k) final_evolution(&rays[k], hit[k], &tris[hit[k] - 1]);
    for (int64_t k = 0; k < n; ++k) {
        if (rays[k].status != O_STATUS_DIFFUSE) continue;
        n_diffuse += 1;
        n_samples += splat_ray(&rays[k], &tris[hit[k] - 1], spectrum, n_lambda, deltas, nd, tex_f32, tex_i32,
                               frac_bits, width, height);
    }
    if (stats) {
        for (int b = 0; b < 6; ++b) stats[b] = per_bounce[b];
        stats[6] = n_diffuse;
        stats[7] = n_samples;
    }
    free(hit);
    free(ids);
    if (!rays_out) free(rays);
}

/* ------------------------------------------------------------------------ */
/* Camera pass, src/geo.jl:183-191, src/ray_generators.jl:18-62,            */
/* src/ray_imagers.jl:383-503                                                */
/* ------------------------------------------------------------------------ */
void o_camera_look_at(const float pos[3], const float look_at[3], const float true_up[3], double fov, o_camera* out) {
    memset(out, 0, sizeof(*out));
    for (int i = 0; i < 3; ++i) {
        out->pos[i] = pos[i];
        out->look_at[i] = look_at[i];
    }
    v3 dir = vnormalize(vsub(V(look_at), V(pos)));
    v3 right = vnormalize(vcross(dir, V(true_up)));
    v3 up = vnormalize(vcross(right, dir));
    vstore(out->dir, dir);
    vstore(out->right, right);
    vstore(out->up, up);
    out->fov_half_sin = (float)sin(fov / 2.0);
}

/* One ForwardDiff partial in double. */
typedef struct { double v, d; } ddual;

void o_camera_rays(const o_camera* cam, int64_t h, int64_t w, float lambda, uint64_t seed, o_adray* out) {
    const double cos45 = 1.0 / sqrt(2.0);
    const double scale = ((double)h * cos45) / (double)cam->fov_half_sin;
    const float m = (float)(h > w ? h : w);
    for (int64_t g = 0; g < h * w; ++g) {
        const int64_t x = g % h + 1, y = g / h + 1;
        uint32_t rnd[4];
        draw4(seed, (uint32_t)g, 0u, 2u, 0u, rnd);
        const float dv[3] = {(o_uniform(rnd[0]) * 0.025f) / m, (o_uniform(rnd[1]) * 0.025f) / m,
                             (o_uniform(rnd[2]) * 0.025f) / m};
        /* x pass: _x carries the partial; y pass: _y does. */
        ddual X = {((double)x - (double)h / 2.0) / scale, 1.0 / scale};
        ddual Y = {((double)y - (double)w / 2.0) / scale, 1.0 / scale};
        const double x2 = X.v * X.v, y2 = Y.v * Y.v;
        const double zz = (1.0 - x2) - y2;
        const double z = sqrt(zz);
        const double dsq = 1.0 / (2.0 * z);
        const double zx = (-((X.d * 2.0) * X.v)) * dsq; /* d(1 - _x^2 - _y^2)/dx through sqrt */
        const double zy = (-((Y.d * 2.0) * Y.v)) * dsq;
        o_adray* r = &out[g];
        memset(r, 0, sizeof(*r));
        for (int i = 0; i < 3; ++i) {
            const double R = cam->right[i], U = cam->up[i], D = cam->dir[i];
            r->pos[i] = cam->pos[i];
            r->dir[i] = (float)((((X.v * R) + (Y.v * U)) + (z * D)) + (double)dv[i]);
            r->dd_dx[i] = (float)((X.d * R) + (zx * D));
            r->dd_dy[i] = (float)((Y.d * U) + (zy * D));
        }
        r->in_medium = 0;
        r->ignore_tri = 1;
        r->dest = (y - 1) * h + x;
        r->lambda = lambda;
        r->x = 0.0f;
        r->y = 0.0f;
        r->status = O_STATUS_ACTIVE;
    }
}

/* CUDA texture fetch at CUDA coordinates (x, y, z) (the reference's
 * 1-based coordinate minus 0.5), linear filter, clamp addressing,
 * unnormalised coordinates: xB = x - 0.5, i = floor(xB), a = xB - i, texels
 * i and i + 1 clamped to the array.  Returns the exactly-weighted value; *spread is the
 * largest difference between the texels that carry weight. */
static double tex_fetch(const float* a, int64_t W, int64_t H, int64_t D, float x, float y, float z, double* spread) {
    if (!isfinite(x) || !isfinite(y) || !isfinite(z)) {
        *spread = INFINITY;
        return NAN;
    }
    const double c[3] = {(double)x - 0.5, (double)y - 0.5, (double)z - 0.5};
    const int64_t ext[3] = {W, H, D};
    int64_t i0[3], i1[3];
    double f[3];
    for (int k = 0; k < 3; ++k) {
        const double fl = floor(c[k]);
        f[k] = c[k] - fl;
        int64_t lo = (int64_t)fl, hi = lo + 1;
        lo = lo < 0 ? 0 : (lo > ext[k] - 1 ? ext[k] - 1 : lo);
        hi = hi < 0 ? 0 : (hi > ext[k] - 1 ? ext[k] - 1 : hi);
        i0[k] = lo;
        i1[k] = hi;
    }
    double v = 0.0, mn = INFINITY, mx = -INFINITY;
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                const double wgt = (dx ? f[0] : 1.0 - f[0]) * (dy ? f[1] : 1.0 - f[1]) * (dz ? f[2] : 1.0 - f[2]);
                const int live = (dx == 0 || f[0] > 0.0) && (dy == 0 || f[1] > 0.0) && (dz == 0 || f[2] > 0.0);
                if (!live) continue;
                const int64_t xi = dx ? i1[0] : i0[0], yi = dy ? i1[1] : i0[1], zi = dz ? i1[2] : i0[2];
                const double t = a[xi + W * (yi + H * zi)];
                v += wgt * t;
                if (t < mn) mn = t;
                if (t > mx) mx = t;
            }
    *spread = mx - mn;
    return v;
}

/* Julia clamp(x, 0, 1): NaN passes through. */
static float clamp01f(float x) { return x > 1.0f ? 1.0f : (x < 0.0f ? 0.0f : x); }

static void put_px(float* rgb, float* tol, int64_t height, int64_t cam_h, int32_t nd, int64_t ray, int i, int j,
                   const double val[3], const double tl[3]) {
    const int64_t gx = ray % cam_h, gy = ray / cam_h;
    const int64_t px = ((int64_t)nd * gx + i) + height * ((int64_t)nd * gy + j);
    for (int c = 0; c < 3; ++c) {
        rgb[3 * px + c] = clamp01f((float)val[c]);
        tol[3 * px + c] = (float)tl[c];
    }
}

void o_continuum_shade(o_adray* rays, int64_t n_rays, const int32_t* hit_idx, const o_ftri* tris,
                       const float* spectrum, const float* retina, int32_t n_lambda, int32_t upscale,
                       const float* tex, int64_t tw, int64_t th, int64_t planes, const float* sky, int64_t sw,
                       int64_t sh, int64_t height, int64_t width, float* rgb, float* tol) {
    float deltas[64];
    const int32_t nd = upscale < 1 ? 1 : (upscale > 64 ? 64 : upscale);
    o_upres(nd, deltas);
    const int64_t cam_h = height / nd;
    const float kPi = 3.14159265358979323846f;
    /* quantised filter weights: 2^-8 per filtered axis, two axes */
    const double q = 0x1p-7;
    (void)width;
    for (int64_t k = 0; k < n_rays; ++k) {
        o_adray* r = &rays[k];
        const int32_t ih = hit_idx[k];
        const o_ftri* T = &tris[ih - 1];
        if (r->status == O_STATUS_DIFFUSE) final_evolution(r, ih, T);
        for (int i = 0; i < nd; ++i) {
            const float xs = r->x + deltas[i];
            for (int j = 0; j < nd; ++j) {
                const float ys = r->y + deltas[j];
                double val[3] = {0, 0, 0}, tl[3] = {0, 0, 0};
                if (r->status == O_STATUS_INFINITY && sky) {
                    v3 d = dval(d_expansion(r, DC(r->lambda), DC(xs), DC(ys)));
                    const float th_ = acosf(d.z);
                    const float ph = atan2f(d.y, d.x);
                    const float vv = ((ph / kPi) + 1.0f) * 0.5f;
                    const float uu = th_ / kPi;
                    const float us = uu * (float)sw, vs = vv * (float)sh;
                    for (int c = 0; c < 3; ++c) {
                        double sp;
                        val[c] = tex_fetch(sky, sw, sh, 3, us - 0.5f, vs - 0.5f, (float)c + 0.5f, &sp);
                        /* + a few ulp of the polar angles (acosf / atan2f differ between libraries) */
                        tl[c] = (q + 0x1p-10) * sp + 0x1p-20 * fabs(val[c]);
                    }
                } else if (r->status == O_STATUS_DIFFUSE) {
                    float R = 0.0f, G = 0.0f, B = 0.0f;
                    for (int32_t il = 0; il < n_lambda; ++il) {
                        v3 pos = dval(p_expansion(r, DC(spectrum[il]), DC(xs), DC(ys)));
                        float bu, bv;
                        reverse_uv_f(pos, T, &bu, &bv);
                        const float bw = (1.0f - bu) - bv;
                        const float U = (T->v[7][0] * bu + T->v[8][0] * bv) + T->v[9][0] * bw;
                        const float Vt = (T->v[7][1] * bu + T->v[8][1] * bv) + T->v[9][1] * bw;
                        if (isnan(U) || isnan(Vt)) continue;
                        double sp;
                        const float X = (float)tex_fetch(tex, tw, th, planes, U * (float)tw - 0.5f,
                                                         Vt * (float)th - 0.5f, (float)(il + 1) - 0.5f, &sp);
                        const float rr = retina[il], gg = retina[n_lambda + il], bb = retina[2 * n_lambda + il];
                        R = R + rr * X;
                        G = G + gg * X;
                        B = B + bb * X;
                        const double e = q * sp + 0x1p-20 * fabs((double)X);
                        tl[0] += fabs((double)rr) * e;
                        tl[1] += fabs((double)gg) * e;
                        tl[2] += fabs((double)bb) * e;
                    }
                    val[0] = R;
                    val[1] = G;
                    val[2] = B;
                    for (int c = 0; c < 3; ++c) tl[c] += 0x1p-20 * fabs(val[c]) * (double)(n_lambda + 1);
                }
                put_px(rgb, tol, height, cam_h, nd, k, i, j, val, tl);
            }
        }
    }
}
