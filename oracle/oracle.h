/*
 * oracle.h -- CPU restatement of SPLAT's forward trace step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * CUDA path in splat_gb300/csrc.  Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / reference leg may load it.  The product never
 * links it and never falls back to it.
 *
 * Every function restates a piece of the reference (Julia, xaellison/SPLAT);
 * the citation is given as path:line inside the reference project.  The
 * arithmetic is IEEE binary32 in the reference's source order, compiled with
 * -ffp-contract=off and without fast-math, so the CUDA path can be compared
 * bit for bit.  Derivatives are forward-mode dual numbers evaluated closure by
 * closure exactly as the reference's ForwardDiff.derivative calls are written
 * (constants stay constants, the differentiated argument is a dual).
 *
 * Parity pins: the reflect / distance_to_plane vectors of test/geo.jl:4-29 and
 * the packed-argmin properties of src/atomic_argmin.jl:32-96 (see tests/).
 * Hit selection, evolve and light-map values have no golden vectors in the
 * reference; for those the restatement itself is the specification.
 */
#ifndef SPLAT_ORACLE_H
#define SPLAT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ADRay, Julia isbits layout (src/geo.jl:60-76): 136 bytes. */
typedef struct o_adray {
    float pos[3];
    float dp_dl[3];
    float dp_dx[3];
    float dp_dy[3];
    float dir[3];
    float dd_dl[3];
    float dd_dx[3];
    float dd_dy[3];
    uint8_t in_medium;
    uint8_t _pad0[7];
    int64_t ignore_tri;
    int64_t dest;
    float lambda;
    float x;
    float y;
    uint8_t status;
    uint8_t _pad1[3];
} o_adray;

/* FTri = SVector{10, R3} (src/geo.jl:18): normal, v1..v3, vertex normals, uvs. */
typedef struct o_ftri {
    float v[10][3];
} o_ftri;

/* RectLight (src/ray_generators.jl:4-11), Julia layout: 64 bytes. */
typedef struct o_rect_light {
    float center[3];
    float dir[3];
    float dim1[3];
    float dim2[3];
    int64_t res1;
    int64_t res2;
} o_rect_light;

enum { O_STATUS_DIFFUSE = 0, O_STATUS_ACTIVE = 1, O_STATUS_INFINITY = 2 };

/* Refractive index model of the glass.  kind 0 is the reference's linear
 * glass (src/material.jl:1-9); 1 is Cauchy n = a + b / lambda_um^2;
 * 2 is Sellmeier with three terms (b[i], c[i] in um^2). */
typedef struct o_material {
    int32_t kind;
    float a, b;
    float sb[3];
    float sc[3];
} o_material;

/* Wavelength assignment of generated rays.  mode 0: fixed lambda0 (the
 * reference hard-codes 550, src/ray_generators.jl:59); 1: uniform in
 * [lambda0, lambda1); 2: stratified, ray k in stratum k mod n_strata. */
typedef struct o_lambda_mode {
    int32_t mode;
    int32_t n_strata;
    float lambda0;
    float lambda1;
} o_lambda_mode;

int o_version(void);

/* Philox4x32-10 (Salmon et al., SC'11). */
void o_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float o_uniform(uint32_t bits);

/* src/atomic_argmin.jl:5-30 */
uint32_t o_monotonic_u32(float f);
float o_monotonic_f32(uint32_t u);
uint64_t o_pack_argmin(float t, uint32_t idx);
uint32_t o_retrieve_arg(uint64_t k);

/* Geometry / optics primitives (src/geo.jl). */
float o_distance_to_plane(const float o[3], const float d[3], const float pp[3], const float n[3]);
int o_in_triangle(const float p[3], const float a[3], const float b[3], const float c[3]);
void o_reflect(const float v[3], const float n[3], float out[3]);
void o_refract(const float v[3], const float n[3], float n1, float n2, float out[3]);
int o_can_refract(const float v[3], const float n[3], float n1, float n2);
float o_reflectance(const float v[3], const float n[3], float n1, float n2);
float o_glass(const o_material* m, float lambda);
void o_upres(int n, float* out);

/* Ray generation (src/ray_generators.jl:64-113). */
void o_rays_from_light(const o_rect_light* light, int64_t upscale, const o_lambda_mode* lm,
                       uint64_t seed, uint32_t light_index, o_adray* out);

/* Brute-force nearest hit, lexicographic (t, idx) minimum over all
 * triangles (src/hitters.jl:24-30).  hit_idx is 1-based, 1 = miss. */
void o_next_hit(const o_adray* rays, int64_t n_rays, const o_ftri* tris, int64_t n_tris,
                int32_t* hit_idx, float* hit_t, int nthreads);

/* One evolve_ray over n rays (src/tracer.jl:181-201). */
void o_evolve(o_adray* rays, int64_t n_rays, const int32_t* hit_idx, const o_ftri* tris,
              const float* rndm, int64_t first_diffuse, const o_material* mat, int ref_quirks,
              int nthreads);

/* Fresnel draw of ray `ray_id` at bounce `bounce` (1-based). */
float o_fresnel_draw(uint64_t seed, uint32_t ray_id, uint32_t bounce);

/* run_evolution! (src/tracer.jl:205-230): depth x {next_hit!, rand!, evolve}.
 * force_rand < 0 means "draw", otherwise every draw is replaced by it.
 * hit_idx receives the hit indices of the last pass (aligned with rays). */
void o_run_evolution(o_adray* rays, int64_t n_rays, const o_ftri* tris, int64_t n_tris,
                     int32_t depth, int64_t first_diffuse, const o_material* mat,
                     float force_rand, uint64_t seed, int ref_quirks, int32_t* hit_idx,
                     int nthreads);

/* final_evolution + atomic_spectrum_kernel2 (src/ray_imagers.jl:4-37,78-113,
 * 142-165).  rays are updated in place (diffuse rays move onto their hit).
 * spectrum == NULL / n_lambda == 0 selects "own wavelength": one plane, each
 * ray splats at its own lambda.  Either tex_f32 (float accumulation in ray
 * order) or tex_i32 (fixed point, round(intensity * 2^frac_bits)) may be NULL. */
void o_continuum_light_map(o_adray* rays, int64_t n_rays, const int32_t* hit_idx,
                           const o_ftri* tris, const float* spectrum, int32_t n_lambda,
                           int32_t upscale, float* tex_f32, int32_t* tex_i32,
                           int32_t frac_bits, int64_t width, int64_t height);

/* Whole forward trace step: rays_from_light -> run_evolution! ->
 * continuum_light_map2!.  Only rays [ray_begin, ray_end) of the generated
 * grid are traced (a bounded sample); ray ids stay the full-grid ids so a
 * sample traces exactly the rays the GPU traces for those ids.  stats
 * (optional, 8 int64): rays per bounce (depth entries, up to 6), diffuse
 * count, splat samples. */
void o_trace_forward(const o_rect_light* light, int64_t upscale, const o_lambda_mode* lm,
                     uint64_t seed, const o_ftri* tris, int64_t n_tris, int64_t first_diffuse,
                     int32_t depth, const o_material* mat, float force_rand, int ref_quirks,
                     const float* spectrum, int32_t n_lambda, float* tex_f32, int32_t* tex_i32,
                     int32_t frac_bits, int64_t width, int64_t height, int64_t ray_begin,
                     int64_t ray_end, o_adray* rays_out, int64_t* stats, int nthreads);

/* Cam (src/geo.jl:50-57): 64 bytes. */
typedef struct o_camera {
    float pos[3];
    float look_at[3];
    float dir[3];
    float up[3];
    float right[3];
    float fov_half_sin;
} o_camera;

/* get_camera (src/geo.jl:183-191). */
void o_camera_look_at(const float pos[3], const float look_at[3], const float true_up[3], double fov, o_camera* out);

/* wrap_ray_gen(camera_ray) (src/ray_generators.jl:18-62) over an h x w grid:
 * ray g = (x - 1) + h (y - 1); jitter dv from Philox(seed) at (g, 0, 2, 0).
 * The direction and its partials are evaluated in double (integer pixel
 * indices promote them) and rounded to float once. */
void o_camera_rays(const o_camera* cam, int64_t h, int64_t w, float lambda, uint64_t seed, o_adray* out);

/* continuum_shade!(ExperimentalImager2) (src/ray_imagers.jl:383-503) with a
 * model of the texture unit's linear filter: exact (unquantised) weights;
 * tol receives, per image value, a bound on what the hardware's 8-bit
 * fractional weights and its math library may change (+inf where the
 * texture coordinate is not finite).  tex: [tw, th, planes] column-major;
 * sky: [sw, sh, 3] or NULL.  rgb / tol: height * width RGB triples,
 * column-major pixels.  Diffuse rays are final-evolved in place. */
void o_continuum_shade(o_adray* rays, int64_t n_rays, const int32_t* hit_idx, const o_ftri* tris,
                       const float* spectrum, const float* retina, int32_t n_lambda, int32_t upscale,
                       const float* tex, int64_t tw, int64_t th, int64_t planes, const float* sky, int64_t sw,
                       int64_t sh, int64_t height, int64_t width, float* rgb, float* tol);

#ifdef __cplusplus
}
#endif

#endif
