/*
 * splat.h -- C ABI of libsplat, the GB300-native (sm_103a) forward trace step
 * of SPLAT, the spectral photon-splatting ray tracer (xaellison/SPLAT).
 *
 * Every entry point returns a splat_status_t (SPLAT_OK == 0) and never
 * throws; the message of the last failure on the calling thread is
 * splat_last_error().  Device pointers are caller-owned and never freed by
 * the library; the only library-owned objects are scenes (resident packed
 * geometry + BVH).  Every call takes the caller's CUDA stream (cudaStream_t
 * passed as void*; NULL is the legacy default stream) and enqueues
 * asynchronously on it; nothing here synchronises the device except the
 * *_host entry points, which wait for their own stream.
 *
 * Records keep the reference's Julia isbits layouts, so the Julia side can
 * pass its own CuArray{ADRay}, CuArray{FTri}, CuArray{Tuple{Int32,Tri}}
 * buffers (pointer(a)) without conversion.  Triangle indices are the
 * reference's 1-based indices; a hit index of 1 means "miss" (index 1 is
 * the all-zero sentinel triangle every scene starts with).
 *
 * Citations are path:line in the reference project.
 */
#ifndef SPLAT_H
#define SPLAT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPLAT_ABI_VERSION 1

typedef int32_t splat_status_t;
enum {
    SPLAT_OK = 0,
    SPLAT_ERR_INVALID = 1,   /* bad argument (null pointer, size, enum) */
    SPLAT_ERR_CUDA = 2,      /* a CUDA runtime call failed */
    SPLAT_ERR_ALLOC = 3,     /* a library-owned allocation failed */
    SPLAT_ERR_WORKSPACE = 4, /* caller workspace smaller than required */
    SPLAT_ERR_DEVICE = 5     /* a kernel reported an error status word */
};

/* ADRay, src/geo.jl:60-76 (136 bytes). status: 0 diffuse, 1 active, 2 infinity
 * (src/geo.jl:78-80). */
typedef struct splat_adray {
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
} splat_adray_t;

/* FTri = SVector{10, R3}, src/geo.jl:18 (120 bytes): plane normal, v1, v2,
 * v3, vertex normals n1..n3, texture coordinates (u, v, 0) of v1..v3. */
typedef struct splat_ftri {
    float v[10][3];
} splat_ftri_t;

/* Tuple{Int32, Tri}, the n_tris element of src/tracer.jl:313 (52 bytes):
 * index, plane normal, v1, v2, v3. */
typedef struct splat_ntri {
    int32_t idx;
    float v[4][3];
} splat_ntri_t;

/* RectLight, src/ray_generators.jl:4-11 (64 bytes). */
typedef struct splat_rect_light {
    float center[3];
    float dir[3];
    float dim1[3];
    float dim2[3];
    int64_t res1;
    int64_t res2;
} splat_rect_light_t;

/* Glass index model.  LINEAR_REF is the reference's glass(lambda)
 * (src/material.jl:1-9); CAUCHY n = a + b / lambda_um^2; SELLMEIER
 * n^2 = 1 + sum_i sb[i] l2 / (l2 - sc[i]), l2 = lambda_um^2.  Air is 1. */
enum { SPLAT_MATERIAL_LINEAR_REF = 0, SPLAT_MATERIAL_CAUCHY = 1, SPLAT_MATERIAL_SELLMEIER = 2 };
typedef struct splat_material {
    int32_t kind;
    float a, b;
    float sb[3];
    float sc[3];
} splat_material_t;

/* Wavelength of generated rays: FIXED lambda0 (the reference hard-codes 550,
 * src/ray_generators.jl:59), UNIFORM in [lambda0, lambda1), STRATIFIED: ray k
 * uniform inside stratum (k mod n_strata). */
enum { SPLAT_LAMBDA_FIXED = 0, SPLAT_LAMBDA_UNIFORM = 1, SPLAT_LAMBDA_STRATIFIED = 2 };
typedef struct splat_lambda_mode {
    int32_t mode;
    int32_t n_strata;
    float lambda0;
    float lambda1;
} splat_lambda_mode_t;

/* Hitters: BRUTE all pairs; BVH the four-wide BVH; BVH2 the binary BVH it is
 * collapsed from.  All three return identical results. */
enum { SPLAT_HITTER_BRUTE = 0, SPLAT_HITTER_BVH = 1, SPLAT_HITTER_BVH2 = 2 };
enum { SPLAT_ACCUM_F32 = 0, SPLAT_ACCUM_I32 = 1 };

/* flags */
#define SPLAT_FLAG_REF_QUIRKS 1u /* reproduce the reference's derivative quirks (default) */

typedef struct splat_scene splat_scene_t;

typedef struct splat_scene_info {
    int64_t n_tris;        /* including the sentinel */
    int64_t first_diffuse; /* 1-based */
    int64_t bvh_nodes;     /* 0 without BVH */
    int64_t bvh_leaves;
    int32_t bvh_depth;
    int32_t bvh_max_leaf;
    int64_t device_bytes;  /* library-owned device memory of this scene */
    float bounds_lo[3];
    float bounds_hi[3];
    float bvh_pad;         /* absolute padding of the BVH boxes */
} splat_scene_info_t;

#define SPLAT_MAX_LAMBDA 64

/* One forward trace step (the forward half of trace!, src/tracer.jl:317-342):
 * rays_from_light -> depth x {next_hit!, rand!, evolve_ray} -> final_evolution
 * -> atomic spectrum splat.  Rays ray_begin .. ray_end-1 of the light grid are
 * traced (ray_end <= 0: the whole grid); ray ids are grid indices. */
typedef struct splat_trace_params {
    splat_rect_light_t light;
    int64_t upscale;           /* forward_upscale: grid res / upscale rays, upscale^2 splat offsets */
    splat_lambda_mode_t lambda_mode;
    uint64_t seed;             /* Philox key: jitter, wavelength and Fresnel draws */
    int32_t depth;
    int32_t hitter;            /* SPLAT_HITTER_* */
    splat_material_t material;
    float force_rand;          /* < 0: draw; else every Fresnel draw is this value */
    uint32_t flags;            /* SPLAT_FLAG_* */
    int32_t n_lambda;          /* 0: each ray splats at its own wavelength into plane 0 */
    float spectrum[SPLAT_MAX_LAMBDA];
    int64_t map_w, map_h;      /* light map [w, h, planes], column-major (u fastest) */
    int32_t accum;             /* SPLAT_ACCUM_* */
    int32_t frac_bits;         /* fixed point: round(intensity * 2^frac_bits) */
    int32_t zero_map;          /* 1: clear the map first; 0: accumulate onto it */
    int32_t _pad;
    int64_t ray_begin, ray_end;
} splat_trace_params_t;

/* Counters of one trace step, written on the device. */
typedef struct splat_trace_stats {
    int64_t rays_per_bounce[8]; /* active rays entering bounce b */
    int64_t diffuse;            /* rays splatted */
    int64_t samples;            /* splat samples accumulated (finite uv) */
    int64_t error;              /* kernel error word, 0 = ok */
    int64_t _pad;
} splat_trace_stats_t;

/* ---------------------------------------------------------------- library */
int32_t splat_abi_version(void);
const char* splat_last_error(void);
/* Number of SMs and the device name of the current device (for reports). */
splat_status_t splat_device_info(int32_t* sm_count, char* name, int32_t name_len);

/* ------------------------------------------------------------------ scene */
/* Resident scene: packed hit records, FTri optical data, optional BVH (host
 * binned-SAH build, padded boxes).  Replaces the hitter constructors
 * (src/alg_types.jl:60-90) and bv_partition / pack_bv_tris (src/bv.jl:68-136).
 * host_tris: reference FTri array, index 1 the sentinel. */
splat_status_t splat_scene_create(const splat_ftri_t* host_tris, int64_t n_tris, int64_t first_diffuse,
                                  int32_t build_bvh, void* stream, splat_scene_t** out);
splat_status_t splat_scene_destroy(splat_scene_t* scene);
/* The scene's device error word, OR of the bits the plugin-level calls
 * (next_hit, evolve, light map, shade) set on bad input -- 16: a hit index
 * outside 1..n_tris, treated as a miss.  Synchronises the stream; with
 * reset != 0 the word is cleared after the read. */
splat_status_t splat_scene_errors(splat_scene_t* scene, int32_t reset, int32_t* out, void* stream);
splat_status_t splat_scene_info(const splat_scene_t* scene, splat_scene_info_t* info);
/* Device-side update from new FTri data of the same count (per-frame
 * geometry upload): repacks the hit records and refits the BVH boxes
 * bottom-up, keeping its topology.  d_tris: device FTri array. */
splat_status_t splat_scene_update(splat_scene_t* scene, const splat_ftri_t* d_tris, void* stream);
/* Device-side geometry replacement with the BVH rebuilt on the GPU: a
 * linear BVH (Morton-ordered centroids, radix tree, bottom-up padded boxes,
 * leaves of at most 4 triangles) in the same node formats, for scenes whose
 * motion a refit would degrade (the reference rebuilds its bounding volumes
 * on the host every frame, src/scenes/splash_scene.jl:41, src/bv.jl:68-121).
 * Hits stay identical to brute force.  The first call allocates the build's
 * scratch; later calls allocate nothing.  After a rebuild,
 * splat_scene_update rebuilds too.  d_tris NULL: rebuild from the scene's
 * current triangles. */
splat_status_t splat_scene_rebuild(splat_scene_t* scene, const splat_ftri_t* d_tris, void* stream);
/* Device pointer of the scene's FTri array (read-only). */
const splat_ftri_t* splat_scene_tris(const splat_scene_t* scene);

/* Mesh ingest: a Wavefront OBJ file -> FTri records (mesh_to_FTri over the
 * faces MeshIO loads, src/geo.jl:289-341): one record per triangle, polygons
 * fan-triangulated, per-corner positions / normals / uvs, plane normal
 * cross(v1 - v2, v2 - v3).  No sentinel is prepended (the scene does that).
 * Call with out = NULL to get the count, then with capacity >= count. */
splat_status_t splat_obj_to_ftri(const char* path, splat_ftri_t* out, int64_t capacity, int64_t* n_tris);

/* -------------------------------------------------------- plugin boundary */
/* rays_from_light (src/ray_generators.jl:64-97): (res1/upscale)*(res2/upscale)
 * rays, column-major over (row, col), jitter from Philox(seed). */
splat_status_t splat_rays_from_light(const splat_rect_light_t* light, int64_t upscale,
                                     const splat_lambda_mode_t* lambda_mode, uint64_t seed, uint32_t light_index,
                                     splat_adray_t* d_rays, void* stream);

/* next_hit!(tracer, ::ExperimentalHitter6, rays, n_tris) (src/hitters.jl:205-226):
 * brute-force nearest hit of every ray over the reference's n_tris array;
 * lexicographic (t, index) minimum, packed into d_tmp (hitter.tmp, caller
 * scratch of n_rays u64) then unpacked into d_hit_idx (tracer.hit_idx). */
splat_status_t splat_next_hit_brute(const splat_adray_t* d_rays, int64_t n_rays, const splat_ntri_t* d_n_tris,
                                    int64_t n_tris, uint64_t* d_tmp, int32_t* d_hit_idx, void* stream);

/* Allocation-free variant of splat_next_hit_brute.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory at the
 * point of the call -- a render callback running under a fixed, pre-admitted
 * memory budget, a Julia finalizer or @cfunction callback where triggering the
 * CUDA.jl allocator (and the garbage collection and synchronisation it may
 * cause) is not allowed, or a host that hands out only the input and output
 * buffers.  The packed (t, index) words that splat_next_hit_brute keeps in the
 * caller's d_tmp live instead in one array of SPLAT_STATIC_HIT_MAX_RAYS
 * 64-bit words (4 MiB) inside the library, which every GPU that loads the
 * library holds until the process exits.  Rules:
 *   - n_rays above SPLAT_STATIC_HIT_MAX_RAYS is rejected (SPLAT_ERR_INVALID);
 *   - the first call on a device looks the array's device address up (once
 *     per device, with that device current); make that first call before
 *     any stream capture.  The address is kept for the life of the process:
 *     after cudaDeviceReset (or any teardown of the device's primary
 *     context) it is stale, so do not call this entry point again on that
 *     device after a reset;
 *   - every call shares the array and first resets the words it uses, so
 *     calls whose kernels overlap on the GPU (other streams, other host
 *     threads) race and must be serialised by the caller;
 *   - no cudaMalloc, cudaFree or allocating library routine is called. */
#define SPLAT_STATIC_HIT_MAX_RAYS (1 << 19)
splat_status_t splat_next_hit_brute_static(const splat_adray_t* d_rays, int64_t n_rays, const splat_ntri_t* d_n_tris,
                                           int64_t n_tris, int32_t* d_hit_idx, void* stream);

/* next_hit! with a resident scene (brute force or BVH,
 * src/hitters.jl:205-226 / 615-647).  d_hit_t (optional) receives the hit
 * distance, Inf on a miss. */
splat_status_t splat_next_hit(const splat_scene_t* scene, int32_t hitter, const splat_adray_t* d_rays,
                              int64_t n_rays, int32_t* d_hit_idx, float* d_hit_t, void* stream);

/* run_evolution! (src/tracer.jl:233-282) on the caller's rays, in place:
 * depth x {hit, Fresnel draw, evolve_ray, compaction}, then the final hit of
 * every ray into d_hit_idx.  Ray slot k draws Philox(seed, (k, 0, 1, bounce)).
 * Workspace: splat_run_evolution_workspace_size(n_rays) bytes. */
size_t splat_run_evolution_workspace_size(int64_t n_rays);
splat_status_t splat_run_evolution(const splat_scene_t* scene, int32_t hitter, splat_adray_t* d_rays,
                                   int64_t n_rays, int32_t depth, const splat_material_t* material,
                                   float force_rand, uint64_t seed, uint32_t flags, int32_t* d_hit_idx,
                                   void* d_workspace, size_t workspace_bytes, void* stream);

/* One evolve_ray broadcast (src/tracer.jl:181-201, as called at
 * src/tracer.jl:246-256: `rays .= evolve_ray.(rays, hit_idx, tri_view, rndm,
 * first_diffuse)`), in place.  Every ACTIVE ray k evolves with hit index
 * d_hit_idx[k] (1-based) and Fresnel draw d_rndm[k] (the reference's rand!
 * array); with d_rndm NULL the draw is force_rand when >= 0, else
 * Philox(seed, (k, 0, 1, bounce)).  Rays that hit a diffuse triangle or
 * nothing change only their status; retired rays are untouched. */
splat_status_t splat_evolve(const splat_scene_t* scene, splat_adray_t* d_rays, int64_t n_rays,
                            const int32_t* d_hit_idx, const float* d_rndm, const splat_material_t* material,
                            float force_rand, uint64_t seed, uint32_t bounce, uint32_t flags, void* stream);

/* partition!(rays, ray_swap; by = status != ACTIVE) (src/partition.jl:122-132,
 * called at src/tracer.jl:263): the ACTIVE rays move to the front of d_rays,
 * in no particular order (the reference's is not stable either), and their
 * count is written to the device int64 *d_n_active -- it is not read back.
 * Workspace: splat_partition_workspace_size(n_rays) bytes (the swap array). */
size_t splat_partition_workspace_size(int64_t n_rays);
splat_status_t splat_partition(splat_adray_t* d_rays, int64_t n_rays, int64_t* d_n_active, void* d_workspace,
                               size_t workspace_bytes, void* stream);

/* continuum_light_map2! (src/ray_imagers.jl:142-165): final_evolution of the
 * diffuse rays (in place) and the atomic spectrum splat into d_tex
 * ([w, h, planes] column-major, float or int32 fixed point).  spectrum is a
 * host array of n_lambda wavelengths (n_lambda 0: own wavelength, 1 plane). */
splat_status_t splat_continuum_light_map(const splat_scene_t* scene, splat_adray_t* d_rays, int64_t n_rays,
                                         const int32_t* d_hit_idx, const float* spectrum, int32_t n_lambda,
                                         int64_t upscale, void* d_tex, int32_t accum, int32_t frac_bits,
                                         int64_t map_w, int64_t map_h, void* stream);

/* ------------------------------------------------------- fused trace step */
/* The GB300 form of the forward half of trace! (src/tracer.jl:317-342):
 * structure-of-arrays ray state, compaction fused into evolve (ballot +
 * block scan, one atomic per block, counts stay on the device), diffuse
 * rays splatted inside the bounce that finds them, no host round trip.
 * d_stats (optional) receives splat_trace_stats_t on the device. */
size_t splat_trace_workspace_size(int64_t n_rays);
splat_status_t splat_trace_forward(const splat_scene_t* scene, const splat_trace_params_t* params, void* d_map,
                                   void* d_workspace, size_t workspace_bytes, splat_trace_stats_t* d_stats,
                                   void* stream);
/* Same step with host buffers: copies host_tris (n_tris FTri, the scene's
 * triangle count) to the device, updates the scene (repack + BVH refit),
 * traces, and copies the map back into host_map.  Pinned host memory is
 * recommended.  Returns after the stream has finished. */
splat_status_t splat_trace_forward_host(splat_scene_t* scene, const splat_ftri_t* host_tris,
                                        const splat_trace_params_t* params, void* host_map, void* d_map,
                                        void* d_workspace, size_t workspace_bytes, splat_trace_stats_t* host_stats,
                                        void* stream);

/* ------------------------------------------------------------ camera pass */
/* The backward half of trace! (src/tracer.jl:345-378): camera rays traced
 * through the same bounce loop, then shaded from the light map the forward
 * step wrote and from a skydome (continuum_shade!, ExperimentalImager2).
 *
 * Cam (src/geo.jl:50-57), Julia layout: 64 bytes. */
typedef struct splat_camera {
    float pos[3];
    float look_at[3];
    float dir[3];
    float up[3];
    float right[3];
    float fov_half_sin;
} splat_camera_t;

/* get_camera (src/geo.jl:183-191): dir = normalize(look_at - pos),
 * right = normalize(dir x true_up), up = normalize(right x dir),
 * fov_half_sin = sin(fov / 2) (fov in radians, evaluated in double). */
splat_status_t splat_camera_look_at(const float pos[3], const float look_at[3], const float true_up[3], double fov,
                                    splat_camera_t* out);

/* wrap_ray_gen(camera_ray) (src/ray_generators.jl:18-62): height * width
 * camera rays, column-major over (x = row 1..height, y = col 1..width), at
 * wavelength lambda; dest = (y - 1) * height + x.  The direction and its x / y
 * derivatives are evaluated in double and rounded once, as the reference's
 * integer pixel indices promote them.  The jitter dv in [0, 1)^3 is
 * Philox(seed) keyed by the ray index (the reference draws CUDA.rand). */
splat_status_t splat_camera_rays(const splat_camera_t* camera, int64_t height, int64_t width, float lambda,
                                 uint64_t seed, splat_adray_t* d_rays, void* stream);

/* _spectrum_datastructs (src/rgb_spectrum.jl:135-149): retina response of
 * each wavelength, out[c * n_lambda + i] for c = red, green, blue: the
 * reference's piecewise-linear retina curves normalised by their sums over
 * 400..700 nm, evaluated in double and rounded to float (host only). */
splat_status_t splat_retina_factors(const float* spectrum, int32_t n_lambda, float* out);

/* Shader: the light map and the skydome as hardware-filtered textures
 * (CuTexture(CuTextureArray(tex); interpolation = LinearInterpolation()),
 * src/tracer.jl:343 and src/scenes/sphere.jl:116-126): 3-D float arrays,
 * linear filtering, clamped addressing, unnormalised coordinates.  Library-
 * owned device arrays, reused frame after frame. */
typedef struct splat_shader splat_shader_t;
/* map: [map_w, map_h, n_planes]; sky: [sky_w, sky_h, 3] (sky_w = 0: no
 * skydome, escaping rays shade black). */
splat_status_t splat_shader_create(int64_t map_w, int64_t map_h, int32_t n_planes, int64_t sky_w, int64_t sky_h,
                                   splat_shader_t** out);
splat_status_t splat_shader_destroy(splat_shader_t* shader);
/* Loads a light map (device, column-major [w, h, planes]); int32 maps are
 * converted to float (value / 2^frac_bits) on the way. */
splat_status_t splat_shader_set_light_map(splat_shader_t* shader, const void* d_map, int32_t accum, int32_t frac_bits,
                                          void* stream);
/* Loads the skydome (device float, [sky_w, sky_h, 3] column-major). */
splat_status_t splat_shader_set_skydome(splat_shader_t* shader, const float* d_sky, void* stream);

/* continuum_shade!(ExperimentalImager2) (src/ray_imagers.jl:441-503) on the
 * caller's rays after splat_run_evolution (ray i at index dest - 1, hit
 * indices realigned): final_evolution of the diffuse rays in place, then
 * for every ray and upscale^2 sub-sample (shade_tex4_kernel,
 * src/ray_imagers.jl:383-438): diffuse -> sum over the spectrum of
 * retina * light map texel at the hit's uv; escaped -> skydome at the
 * direction's polar angles; otherwise black; each channel clamped to
 * [0, 1].  d_rgb: height * width RGB float triples, column-major pixels
 * (the reference's RGBf image); camera ray (x, y) sub-sample (i, j) lands on
 * pixel (upscale (x-1) + i, upscale (y-1) + j).  retina: [3][n_lambda]. */
splat_status_t splat_continuum_shade(const splat_scene_t* scene, const splat_shader_t* shader, splat_adray_t* d_rays,
                                     int64_t n_rays, const int32_t* d_hit_idx, const float* spectrum,
                                     const float* retina, int32_t n_lambda, int64_t upscale, int64_t height,
                                     int64_t width, float* d_rgb, void* stream);

/* One camera pass in the fused form (SoA, compacted bounce loop). */
typedef struct splat_render_params {
    splat_camera_t camera;
    int64_t height, width;  /* image in pixels; camera rays (height / upscale) x (width / upscale) */
    int64_t upscale;        /* backward_upscale */
    uint64_t seed;          /* Philox key: camera jitter and Fresnel draws */
    int32_t depth;
    int32_t hitter;         /* SPLAT_HITTER_* */
    splat_material_t material;
    float force_rand;       /* < 0: draw */
    uint32_t flags;         /* SPLAT_FLAG_* */
    float lambda;           /* camera rays' wavelength (the reference uses 550) */
    int32_t n_lambda;       /* shading spectrum = the light map's planes */
    float spectrum[SPLAT_MAX_LAMBDA];
    float retina[3][SPLAT_MAX_LAMBDA];
} splat_render_params_t;

size_t splat_render_workspace_size(int64_t n_camera_rays);
/* Camera rays -> depth x {hit, evolve} with diffuse rays final-evolved into
 * a shading queue and escaping rays into a sky queue -> shading straight
 * into their pixels (the rest stay black).  The image equals
 * splat_camera_rays + splat_run_evolution + splat_continuum_shade. */
splat_status_t splat_render_camera(const splat_scene_t* scene, const splat_shader_t* shader,
                                   const splat_render_params_t* params, float* d_rgb, void* d_workspace,
                                   size_t workspace_bytes, void* stream);
/* The same, with the shading held back until map_ready (a cudaEvent_t, e.g.
 * recorded after splat_shader_set_light_map on another stream) has
 * completed.  The camera rays' bounce loop does not read the light map, so
 * on its own stream it runs while the frame's forward step is still
 * tracing.  map_ready NULL: as splat_render_camera. */
splat_status_t splat_render_camera_after(const splat_scene_t* scene, const splat_shader_t* shader,
                                         const splat_render_params_t* params, float* d_rgb, void* d_workspace,
                                         size_t workspace_bytes, void* stream, void* map_ready);

/* Running average of a frame's iterations (src/tracer.jl:380-384):
 * iteration k = 1 copies rgb into out; k > 1 sets
 * out = out * (k - 1) / k + rgb / k.  n: floats. */
splat_status_t splat_image_accumulate(float* d_out, const float* d_rgb, int64_t n, int32_t iteration, void* stream);

/* ----------------------------------------------------------- batch engine */
/* Many frames of many scenes traced together (the batched and served
 * forms).  An item is one frame: a resident scene, its trace parameters and
 * its light map.  splat_batch_tick advances every in-flight item by one
 * bounce in one launch sequence; an item admitted between ticks starts at the
 * next tick, so requests join and leave at bounce granularity while others
 * are in flight (continuous batching).  Draws are keyed by the item's seed
 * and each ray's grid index and int32 maps add exactly, so an item's map is
 * the one splat_trace_forward produces, alone or in any mix.
 * The pool holds max_pool_rays rays of items in flight (library-owned device
 * memory, splat_batch_device_bytes).  Items keep pointers into their scene:
 * a scene must outlive its items.  BVH2 items use the four-wide BVH. */
typedef struct splat_batch splat_batch_t;
size_t splat_batch_device_bytes(int32_t max_items, int64_t max_pool_rays);
splat_status_t splat_batch_create(int32_t max_items, int64_t max_pool_rays, splat_batch_t** out);
splat_status_t splat_batch_destroy(splat_batch_t* batch);
/* Admits one frame; SPLAT_ERR_WORKSPACE when no slot or pool room is free
 * (retry after a tick).  The map is cleared at the item's first tick when
 * params->zero_map is set. */
splat_status_t splat_batch_admit(splat_batch_t* batch, const splat_scene_t* scene,
                                 const splat_trace_params_t* params, void* d_map, int32_t* slot);
/* Enqueues one tick on the stream.  done_slots receives the items whose last
 * bounce runs in this tick: their maps are complete once the stream reaches
 * this point. */
splat_status_t splat_batch_tick(splat_batch_t* batch, void* stream, int32_t* done_slots, int32_t max_done,
                                int32_t* n_done);
/* Frees a completed item's slot. */
splat_status_t splat_batch_release(splat_batch_t* batch, int32_t slot);
splat_status_t splat_batch_status(const splat_batch_t* batch, int32_t* in_flight, int64_t* pool_rays, int32_t* tick);
/* Captures the ticks that run every admitted item to completion into a CUDA
 * graph (all items must start at the current tick; the stream must be a
 * created stream, not a default one).  splat_batch_replay
 * launches it again, optionally with new per-slot seeds. */
splat_status_t splat_batch_capture(splat_batch_t* batch, void* stream, int32_t* n_ticks);
splat_status_t splat_batch_replay(splat_batch_t* batch, const uint64_t* seeds, int32_t n_seeds, void* stream);

/* ---------------------------------------------------------------- server */
/* Continuous-batching render server over one batch engine (the served form).
 * splat_server_submit queues a request (a resident caller-owned scene, trace
 * parameters, a caller-owned device light map) in arrival order;
 * splat_server_step admits what fits -- a free slot, room in the engine's
 * ray pool, and the request's light map within map_budget_bytes of maps in
 * flight -- and enqueues one tick on the stream, staying at most
 * max_ticks_ahead ticks ahead of the device.  splat_server_poll returns the
 * requests whose maps are complete (block != 0: waits for every request
 * already given its last tick) with their completion time on the device, in
 * ms since the server's first step.  A request's map is the one
 * splat_trace_forward produces alone. */
typedef struct splat_server splat_server_t;
splat_status_t splat_server_create(int32_t max_items, int64_t max_pool_rays, int64_t map_budget_bytes,
                                   int32_t max_ticks_ahead, splat_server_t** out);
splat_status_t splat_server_destroy(splat_server_t* server);
splat_status_t splat_server_submit(splat_server_t* server, const splat_scene_t* scene,
                                   const splat_trace_params_t* params, void* d_map, int64_t* request_id);
splat_status_t splat_server_step(splat_server_t* server, void* stream, int32_t* in_flight, int32_t* queued);
splat_status_t splat_server_poll(splat_server_t* server, int32_t block, int64_t* request_ids, double* device_ms,
                                 int32_t max_ids, int32_t* n_ids);
splat_status_t splat_server_status(const splat_server_t* server, int32_t* queued, int32_t* in_flight,
                                   int64_t* map_bytes_in_use);

/* ---------------------------------------------------------------- tuning */
/* Launch-shape knobs (process-wide): blocks per SM of the grid-stride
 * kernels (1..256), and the splat's block-level texel aggregation (0 or 1).
 * They change only how work is spread over the GPU, never a result (float
 * maps: summation order only); the autotuner (splat_gb300/autotune.py)
 * picks them per workload. */
enum {
    SPLAT_TUNE_BRUTE_BLOCKS_PER_SM = 0, /* brute force: triangle-range splits target (default 4) */
    SPLAT_TUNE_BVH_BLOCKS_PER_SM = 1,   /* BVH traversal grid (default 16) */
    SPLAT_TUNE_EVOLVE_BLOCKS_PER_SM = 2, /* evolve grid (default 8) */
    SPLAT_TUNE_SPLAT_BLOCKS_PER_SM = 3,  /* splat grid (default 8) */
    SPLAT_TUNE_SPLAT_AGGREGATE = 4,      /* splat sums samples per texel in shared memory first (default 0) */
    SPLAT_TUNE_BVH_PACKET = 5,           /* four-wide BVH warp packets: 0 never, 1 first bounce (default), 2 every bounce,
                                            3 / 4 first bounce + per-warp choice by ray spread after (loose /
                                            tight), 5 per-warp choice everywhere */
    SPLAT_TUNE_SPLAT_OVERLAP = 6,        /* fused trace step: 0 one splat after the last bounce; 1 the diffuse rays
                                            of the earlier bounces splatted on a side stream while the last bounce
                                            runs; 2 one splat per bounce on the side stream (default 2) */
    SPLAT_TUNE_BVH_REFILL = 7,           /* four-wide BVH, per-ray form: 0 a warp takes 32 new rays when all 32 are
                                            done; 1..32 a warp refills its finished lanes once that many are done */
    SPLAT_TUNE_TRACE_SPLIT = 8,          /* fused trace step: the rays as 1..4 independent ranges traced on
                                            concurrent streams (steps of at least 2^17 rays; default 2) */
    SPLAT_TUNE_TEST_WAIT_STALL = 9,      /* test only (default 0, off): k > 0 makes the brute-force hitter's wait for
                                            tile k - 1 of every block poll a barrier that nothing completes (64
                                            polls), so each block takes the failure path of its bounded waits:
                                            error bit 1, bounded drain of its copies in flight, early return */
    SPLAT_TUNE_RAY_ORDER = 10,           /* fused trace step, four-wide BVH: 0 secondary rays traced in compaction
                                            order; 4..22 each bounce after the first groups its rays by (direction
                                            octant, BVH position of the triangle they leave), a key of that many
                                            bits, before the hit launch (default 0).  Batch engine (any value
                                            above 0): every tick's rays grouped by (item, BVH position of the
                                            triangle left, octant) before its hit kernel, up to 2^24 buckets
                                            (positions coarsened by one shift when the items' triangles do not
                                            fit) */
    SPLAT_TUNE_BRUTE_TILE = 11,          /* brute-force hitter: hit records per stage of its shared-memory ring,
                                            32, 64 (default) or 128 */
    SPLAT_TUNE_COUNT_WORK = 12,          /* four-wide BVH: 0 (default) plain kernels; 1 counting kernels that add
                                            their traversal work to counters read by splat_hit_work */
    SPLAT_TUNE_BATCH_PERSISTENT = 13,    /* splat_batch_capture: 0 (default) one tick at a time (five launches
                                            per tick); k = 1..8 the whole pass as one persistent cooperative
                                            launch over 1/k of the GPU's resident blocks (k engines replaying
                                            side by side), grid-wide waits between its phases */
    SPLAT_TUNE_KEYS = 14
};
splat_status_t splat_set_tuning(int32_t key, int32_t value);
int32_t splat_get_tuning(int32_t key);

/* Traversal work of the four-wide BVH hitter counted while
 * SPLAT_TUNE_COUNT_WORK is 1, over every device call since the last reset:
 * out[0] nodes visited, out[1] triangle pre-tests (plane distance and the
 * conservative "in front of the ray, before the best hit" test), out[2] full
 * triangle tests (the reference's in_triangle), out[3] rays traced; per ray
 * lane, so a packet's node visit counts once per valid lane.  No counterpart
 * in the reference: it feeds the traversal's instruction-issue roofline.
 * Synchronises the stream; reset != 0 clears the counters after the read. */
splat_status_t splat_hit_work(int64_t out[4], int32_t reset, void* stream);

/* ------------------------------------------------------------- profiling */
/* Launch profiling: while a profile is attached to the calling thread, every
 * kernel libsplat launches from that thread is bracketed by CUDA events on
 * the launch stream, per kernel kind.  splat_profile_read synchronises those
 * events and returns the launch count and summed device time of one kind. */
enum {
    SPLAT_KERNEL_GENERATE = 0,
    SPLAT_KERNEL_HIT_BRUTE = 1,
    SPLAT_KERNEL_HIT_BVH = 2,
    SPLAT_KERNEL_EVOLVE = 3,
    SPLAT_KERNEL_AUX = 4, /* fills, unpacks, conversions, stats, refit, packing */
    SPLAT_KERNEL_SPLAT = 5,
    SPLAT_KERNEL_BATCH = 6, /* one whole batch tick */
    SPLAT_KERNEL_SHADE = 7, /* camera pass: camera rays, light-map / skydome shading, texture uploads */
    SPLAT_KERNEL_KINDS = 8
};
typedef struct splat_profile splat_profile_t;
splat_status_t splat_profile_create(int32_t max_launches, splat_profile_t** out);
splat_status_t splat_profile_attach(splat_profile_t* profile); /* NULL detaches */
splat_status_t splat_profile_read(splat_profile_t* profile, int32_t kind, int64_t* launches, double* total_ms);
splat_status_t splat_profile_reset(splat_profile_t* profile);
splat_status_t splat_profile_destroy(splat_profile_t* profile);

#ifdef __cplusplus
}
#endif

#endif /* SPLAT_H */
