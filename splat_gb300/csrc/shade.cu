// shade.cu -- the camera pass: camera rays, and the light-map / skydome
// shading of the rays the bounce loop retires.
//
//   camera_ray     src/ray_generators.jl:18-50 (rays of one camera grid)
//   shade          shade_tex4_kernel, src/ray_imagers.jl:383-438: per ray and
//                  upscale^2 sub-sample, a diffuse ray sums retina-weighted
//                  light-map texels over the spectrum at its hit's uv, an
//                  escaped ray reads the skydome at its direction's polar
//                  angles; channels clamp to [0, 1]
//
// Textures are the reference's CuTexture objects: 3-D float arrays with
// hardware linear filtering, clamped addressing and unnormalised coordinates,
// sampled at (u, v, plane) - 0.5 (Julia's 1-based texel centres).
#include <cmath>

#include "optics.cuh"

namespace splat {

// ---------------------------------------------------------------------------
// camera rays
// ---------------------------------------------------------------------------

// dir(x, y, dv) of camera_ray and its x / y derivatives.  The reference's
// pixel indices are integers, so the direction is evaluated in double (one
// ForwardDiff partial per pass) and rounded to float once:
//   scale = height cos45 / fov_half_sin, _x = (x - height/2) / scale,
//   _y = (y - width/2) / scale, _z = sqrt((1 - _x^2) - _y^2)
//   dir = ((_x right + _y up) + _z dir) + (dv 0.025f) / max(height, width)
// with d(_x^2) = (p 2) _x and d sqrt(a) = (1 / (2 sqrt a)) p.
__device__ __forceinline__ void camera_dir(const CameraParams& c, int64_t x, int64_t y, F3 dvt, F3& dir, F3& ddx,
                                           F3& ddy) {
    const double scale = ((double)c.h * c.cos45) / (double)c.cam.fov_half_sin;
    const double vx = ((double)x - (double)c.h / 2.0) / scale;
    const double vy = ((double)y - (double)c.w / 2.0) / scale;
    const double px = 1.0 / scale;
    const double py = 1.0 / scale;
    const double vz = sqrt((1.0 - vx * vx) - vy * vy);
    const double dsq = 1.0 / (2.0 * vz);
    const double pzx = (-((px * 2.0) * vx)) * dsq;
    const double pzy = (-((py * 2.0) * vy)) * dsq;
    const float* R = c.cam.right;
    const float* U = c.cam.up;
    const float* Dd = c.cam.dir;
    const float dv[3] = {dvt.x, dvt.y, dvt.z};
    float o[3], ox[3], oy[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double r = R[i], u = U[i], d = Dd[i];
        o[i] = (float)((((vx * r) + (vy * u)) + (vz * d)) + (double)dv[i]);
        ox[i] = (float)((px * r) + (pzx * d));
        oy[i] = (float)((py * u) + (pzy * d));
    }
    dir = {o[0], o[1], o[2]};
    ddx = {ox[0], ox[1], ox[2]};
    ddy = {oy[0], oy[1], oy[2]};
}

// Camera ray g (0-based, column-major over the h x w grid: x = g mod h + 1,
// y = g div h + 1); its jitter dv = three uniforms of Philox(seed) at
// (g, 0, 2, 0).
__device__ __forceinline__ RayState camera_ray(const CameraParams& c, int64_t g) {
    const int64_t x = g % c.h + 1, y = g / c.h + 1;
    const uint4 rnd = philox(make_uint4((uint32_t)g, 0u, 2u, 0u), (uint32_t)c.seed, (uint32_t)(c.seed >> 32));
    const float m = (float)(c.h > c.w ? c.h : c.w);
    const F3 dvt = {(uniform24(rnd.x) * 0.025f) / m, (uniform24(rnd.y) * 0.025f) / m, (uniform24(rnd.z) * 0.025f) / m};
    RayState r;
    r.pos = {c.cam.pos[0], c.cam.pos[1], c.cam.pos[2]};
    const F3 z = {0.0f, 0.0f, 0.0f};
    r.dpl = z;
    r.dpx = z;
    r.dpy = z;
    r.ddl = z;
    camera_dir(c, x, y, dvt, r.dir, r.ddx, r.ddy);
    r.lam = c.lambda;
    r.x = 0.0f;
    r.y = 0.0f;
    r.ignore = 1;
    r.medium = 0;
    return r;
}

__global__ void camera_soa_kernel(CameraParams c, int64_t n, RaySoA out, int64_t* count) {
    const int64_t g0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (g0 == 0) *count = n;
    for (int64_t g = g0; g < n; g += (int64_t)gridDim.x * blockDim.x) store_ray(out, g, camera_ray(c, g), (uint32_t)g);
}

__global__ void camera_aos_kernel(CameraParams c, int64_t n, splat_adray_t* out) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
        const RayState r = camera_ray(c, g);
        splat_adray_t& a = out[g];
        ray_to_aos(a, r, kStatusActive);
        a.dest = g + 1;
    }
}

static int grid_for_rays(int64_t n, int threads, int sm_count, int per_sm) {
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count * per_sm;
    if (b > cap) b = cap;
    return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_camera_soa(const CameraParams& c, int64_t n, RaySoA out, int64_t* count, int sm_count,
                              cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    camera_soa_kernel<<<grid_for_rays(n, 256, sm_count, 8), 256, 0, s>>>(c, n, out, count);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t launch_camera_aos(const CameraParams& c, int64_t n, splat_adray_t* out, int sm_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    camera_aos_kernel<<<grid_for_rays(n, 256, sm_count, 8), 256, 0, s>>>(c, n, out);
    ++g_launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// shading
// ---------------------------------------------------------------------------

// Julia clamp(x, 0, 1): NaN passes through.
__device__ __forceinline__ float clamp01(float x) { return x > 1.0f ? 1.0f : (x < 0.0f ? 0.0f : x); }

__device__ __forceinline__ void put_pixel(const ShadeParams& p, int64_t ray, int i, int j, float R, float G, float B) {
    const int64_t gx = ray % p.cam_h, gy = ray / p.cam_h;
    const int64_t row = (int64_t)p.nd * gx + i, col = (int64_t)p.nd * gy + j;
    float* o = p.rgb + 3 * (row + p.height * col);
    o[0] = clamp01(R);
    o[1] = clamp01(G);
    o[2] = clamp01(B);
}

// Diffuse ray (final-evolved, ignore = its hit triangle): every sub-sample
// sums retina x texel over the spectrum.  tex_uv (src/geo.jl:222-229) of the
// expanded position; a NaN uv skips that wavelength.
__device__ __forceinline__ void shade_diffuse(const ShadeParams& p, const RayState& r, const Tri& T, const TriUV& q,
                                              int64_t ray) {
    const float Wf = (float)p.map_w, Hf = (float)p.map_h;
    for (int i = 0; i < p.nd; ++i) {
        const float xs = r.x + p.deltas[i];
        for (int j = 0; j < p.nd; ++j) {
            const float ys = r.y + p.deltas[j];
            float R = 0.0f, G = 0.0f, B = 0.0f;
            for (int il = 0; il < p.n_lambda; ++il) {
                const F3 pos = p_expansion(r, p.spectrum[il], xs, ys);
                const float bu = dot(q.N, cross(q.e1, pos - T.b)) / q.denom;
                const float bv = dot(q.N, cross(q.e2, pos - T.c)) / q.denom;
                const float bw = (1.0f - bu) - bv;
                const float U = (T.ta.x * bu + T.tb.x * bv) + T.tc.x * bw;
                const float V = (T.ta.y * bu + T.tb.y * bv) + T.tc.y * bw;
                if (isnan(U) || isnan(V)) continue;
                const float X =
                    tex3D<float>(p.map_tex, U * Wf - 0.5f, V * Hf - 0.5f, (float)(il + 1) - 0.5f);
                R = R + p.retina[0][il] * X;
                G = G + p.retina[1][il] * X;
                B = B + p.retina[2][il] * X;
            }
            put_pixel(p, ray, i, j, R, G, B);
        }
    }
}

// Escaped ray: the skydome at theta = acos(dir_z), phi = atan(dir_y, dir_x)
// of each sub-sample's expanded direction, u = theta / pi * sky_w,
// v = ((phi / pi) + 1) / 2 * sky_h.
__device__ __forceinline__ void shade_sky(const ShadeParams& p, const RayState& r, int64_t ray) {
    const float kPi = 3.14159265358979323846f;
    for (int i = 0; i < p.nd; ++i) {
        const float xs = r.x + p.deltas[i];
        for (int j = 0; j < p.nd; ++j) {
            const float ys = r.y + p.deltas[j];
            float R = 0.0f, G = 0.0f, B = 0.0f;
            if (p.has_sky) {
                const F3 d = d_expansion(r, r.lam, xs, ys);
                const float th = acosf(d.z);
                const float ph = atan2f(d.y, d.x);
                const float v = ((ph / kPi) + 1.0f) * 0.5f;
                const float u = th / kPi;
                const float us = u * (float)p.sky_w, vs = v * (float)p.sky_h;
                R = tex3D<float>(p.sky_tex, us - 0.5f, vs - 0.5f, 0.5f);
                G = tex3D<float>(p.sky_tex, us - 0.5f, vs - 0.5f, 1.5f);
                B = tex3D<float>(p.sky_tex, us - 0.5f, vs - 0.5f, 2.5f);
            }
            put_pixel(p, ray, i, j, R, G, B);
        }
    }
}

// Fused form: the diffuse queue (final-evolved) and the sky queue of the
// camera bounce loop, one lane per queued ray.
__global__ void __launch_bounds__(256) shade_diffuse_kernel(RaySoA q, const int64_t* __restrict__ count,
                                                            const splat_ftri_t* __restrict__ tris, ShadeParams p) {
    const int64_t n = *count;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const RayState r = load_ray(q, k);
        const Tri T = load_tri(tris, r.ignore);
        shade_diffuse(p, r, T, tri_uv(T), (int64_t)q.id[k]);
    }
}

__global__ void __launch_bounds__(256) shade_sky_kernel(RaySoA q, const int64_t* __restrict__ count, ShadeParams p) {
    const int64_t n = *count;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        shade_sky(p, load_ray(q, k), (int64_t)q.id[k]);
}

// Plugin form (continuum_shade!): the caller's AoS rays in pixel order after
// run_evolution!; diffuse rays are final-evolved in place first.
__global__ void __launch_bounds__(256) shade_aos_kernel(splat_adray_t* rays, int64_t n,
                                                        const int32_t* __restrict__ hit_idx,
                                                        const splat_ftri_t* __restrict__ tris, int64_t n_tris,
                                                        int32_t* err, ShadeParams p) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int status = rays[k].status;
        if (status == kStatusDiffuse) {
            const int32_t i = hit_idx[k];
            if (i >= 1 && i <= n_tris) {
                const RayState r = ray_from_aos(rays[k]);
                const Tri T = load_tri(tris, i);
                HitDerivs h;
                const int32_t ih = get_hit_ad(r, i, T, h);
                RayState o;
                final_evolution(r, h, ih, o);
                ray_to_aos(rays[k], o, kStatusDiffuse);
                shade_diffuse(p, o, T, tri_uv(T), k);  // tri_view[ray_index]: the hit_idx triangle
                continue;
            }
            atomicOr(err, 16);
        } else if (status == kStatusInfinity) {
            shade_sky(p, ray_from_aos(rays[k]), k);
            continue;
        }
        for (int a = 0; a < p.nd; ++a)
            for (int b = 0; b < p.nd; ++b) put_pixel(p, k, a, b, 0.0f, 0.0f, 0.0f);
    }
}

cudaError_t launch_shade_queues(const RaySoA& dq, const int64_t* d_count, const RaySoA& sq, const int64_t* s_count,
                                const splat_ftri_t* tris, const ShadeParams& p, int64_t cap, int sm_count,
                                cudaStream_t s) {
    if (cap <= 0) return cudaSuccess;
    shade_diffuse_kernel<<<grid_for_rays(cap, 256, sm_count, 8), 256, 0, s>>>(dq, d_count, tris, p);
    ++g_launches;
    shade_sky_kernel<<<grid_for_rays(cap, 256, sm_count, 8), 256, 0, s>>>(sq, s_count, p);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t launch_shade_aos(splat_adray_t* rays, int64_t n, const int32_t* hit_idx, const splat_ftri_t* tris,
                             int64_t n_tris, int32_t* err, const ShadeParams& p, int sm_count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    shade_aos_kernel<<<grid_for_rays(n, 256, sm_count, 8), 256, 0, s>>>(rays, n, hit_idx, tris, n_tris, err, p);
    ++g_launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// light map -> texture array
// ---------------------------------------------------------------------------

// int32 fixed point -> float texels (value / 2^frac_bits) through a surface.
__global__ void map_to_array_kernel(const int32_t* __restrict__ map, int64_t w, int64_t h, int64_t planes,
                                    float inv_scale, cudaSurfaceObject_t surf) {
    const int64_t n = w * h * planes;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = k % w, y = (k / w) % h, z = k / (w * h);
        surf3Dwrite(__int2float_rn(map[k]) * inv_scale, surf, (int)(x * 4), (int)y, (int)z);
    }
}

cudaError_t launch_map_to_array(const int32_t* map, int64_t w, int64_t h, int64_t planes, float inv_scale,
                                cudaSurfaceObject_t surf, int sm_count, cudaStream_t s) {
    const int64_t n = w * h * planes;
    if (n <= 0) return cudaSuccess;
    map_to_array_kernel<<<grid_for_rays(n, 256, sm_count, 16), 256, 0, s>>>(map, w, h, planes, inv_scale, surf);
    ++g_launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// iterations of one frame: out = out (k - 1) / k + rgb / k
// (src/tracer.jl:380-384; the first iteration copies)
// ---------------------------------------------------------------------------
__global__ void image_accumulate_kernel(float* __restrict__ out, const float* __restrict__ rgb, int64_t n, int32_t k) {
    const float kf = (float)k, km = (float)(k - 1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = k == 1 ? rgb[i] : (out[i] * km) / kf + rgb[i] / kf;
}

cudaError_t launch_image_accumulate(float* out, const float* rgb, int64_t n, int32_t k, int sm_count,
                                    cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    image_accumulate_kernel<<<grid_for_rays(n, 256, sm_count, 8), 256, 0, s>>>(out, rgb, n, k);
    ++g_launches;
    return cudaGetLastError();
}

}  // namespace splat
