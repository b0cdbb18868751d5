// lbvh.cu -- BVH rebuild on the GPU for scenes whose geometry changes every
// frame (the reference rebuilds its bounding volumes on the host each frame,
// src/scenes/splash_scene.jl:41, src/bv.jl:68-121).
//
// A linear BVH: triangle centroids are quantised to 10 bits per axis and
// ordered by their Morton code (a stable least-significant-digit radix sort,
// 8 bits per pass); the binary radix tree over the sorted codes is built with
// one thread per inner node (Karras, "Maximizing Parallelism in the
// Construction of BVHs, Octrees, and k-d Trees", HPG 2012, codes made unique
// by appending the sorted position); boxes are merged bottom-up by the second
// thread to reach each node.  Subtrees of at most `leaf_max` triangles become
// leaves (their triangles are contiguous in sorted order), and the tree is
// written in the traversal formats the host builder produces: two-child
// nodes indexed like the radix tree, and four-wide nodes for the inner nodes
// at even depth (each takes its children, or its grandchildren through an
// odd-depth inner child).  Boxes are padded exactly as the host builder pads
// them, so traversal results equal brute force bit for bit.
#include "hitcore.cuh"

namespace splat {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 4;
constexpr int kTile = kSortThreads * kSortItems;  // 1024 keys per tile

__host__ __device__ __forceinline__ int64_t n_tiles_of(int64_t n) { return (n + kTile - 1) / kTile; }

// -------------------------------------------------------------- scan (u32)
// In-place exclusive scan of a[0, m): tiles of 1024 scanned in shared memory,
// the tile sums scanned by one block, then added back.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    if (warp == 0) {
        uint32_t w = lane < nw ? warp_sum[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_sum[lane] = w;
    }
    __syncthreads();
    const uint32_t before = warp ? warp_sum[warp - 1] : 0u;
    if (total) *total = warp_sum[nw - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void scan_tiles_kernel(uint32_t* a, int64_t m, uint32_t* sums) {
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kSortItems;
    uint32_t v[kSortItems];
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        v[j] = base + j < m ? a[base + j] : 0u;
        s += v[j];
    }
    uint32_t tot;
    uint32_t off = block_exclusive_scan(s, &tot);
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        if (base + j < m) a[base + j] = off;
        off += v[j];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan_sums_kernel(uint32_t* sums, int64_t n) {
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < n; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const uint32_t v = i < n ? sums[i] : 0u;
        uint32_t tot;
        const uint32_t off = block_exclusive_scan(v, &tot);
        if (i < n) sums[i] = carry + off;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

__global__ void scan_add_kernel(uint32_t* a, int64_t m, const uint32_t* sums) {
    const uint32_t add = sums[blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * kTile;
    for (int j = threadIdx.x; j < kTile; j += blockDim.x)
        if (base + j < m) a[base + j] += add;
}

cudaError_t scan_u32(uint32_t* a, int64_t m, uint32_t* sums, cudaStream_t s) {
    const int64_t tiles = n_tiles_of(m);
    scan_tiles_kernel<<<(unsigned)tiles, kSortThreads, 0, s>>>(a, m, sums);
    scan_sums_kernel<<<1, 1024, 0, s>>>(sums, tiles);
    scan_add_kernel<<<(unsigned)tiles, kSortThreads, 0, s>>>(a, m, sums);
    g_launches += 3;
    return cudaGetLastError();
}

// ------------------------------------------------------------ radix sort
// Digit histogram of one tile, digit-major: hist[d * tiles + tile].  After an
// exclusive scan of the whole array, hist[d * tiles + tile] is where the
// tile's first key with digit d goes.
__global__ void radix_hist_kernel(const uint32_t* __restrict__ keys, int64_t n, int shift, uint32_t* hist,
                                  int64_t tiles, const int64_t* d_n) {
    __shared__ uint32_t cnt[256];
    if (d_n) n = min(n, *d_n);  // key count on the device (at most n)
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const int64_t i = base + j * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

// Stable scatter: a key's rank among the tile's keys with its digit is the
// count in the tile's earlier passes of the block, in earlier warps of this
// pass, and in earlier lanes of its warp (__match_any_sync peers).
__global__ void radix_scatter_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int64_t n,
                                     int shift, const uint32_t* __restrict__ hist, int64_t tiles, uint32_t* keys_out,
                                     uint32_t* vals_out, const int64_t* d_n) {
    __shared__ uint32_t s_run[256];
    if (d_n) n = min(n, *d_n);
    __shared__ uint32_t s_warp[kSortThreads / 32][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s_run[threadIdx.x] = 0;
    for (int w = 0; w < kSortThreads / 32; ++w) s_warp[w][threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
    const unsigned below = (1u << lane) - 1u;
    for (int j = 0; j < kSortItems; ++j) {
        const int64_t i = base + j * kSortThreads + threadIdx.x;
        const bool valid = i < n;
        const uint32_t key = valid ? keys[i] : 0u;
        const uint32_t d = valid ? (key >> shift) & 255u : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & below);
        if (valid && rank == 0) s_warp[warp][d] = (uint32_t)__popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t before = s_run[d];
            for (int w = 0; w < warp; ++w) before += s_warp[w][d];
            const uint32_t pos = hist[(int64_t)d * tiles + blockIdx.x] + before + (uint32_t)rank;
            keys_out[pos] = key;
            vals_out[pos] = vals[i];
        }
        __syncthreads();
        uint32_t add = 0;
        for (int w = 0; w < kSortThreads / 32; ++w) {
            add += s_warp[w][threadIdx.x];
            s_warp[w][threadIdx.x] = 0;
        }
        s_run[threadIdx.x] += add;
        __syncthreads();
    }
}

// --------------------------------------------------------- Morton codes
// bounds: [0..2] centroid min, [3..5] centroid max (order-preserving u32),
// [6] max |vertex coordinate| (float bits, NaN skipped).
__device__ __forceinline__ float tri_centroid(const float* p, int a) {
    const float l = fminf(fminf(p[a], p[3 + a]), p[6 + a]);
    const float h = fmaxf(fmaxf(p[a], p[3 + a]), p[6 + a]);
    const float c = 0.5f * (l + h);
    return isfinite(c) ? c : 0.0f;
}

__global__ void lbvh_init_kernel(uint32_t* bounds) {
    if (threadIdx.x < 3) {
        bounds[threadIdx.x] = 0xffffffffu;
        bounds[3 + threadIdx.x] = 0u;
    }
    if (threadIdx.x == 3) bounds[6] = 0u;
}

__global__ void lbvh_bounds_kernel(const splat_ftri_t* __restrict__ ftri, int64_t np, uint32_t* bounds) {
    uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u}, m = 0u;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < np; k += (int64_t)gridDim.x * blockDim.x) {
        const float* p = ftri[k + 1].v[1];
        for (int a = 0; a < 3; ++a) {
            const uint32_t u = monotonic_u32(tri_centroid(p, a));
            lo[a] = min(lo[a], u);
            hi[a] = max(hi[a], u);
        }
        for (int v = 0; v < 9; ++v) {
            const float x = fabsf(p[v]);
            if (x == x) m = max(m, __float_as_uint(x));
        }
    }
    for (int o = 16; o; o >>= 1) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
        m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; ++a) {
            atomicMin(&bounds[a], lo[a]);
            atomicMax(&bounds[3 + a], hi[a]);
        }
        atomicMax(&bounds[6], m);
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__global__ void lbvh_morton_kernel(const splat_ftri_t* __restrict__ ftri, int64_t np, const uint32_t* bounds,
                                   uint32_t* keys, uint32_t* vals) {
    float lo[3], ext[3];
    for (int a = 0; a < 3; ++a) {
        lo[a] = monotonic_f32(bounds[a]);
        ext[a] = monotonic_f32(bounds[3 + a]) - lo[a];
    }
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < np; k += (int64_t)gridDim.x * blockDim.x) {
        const float* p = ftri[k + 1].v[1];
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            const float f = ext[a] > 0.0f ? (tri_centroid(p, a) - lo[a]) / ext[a] : 0.5f;
            q[a] = (uint32_t)fminf(fmaxf(f * 1024.0f, 0.0f), 1023.0f);
        }
        keys[k] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
        vals[k] = (uint32_t)k;
    }
}

// ------------------------------------------------------- radix tree
// delta(i, j): common prefix length of the unique 64-bit codes (code, position).
__device__ __forceinline__ int delta(const uint32_t* keys, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = ((uint64_t)keys[i] << 32) | (uint64_t)i;
    const uint64_t b = ((uint64_t)keys[j] << 32) | (uint64_t)j;
    return __clzll((long long)(a ^ b));
}

// Inner node i of n - 1: its key range [first, last], split and children
// (>= 0 inner node, < 0 leaf ~k for sorted triangle k); parent links for
// inner nodes in parent[0, n-1) and for leaves in parent[n-1, 2n-1).
__global__ void lbvh_tree_kernel(const uint32_t* __restrict__ keys, int64_t n, int32_t* parent, int32_t* lch,
                                 int32_t* rch, int32_t* first, int32_t* last) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n - 1; i += (int64_t)gridDim.x * blockDim.x) {
        const int d = delta(keys, n, i, i + 1) > delta(keys, n, i, i - 1) ? 1 : -1;
        const int dmin = delta(keys, n, i, i - d);
        int64_t lmax = 2;
        while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int64_t l = 0;
        for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
        const int64_t j = i + l * d;
        const int dnode = delta(keys, n, i, j);
        int64_t s = 0;
        for (int64_t div = 2;; div <<= 1) {
            const int64_t t = (l + div - 1) / div;
            if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
            if (t <= 1) break;
        }
        const int64_t g = i + s * d + (d < 0 ? -1 : 0);
        const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
        const int32_t left = lo == g ? ~(int32_t)g : (int32_t)g;
        const int32_t right = hi == g + 1 ? ~(int32_t)(g + 1) : (int32_t)(g + 1);
        lch[i] = left;
        rch[i] = right;
        first[i] = (int32_t)lo;
        last[i] = (int32_t)hi;
        parent[left >= 0 ? left : (n - 1) + ~left] = (int32_t)i;
        parent[right >= 0 ? right : (n - 1) + ~right] = (int32_t)i;
        if (i == 0) parent[0] = -1;
    }
}

__device__ __forceinline__ float pad_abs_of(const uint32_t* bounds) {
    return 1.0e-4f * fmaxf(1.0f, __uint_as_float(bounds[6]));
}

// Leaf boxes (the host builder's padded triangle boxes), then each inner
// node's box once both children are done: the second thread to arrive merges.
__global__ void lbvh_boxes_kernel(const splat_ftri_t* __restrict__ ftri, const uint32_t* __restrict__ vals, int64_t n,
                                  const int32_t* __restrict__ parent, const int32_t* __restrict__ lch,
                                  const int32_t* __restrict__ rch, float* box, unsigned* flag,
                                  const uint32_t* bounds) {
    const float pad_abs = pad_abs_of(bounds), pad_rel = 1.0e-3f;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const float* p = ftri[vals[k] + 1].v[1];
        float tl[3], th[3];
        for (int a = 0; a < 3; ++a) {
            tl[a] = fminf(fminf(p[a], p[3 + a]), p[6 + a]);
            th[a] = fmaxf(fmaxf(p[a], p[3 + a]), p[6 + a]);
        }
        const float dx = th[0] - tl[0], dy = th[1] - tl[1], dz = th[2] - tl[2];
        const float pad = pad_abs + pad_rel * sqrtf(dx * dx + dy * dy + dz * dz);
        float* b = box + 6 * ((n - 1) + k);
        for (int a = 0; a < 3; ++a) {
            b[a] = tl[a] - pad;
            b[3 + a] = th[a] + pad;
        }
        int32_t node = n > 1 ? parent[(n - 1) + k] : -1;
        while (node >= 0) {
            __threadfence();
            if (atomicAdd(&flag[node], 1u) == 0u) break;
            const int32_t c0 = lch[node], c1 = rch[node];
            const float* b0 = box + 6 * (c0 >= 0 ? (int64_t)c0 : (n - 1) + ~c0);
            const float* b1 = box + 6 * (c1 >= 0 ? (int64_t)c1 : (n - 1) + ~c1);
            float* bn = box + 6 * (int64_t)node;
            for (int a = 0; a < 3; ++a) {
                bn[a] = fminf(__ldcg(b0 + a), __ldcg(b1 + a));
                bn[3 + a] = fmaxf(__ldcg(b0 + 3 + a), __ldcg(b1 + 3 + a));
            }
            node = parent[node];
        }
    }
}

// Depth of every inner node (parent hops to the root) and the flag of the
// inner nodes that become four-wide nodes: kept (not folded into a leaf) and
// at even depth.
__global__ void lbvh_depth_kernel(const int32_t* __restrict__ parent, const int32_t* __restrict__ first,
                                  const int32_t* __restrict__ last, int64_t n, int leaf_max, uint8_t* odd,
                                  uint32_t* flag4) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n - 1; i += (int64_t)gridDim.x * blockDim.x) {
        int d = 0;
        for (int32_t p = parent[i]; p >= 0 && d < n; p = parent[p]) ++d;
        const bool kept = i == 0 || last[i] - first[i] + 1 > leaf_max;
        odd[i] = (uint8_t)(d & 1);
        flag4[i] = kept && !(d & 1) ? 1u : 0u;
    }
}

__device__ __forceinline__ int leaf_ref(int32_t first, int32_t count) { return ~((first << 4) | (count - 1)); }

struct LbvhView {
    const int32_t *lch, *rch, *first, *last;
    const float* box;
    int64_t n;
    int leaf_max;
};

// A child of an inner node: its box, and whether it is folded into a leaf.
__device__ __forceinline__ const float* child_box(const LbvhView& v, int32_t c) {
    return v.box + 6 * (c >= 0 ? (int64_t)c : (v.n - 1) + ~c);
}
__device__ __forceinline__ bool folded(const LbvhView& v, int32_t c) {
    return c < 0 || v.last[c] - v.first[c] + 1 <= v.leaf_max;
}
__device__ __forceinline__ int folded_ref(const LbvhView& v, int32_t c) {
    return c < 0 ? leaf_ref(~c, 1) : leaf_ref(v.first[c], v.last[c] - v.first[c] + 1);
}

__global__ void lbvh_emit_kernel(LbvhView v, const uint32_t* __restrict__ flag4, const uint32_t* __restrict__ idx4,
                                 BvhNode* nodes2, Bvh4Node* nodes4) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n - 1; i += (int64_t)gridDim.x * blockDim.x) {
        if (i != 0 && folded(v, (int32_t)i)) continue;
        const int32_t c[2] = {v.lch[i], v.rch[i]};
        // two-child node i
        {
            const float* b0 = child_box(v, c[0]);
            const float* b1 = child_box(v, c[1]);
            BvhNode nd;
            nd.x = make_float4(b0[0], b0[3], b1[0], b1[3]);
            nd.y = make_float4(b0[1], b0[4], b1[1], b1[4]);
            nd.z = make_float4(b0[2], b0[5], b1[2], b1[5]);
            nd.c = make_int4(folded(v, c[0]) ? folded_ref(v, c[0]) : c[0], folded(v, c[1]) ? folded_ref(v, c[1]) : c[1],
                             0, 0);
            nodes2[i] = nd;
        }
        if (!flag4[i]) continue;
        // four-wide node: children, or grandchildren through an unfolded child
        float lo[3][4], hi[3][4];
        int ref[4];
        int nc = 0;
        for (int a = 0; a < 2; ++a) {
            if (folded(v, c[a])) {
                const float* b = child_box(v, c[a]);
                for (int x = 0; x < 3; ++x) {
                    lo[x][nc] = b[x];
                    hi[x][nc] = b[3 + x];
                }
                ref[nc++] = folded_ref(v, c[a]);
                continue;
            }
            const int32_t g[2] = {v.lch[c[a]], v.rch[c[a]]};
            for (int e = 0; e < 2; ++e) {
                const float* b = child_box(v, g[e]);
                for (int x = 0; x < 3; ++x) {
                    lo[x][nc] = b[x];
                    hi[x][nc] = b[3 + x];
                }
                ref[nc++] = folded(v, g[e]) ? folded_ref(v, g[e]) : (int)idx4[g[e]];
            }
        }
        for (int s = nc; s < 4; ++s) {  // empty slots: a box no ray enters
            for (int x = 0; x < 3; ++x) {
                lo[x][s] = __int_as_float(0x7f800000);
                hi[x][s] = -__int_as_float(0x7f800000);
            }
            ref[s] = ref[0];
        }
        Bvh4Node q;
        q.lox = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
        q.hix = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
        q.loy = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
        q.hiy = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
        q.loz = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
        q.hiz = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
        q.c = make_int4(ref[0], ref[1], ref[2], ref[3]);
        q.meta = make_int4(nc, 0, 0, 0);
        nodes4[idx4[i]] = q;
    }
}

// A single triangle: both trees are a root whose two children are that leaf.
__global__ void lbvh_single_kernel(const float* box, BvhNode* nodes2, Bvh4Node* nodes4) {
    const float* b = box;
    BvhNode nd;
    nd.x = make_float4(b[0], b[3], b[0], b[3]);
    nd.y = make_float4(b[1], b[4], b[1], b[4]);
    nd.z = make_float4(b[2], b[5], b[2], b[5]);
    nd.c = make_int4(leaf_ref(0, 1), leaf_ref(0, 1), 0, 0);
    nodes2[0] = nd;
    const float inf = __int_as_float(0x7f800000);  // slots 2 and 3 empty
    Bvh4Node q;
    q.lox = make_float4(b[0], b[0], inf, inf);
    q.hix = make_float4(b[3], b[3], -inf, -inf);
    q.loy = make_float4(b[1], b[1], inf, inf);
    q.hiy = make_float4(b[4], b[4], -inf, -inf);
    q.loz = make_float4(b[2], b[2], inf, inf);
    q.hiz = make_float4(b[5], b[5], -inf, -inf);
    q.c = make_int4(leaf_ref(0, 1), leaf_ref(0, 1), leaf_ref(0, 1), leaf_ref(0, 1));
    q.meta = make_int4(2, 0, 0, 0);
    nodes4[0] = q;
}

__global__ void lbvh_order_kernel(const uint32_t* __restrict__ vals, int64_t n, int32_t* order) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        order[k] = (int32_t)vals[k] + 2;
}

struct Carve {
    char* p;
    template <class T>
    T* take(int64_t count) {
        T* r = reinterpret_cast<T*>(p);
        p += ((size_t)count * sizeof(T) + 255) / 256 * 256;
        return r;
    }
};

}  // namespace

size_t lbvh_scratch_bytes(int64_t np) {
    if (np < 1) return 256;
    const int64_t tiles = n_tiles_of(np), inner = np > 1 ? np - 1 : 1;
    const int64_t m_hist = 256 * tiles, sum_tiles = n_tiles_of(m_hist > inner ? m_hist : inner);
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    return 256 + 4 * al(4 * (size_t)np) + al(4 * (size_t)m_hist) + al(4 * (size_t)sum_tiles) + al(4 * 8) +
           al(4 * (size_t)(2 * np)) + 4 * al(4 * (size_t)inner) + al(4 * 6 * (size_t)(2 * np)) + al(4 * (size_t)inner) +
           al((size_t)inner) + 2 * al(4 * (size_t)inner);
}

cudaError_t launch_lbvh_build(const splat_ftri_t* ftri, int64_t n_tris, int leaf_max, void* scratch,
                              BvhNode* nodes2, Bvh4Node* nodes4, int32_t* order, int sm_count, cudaStream_t s) {
    const int64_t n = n_tris - 1;  // the sentinel (index 1) is never hit
    if (n < 1) return cudaSuccess;
    const int64_t tiles = n_tiles_of(n), inner = n > 1 ? n - 1 : 1;
    const int64_t m_hist = 256 * tiles;
    Carve c{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(scratch) + 255) / 256 * 256)};
    uint32_t* keys[2] = {c.take<uint32_t>(n), c.take<uint32_t>(n)};
    uint32_t* vals[2] = {c.take<uint32_t>(n), c.take<uint32_t>(n)};
    uint32_t* hist = c.take<uint32_t>(m_hist);
    uint32_t* sums = c.take<uint32_t>(n_tiles_of(m_hist > inner ? m_hist : inner));
    uint32_t* bounds = c.take<uint32_t>(8);
    int32_t* parent = c.take<int32_t>(2 * n);
    int32_t* lch = c.take<int32_t>(inner);
    int32_t* rch = c.take<int32_t>(inner);
    int32_t* first = c.take<int32_t>(inner);
    int32_t* last = c.take<int32_t>(inner);
    float* box = c.take<float>(6 * (2 * n));
    unsigned* flag = c.take<unsigned>(inner);
    uint8_t* odd = c.take<uint8_t>(inner);
    uint32_t* flag4 = c.take<uint32_t>(inner);
    uint32_t* idx4 = c.take<uint32_t>(inner);

    auto grid = [&](int64_t items) {
        int64_t b = (items + 255) / 256;
        const int64_t cap = (int64_t)sm_count * 8;
        return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
    };
    cudaError_t e;
    lbvh_init_kernel<<<1, 32, 0, s>>>(bounds);
    lbvh_bounds_kernel<<<grid(n), 256, 0, s>>>(ftri, n, bounds);
    lbvh_morton_kernel<<<grid(n), 256, 0, s>>>(ftri, n, bounds, keys[0], vals[0]);
    g_launches += 3;
    int cur = 0;
    for (int shift = 0; shift < 32; shift += 8) {
        radix_hist_kernel<<<(unsigned)tiles, kSortThreads, 0, s>>>(keys[cur], n, shift, hist, tiles, nullptr);
        ++g_launches;
        if ((e = scan_u32(hist, m_hist, sums, s)) != cudaSuccess) return e;
        radix_scatter_kernel<<<(unsigned)tiles, kSortThreads, 0, s>>>(keys[cur], vals[cur], n, shift, hist, tiles,
                                                                      keys[cur ^ 1], vals[cur ^ 1], nullptr);
        ++g_launches;
        cur ^= 1;
    }
    if ((e = cudaMemsetAsync(flag, 0, sizeof(unsigned) * (size_t)inner, s)) != cudaSuccess) return e;
    if (n > 1) {
        lbvh_tree_kernel<<<grid(n - 1), 256, 0, s>>>(keys[cur], n, parent, lch, rch, first, last);
        ++g_launches;
    }
    lbvh_boxes_kernel<<<grid(n), 256, 0, s>>>(ftri, vals[cur], n, parent, lch, rch, box, flag, bounds);
    ++g_launches;
    if (n == 1) {
        lbvh_single_kernel<<<1, 1, 0, s>>>(box, nodes2, nodes4);
        ++g_launches;
    } else {
        lbvh_depth_kernel<<<grid(n - 1), 256, 0, s>>>(parent, first, last, n, leaf_max, odd, flag4);
        if ((e = cudaMemcpyAsync(idx4, flag4, sizeof(uint32_t) * (size_t)(n - 1), cudaMemcpyDeviceToDevice, s)) !=
            cudaSuccess)
            return e;
        ++g_launches;
        if ((e = scan_u32(idx4, n - 1, sums, s)) != cudaSuccess) return e;
        LbvhView v{lch, rch, first, last, box, n, leaf_max};
        lbvh_emit_kernel<<<grid(n - 1), 256, 0, s>>>(v, flag4, idx4, nodes2, nodes4);
        ++g_launches;
    }
    lbvh_order_kernel<<<grid(n), 256, 0, s>>>(vals[cur], n, order);
    ++g_launches;
    return cudaGetLastError();
}

// ---------------------------------------------------------- ray order
// A counting sort of the active rays by key: the direction octant above the
// BVH-order position of the triangle the ray leaves (ignore_tri), the
// position's low bits dropped so that the key has key_bits bits.  Bucket
// sizes are counted with global atomics, scanned into offsets, and every ray
// takes a slot in its bucket with one atomic per group of equal keys in a
// warp (__match_any_sync), so a warp's rays of one bucket stay together.
// The order inside a bucket is the atomics' order: only which rays share a
// warp changes with it, never a result.
constexpr int kOrderMaxBits = 22;
constexpr int kDirClasses = 8, kDirBits = 3;  // direction octants

__device__ __forceinline__ uint32_t ray_key(const float* __restrict__ f, int64_t cap, const int32_t* __restrict__ ignore,
                                            const int32_t* __restrict__ bvh_pos, int64_t n_tris, int pos_shift,
                                            uint32_t n_pos, int64_t k) {
    const uint32_t cls = (f[3 * cap + k] < 0.0f ? 1u : 0u) | (f[4 * cap + k] < 0.0f ? 2u : 0u) |
                         (f[5 * cap + k] < 0.0f ? 4u : 0u);
    const int32_t ig = ignore[k];
    const uint32_t pos = (ig >= 1 && (int64_t)ig <= n_tris) ? (uint32_t)bvh_pos[ig] : 0u;
    return cls * n_pos + (pos >> pos_shift);
}

// Bucket sizes: one atomic per group of equal keys in a warp.
__global__ void ray_bucket_count_kernel(const float* __restrict__ f, int64_t cap, const int32_t* __restrict__ ignore,
                                        const int64_t* __restrict__ d_count, const int32_t* __restrict__ bvh_pos,
                                        int64_t n_tris, int pos_shift, uint32_t n_pos, uint32_t* keys,
                                        uint32_t* cnt) {
    const int64_t n = min(cap, *d_count);
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride) {
        const int64_t k = base + lane;
        const bool valid = k < n;
        const uint32_t key = valid ? ray_key(f, cap, ignore, bvh_pos, n_tris, pos_shift, n_pos, k) : 0xffffffffu;
        if (valid) keys[k] = key;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (valid && lane == __ffs(peers) - 1) atomicAdd(&cnt[key], (uint32_t)__popc(peers));
    }
}

__global__ void ray_bucket_place_kernel(const uint32_t* __restrict__ keys, int64_t cap,
                                        const int64_t* __restrict__ d_count, uint32_t* off, int32_t* perm) {
    const int64_t n = min(cap, *d_count);
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // warp-uniform trip count: every lane takes part in the vote
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < n; base += stride) {
        const int64_t k = base + lane;
        const bool valid = k < n;
        const uint32_t key = valid ? keys[k] : 0xffffffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        uint32_t slot = 0;
        if (valid && lane == leader) slot = atomicAdd(&off[key], (uint32_t)__popc(peers));
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (valid) perm[slot + (uint32_t)__popc(peers & below)] = (int32_t)k;
    }
}

size_t ray_order_bytes(int64_t cap) {
    if (cap < 1) return 256;
    const int64_t buckets = int64_t(1) << kOrderMaxBits;
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    return 256 + 2 * al(4 * (size_t)cap) + al(4 * (size_t)buckets) + al(4 * (size_t)n_tiles_of(buckets));
}

cudaError_t launch_ray_order(const float* soa_f, const int32_t* ignore, int64_t cap, const int64_t* d_count,
                             const int32_t* bvh_pos, int64_t n_tris, int key_bits, void* scratch,
                             const int32_t** perm_out, int sm_count, cudaStream_t s) {
    if (cap < 1) return cudaSuccess;
    if (key_bits < 4) key_bits = 4;
    if (key_bits > kOrderMaxBits) key_bits = kOrderMaxBits;
    Carve c{reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(scratch) + 255) / 256 * 256)};
    uint32_t* keys = c.take<uint32_t>(cap);
    int32_t* perm = c.take<int32_t>(cap);
    uint32_t* cnt = c.take<uint32_t>(int64_t(1) << kOrderMaxBits);
    uint32_t* sums = c.take<uint32_t>(n_tiles_of(int64_t(1) << kOrderMaxBits));
    // positions 0 .. n_tris - 2 (the records); keep the high bits that fit
    int full_bits = 1;
    while (full_bits < 31 && (int64_t(1) << full_bits) < n_tris + 1) ++full_bits;
    const int pos_bits = full_bits < key_bits - kDirBits ? full_bits : key_bits - kDirBits;
    const int pos_shift = full_bits - pos_bits;
    const uint32_t n_pos = (uint32_t)((n_tris >> pos_shift) + 1);  // positions after the shift, all < n_pos
    const int64_t buckets = kDirClasses * (int64_t)n_pos;           // <= 2^key_bits
    int64_t b = (cap + 255) / 256;
    if (b > (int64_t)sm_count * 8) b = (int64_t)sm_count * 8;
    if (b < 1) b = 1;
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (size_t)buckets, s);
    if (e != cudaSuccess) return e;
    ray_bucket_count_kernel<<<(unsigned)b, 256, 0, s>>>(soa_f, cap, ignore, d_count, bvh_pos, n_tris, pos_shift,
                                                        n_pos, keys, cnt);
    ++g_launches;
    if ((e = scan_u32(cnt, buckets, sums, s)) != cudaSuccess) return e;
    // one block per 256 rays (blocks start in index order), so a bucket's
    // slots go to its rays nearly in position order: the input order carries
    // the first bounce's tiles
    const int64_t bp = (cap + 255) / 256;
    ray_bucket_place_kernel<<<(unsigned)(bp < 1 ? 1 : bp), 256, 0, s>>>(keys, cap, d_count, cnt, perm);
    ++g_launches;
    *perm_out = perm;
    return cudaGetLastError();
}

size_t order_sums_count(int64_t buckets) { return (size_t)n_tiles_of(buckets < 1 ? 1 : buckets); }

cudaError_t launch_order_scan(uint32_t* cnt, int64_t buckets, uint32_t* sums, cudaStream_t s) {
    if (buckets < 1) return cudaSuccess;
    return scan_u32(cnt, buckets, sums, s);
}

}  // namespace splat
