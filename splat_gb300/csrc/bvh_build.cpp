// bvh_build.cpp -- host build of the flattened BVH2 the BVH hitter walks.
//
// Replaces the reference's one-level bounding-volume "shrub" (bv_partition /
// spatial_partition / pack_bv_tris, src/bv.jl:68-136: 2^d median-split
// leaf boxes, triangles duplicated across leaves) with a binned-SAH binary
// BVH (32 bins per axis on triangle centroids, leaves of at most 16
// triangles, object-median splits when centroids coincide), flattened in
// depth-first order into two-child nodes.
//
// Conservativeness.  The hit test accepts p = o + d t by barycentrics
// computed in binary32, so an accepted p can lie a few ulps outside the exact
// triangle.  Every triangle box is therefore padded by
//   pad = pad_abs + pad_rel * |box diagonal|,
//   pad_abs = 1e-4 * max(1, max |coordinate|),  pad_rel = 1e-3,
// orders of magnitude above that rounding band, and traversal keeps every
// node whose padded box the ray enters at or before the current best t.  The
// BVH hitter therefore tests every triangle whose test can succeed at
// t <= best, and with the lexicographic (t, index) rule returns exactly the
// brute-force result.  (Compiled with -ffp-contract=off like the device
// refit, so both compute the same padded boxes.)
#include "bvh_build.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>

namespace splat {

namespace {

constexpr int kBins = 32;
constexpr int kSahLeaf = 8;
constexpr int kMaxDepth = 56;

struct Prim {
    float lo[3], hi[3], c[3];
    int32_t idx;
};

struct Box {
    float lo[3], hi[3];
    Box() {
        for (int a = 0; a < 3; ++a) {
            lo[a] = INFINITY;
            hi[a] = -INFINITY;
        }
    }
    void grow(const float l[3], const float h[3]) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], l[a]);
            hi[a] = std::max(hi[a], h[a]);
        }
    }
    void grow(const Box& b) { grow(b.lo, b.hi); }
    float area() const {
        float d[3];
        for (int a = 0; a < 3; ++a) d[a] = std::max(0.0f, hi[a] - lo[a]);
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

struct BNode {
    Box box;
    int32_t left = -1, right = -1;
    int32_t first = 0, count = 0;  // leaf when count > 0
};

struct Builder {
    std::vector<Prim>& P;
    std::vector<BNode> nodes;
    int max_depth = 0;

    explicit Builder(std::vector<Prim>& p) : P(p) {}

    int make_leaf(int b, int e, const Box& box) {
        BNode n;
        n.box = box;
        n.first = b;
        n.count = e - b;
        nodes.push_back(n);
        return (int)nodes.size() - 1;
    }

    int build(int b, int e, int depth) {
        max_depth = std::max(max_depth, depth);
        Box box, cbox;
        for (int i = b; i < e; ++i) {
            box.grow(P[i].lo, P[i].hi);
            cbox.grow(P[i].c, P[i].c);
        }
        const int n = e - b;
        if (n <= 2 && depth > 0) return make_leaf(b, e, box);
        int mid = -1;
        float best_cost = INFINITY;
        int best_axis = -1, best_split = -1;
        for (int a = 0; a < 3; ++a) {
            const float ext = cbox.hi[a] - cbox.lo[a];
            if (!(ext > 0.0f)) continue;
            Box bins[kBins];
            int cnt[kBins] = {0};
            const float scale = (float)kBins / ext;
            for (int i = b; i < e; ++i) {
                int k = (int)((P[i].c[a] - cbox.lo[a]) * scale);
                k = std::min(std::max(k, 0), kBins - 1);
                cnt[k]++;
                bins[k].grow(P[i].lo, P[i].hi);
            }
            float rarea[kBins];
            int rcnt[kBins];
            Box acc;
            int ac = 0;
            for (int k = kBins - 1; k > 0; --k) {
                acc.grow(bins[k]);
                ac += cnt[k];
                rarea[k] = acc.area();
                rcnt[k] = ac;
            }
            Box lacc;
            int lc = 0;
            for (int k = 0; k < kBins - 1; ++k) {
                lacc.grow(bins[k]);
                lc += cnt[k];
                if (lc == 0 || rcnt[k + 1] == 0) continue;
                const float cost = lacc.area() * (float)lc + rarea[k + 1] * (float)rcnt[k + 1];
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = a;
                    best_split = k;
                }
            }
        }
        const float parea = box.area();
        const bool sah_leaf = best_axis < 0 || (parea > 0.0f && 1.0f + best_cost / parea >= (float)n);
        if (depth > 0 && n <= kSahLeaf && sah_leaf) return make_leaf(b, e, box);
        if (depth >= kMaxDepth && n <= kLeafMax) return make_leaf(b, e, box);
        if (best_axis >= 0 && depth < kMaxDepth) {
            const float ext = cbox.hi[best_axis] - cbox.lo[best_axis];
            const float scale = (float)kBins / ext;
            Prim* it = std::partition(P.data() + b, P.data() + e, [&](const Prim& p) {
                int k = (int)((p.c[best_axis] - cbox.lo[best_axis]) * scale);
                k = std::min(std::max(k, 0), kBins - 1);
                return k <= best_split;
            });
            mid = (int)(it - P.data());
        }
        if (mid <= b || mid >= e) {
            // coincident centroids (or depth cap): object median by index
            mid = b + n / 2;
            std::nth_element(P.data() + b, P.data() + mid, P.data() + e,
                             [](const Prim& x, const Prim& y) { return x.idx < y.idx; });
        }
        const int me = (int)nodes.size();
        nodes.push_back(BNode());
        nodes[me].box = box;
        const int l = build(b, mid, depth + 1);
        const int r = build(mid, e, depth + 1);
        nodes[me].left = l;
        nodes[me].right = r;
        return me;
    }
};

}  // namespace

void prim_box(const splat_ftri_t& t, float pad_abs, float pad_rel, float lo[3], float hi[3]) {
    float tl[3], th[3];
    for (int a = 0; a < 3; ++a) {
        tl[a] = std::fmin(std::fmin(t.v[1][a], t.v[2][a]), t.v[3][a]);
        th[a] = std::fmax(std::fmax(t.v[1][a], t.v[2][a]), t.v[3][a]);
    }
    const float dx = th[0] - tl[0], dy = th[1] - tl[1], dz = th[2] - tl[2];
    const float pad = pad_abs + pad_rel * std::sqrt(dx * dx + dy * dy + dz * dz);
    for (int a = 0; a < 3; ++a) {
        lo[a] = tl[a] - pad;
        hi[a] = th[a] + pad;
    }
}

bool build_bvh(const splat_ftri_t* tris, int64_t n_tris, BvhHost& out, std::string& err) {
    out = BvhHost();
    const int64_t np = n_tris - 1;  // the sentinel (index 1) is never hit
    if (np <= 0) return true;
    if (np >= (int64_t(1) << 27)) {
        err = "BVH supports at most 2^27 triangles";
        return false;
    }
    float M = 1.0f;
    for (int64_t j = 1; j < n_tris; ++j)
        for (int v = 1; v < 4; ++v)
            for (int a = 0; a < 3; ++a) M = std::max(M, std::fabs(tris[j].v[v][a]));
    out.pad_abs = 1.0e-4f * M;
    out.pad_rel = 1.0e-3f;

    std::vector<Prim> P((size_t)np);
    for (int64_t j = 0; j < np; ++j) {
        const splat_ftri_t& t = tris[j + 1];
        Prim& p = P[(size_t)j];
        prim_box(t, out.pad_abs, out.pad_rel, p.lo, p.hi);
        for (int a = 0; a < 3; ++a) {
            const float l = std::fmin(std::fmin(t.v[1][a], t.v[2][a]), t.v[3][a]);
            const float h = std::fmax(std::fmax(t.v[1][a], t.v[2][a]), t.v[3][a]);
            p.c[a] = 0.5f * (l + h);
            if (!std::isfinite(p.c[a])) p.c[a] = 0.0f;
        }
        p.idx = (int32_t)(j + 2);
    }
    Builder B(P);
    if (np == 1) {
        // a lone triangle: root with the same one-triangle leaf on both sides
        BNode root, leaf;
        leaf.first = 0;
        leaf.count = 1;
        leaf.box.grow(P[0].lo, P[0].hi);
        B.nodes.push_back(root);
        B.nodes.push_back(leaf);
        B.nodes[0].box = leaf.box;
        B.nodes[0].left = 1;
        B.nodes[0].right = 1;
    } else {
        B.build(0, (int)np, 0);
    }

    // flatten depth first: one BvhNode per inner BNode
    std::vector<int32_t> flat_of(B.nodes.size(), -1);
    std::vector<int32_t> depth_of;
    struct Item {
        int bnode, depth;
    };
    std::vector<Item> stack{{0, 0}};
    std::vector<int> order_inner;
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        const BNode& bn = B.nodes[(size_t)it.bnode];
        flat_of[(size_t)it.bnode] = (int32_t)order_inner.size();
        order_inner.push_back(it.bnode);
        depth_of.push_back(it.depth);
        if (B.nodes[(size_t)bn.right].count == 0) stack.push_back({bn.right, it.depth + 1});
        if (B.nodes[(size_t)bn.left].count == 0) stack.push_back({bn.left, it.depth + 1});
    }
    auto ref_of = [&](int c) -> int32_t {
        const BNode& bn = B.nodes[(size_t)c];
        if (bn.count == 0) return flat_of[(size_t)c];
        int64_t first = bn.first;
        int count = bn.count;
        const uint32_t enc = (uint32_t)((first << 4) | (int64_t)(count - 1));
        return (int32_t)~enc;
    };
    out.nodes.resize(order_inner.size());
    int max_leaf = 0;
    int64_t leaves = 0;
    for (size_t q = 0; q < order_inner.size(); ++q) {
        const BNode& bn = B.nodes[(size_t)order_inner[q]];
        const BNode& L = B.nodes[(size_t)bn.left];
        const BNode& R = B.nodes[(size_t)bn.right];
        for (const BNode* c : {&L, &R})
            if (c->count > 0) {
                max_leaf = std::max(max_leaf, c->count);
                ++leaves;
            }
        if (L.count > kLeafMax || R.count > kLeafMax) {
            err = "BVH leaf larger than 16 triangles";
            return false;
        }
        BvhNode& f = out.nodes[q];
        f.x = make_float4(L.box.lo[0], L.box.hi[0], R.box.lo[0], R.box.hi[0]);
        f.y = make_float4(L.box.lo[1], L.box.hi[1], R.box.lo[1], R.box.hi[1]);
        f.z = make_float4(L.box.lo[2], L.box.hi[2], R.box.lo[2], R.box.hi[2]);
        f.c = make_int4(ref_of(bn.left), ref_of(bn.right), 0, 0);
    }
    out.order.resize((size_t)np);
    for (int64_t j = 0; j < np; ++j) out.order[(size_t)j] = P[(size_t)j].idx;

    int maxd = 0;
    for (int d : depth_of) maxd = std::max(maxd, d);
    out.depth = maxd + 1;
    // refit links: parent of each node, then its number of inner children
    out.links.assign(2 * out.nodes.size(), 0);
    out.links[0] = -1;
    for (size_t q = 0; q < out.nodes.size(); ++q)
        for (int c : {out.nodes[q].c.x, out.nodes[q].c.y})
            if (c >= 0 && c != (int)q) {
                out.links[(size_t)c] = (int32_t)q;
                out.links[out.nodes.size() + q] += 1;
            }
    if (out.depth + 1 >= kBvhStack) {
        err = "BVH deeper than the traversal stack";
        return false;
    }
    out.max_leaf = max_leaf;
    out.leaves = leaves;

    // Collapse into a four-wide tree: starting from a binary node's two
    // children, repeatedly open the inner child with the largest surface area
    // until four children are reached or only leaves remain.
    std::vector<int> depth4_of;
    std::function<int(int, int)> emit = [&](int b, int depth) -> int {
        std::vector<int> ch = {B.nodes[(size_t)b].left, B.nodes[(size_t)b].right};
        while (ch.size() < 4) {
            int pick = -1;
            float best_area = -1.0f;
            for (size_t i = 0; i < ch.size(); ++i) {
                const BNode& c = B.nodes[(size_t)ch[i]];
                if (c.count == 0 && c.box.area() > best_area) {
                    best_area = c.box.area();
                    pick = (int)i;
                }
            }
            if (pick < 0) break;
            const int c = ch[(size_t)pick];
            ch.erase(ch.begin() + pick);
            ch.push_back(B.nodes[(size_t)c].left);
            ch.push_back(B.nodes[(size_t)c].right);
        }
        const int me = (int)out.nodes4.size();
        out.nodes4.emplace_back();
        depth4_of.push_back(depth);
        int refs[4] = {0, 0, 0, 0};
        for (size_t i = 0; i < ch.size(); ++i)
            refs[i] = B.nodes[(size_t)ch[i]].count > 0 ? ref_of(ch[i]) : emit(ch[i], depth + 1);
        Bvh4Node& f = out.nodes4[(size_t)me];
        float lo[3][4], hi[3][4];
        for (int a = 0; a < 3; ++a)
            for (int i = 0; i < 4; ++i) {
                lo[a][i] = INFINITY;
                hi[a][i] = -INFINITY;
            }
        for (size_t i = 0; i < ch.size(); ++i)
            for (int a = 0; a < 3; ++a) {
                lo[a][i] = B.nodes[(size_t)ch[i]].box.lo[a];
                hi[a][i] = B.nodes[(size_t)ch[i]].box.hi[a];
            }
        f.lox = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
        f.hix = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
        f.loy = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
        f.hiy = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
        f.loz = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
        f.hiz = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
        f.c = make_int4(refs[0], refs[1], refs[2], refs[3]);
        f.meta = make_int4((int)ch.size(), 0, 0, 0);
        return me;
    };
    emit(0, 0);
    int maxd4 = 0;
    for (int d : depth4_of) maxd4 = std::max(maxd4, d);
    out.depth4 = maxd4 + 1;
    out.links4.assign(2 * out.nodes4.size(), 0);
    out.links4[0] = -1;
    for (size_t q = 0; q < out.nodes4.size(); ++q) {
        const Bvh4Node& f = out.nodes4[q];
        const int refs[4] = {f.c.x, f.c.y, f.c.z, f.c.w};
        for (int i = 0; i < f.meta.x; ++i)
            if (refs[i] >= 0) {
                out.links4[(size_t)refs[i]] = (int32_t)q;
                out.links4[out.nodes4.size() + q] += 1;
            }
    }
    if (3 * out.depth4 + 1 >= kBvhStack) {
        err = "four-wide BVH deeper than the traversal stack";
        return false;
    }
    return true;
}

}  // namespace splat
