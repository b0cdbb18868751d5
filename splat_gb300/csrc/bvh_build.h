// bvh_build.h -- host BVH build (see bvh_build.cpp).
#pragma once

#include <string>
#include <vector>

#include "kernels.h"

namespace splat {

struct BvhHost {
    std::vector<BvhNode> nodes;
    std::vector<int32_t> order;        // reference index of each BVH-ordered record
    std::vector<int32_t> links;  // refit: parent per node (-1 root), then inner-child count per node
    int depth = 0;
    int max_leaf = 0;
    int64_t leaves = 0;
    float pad_abs = 0.f, pad_rel = 0.f;
    // four-wide tree collapsed from the binary one (same leaves)
    std::vector<Bvh4Node> nodes4;
    std::vector<int32_t> links4;
    int depth4 = 0;
};

bool build_bvh(const splat_ftri_t* tris, int64_t n_tris, BvhHost& out, std::string& err);
void prim_box(const splat_ftri_t& t, float pad_abs, float pad_rel, float lo[3], float hi[3]);

}  // namespace splat
