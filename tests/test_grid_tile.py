"""The first-bounce tiling map (grid_tile_ray, csrc/common.cuh) is a
bijection of the positions 0 .. n - 1 for every grid shape, so that tiling
the first bounce's packets changes only which rays share a warp.  The
header's host form is compiled here and checked on the CPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SOURCE = r'''
#include <cstdio>
#include <vector>
#include "common.cuh"
using namespace splat;
int main() {
    const unsigned cases[][2] = {{1u << 20, 1024}, {1u << 21, 2048}, {135 * 135, 135}, {128 * 131, 131},
                                 {1000, 7}, {5000, 13}, {360 * 640, 360}, {129 * 129 + 5, 129}, {100, 3},
                                 {64, 16}, {1, 1}, {33, 1}, {4 * 8 * 3 + 31, 8}};
    for (auto& c : cases) {
        const unsigned n = c[0], h = c[1];
        std::vector<unsigned char> seen(n, 0);
        for (unsigned p = 0; p < n; ++p) {
            const unsigned k = grid_tile_ray(p, h, n);
            if (k >= n || seen[k]) { std::printf("FAIL n=%u h=%u p=%u k=%u\n", n, h, p, k); return 1; }
            seen[k] = 1;
        }
        // a full 8 x 4 tile: the first 32 positions of a grid of >= 8 rows
        if (h >= 8 && n >= kGridTileCols * h) {
            for (unsigned p = 0; p < 32; ++p) {
                const unsigned k = grid_tile_ray(p, h, n);
                if (k % h != p % 8 || k / h != p / 8) { std::printf("TILE n=%u h=%u p=%u\n", n, h, p); return 1; }
            }
        }
    }
    std::printf("ok\n");
    return 0;
}
'''


def test_grid_tile_ray_is_a_bijection(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    src = tmp_path / "grid_tile_check.cu"
    src.write_text(SOURCE)
    exe = tmp_path / "grid_tile_check"
    inc = os.path.join(ROOT, "splat_gb300", "csrc")
    r = subprocess.run([nvcc, "-O2", "-std=c++17", "-I", inc, "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
