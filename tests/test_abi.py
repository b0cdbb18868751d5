"""The C ABI without a GPU: libsplat.so loads, exports every function
include/splat.h declares, and the ctypes records match the header's layout
(checked by compiling a C program against the header)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from splat_gb300 import _lib as L
from splat_gb300 import types as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "splat.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(splat_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = L.load()
    declared = header_functions()
    assert len(declared) >= 15
    missing = [f for f in declared if not hasattr(lib, f)]
    assert not missing, f"not exported: {missing}"
    assert set(declared) == set(L.SIGNATURES), "ctypes signatures out of sync with the header"
    assert lib.splat_abi_version() == 1


LAYOUT_C = r"""
#include <stddef.h>
#include <stdio.h>
#include "splat.h"
#define P(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  P(splat_adray_t) P(splat_ftri_t) P(splat_ntri_t) P(splat_rect_light_t) P(splat_material_t)
  P(splat_lambda_mode_t) P(splat_trace_params_t) P(splat_trace_stats_t) P(splat_scene_info_t)
  O(splat_adray_t, in_medium) O(splat_adray_t, ignore_tri) O(splat_adray_t, dest) O(splat_adray_t, lambda)
  O(splat_adray_t, status)
  O(splat_trace_params_t, upscale) O(splat_trace_params_t, seed) O(splat_trace_params_t, material)
  O(splat_trace_params_t, force_rand) O(splat_trace_params_t, spectrum) O(splat_trace_params_t, map_w)
  O(splat_trace_params_t, accum) O(splat_trace_params_t, ray_begin) O(splat_trace_params_t, ray_end)
  O(splat_scene_info_t, device_bytes) O(splat_scene_info_t, bvh_pad)
  P(splat_camera_t) P(splat_render_params_t)
  O(splat_camera_t, right) O(splat_camera_t, fov_half_sin)
  O(splat_render_params_t, height) O(splat_render_params_t, seed) O(splat_render_params_t, material)
  O(splat_render_params_t, lambda) O(splat_render_params_t, spectrum) O(splat_render_params_t, retina)
  return 0;
}
"""


def c_layout():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(src, "w").write(LAYOUT_C)
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


def test_record_layouts_match_header():
    c = c_layout()
    # Julia isbits layouts of the reference (src/geo.jl:60-76, :18; src/ray_generators.jl:4-11)
    assert c["splat_adray_t"] == 136 == T.ADRAY.itemsize
    assert c["splat_adray_t.ignore_tri"] == 104 and c["splat_adray_t.dest"] == 112
    assert c["splat_adray_t.lambda"] == 120 and c["splat_adray_t.status"] == 132
    assert c["splat_ftri_t"] == T.FTRI_BYTES
    assert c["splat_ntri_t"] == 52
    assert c["splat_rect_light_t"] == 64 == T.RECT_LIGHT.itemsize
    for name, cls in [("splat_trace_params_t", L.TraceParams), ("splat_trace_stats_t", L.TraceStats),
                      ("splat_scene_info_t", L.SceneInfo), ("splat_material_t", L.Material),
                      ("splat_lambda_mode_t", L.LambdaMode), ("splat_rect_light_t", L.RectLight)]:
        assert c[name] == C.sizeof(cls), name
    for f in ["upscale", "seed", "material", "force_rand", "spectrum", "map_w", "accum", "ray_begin", "ray_end"]:
        assert c[f"splat_trace_params_t.{f}"] == getattr(L.TraceParams, f).offset, f
    assert c["splat_scene_info_t.bvh_pad"] == L.SceneInfo.bvh_pad.offset
    for f, off in [("in_medium", 96), ("ignore_tri", 104), ("dest", 112), ("lam", 120), ("status", 132)]:
        assert T.ADRAY.fields[f][1] == off
    # Cam (src/geo.jl:50-57): five R3 and a Float32
    assert c["splat_camera_t"] == 64 == C.sizeof(L.Camera)
    assert c["splat_camera_t.right"] == 48 and c["splat_camera_t.fov_half_sin"] == 60
    assert c["splat_render_params_t"] == C.sizeof(L.RenderParams)
    for f in ["height", "seed", "material", "spectrum", "retina"]:
        assert c[f"splat_render_params_t.{f}"] == getattr(L.RenderParams, f).offset, f
    assert c["splat_render_params_t.lambda"] == L.RenderParams.lambda_.offset


def test_invalid_arguments_fail_cleanly_without_gpu():
    """Argument validation happens before any CUDA call."""
    lib = L.load()
    P = L.TraceParams()
    rc = lib.splat_trace_forward(None, C.byref(P), None, None, 0, None, None)
    assert rc == L.ERR_INVALID
    assert b"null" in lib.splat_last_error()
    rc = lib.splat_scene_create(None, 0, 2, 0, None, None)
    assert rc == L.ERR_INVALID
    assert lib.splat_trace_workspace_size(1000) > 1000 * 117 * 2
    with pytest.raises(L.SplatError):
        L.check(L.ERR_INVALID)


def test_tuning_knobs_validate_and_round_trip_without_gpu():
    """splat_set_tuning / splat_get_tuning are host-only: ranges are checked
    and values read back; unknown keys fail."""
    lib = L.load()
    old = {k: lib.splat_get_tuning(k) for k in range(L.TUNE_KEYS)}
    try:
        assert old[L.TUNE_SPLAT_AGGREGATE] in (0, 1)
        assert lib.splat_set_tuning(L.TUNE_SPLAT_AGGREGATE, 2) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_SPLAT_AGGREGATE, 0) == L.OK
        assert lib.splat_get_tuning(L.TUNE_SPLAT_AGGREGATE) == 0
        assert lib.splat_set_tuning(L.TUNE_BVH_BLOCKS_PER_SM, 0) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_BVH_BLOCKS_PER_SM, 257) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_BVH_BLOCKS_PER_SM, 12) == L.OK
        assert lib.splat_get_tuning(L.TUNE_BVH_BLOCKS_PER_SM) == 12
        assert lib.splat_set_tuning(L.TUNE_BVH_PACKET, 6) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_BVH_PACKET, 2) == L.OK
        assert lib.splat_set_tuning(L.TUNE_SPLAT_OVERLAP, 3) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_SPLAT_OVERLAP, 2) == L.OK
        assert lib.splat_get_tuning(L.TUNE_SPLAT_OVERLAP) == 2
        assert lib.splat_set_tuning(L.TUNE_BVH_REFILL, 33) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_BVH_REFILL, 16) == L.OK
        assert lib.splat_get_tuning(L.TUNE_BVH_REFILL) == 16
        assert lib.splat_set_tuning(L.TUNE_TRACE_SPLIT, 0) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_TRACE_SPLIT, 5) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_TRACE_SPLIT, 2) == L.OK
        assert lib.splat_get_tuning(L.TUNE_BRUTE_TILE) == 64
        assert lib.splat_set_tuning(L.TUNE_BRUTE_TILE, 48) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_BRUTE_TILE, 128) == L.OK
        assert lib.splat_set_tuning(L.TUNE_RAY_ORDER, 3) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_RAY_ORDER, 23) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_RAY_ORDER, 20) == L.OK
        assert lib.splat_get_tuning(L.TUNE_COUNT_WORK) == 0 and lib.splat_get_tuning(L.TUNE_BATCH_PERSISTENT) == 0
        assert lib.splat_set_tuning(L.TUNE_COUNT_WORK, 2) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_BATCH_PERSISTENT, 9) == L.ERR_INVALID
        assert lib.splat_hit_work(None, 0, None) == L.ERR_INVALID
        assert lib.splat_get_tuning(L.TUNE_TEST_WAIT_STALL) == 0  # off by default
        assert lib.splat_set_tuning(L.TUNE_TEST_WAIT_STALL, -1) == L.ERR_INVALID
        assert lib.splat_set_tuning(L.TUNE_TEST_WAIT_STALL, 0) == L.OK
        assert lib.splat_set_tuning(L.TUNE_KEYS, 1) == L.ERR_INVALID
        assert lib.splat_get_tuning(L.TUNE_KEYS) == -1 and lib.splat_get_tuning(-1) == -1
    finally:
        for k, v in old.items():
            L.check(lib.splat_set_tuning(k, v))
