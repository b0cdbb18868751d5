"""Autotuner: hitter choice per scene size and launch shapes per workload.

Two decisions are tuned on the GPU the library runs on, with CUDA-event
timings, and cached in a JSON file (``$SPLAT_TUNE_CACHE`` or
``~/.cache/splat_gb300/tuning.json``):

* the hitter of a scene: brute force, the four-wide BVH or the binary BVH,
  timed on a sample of the workload's primary rays (the BVH-vs-brute-force
  crossover by triangle count comes out of this per scene size);
* the launch-shape knobs (blocks per SM of the grid-stride kernels), by
  coordinate descent on the time of the whole trace step.

None of these changes a result: every hitter returns identical hits and the
knobs only change grid sizes.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from typing import Dict, Optional, Sequence

from . import _lib as L
from . import tracer

KNOB_CHOICES = {
    L.TUNE_BRUTE_BLOCKS_PER_SM: (2, 4, 8, 16),
    L.TUNE_BVH_BLOCKS_PER_SM: (4, 8, 16, 32),
    L.TUNE_EVOLVE_BLOCKS_PER_SM: (4, 8, 16),
    L.TUNE_SPLAT_BLOCKS_PER_SM: (4, 8, 16),
    L.TUNE_SPLAT_AGGREGATE: (0, 1),
    L.TUNE_BVH_PACKET: (0, 1, 2, 3, 4, 5),
    L.TUNE_SPLAT_OVERLAP: (0, 1, 2),
    L.TUNE_BVH_REFILL: (0, 16, 24),
    L.TUNE_TRACE_SPLIT: (1, 2, 3),
}


def cache_path() -> str:
    return os.environ.get("SPLAT_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "splat_gb300",
                                                           "tuning.json"))


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    p = cache_path()
    os.makedirs(os.path.dirname(p), exist_ok=True)
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def _gpu_name() -> str:
    sm = C.c_int32()
    name = C.create_string_buffer(128)
    L.check(L.load().splat_device_info(C.byref(sm), name, 128))
    return name.value.decode()


def _bucket(x: int) -> int:
    return int(round(math.log2(max(1, x)) * 2))


def time_ms(fn, reps: int = 3, warmup: int = 1) -> float:
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def choose_hitter(scene: "tracer.Scene", wl, sample_rays: int = 1 << 15, candidates: Sequence[str] = ("bvh", "bvh2",
                  "brute"), use_cache: bool = True) -> Dict[str, object]:
    """Fastest hitter of a scene for a workload's first-bounce rays."""
    key = f"hitter|{_gpu_name()}|T{_bucket(scene.n_tris)}|R{_bucket(wl.n_rays)}"
    cache = _load() if use_cache else {}
    if key in cache:
        return cache[key]
    res = max(8, int(math.sqrt(min(sample_rays, wl.n_rays))))
    light = wl.light.copy()
    light["res1"] = res
    light["res2"] = res
    rays = tracer.rays_from_light(light, 1, wl.lambda_mode, wl.seed)
    codes = {"bvh": tracer.BVH, "bvh2": tracer.BVH2, "brute": tracer.BRUTE}
    times = {}
    for name in candidates:
        if name != "brute" and not scene.has_bvh:
            continue
        times[name] = time_ms(lambda c=codes[name]: tracer.next_hit(scene, c, rays))
    best = min(times, key=times.get)
    out = {"hitter": best, "ms": times, "n_tris": scene.n_tris, "sample_rays": res * res}
    if use_cache:
        cache = _load()
        cache[key] = out
        _store(cache)
    return out


def crossover(tri_counts: Sequence[int], make_scene, wl_of, sample_rays: int = 1 << 15) -> list:
    """Hitter timings over a sweep of triangle counts: where brute force
    stops winning against the BVH."""
    rows = []
    for t in tri_counts:
        tris, fd = make_scene(t)
        sc = tracer.Scene(tris, fd, bvh=True)
        r = choose_hitter(sc, wl_of(tris, fd), sample_rays, use_cache=False)
        rows.append({"n_tris": int(t), **r})
        sc.close()
    return rows


def set_knobs(knobs: Dict[int, int]) -> None:
    for k, v in knobs.items():
        L.check(L.load().splat_set_tuning(int(k), int(v)))


def get_knobs() -> Dict[int, int]:
    return {k: int(L.load().splat_get_tuning(k)) for k in KNOB_CHOICES}


def tune_knobs(step: "tracer.TraceStep", reps: int = 3, use_cache: bool = True) -> Dict[str, object]:
    """Coordinate descent over the launch-shape knobs on one trace step."""
    key = f"knobs|{_gpu_name()}|{step.wl.name}"
    cache = _load() if use_cache else {}
    if key in cache:
        knobs = {int(k): v for k, v in cache[key]["knobs"].items()}
        set_knobs(knobs)
        return cache[key]
    best = get_knobs()
    best_ms = time_ms(step.run, reps)
    for k, choices in KNOB_CHOICES.items():
        for v in choices:
            if v == best[k]:
                continue
            set_knobs({**best, k: v})
            ms = time_ms(step.run, reps)
            if ms < best_ms:
                best_ms, best = ms, {**best, k: v}
        set_knobs(best)
    out = {"knobs": {str(k): v for k, v in best.items()}, "ms": best_ms}
    if use_cache:
        cache = _load()
        cache[key] = out
        _store(cache)
    return out


def apply_cached(wl_name: str) -> Optional[Dict[int, int]]:
    """Set the knobs cached for a workload, if any."""
    d = _load().get(f"knobs|{_gpu_name()}|{wl_name}")
    if not d:
        return None
    knobs = {int(k): v for k, v in d["knobs"].items()}
    set_knobs(knobs)
    return knobs
