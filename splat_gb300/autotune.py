"""Autotuner: hitter choice per scene size and launch shapes per workload.

Decisions are tuned on the GPU the library runs on, with CUDA-event
timings, and cached in a JSON file (``$SPLAT_TUNE_CACHE`` or
``~/.cache/splat_gb300/tuning.json``) under the GPU's name:

* the brute-force vs bounding-volume crossover of the batch engine: one
  frame at a time through the engine, each hitter, over a sweep of scene
  sizes; frames below the crossover's triangle count are traced by brute
  force, the others by the four-wide BVH (``batch_crossover``,
  ``hitter_for``).  The sweep follows the reference's hitter benchmark
  (rays x triangles, src/scenes/perf_test.jl:9-45);
* the launch shapes of the batch engine (its rays' order, the packet form,
  blocks per SM of its hit, evolve and splat kernels, the splat's texel
  aggregation), by coordinate descent
  on the time of a captured pass (``tune_batch``); the reference sizes its
  hitter launches with the occupancy API (src/hitters.jl:75,149,214,297,390);
* the knobs of the plain trace step, including the brute-force tile size,
  the secondary rays' order and the packet form, by coordinate descent on
  the time of the step (``tune_knobs``);
* the hitter of one scene for a workload's primary rays (``choose_hitter``).

None of these changes a result: every hitter returns identical hits, ray
order only decides which rays share a warp, and the knobs only change grid
sizes, so every int32 light map is the same bit for bit whatever is chosen.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os
from typing import Callable, Dict, List, Optional, Sequence

from . import _lib as L

# the traversal's form first: the secondary rays' order and the packet form
# interact, and the descent takes two rounds
KNOB_CHOICES = {
    L.TUNE_RAY_ORDER: (0, 16, 20),
    L.TUNE_BVH_PACKET: (0, 1, 2, 3, 4, 5),
    L.TUNE_BRUTE_BLOCKS_PER_SM: (2, 4, 8, 16),
    L.TUNE_BVH_BLOCKS_PER_SM: (4, 8, 16, 32),
    L.TUNE_EVOLVE_BLOCKS_PER_SM: (4, 8, 16),
    L.TUNE_SPLAT_BLOCKS_PER_SM: (4, 8, 16),
    L.TUNE_SPLAT_AGGREGATE: (0, 1),
    L.TUNE_SPLAT_OVERLAP: (0, 1, 2),
    L.TUNE_BVH_REFILL: (0, 16, 24),
    L.TUNE_TRACE_SPLIT: (1, 2, 3),
    L.TUNE_BRUTE_TILE: (32, 64, 128),
}

# knobs that the batch engine's kernels read
BATCH_KNOB_CHOICES = {
    L.TUNE_RAY_ORDER: (0, 20),
    L.TUNE_BVH_PACKET: (0, 1, 2, 3, 4, 5),
    L.TUNE_BVH_BLOCKS_PER_SM: (8, 16, 32),
    L.TUNE_EVOLVE_BLOCKS_PER_SM: (4, 8, 16),
    L.TUNE_SPLAT_BLOCKS_PER_SM: (4, 8, 16),
    L.TUNE_SPLAT_AGGREGATE: (0, 1),
}

# scene sizes of the crossover sweep (triangles of glass)
CROSSOVER_SIZES = (32, 128, 512, 2048, 8192)


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
    os.makedirs(os.path.dirname(p) or ".", exist_ok=True)
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def cache_get(key: str):
    return _load().get(key)


def cache_put(key: str, value) -> None:
    d = _load()
    d[key] = value
    _store(d)


def _gpu_name() -> str:
    sm = C.c_int32()
    name = C.create_string_buffer(128)
    L.check(L.load().splat_device_info(C.byref(sm), name, 128))
    return name.value.decode()


def _bucket(x: int) -> int:
    """Half-octave bucket of a size (sizes within ~41 % share a bucket)."""
    return int(round(math.log2(max(1, x)) * 2))


# --------------------------------------------------------------- decisions
def crossover_from(rows: Sequence[dict]) -> int:
    """The triangle count from which the BVH wins: the smallest swept size
    at which the BVH is at least as fast as brute force and stays so for
    every larger size.  rows: {"n_tris": T, "ms": {"bvh": x, "brute": y}}.
    No size where the BVH wins: one past the largest size swept."""
    rows = sorted(rows, key=lambda r: r["n_tris"])
    cross = rows[-1]["n_tris"] + 1 if rows else 0
    for r in reversed(rows):
        if r["ms"]["bvh"] <= r["ms"]["brute"]:
            cross = r["n_tris"]
        else:
            break
    return int(cross)


def hitter_for(n_tris: int, crossover_tris: int) -> str:
    """Brute force below the crossover, the four-wide BVH from it on."""
    return "brute" if n_tris < crossover_tris else "bvh"


def descend(choices: Dict[int, Sequence[int]], start: Dict[int, int], cost: Callable[[Dict[int, int]], float],
            rounds: int = 1):
    """Coordinate descent: each knob in turn takes the value of lowest cost
    with the others held; returns (best knobs, best cost, trials)."""
    best = dict(start)
    best_cost = cost(best)
    trials = [(dict(best), best_cost)]
    for _ in range(rounds):
        changed = False
        for k, vals in choices.items():
            for v in vals:
                if v == best.get(k):
                    continue
                cand = {**best, k: v}
                c = cost(cand)
                trials.append((cand, c))
                if c < best_cost:
                    best, best_cost, changed = cand, c, True
        if not changed:
            break
    return best, best_cost, trials


# --------------------------------------------------------------- timing
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


def set_knobs(knobs: Dict[int, int]) -> None:
    for k, v in knobs.items():
        L.check(L.load().splat_set_tuning(int(k), int(v)))


def get_knobs(choices: Optional[Dict[int, Sequence[int]]] = None) -> Dict[int, int]:
    return {k: int(L.load().splat_get_tuning(k)) for k in (choices or KNOB_CHOICES)}


KNOB_NAMES = {L.TUNE_BRUTE_BLOCKS_PER_SM: "brute_blocks_per_sm", L.TUNE_BVH_BLOCKS_PER_SM: "bvh_blocks_per_sm",
              L.TUNE_EVOLVE_BLOCKS_PER_SM: "evolve_blocks_per_sm", L.TUNE_SPLAT_BLOCKS_PER_SM: "splat_blocks_per_sm",
              L.TUNE_SPLAT_AGGREGATE: "splat_aggregate", L.TUNE_BVH_PACKET: "bvh_packet",
              L.TUNE_SPLAT_OVERLAP: "splat_overlap", L.TUNE_BVH_REFILL: "bvh_refill",
              L.TUNE_TRACE_SPLIT: "trace_split", L.TUNE_RAY_ORDER: "ray_order_bits",
              L.TUNE_BRUTE_TILE: "brute_tile", L.TUNE_BATCH_PERSISTENT: "batch_persistent_share"}


def named(knobs: Dict) -> Dict[str, int]:
    """Knobs by name (keys may be ints or their strings)."""
    return {KNOB_NAMES.get(int(k), str(k)): int(v) for k, v in knobs.items()}


def choose_hitter(scene, wl, sample_rays: int = 1 << 15, candidates: Sequence[str] = ("bvh", "bvh2", "brute"),
                  use_cache: bool = True) -> Dict[str, object]:
    """Fastest hitter of a scene for a workload's first-bounce rays."""
    from . import tracer

    key = f"hitter|{_gpu_name()}|T{_bucket(scene.n_tris)}|R{_bucket(wl.n_rays)}"
    if use_cache and cache_get(key):
        return cache_get(key)
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
        cache_put(key, out)
    return out


def crossover_frame(n_tris: int, n_rays: int, seed: int = 3):
    """The sweep's frame: n_tris of displaced-icosphere glass over the floor,
    a hemisphere light of n_rays rays, depth 3, 4 wavelengths, 256^2 int32."""
    from . import scenes as S
    from . import types as T

    glass = S.sphere_tris(next(k for k in range(1, 9) if 20 * 4 ** k >= n_tris), noise_amp=0.05,
                          noise_seed=seed)[:n_tris]
    tris, fd = S.assemble(glass, S.floor_tris(-1.5, 4.0))
    res = max(16, int(round(math.sqrt(n_rays))))
    return S.Workload(name=f"crossover-{n_tris}tris-{res * res}rays", tris=tris, first_diffuse=fd,
                      light=S.hemisphere_light(seed, res, 1.1), upscale=1,
                      lambda_mode=(T.LAMBDA_STRATIFIED, 4, 400.0, 700.0), spectrum=S.stratified_spectrum(4),
                      depth=3, material=S.CAUCHY_GLASS, map_w=256, map_h=256, accum="i32", hitter="bvh", seed=seed)


def batch_crossover(sizes: Sequence[int] = CROSSOVER_SIZES, n_rays: int = 1 << 16, reps: int = 3,
                    use_cache: bool = True) -> dict:
    """Brute force vs BVH in the batch engine, one frame of n_rays rays per
    scene size, each hitter timed over captured passes; returns
    {"crossover_tris": T, "rows": [...]}, cached per GPU."""
    from . import batch as B
    from . import tracer

    key = f"batch-crossover|{_gpu_name()}|R{_bucket(n_rays)}|{','.join(str(s) for s in sizes)}"
    if use_cache and cache_get(key):
        return cache_get(key)
    rows = []
    for n in sizes:
        wl = crossover_frame(int(n), n_rays)
        scene = tracer.Scene(wl.tris, wl.first_diffuse, bvh=True)
        ms = {}
        for hitter in ("brute", "bvh"):
            w = wl.with_(hitter=hitter)
            tex = tracer.new_light_map(w.map_w, w.map_h, w.n_planes, w.accum)
            eng = B.Batch(1, w.n_rays + 1024)
            eng.admit(scene, w, tex)
            eng.capture()
            ms[hitter] = time_ms(lambda: eng.replay([w.seed]), reps)
            eng.close()
        scene.close()
        rows.append({"n_tris": int(n), "ms": ms})
    out = {"crossover_tris": crossover_from(rows), "rows": rows, "n_rays": int(n_rays)}
    if use_cache:
        cache_put(key, out)
    return out


def tune_batch(lanes, seeds: Sequence[int], reps: int = 2, use_cache: bool = True,
               signature: Optional[str] = None) -> dict:
    """Coordinate descent over the batch engine's launch shapes on the time
    of one captured pass of `lanes` (re-captured for every trial: grid sizes
    are fixed when a graph is captured).  Leaves the best knobs set and
    `lanes` captured with them."""
    key = f"batch-knobs|{_gpu_name()}|{signature}" if signature else None
    if use_cache and key and cache_get(key):
        d = cache_get(key)
        set_knobs({int(k): v for k, v in d["knobs"].items()})
        lanes.capture()
        return d

    def cost(knobs):
        set_knobs(knobs)
        lanes.capture()
        return time_ms(lambda: lanes.replay(seeds), reps)

    # the pass tick by tick, or as one persistent launch per engine over its
    # share of the GPU
    choices = {**BATCH_KNOB_CHOICES, L.TUNE_BATCH_PERSISTENT: (0, len(lanes.engines))}
    best, best_ms, trials = descend(choices, get_knobs(choices), cost)
    set_knobs(best)
    lanes.capture()
    out = {"knobs": {str(k): v for k, v in best.items()}, "ms": best_ms, "trials": len(trials),
           "trial_ms": [(named(k), round(c, 4)) for k, c in trials]}
    if use_cache and key:
        cache_put(key, out)
    return out


def tune_knobs(step, reps: int = 3, use_cache: bool = True, rounds: int = 2) -> Dict[str, object]:
    """Coordinate descent over the plain step's knobs on one trace step;
    leaves the best knobs set."""
    key = f"knobs|{_gpu_name()}|{step.wl.name}"
    if use_cache and cache_get(key):
        d = cache_get(key)
        set_knobs({int(k): v for k, v in d["knobs"].items()})
        return d
    start = get_knobs()
    best, best_ms, trials = descend(KNOB_CHOICES, start, lambda k: (set_knobs(k), time_ms(step.run, reps))[1],
                                    rounds=rounds)
    set_knobs(best)
    out = {"knobs": {str(k): v for k, v in best.items()}, "ms": best_ms, "trials": len(trials),
           "default_ms": trials[0][1]}
    if use_cache:
        cache_put(key, out)
    return out


def apply_cached(wl_name: str) -> Optional[Dict[int, int]]:
    """Set the knobs cached for a workload, if any."""
    d = cache_get(f"knobs|{_gpu_name()}|{wl_name}")
    if not d:
        return None
    knobs = {int(k): v for k, v in d["knobs"].items()}
    set_knobs(knobs)
    return knobs


def tuned_hitters(frames: Sequence, crossover_tris: int) -> List[str]:
    """The hitter of each frame under the crossover."""
    return [hitter_for(int(w.n_tris), crossover_tris) for w in frames]
