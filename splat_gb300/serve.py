"""Serving loop: render requests admitted by HBM budget onto the batch engine.

A request names a scene (from a pool of scene factories), light and trace
parameters.  The server keeps scenes resident on the device (geometry,
hit records, BVH) and evicts the least recently used idle scene when the
HBM budget would be exceeded.  Admitted requests join the batch engine's next
tick -- requests arriving while others are on the GPU overlap with them
(continuous batching) -- and leave when their last bounce has run.  The
light map of a request is device memory owned by the request until it is
delivered.

The queue, admission, tick loop and completion tracking are native
(splat_server_*, csrc/serve.cpp); this module keeps the scene pool and maps
arrivals on the host clock to submissions.

Latency is measured on the device clock: the native server's start event and
the event after each request's last tick give its completion time on the
host clock, from which the arrival time is subtracted.
"""
from __future__ import annotations

import collections
import heapq
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional

import numpy as np

from . import batch as B
from . import tracer

SCENE_OVERHEAD = 1 << 20


@dataclass(order=True)
class Request:
    arrival: float
    rid: int = field(compare=False)
    scene_id: int = field(compare=False)
    wl: object = field(compare=False)   # scenes.Workload without geometry needs (tris come from the scene)
    done_at: Optional[float] = field(default=None, compare=False)
    tex: object = field(default=None, compare=False)


def map_bytes(wl) -> int:
    return int(wl.map_w) * int(wl.map_h) * int(wl.n_planes) * 4


def pool_ray_bytes(n_rays: int) -> int:
    return int(n_rays) * 117 * 3 + 4 * int(n_rays)


class ScenePool:
    """Resident scenes with LRU eviction under a byte budget.  `factory(id)`
    returns (tris, first_diffuse)."""

    def __init__(self, factory: Callable[[int], tuple], budget_bytes: int, make_scene: Optional[Callable] = None):
        self.factory = factory
        self.make_scene = make_scene or (lambda tris, fd: tracer.Scene(tris, fd, bvh=True))
        self.budget = int(budget_bytes)
        self.resident: "collections.OrderedDict[int, tracer.Scene]" = collections.OrderedDict()
        self.bytes: Dict[int, int] = {}
        self.busy: Dict[int, int] = collections.defaultdict(int)
        self.evictions = 0
        self.loads = 0

    def used(self) -> int:
        return sum(self.bytes.values())

    def acquire(self, sid: int, other_bytes: int) -> Optional["tracer.Scene"]:
        """The scene, loading it if needed; None when it cannot fit."""
        if sid in self.resident:
            self.resident.move_to_end(sid)
            self.busy[sid] += 1
            return self.resident[sid]
        tris, fd = self.factory(sid)
        need = int(tris.nbytes) * 3 + SCENE_OVERHEAD
        while self.used() + need + other_bytes > self.budget:
            victim = next((s for s in self.resident if self.busy[s] == 0), None)
            if victim is None:
                return None
            self.resident.pop(victim).close()
            self.bytes.pop(victim)
            self.evictions += 1
        sc = self.make_scene(tris, fd)
        self.resident[sid] = sc
        self.bytes[sid] = int(sc.info()["device_bytes"]) + SCENE_OVERHEAD
        self.busy[sid] += 1
        self.loads += 1
        return sc

    def release(self, sid: int) -> None:
        self.busy[sid] -= 1


class Server:
    """Continuous-batching renderer: native servers (splat_server_*: arrival
    order, admission by engine slot, ray-pool room and light-map budget, one
    tick per step, bounded run-ahead, completion on the device) with scenes
    kept resident by a ScenePool.  A request is handed to a native server once
    it has arrived on the host clock, with its scene acquired; the scene is
    released when the request completes.  With lanes > 1 there is one native
    server per lane, each stepping on its own stream; a request goes to the
    lane with the fewest rays in flight, or (split_min_rays set), from that
    many rays on, to every lane as disjoint ray ranges; one lane's
    latency-bound last ticks overlap the others' work.

    A completed request is delivered: with on_done set, on_done(request) is
    called once its map is complete on the device (the callback may copy
    request.tex out or keep a reference), then the server drops its own
    reference to the map, so a long-running server holds only the maps in
    flight; without on_done, completed requests keep their maps in `done`.

    max_pool_rays bounds the rays in flight (split evenly over the lanes).
    Every tick advances all of a lane's requests by one bounce, so a tick
    lasts about as long as its lane's rays take; the bound keeps a burst of
    arrivals from stretching every tick (and every request's latency) and
    leaves the excess queued in arrival order.  Each lane must hold the
    largest request.  Measured on Poisson Menger requests of up to 2^22
    rays at 400 req/s: p99 244 ms with 2^26 rays in flight, 38 ms with 2^24
    (the default), p50 5.6 -> 5.1 ms; at 200 req/s no change."""

    def __init__(self, scenes: ScenePool, budget_bytes: int, max_items: int = 128, max_pool_rays: int = 1 << 24,
                 max_ticks_ahead: int = 4, lanes: int = 2, split_min_rays: Optional[int] = None,
                 on_done: Optional[Callable[[Request], None]] = None, crossover_tris: Optional[int] = None):
        import ctypes as C

        import torch

        from . import _lib as L

        self.torch, self.C, self.L = torch, C, L
        self.lib = L.load()
        self.scenes = scenes
        self.budget = int(budget_bytes)
        self.on_done = on_done
        # autotune.batch_crossover: requests on scenes below it are traced by
        # brute force, the others by the four-wide BVH (None: the request's own)
        self.crossover_tris = crossover_tris
        self.hitter_counts: Dict[str, int] = {}
        n = max(1, int(lanes))
        items, pool = max(1, int(max_items) // n), max(1, int(max_pool_rays) // n)
        self.engine_bytes = n * B.Batch.device_bytes(items, pool)
        self.max_items = items * n
        map_budget = max(0, self.budget - self.engine_bytes) // n
        self.handles, self.streams = [], []
        for _ in range(n):
            h = C.c_void_p()
            L.check(self.lib.splat_server_create(items, pool, map_budget, int(max_ticks_ahead), C.byref(h)))
            self.handles.append(h)
            self.streams.append(torch.cuda.Stream())
        self.lane_rays = [0] * n
        # off by default: measured on the Poisson stream, p50 2.39 -> 2.42 ms
        self.split_min_rays = int(split_min_rays) if split_min_rays else 1 << 62
        self.map_bytes_in_use = 0
        self.inflight: Dict[tuple, tuple] = {}     # (lane, native request id) -> (request, rays)
        self._parts: Dict[int, list] = {}          # id(request) -> [parts left, latest completion]
        self.pending: List[Request] = []
        self.done: List[Request] = []
        self._ids = (C.c_int64 * 256)()
        self._ms = (C.c_double * 256)()
        # each native server's device clock starts at its first step; the
        # host clock is read right after them, with the streams idle
        torch.cuda.synchronize()
        for lane in range(n):
            self._native_step(lane)
        torch.cuda.synchronize()
        self.host0 = time.perf_counter()

    def now(self) -> float:
        return time.perf_counter() - self.host0

    def submit(self, req: Request) -> None:
        heapq.heappush(self.pending, req)

    def _native_step(self, lane: int):
        C = self.C
        fl, q = C.c_int32(), C.c_int32()
        self.L.check(self.lib.splat_server_step(self.handles[lane], self.streams[lane].cuda_stream, C.byref(fl),
                                                C.byref(q)))
        return fl.value, q.value

    def _arrive(self) -> None:
        """Hands every request that has arrived to the least loaded lane."""
        from . import tracer

        C = self.C
        t = self.now()
        while self.pending and self.pending[0].arrival <= t:
            req = self.pending[0]
            mb = map_bytes(req.wl)
            sc = self.scenes.acquire(req.scene_id, self.engine_bytes + self.map_bytes_in_use + mb)
            if sc is None:
                return  # its scene fits only after requests in flight release theirs
            heapq.heappop(self.pending)
            if self.crossover_tris is not None:
                from .autotune import hitter_for

                req.wl = req.wl.with_(hitter=hitter_for(int(sc.n_tris), int(self.crossover_tris)))
            self.hitter_counts[req.wl.hitter] = self.hitter_counts.get(req.wl.hitter, 0) + 1
            # the new map is zeroed on the current stream; a large request goes
            # to every lane as disjoint ray ranges adding into that map (ray
            # ids are grid indices, so the map is the same as in one piece)
            req.tex = tracer.new_light_map(req.wl.map_w, req.wl.map_h, req.wl.n_planes, req.wl.accum)
            n_rays = req.wl.n_rays
            k = len(self.handles) if n_rays >= self.split_min_rays else 1
            order = sorted(range(len(self.handles)), key=lambda j: self.lane_rays[j])[:k]
            each = -(-n_rays // k)
            self._parts[id(req)] = [k, 0.0]
            for part, lane in enumerate(order):
                lo, hi = part * each, min(n_rays, (part + 1) * each)
                req.tex.record_stream(self.streams[lane])
                self.streams[lane].wait_stream(self.torch.cuda.current_stream())  # the map's allocation
                P = tracer.trace_params(req.wl, lo, hi if k > 1 else 0, zero_map=False)
                rid = C.c_int64()
                self.L.check(self.lib.splat_server_submit(self.handles[lane], sc.handle, C.byref(P),
                                                          req.tex.data_ptr(), C.byref(rid)))
                self.inflight[(lane, int(rid.value))] = (req, hi - lo)
                self.lane_rays[lane] += hi - lo
            self.map_bytes_in_use += mb

    def step(self) -> int:
        """Hands over what has arrived, enqueues one tick per lane; returns the
        number of requests completed so far."""
        self._arrive()
        for lane in range(len(self.handles)):
            self._native_step(lane)
        self._collect()
        return len(self.done)

    def _collect(self, block: bool = False) -> None:
        C = self.C
        for lane, h in enumerate(self.handles):
            while True:
                n = C.c_int32()
                self.L.check(self.lib.splat_server_poll(h, int(block), self._ids, self._ms, len(self._ids),
                                                        C.byref(n)))
                for i in range(n.value):
                    req, rays = self.inflight.pop((lane, int(self._ids[i])))
                    self.lane_rays[lane] -= rays
                    left = self._parts[id(req)]
                    left[0] -= 1
                    left[1] = max(left[1], self._ms[i] / 1e3)
                    if left[0] > 0:
                        continue
                    del self._parts[id(req)]
                    req.done_at = left[1]
                    self.scenes.release(req.scene_id)
                    self.map_bytes_in_use -= map_bytes(req.wl)
                    if self.on_done is not None:
                        self.on_done(req)
                        req.tex = None
                    self.done.append(req)
                if n.value < len(self._ids):
                    break

    def drain(self) -> None:
        while self.pending or self.inflight:
            if not self.inflight and self.pending and self.pending[0].arrival > self.now():
                time.sleep(max(0.0, min(0.001, self.pending[0].arrival - self.now())))
            if self.pending and not self.inflight and self.pending[0].arrival <= self.now():
                self._arrive()
                if not self.inflight:
                    raise RuntimeError(f"request {self.pending[0].rid} can never fit the budget")
            self.step()
        self._collect(block=True)
        cur = self.torch.cuda.current_stream()
        for st in self.streams:
            cur.wait_stream(st)

    def latencies(self) -> np.ndarray:
        return np.array([r.done_at - r.arrival for r in self.done])

    def close(self) -> None:
        for h in getattr(self, "handles", []):
            if h is not None and h.value:
                self.lib.splat_server_destroy(h)
        self.handles = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_arrivals(rate: float, duration: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return np.array(out)
        out.append(t)
