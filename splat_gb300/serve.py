"""Serving loop: render requests admitted by HBM budget onto the batch engine.

A request names a scene (from a pool of scene factories), light and trace
parameters.  The server keeps scenes resident on the device (geometry,
hit records, BVH) and evicts the least recently used idle scene when the
HBM budget would be exceeded.  Admitted requests join the batch engine's next
tick -- requests arriving while others are on the GPU overlap with them
(continuous batching) -- and leave when their last bounce has run.  The
light map of a request is device memory owned by the request until it is
delivered.

Latency is measured on the device clock: an event recorded at start-up and
one after each request's last tick give its completion time on the host
clock, from which the arrival time is subtracted.
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
    """Continuous-batching renderer over one batch engine."""

    def __init__(self, scenes: ScenePool, budget_bytes: int, max_items: int = 128, max_pool_rays: int = 1 << 26,
                 max_ticks_ahead: int = 4):
        import torch

        self.torch = torch
        self.scenes = scenes
        self.budget = int(budget_bytes)
        self.engine = B.Batch(max_items, max_pool_rays)
        self.engine_bytes = B.Batch.device_bytes(max_items, max_pool_rays)
        self.max_pool_rays = int(max_pool_rays)
        self.stream = torch.cuda.current_stream()
        self.map_bytes_in_use = 0
        self.inflight: Dict[int, Request] = {}
        self.pending: List[Request] = []
        self.done: List[Request] = []
        self.max_ticks_ahead = max_ticks_ahead
        self._tick_events = collections.deque()
        self.ev0 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        self.ev0.record(self.stream)
        torch.cuda.synchronize()
        self.host0 = time.perf_counter()
        self._completion = []  # (event, request)

    def now(self) -> float:
        return time.perf_counter() - self.host0

    def submit(self, req: Request) -> None:
        heapq.heappush(self.pending, req)

    def _try_admit(self, req: Request) -> bool:
        mb = map_bytes(req.wl)
        other = self.engine_bytes + self.map_bytes_in_use + mb
        sc = self.scenes.acquire(req.scene_id, other)
        if sc is None:
            return False
        tex = tracer.new_light_map(req.wl.map_w, req.wl.map_h, req.wl.n_planes, req.wl.accum)
        try:
            slot = self.engine.admit(sc, req.wl, tex)
        except B.PoolFull:
            self.scenes.release(req.scene_id)
            del tex
            return False
        req.tex = tex
        self.map_bytes_in_use += mb
        self.inflight[slot] = req
        return True

    def step(self) -> int:
        """Admits what has arrived and fits, enqueues one tick; returns the
        number of requests completed on the device so far."""
        self._collect()
        t = self.now()
        while self.pending and self.pending[0].arrival <= t:
            if not self._try_admit(self.pending[0]):
                if not self.inflight:
                    if not self._completion:
                        raise RuntimeError(f"request {self.pending[0].rid} can never fit the budget or the pool")
                    self._collect(block=True)  # room held only by delivered-but-uncollected maps
                    continue
                break
            heapq.heappop(self.pending)
        if self.engine.status()["in_flight"] == 0:
            return len(self.done)
        # keep the host at most a few ticks ahead of the device
        while len(self._tick_events) >= self.max_ticks_ahead:
            self._tick_events.popleft().synchronize()
        finished = self.engine.tick(self.stream.cuda_stream)
        ev = self.torch.cuda.Event(enable_timing=True)
        ev.record(self.stream)
        self._tick_events.append(ev)
        for slot in finished:
            req = self.inflight.pop(slot)
            self._completion.append((ev, req, slot))
        self._collect()
        return len(self.done)

    def _collect(self, block: bool = False) -> None:
        keep = []
        for ev, req, slot in self._completion:
            if block or ev.query():
                ev.synchronize()
                req.done_at = self.ev0.elapsed_time(ev) / 1e3
                self.engine.release(slot)
                self.scenes.release(req.scene_id)
                self.map_bytes_in_use -= map_bytes(req.wl)
                self.done.append(req)
            else:
                keep.append((ev, req, slot))
        self._completion = keep

    def drain(self) -> None:
        while self.pending or self.inflight:
            if not self.inflight and self.pending and self.pending[0].arrival > self.now():
                time.sleep(max(0.0, min(0.001, self.pending[0].arrival - self.now())))
            self.step()
        self._collect(block=True)

    def latencies(self) -> np.ndarray:
        return np.array([r.done_at - r.arrival for r in self.done])


def poisson_arrivals(rate: float, duration: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return np.array(out)
        out.append(t)
