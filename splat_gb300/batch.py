"""Batched and served forms: many frames of many scenes in one launch
sequence (libsplat's batch engine, include/splat.h splat_batch_*).

Batch.admit queues a frame (scene + workload parameters + light map);
Batch.tick advances every in-flight frame by one bounce; frames admitted
between ticks join at the next tick.  capture() / replay() turn a fixed set of
admitted frames into one CUDA graph.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

from . import _lib as L
from . import tracer


class PoolFull(RuntimeError):
    """No slot or pool room for the frame right now; retry after a tick."""


class Batch:
    def __init__(self, max_items: int, max_pool_rays: int):
        lib = L.load()
        h = C.c_void_p()
        L.check(lib.splat_batch_create(int(max_items), int(max_pool_rays), C.byref(h)))
        self._h = h
        self.max_items = int(max_items)
        self.max_pool_rays = int(max_pool_rays)
        self._done = (C.c_int32 * self.max_items)()
        self.items = {}

    @staticmethod
    def device_bytes(max_items: int, max_pool_rays: int) -> int:
        return int(L.load().splat_batch_device_bytes(int(max_items), int(max_pool_rays)))

    def admit(self, scene: "tracer.Scene", wl, tex, seed: Optional[int] = None, ray_begin: int = 0,
              ray_end: int = 0) -> int:
        P = tracer.trace_params(wl, ray_begin, ray_end)
        if seed is not None:
            P.seed = int(seed)
        slot = C.c_int32(-1)
        rc = L.load().splat_batch_admit(self._h, scene.handle, C.byref(P), tex.data_ptr(), C.byref(slot))
        if rc == L.ERR_WORKSPACE:
            raise PoolFull(L.load().splat_last_error().decode())
        L.check(rc)
        self.items[slot.value] = (scene, wl, tex)
        return slot.value

    def tick(self, stream: Optional[int] = None) -> List[int]:
        n = C.c_int32(0)
        st = tracer._stream() if stream is None else stream
        L.check(L.load().splat_batch_tick(self._h, st, self._done, self.max_items, C.byref(n)))
        return [self._done[i] for i in range(n.value)]

    def release(self, slot: int) -> None:
        L.check(L.load().splat_batch_release(self._h, int(slot)))
        self.items.pop(slot, None)

    def status(self):
        f, r, t = C.c_int32(), C.c_int64(), C.c_int32()
        L.check(L.load().splat_batch_status(self._h, C.byref(f), C.byref(r), C.byref(t)))
        return {"in_flight": f.value, "pool_rays": r.value, "tick": t.value}

    def run(self) -> List[int]:
        """Ticks until nothing is in flight; returns slots in completion order."""
        done = []
        while self.status()["in_flight"] > 0:
            done += self.tick()
        return done

    def _graph_stream(self):
        """Capture and replay run on a stream of their own (the default stream
        cannot be captured), ordered after and before the current stream."""
        import torch

        if getattr(self, "_gs", None) is None:
            self._gs = torch.cuda.Stream()
        self._gs.wait_stream(torch.cuda.current_stream())
        return self._gs

    def capture(self) -> int:
        import torch

        n = C.c_int32(0)
        gs = self._graph_stream()
        L.check(L.load().splat_batch_capture(self._h, gs.cuda_stream, C.byref(n)))
        torch.cuda.current_stream().wait_stream(gs)
        return n.value

    def replay(self, seeds: Optional[Sequence[int]] = None) -> None:
        import torch

        gs = self.replay_async(seeds)
        torch.cuda.current_stream().wait_stream(gs)

    def replay_async(self, seeds: Optional[Sequence[int]] = None):
        """Launches the captured graph on this engine's graph stream after the
        current stream's work, without joining it back; returns the stream."""
        gs = self._graph_stream()
        if seeds:
            arr = (C.c_uint64 * len(seeds))(*[int(x) for x in seeds])
            L.check(L.load().splat_batch_replay(self._h, arr, len(seeds), gs.cuda_stream))
        else:
            L.check(L.load().splat_batch_replay(self._h, None, 0, gs.cuda_stream))
        return gs

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            L.load().splat_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Lanes:
    """Frames dealt to several batch engines ("lanes") whose captured graphs
    replay concurrently, each on its own stream.  Frames go to the lane with
    the fewest rays so far, largest first; one lane's latency-bound last
    ticks then overlap the other lanes' work.  Every frame's map is still
    the one it gets alone."""

    def __init__(self, n_lanes: int, frames: Sequence, scenes: Sequence, maps: Sequence,
                 crossover_tris: Optional[int] = None):
        """crossover_tris (autotune.batch_crossover): frames with fewer
        triangles are traced by brute force, the others by the four-wide
        BVH; None keeps each frame's own hitter.  The choices are in
        `hitters`."""
        if crossover_tris is not None:
            from .autotune import hitter_for

            frames = [w.with_(hitter=hitter_for(int(w.n_tris), int(crossover_tris))) for w in frames]
        self.hitters = [w.hitter for w in frames]
        order = sorted(range(len(frames)), key=lambda i: -frames[i].n_rays)
        load = [0] * n_lanes
        self.members: List[List[int]] = [[] for _ in range(n_lanes)]
        for i in order:
            lane = min(range(n_lanes), key=lambda j: load[j])
            self.members[lane].append(i)
            load[lane] += frames[i].n_rays
        self.engines = []
        for lane in range(n_lanes):
            idx = self.members[lane]
            eng = Batch(max(1, len(idx)), max(1, sum(frames[i].n_rays for i in idx)) + 1024)
            for i in idx:
                eng.admit(scenes[i], frames[i], maps[i])
            self.engines.append(eng)

    def capture(self) -> int:
        """Captures every engine's pass; with SPLAT_TUNE_BATCH_PERSISTENT set
        each pass is one persistent launch (see persistent())."""
        return max(e.capture() for e in self.engines)

    def persistent(self, on: bool = True) -> int:
        """Re-captures the passes as persistent launches (each engine over
        1/n_lanes of the GPU, so the lanes' launches run side by side) or,
        with on=False, tick by tick; returns the ticks per pass."""
        lib = L.load()
        old = lib.splat_get_tuning(L.TUNE_BATCH_PERSISTENT)
        L.check(lib.splat_set_tuning(L.TUNE_BATCH_PERSISTENT, len(self.engines) if on else 0))
        try:
            return self.capture()
        finally:
            L.check(lib.splat_set_tuning(L.TUNE_BATCH_PERSISTENT, old))

    def replay(self, seeds: Optional[Sequence[int]] = None) -> None:
        """seeds: one per frame, in the order the frames were given."""
        import torch

        streams = [e.replay_async(None if seeds is None else [seeds[i] for i in idx])
                   for e, idx in zip(self.engines, self.members)]
        cur = torch.cuda.current_stream()
        for gs in streams:
            cur.wait_stream(gs)
