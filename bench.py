"""Benchmark of the GB300 forward trace step (SPLAT's forward half of trace!).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload realtime|plain_small|menger]

One step = one frame of the workload: clear the light map, generate the
light's rays, depth x {nearest hit, evolve + compaction + diffuse splat},
statistics.  The metric is rays/s: ray segments traced (sum over bounces of
the rays active in that bounce) per second of device time, whole job.

* value:  K steps on resident inputs, each step bracketed by CUDA events on
          the launch stream; a 256 MiB write flushes L2 between steps
          (outside the events).  Max over ranks, rays summed over ranks.
* e2e:    the same step through the host-buffer C ABI entry point
          (splat_trace_forward_host): host triangles uploaded (pinned), scene
          repacked + BVH refit, traced, light map downloaded (pinned).
* roofline: the kernel kind with the largest share of device time, its
          algorithmic bytes per launch over its event-timed launch duration,
          against the measured HBM copy bandwidth.
* cpu_baseline: the CPU restatement of the reference (oracle/, OpenMP over
          all host cores) on a bounded sample of the same workload.
* --impl reference: that CPU implementation timed alone as the reference arm.

Multi-GPU: replicas (each rank renders its own frames, seeds offset by
rank); no collective on the data path.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from splat_gb300 import scenes as S  # noqa: E402

WORKLOADS = {"realtime": S.realtime, "plain_small": S.plain_small, "menger": S.menger}
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="realtime", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the cpu_baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": PEAKS_FALLBACK["hbm_gbs"], "source": "fallback"}


def profile_traffic(kernel: str):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary
    (profiles/traffic.txt, lines 'kernel: bytes_per_launch ...')."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(kernel + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------- clocks
CLOCK_QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


class ClockSampler:
    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={CLOCK_QUERY}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU side
def cpu_sample_ranges(wl, n_rays_target: int, chunks: int = 16):
    """Disjoint ray ranges spread evenly over the light grid."""
    n = wl.n_rays
    per = max(1, n_rays_target // chunks)
    starts = np.linspace(0, n - per, chunks).astype(np.int64)
    return [(int(s), int(s) + per) for s in starts]


def cpu_trace(wl, ranges, threads: int):
    from oracle import oracle as O

    t0 = time.perf_counter()
    seg = 0
    for lo, hi in ranges:
        _, st, _ = O.trace_forward(wl, lo, hi, nthreads=threads)
        seg += int(st[: wl.depth].sum())
    return seg, time.perf_counter() - t0


def cpu_calibrate(wl, threads: int, target_s: float):
    """Rays per chunk-set so that one sample costs about target_s seconds."""
    probe = cpu_sample_ranges(wl, 256, 8)
    seg, dt = cpu_trace(wl, probe, threads)
    rays = sum(hi - lo for lo, hi in probe)
    per_ray = dt / rays
    return max(64, int(target_s / max(per_ray, 1e-9)))


def cpu_baseline(wl, target_s: float):
    threads = os.cpu_count() or 1
    n = cpu_calibrate(wl, threads, target_s)
    ranges = cpu_sample_ranges(wl, n)
    seg, dt = cpu_trace(wl, ranges, threads)
    rays = sum(hi - lo for lo, hi in ranges)
    return {"value": seg / dt, "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": f"{rays} of {wl.n_rays} rays ({len(ranges)} ranges spread over the light grid), "
                      f"{seg} ray segments in {dt:.1f} s; CPU restatement of the reference (oracle/), "
                      f"brute-force nearest hit, OpenMP"}


# ---------------------------------------------------------------- GPU side
def config_of(wl, l2_note):
    return {
        "workload": wl.name, "rays_per_frame": wl.n_rays, "triangles": wl.n_tris, "depth": wl.depth,
        "lambda_planes": wl.n_planes, "forward_upscale": wl.upscale,
        "light_map": f"{wl.map_w}x{wl.map_h}x{wl.n_planes} {'int32 fixed point 2^' + str(wl.frac_bits) if wl.accum == 'i32' else 'float32'}",
        "hitter": wl.hitter, "material": "Cauchy n=1.5+0.004/lambda_um^2" if wl.material[0] == 1 else str(wl.material),
        "l2": l2_note, "parallelism": "replicas",
    }


def algorithmic_bytes(kind: str, wl, per_step_bounces, n_tris: int, diffuse: int, samples: int):
    """Compulsory bytes of one step of a kernel kind, with the reference's
    AoS record sizes: hit R_b (24 pos+dir + 4 ignore + 8 hit) + T 48 per
    bounce; evolve R_b (136 read + 4 hit + 84 tri gather + 136 write) per
    bounce; splat D (136 + 4 + 120) + 4 per sample + 2 x map bytes (clear +
    final read); generate R 136."""
    if kind in ("hit_bvh", "hit_brute"):
        return sum(r * 36 + n_tris * 48 for r in per_step_bounces)
    if kind == "evolve":
        return sum(r * 360 for r in per_step_bounces)
    if kind == "splat":
        map_bytes = wl.map_w * wl.map_h * wl.n_planes * 4
        return diffuse * 260 + 4 * samples + 2 * map_bytes
    if kind == "generate":
        return per_step_bounces[0] * 136
    return None


def run_ours(args):
    import torch

    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    lib = L.load()
    wl = WORKLOADS[args.workload]()
    step = tracer.TraceStep(wl)
    stream = torch.cuda.current_stream()
    K, W = args.steps, args.warmup
    stats = torch.zeros((K, 16), dtype=torch.int64, device="cuda")
    base_seed = wl.seed + 1000003 * rank

    def run_step(i, st_ptr):
        step.params.seed = base_seed + i
        L.check(lib.splat_trace_forward(step.scene.handle, C.byref(step.params), step.tex.data_ptr(),
                                        step.ws.data_ptr(), step.ws.numel(), st_ptr, stream.cuda_stream))

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for i in range(W):
        run_step(i, step.d_stats.data_ptr())
    torch.cuda.synchronize()

    prof = C.c_void_p()
    L.check(lib.splat_profile_create(64 * (K + 1), C.byref(prof)))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    L.check(lib.splat_profile_attach(prof))
    for i in range(K):
        flush.zero_()
        starts[i].record(stream)
        run_step(W + i, stats[i].data_ptr())
        ends[i].record(stream)
    torch.cuda.synchronize()
    L.check(lib.splat_profile_attach(None))
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = float(sum(step_ms))
    st = stats.cpu().numpy()
    per_step = [[int(x) for x in st[i, : wl.depth]] for i in range(K)]
    segments = int(sum(sum(p) for p in per_step))
    diffuse = int(st[:, 8].sum())
    samples = int(st[:, 9].sum())
    errors = int(np.abs(st[:, 10]).sum())

    kinds = {"generate": L.KERNEL_GENERATE, "hit_brute": L.KERNEL_HIT_BRUTE, "hit_bvh": L.KERNEL_HIT_BVH,
             "evolve": L.KERNEL_EVOLVE, "splat": L.KERNEL_SPLAT, "aux": L.KERNEL_AUX}
    prof_res = {}
    for name, kd in kinds.items():
        n = C.c_int64()
        ms = C.c_double()
        L.check(lib.splat_profile_read(prof, kd, C.byref(n), C.byref(ms)))
        prof_res[name] = (int(n.value), float(ms.value))
    n_all = C.c_int64()
    ms_all = C.c_double()
    L.check(lib.splat_profile_read(prof, L.KERNEL_ALL, C.byref(n_all), C.byref(ms_all)))
    lib.splat_profile_destroy(prof)

    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        seg_t = torch.tensor([segments], dtype=torch.int64, device="cuda")
        dist.all_reduce(seg_t)
        total_ms_max, segments_all = float(t.item()), int(seg_t.item())
    else:
        total_ms_max, segments_all = total_ms, segments
    value = segments_all / (total_ms_max / 1e3)

    # roofline of the dominant kernel kind
    pk = peaks()
    dom = max((k for k in prof_res if k != "aux"), key=lambda k: prof_res[k][1])
    n_launch, dom_ms = prof_res[dom]
    launches_of_kind = {"hit_bvh": wl.depth, "hit_brute": wl.depth, "evolve": wl.depth, "splat": 1,
                        "generate": 1}[dom]
    alg = sum(algorithmic_bytes(dom, wl, p, wl.n_tris, int(st[i, 8]), int(st[i, 9])) for i, p in enumerate(per_step))
    n_kind_launches = K * launches_of_kind
    bytes_per_launch = alg / n_kind_launches
    avg_launch_s = dom_ms / 1e3 / n_kind_launches
    achieved = bytes_per_launch / avg_launch_s / 1e9
    kernel_name = {"hit_bvh": "hit_bvh_kernel", "hit_brute": "hit_brute_kernel", "evolve": "evolve_kernel",
                   "splat": "splat_kernel", "generate": "generate_soa_kernel"}[dom]
    traffic = profile_traffic(kernel_name)
    roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / pk["hbm_gbs"], 5), "traffic": traffic, "kernel": kernel_name,
                "peak_source": pk["source"], "algorithmic_bytes_per_launch": round(bytes_per_launch),
                "avg_launch_ms": round(avg_launch_s * 1e3, 4),
                "share": {k: round(v[1] / max(ms_all.value, 1e-12), 4) for k, v in prof_res.items()}}

    out = {
        "metric": "rays/s", "value": value, "unit": "rays/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: seeded procedural scene and light (no dataset)",
        "config": config_of(wl, "flushed between steps (256 MiB write outside the step events); per-step ray "
                                "state (2 x 117 B x rays) exceeds L2"),
        "frames_per_s": world * K / (total_ms_max / 1e3),
        "primary_rays_per_s": world * K * wl.n_rays / (total_ms_max / 1e3),
        "rays_per_bounce": per_step[0], "diffuse_rays_per_frame": diffuse // K, "splat_samples_per_frame": samples // K,
        "kernel_error_words": errors,
        "gpu_launches": int(n_all.value),
        "roofline": roofline,
        "clocks": clocks,
    }

    if not args.no_e2e:
        out["e2e"] = e2e(step, wl, K, W, stream, world, rank)
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def e2e(step, wl, K, W, stream, world, rank):
    """rays/s through splat_trace_forward_host with host buffers: per step the
    pinned host FTri array goes up, the scene is repacked and its BVH refit,
    the frame is traced and the light map comes back to pinned host memory."""
    import torch

    tris_pinned = torch.from_numpy(np.ascontiguousarray(wl.tris).reshape(-1)).pin_memory()
    host_tris = tris_pinned.numpy().reshape(wl.tris.shape)
    map_pinned = torch.empty(step.tex.numel(), dtype=step.tex.dtype).pin_memory()
    host_map = map_pinned.numpy()
    segs = 0
    for i in range(W):
        step.params.seed = wl.seed + 7 * i
        step.run_host(host_tris, host_map, stream.cuda_stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for i in range(K):
        step.params.seed = wl.seed + 7 * (W + i) + 1000003 * rank
        st = step.run_host(host_tris, host_map, stream.cuda_stream)
        segs += int(sum(st["rays_per_bounce"]))
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        s = torch.tensor([segs], dtype=torch.int64, device="cuda")
        dist.all_reduce(s)
        ms, segs = float(t.item()), int(s.item())
    return {"value": segs / (ms / 1e3), "unit": "rays/s", "h2d_bytes_per_step": int(wl.tris.nbytes),
            "d2h_bytes_per_step": int(step.tex.numel() * step.tex.element_size() + 8 * wl.depth),
            "ms_per_step": ms / K, "api": "splat_trace_forward_host"}


def run_reference(args):
    """The reference's path on the host cores: the CPU restatement (the
    reference is Julia and does not run here), all threads, each step a
    bounded sample of the workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]()
    threads = os.cpu_count() or 1
    per_step_target = max(0.05, min(8.0, 120.0 / max(1, args.steps + args.warmup)))
    n = cpu_calibrate(wl, threads, per_step_target)
    per = max(1, n // 16)
    total_seg, total_s, steps = 0, 0.0, []
    grid = wl.n_rays
    for i in range(args.warmup + args.steps):
        off = (i * 7919 * per) % max(1, grid - per)
        ranges = [((off + j * (grid // 16)) % (grid - per), (off + j * (grid // 16)) % (grid - per) + per)
                  for j in range(16)]
        seg, dt = cpu_trace(wl, ranges, threads)
        if i >= args.warmup:
            total_seg += seg
            total_s += dt
            steps.append(dt)
    value = total_seg / total_s
    sample = (f"{16 * per} of {grid} rays per step (16 ranges spread over the light grid); CPU restatement "
              f"of the reference (oracle/), brute-force nearest hit, OpenMP")
    out = {"impl": "reference", "metric": "rays/s", "value": value, "unit": "rays/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic: seeded procedural scene and light (no dataset)",
           "config": config_of(wl, "CPU run"),
           "cpu_baseline": {"value": value, "unit": "rays/s", "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
