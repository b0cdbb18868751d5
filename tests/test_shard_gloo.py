"""Sharded frame on two CPU ranks (gloo): the ray ranges partition the grid
and the int32 sum of the partial light maps equals the single-rank map bit
for bit.  Without a GPU the partial maps come from the CPU oracle; what is
under test is the partition and the reduction of splat_gb300.shard."""
import os
import socket

import numpy as np
import pytest

from splat_gb300 import shard


def test_ray_ranges_partition():
    for n in (0, 1, 7, 1000, 1 << 20):
        for w in (1, 2, 3, 8):
            rr = shard.ray_ranges(n, w)
            assert len(rr) == w and rr[0][0] == 0 and rr[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rr[:-1], rr[1:]))
            sizes = [hi - lo for lo, hi in rr]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.ray_ranges(10, 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _small_wl():
    from splat_gb300 import scenes as S
    from splat_gb300 import types as T

    tris, fd = S.assemble(S.sphere_tris(2), S.floor_tris(-1.5, 4.0))
    return S.Workload(name="shard", tris=tris, first_diffuse=fd, light=S.hemisphere_light(1, 40, 1.05),
                      depth=3, material=S.CAUCHY_GLASS, map_w=32, map_h=32, accum="i32",
                      spectrum=S.stratified_spectrum(2), lambda_mode=(T.LAMBDA_UNIFORM, 1, 400.0, 700.0))


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl = _small_wl()
    lo, hi = shard.ray_ranges(wl.n_rays, world)[rank]
    part, _, _ = O.trace_forward(wl, lo, hi, nthreads=1)
    tex = torch.from_numpy(np.ascontiguousarray(part.transpose(2, 1, 0)))
    shard.reduce_maps(tex)
    if rank == 0:
        np.save(out, tex.numpy())
    dist.destroy_process_group()


def test_sharded_frame_equals_single_rank(tmp_path):
    import torch.multiprocessing as mp

    from oracle import oracle as O

    O.build()
    out = str(tmp_path / "map.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, start_method="spawn", join=True)
    full, _, _ = O.trace_forward(_small_wl(), nthreads=1)
    got = np.load(out)
    assert np.array_equal(got, full.transpose(2, 1, 0))
    assert got.sum() > 0
