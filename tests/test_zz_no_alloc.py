"""splat_next_hit_brute_static -- the brute-force hitter for callers that
cannot allocate device memory when they call it (a render callback under a
fixed, pre-admitted memory budget; a Julia finalizer or @cfunction callback
that must not trigger the CUDA.jl allocator).  Its scratch is an array inside
the library, so the caller passes only rays, triangles and the hit-index
output.  Checked through the C ABI against splat_next_hit_brute (the entry
point that takes caller scratch), exactly, on two calls in a row; the second
call is smaller, so stale words from the first call would show.  Collected
last so that a failure here comes after every other test has run."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from helpers import random_rays, small_scene

pytestmark = pytest.mark.gpu


def test_static_scratch_hitter_matches_the_allocating_one():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from splat_gb300 import _lib as L
    from splat_gb300 import tracer

    lib = L.load()
    stream = torch.cuda.current_stream().cuda_stream
    tris, _ = small_scene(3, 0.05)
    d_nt = tracer.n_tris_array(tris)
    nt = tris.shape[0]
    for call, n in enumerate((40000, 9000)):
        rays = random_rays(n, 100 + call, nt)
        d_rays = tracer.rays_to_device(rays)
        ref_hit, _ = tracer.next_hit_brute(d_rays, d_nt)
        hit = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        L.check(lib.splat_next_hit_brute_static(d_rays.data_ptr(), n, d_nt.data_ptr(), nt, hit.data_ptr(), stream))
        torch.cuda.synchronize()
        got, ref = hit.cpu().numpy(), ref_hit.cpu().numpy()
        assert np.array_equal(got, ref), f"call {call}: {np.nonzero(got != ref)[0][:10]}"
        assert (ref > 1).sum() > n // 4

    # the Python constant is the header's cap
    header = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                               "splat.h")).read()
    cap = re.search(r"#define SPLAT_STATIC_HIT_MAX_RAYS \(1 << (\d+)\)", header)
    assert cap and (1 << int(cap.group(1))) == L.STATIC_HIT_MAX_RAYS

    # sizes beyond the library's scratch are refused with a clear message;
    # the size check comes before any launch, so the short hit buffer of the
    # last call above is never written
    too_many = L.STATIC_HIT_MAX_RAYS + 1
    rc = lib.splat_next_hit_brute_static(d_rays.data_ptr(), too_many, d_nt.data_ptr(), nt, hit.data_ptr(), stream)
    assert rc == L.ERR_INVALID
    assert b"exceeds the static scratch" in lib.splat_last_error()
    assert C.sizeof(C.c_uint64) * L.STATIC_HIT_MAX_RAYS == 4 << 20
