"""The autotuner's decision logic and cache, without a GPU: the crossover
from sweep timings, the per-frame hitter it implies, coordinate descent over
knobs with a cost model, and the JSON cache round trip."""
import pytest

from splat_gb300 import _lib as L
from splat_gb300 import autotune as A


def test_crossover_from_sweep_rows():
    rows = [{"n_tris": 32, "ms": {"brute": 1.0, "bvh": 2.0}},
            {"n_tris": 128, "ms": {"brute": 2.0, "bvh": 1.5}},
            {"n_tris": 512, "ms": {"brute": 8.0, "bvh": 2.0}}]
    assert A.crossover_from(rows) == 128
    # a noisy win below a loss does not move the crossover down
    rows2 = [{"n_tris": 32, "ms": {"brute": 3.0, "bvh": 2.0}}] + rows[1:]
    rows2.insert(1, {"n_tris": 64, "ms": {"brute": 1.0, "bvh": 1.2}})
    assert A.crossover_from(rows2) == 128
    # the BVH wins everywhere / nowhere
    assert A.crossover_from([{"n_tris": 32, "ms": {"brute": 2.0, "bvh": 1.0}}]) == 32
    assert A.crossover_from([{"n_tris": 32, "ms": {"brute": 1.0, "bvh": 2.0}}]) == 33
    assert A.crossover_from(list(reversed(rows))) == 128


def test_hitter_for_and_tuned_hitters():
    assert A.hitter_for(100, 128) == "brute" and A.hitter_for(128, 128) == "bvh"

    class W:
        def __init__(self, n):
            self.n_tris = n

    assert A.tuned_hitters([W(10), W(512), W(200000)], 512) == ["brute", "bvh", "bvh"]


def test_descend_finds_the_cheapest_corner():
    choices = {1: (4, 8, 16), 2: (0, 1)}

    def cost(k):
        return abs(k[1] - 8) + 3 * (k[2] == 0)

    best, c, trials = A.descend(choices, {1: 16, 2: 0}, cost)
    assert best == {1: 8, 2: 1} and c == 0
    assert len(trials) >= 4 and trials[0] == ({1: 16, 2: 0}, 11)


def test_bucket_groups_nearby_sizes():
    assert A._bucket(1000) == A._bucket(1100)
    assert A._bucket(1000) != A._bucket(2000)
    assert A._bucket(0) == A._bucket(1) == 0


def test_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("SPLAT_TUNE_CACHE", str(tmp_path / "sub" / "tuning.json"))
    assert A.cache_get("x") is None
    A.cache_put("x", {"crossover_tris": 256})
    A.cache_put("y", [1, 2])
    assert A.cache_get("x") == {"crossover_tris": 256} and A.cache_get("y") == [1, 2]
    # a damaged file reads as empty, and is replaced on the next write
    (tmp_path / "sub" / "tuning.json").write_text("{not json")
    assert A.cache_get("x") is None
    A.cache_put("z", 1)
    assert A.cache_get("z") == 1


def test_knob_choices_are_accepted_by_the_library():
    """Every value the tuner may set passes splat_set_tuning's checks."""
    lib = L.load()
    for choices in (A.KNOB_CHOICES, A.BATCH_KNOB_CHOICES):
        old = {k: lib.splat_get_tuning(k) for k in choices}
        try:
            for k, vals in choices.items():
                for v in vals:
                    assert lib.splat_set_tuning(k, v) == L.OK, (k, v)
        finally:
            for k, v in old.items():
                L.check(lib.splat_set_tuning(k, v))


def test_crossover_frame_has_the_requested_size():
    wl = A.crossover_frame(500, 1 << 12)
    assert wl.n_tris == 1 + 500 + 2 and wl.n_rays == 64 * 64 and wl.hitter == "bvh"
