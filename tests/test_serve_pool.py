"""Scene pool of the serving loop on CPU: LRU eviction of idle scenes under
the HBM budget, never of scenes in use."""
import numpy as np

from splat_gb300 import serve


class FakeScene:
    def __init__(self, tris, fd):
        self.n = tris.nbytes
        self.closed = False

    def info(self):
        return {"device_bytes": 3 * self.n}

    def close(self):
        self.closed = True


def _pool(budget):
    def factory(sid):
        return np.zeros((1000 * (sid + 1), 10, 3), np.float32), 2

    return serve.ScenePool(factory, budget, make_scene=FakeScene)


def test_lru_eviction_respects_budget_and_busy_scenes():
    one = 3 * 120000 + serve.SCENE_OVERHEAD  # bytes of scene 0
    pool = _pool(budget=int(one * 3.5))
    a = pool.acquire(0, 0)
    pool.release(0)
    pool.acquire(1, 0)  # stays busy
    pool.acquire(0, 0)
    pool.release(0)     # 0 is now the most recently used
    assert pool.loads == 2 and pool.evictions == 0
    c = pool.acquire(2, 0)  # needs room: evicts nothing busy; 0 is idle
    assert c is not None
    assert pool.evictions >= 1 and 1 in pool.resident and a.closed
    assert pool.used() <= pool.budget
    # nothing idle left to evict and no room: refused
    assert pool.acquire(9, 0) is None
    pool.release(1)
    pool.release(2)
    assert pool.acquire(3, 0) is not None


def test_poisson_arrivals_are_seeded():
    a = serve.poisson_arrivals(200.0, 2.0, seed=6)
    b = serve.poisson_arrivals(200.0, 2.0, seed=6)
    assert np.array_equal(a, b) and np.all(np.diff(a) > 0) and 300 < len(a) < 500
