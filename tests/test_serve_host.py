"""Host-side logic of the render server: the output arena's first-fit
allocator and the request stream (no GPU needed)."""
import math

import numpy as np

from voxurf_gb300 import serve


def test_arena_first_fit_and_merge():
    a = serve.OutputArena(100)
    x = a.alloc(40)
    y = a.alloc(40)
    assert (x, y) == (0, 40)
    assert a.alloc(30) is None          # only 20 left
    a.release(x, 40)
    assert a.alloc(30) == 0             # first fit in the freed range
    a.release(0, 30)
    a.release(y, 40)
    assert a.free == [(0, 100)] and a.used() == 0


def test_request_stream_is_seeded_and_poisson():
    s1 = serve.request_stream(2000, 50.0, 4, seed=3)
    s2 = serve.request_stream(2000, 50.0, 4, seed=3)
    assert [r[0] for r in s1] == [r[0] for r in s2]
    t = np.array([r[0] for r in s1])
    assert np.all(np.diff(t) >= 0)
    assert abs(np.mean(np.diff(t)) - 0.02) < 0.002       # mean inter-arrival 1/rate
    assert {r[1] for r in s1} == {0, 1, 2, 3}
    assert {(r[3], r[4]) for r in s1} == set(serve.RESOLUTIONS)
    for _, _, c2w, _, _ in s1[:50]:
        pos = c2w[:3, 3]
        assert math.isclose(np.linalg.norm(pos), 3.0, rel_tol=1e-9)
        fwd = c2w[:3, 2]
        assert np.allclose(fwd, -pos / 3.0)             # looks at the origin
        R = c2w[:3, :3]
        assert np.allclose(R.T @ R, np.eye(3), atol=1e-9)
    assert all(r[0] == 0.0 for r in serve.request_stream(10, float("inf"), 2))


def test_summarize_percentiles():
    class R:
        def __init__(self, lat, H, W):
            self.latency, self.H, self.W, self.n_pix = lat, H, W, H * W

    reqs = [R(0.010 * (i + 1), 120, 160) for i in range(100)]
    out = serve.summarize(reqs, 2.0)
    assert out["requests"] == 100
    assert math.isclose(out["mpix_s"], 100 * 19200 / 2.0 / 1e6)
    assert math.isclose(out["p50_ms"], 505.0)
    assert "p99_ms_160x120" in out
