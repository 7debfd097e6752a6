"""The committed golden fixtures are what tests/golden/make_golden.py makes
now: regenerating them (the reference's own Python code over the oracle's
restatement of its CUDA ops) into a temporary directory reproduces every
array of the committed files: bit for bit, except float64 results that go
through multi-threaded sums (to 1e-12).  A change of the restatement that
moves a fixture (as a change of its float forms does) fails here until the
fixtures are regenerated.  Runs where a reference checkout is present
($VOXURF_REFERENCE, or the recipe's default location); skips elsewhere.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import ref_build

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")

# fixture name -> files it writes (npz files compared array by array)
FIXTURES = {
    "fine": ["fine_step_golden.npz"],
    "coarse": ["coarse_step_golden.npz"],
    "ckpt": ["ckpt_golden.npz"],
    "womask": ["womask_step_golden.npz"],
    "womask_coarse": ["womask_coarse_step_golden.npz"],
    "bg": ["bg_golden.npz"],
    "tv": ["tv_golden.npz"],
    "ops": ["ops_golden.npz"],
    "mesh": ["mesh_golden.npz"],
}


@pytest.mark.skipif(ref_build.reference_root() is None, reason="the reference checkout is not present here")
def test_fixtures_regenerate_bit_for_bit(tmp_path):
    env = dict(os.environ, VOXURF_REFERENCE=ref_build.reference_root(), VOXURF_GOLDEN_OUT=str(tmp_path),
               PYTHONDONTWRITEBYTECODE="1", OMP_NUM_THREADS="4")
    r = subprocess.run([sys.executable, os.path.join(GOLDEN, "make_golden.py"), *FIXTURES], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    for files in FIXTURES.values():
        for f in files:
            new, old = np.load(tmp_path / f), np.load(os.path.join(GOLDEN, f))
            assert sorted(new.files) == sorted(old.files), f
            diff = []
            for k in old.files:
                a, b = old[k], new[k]
                if a.shape != b.shape:
                    diff.append(k)
                elif a.dtype.kind == "f" and a.dtype.itemsize == 8:
                    # float64 sums (BLAS) depend on the host's thread count
                    if not np.allclose(b, a, rtol=1e-12, atol=1e-300 + 1e-12 * float(np.abs(a).max(initial=0))):
                        diff.append(k)
                elif not np.array_equal(a, b):
                    diff.append(k)
            assert not diff, (f, diff[:10])
