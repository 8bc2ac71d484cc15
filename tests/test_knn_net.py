"""The comparator networks of k_knn_t33's queue flush: the generator's 0-1
principle checks pass, the committed header is the generator's output, and the
flush semantics (sorted 33 smallest, the 34th smallest) hold on random data."""
import importlib.util
import os

import numpy as np

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "asmooth_gb300",
                    "csrc")


def _gen():
    spec = importlib.util.spec_from_file_location("gen_knn_net", os.path.join(CSRC, "gen_knn_net.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_header_is_generated():
    gen = _gen()
    with open(os.path.join(CSRC, "asg_knn_net.cuh")) as f:
        assert f.read() == gen.header()


def test_flush_on_random_values():
    gen = _gen()
    sort, merge, order = gen.networks()
    rng = np.random.default_rng(5)
    for trial in range(300):
        # values with repeats, +inf padding and a sorted resident set
        pool = rng.integers(0, 40, 200).astype(np.float64)
        a = np.sort(rng.choice(pool, gen.KA))
        if trial % 3 == 0:
            a[rng.integers(0, gen.KA):] = np.inf
        v = rng.choice(pool, gen.KQ)
        v[rng.integers(0, gen.KQ + 1):] = np.inf
        vs = gen.run(sort, list(v))
        assert vs == sorted(v)
        out = gen.run(merge, list(a) + vs, order)
        want = sorted(list(a) + list(v))
        assert out[:gen.KA + 1] == want[:gen.KA + 1]


def test_queued_flush_model(tmp_path):
    """The queue-and-merge top-33 (CPU model over the generated networks) gives
    the exact 33rd distance and flags every exact tie."""
    import shutil
    import subprocess

    cxx = shutil.which("g++")
    if cxx is None:
        import pytest

        pytest.skip("g++ not available")
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "knn_flush_model.cpp")
    exe = str(tmp_path / "knn_flush_model")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", src, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
