"""The served request stream of bench.py (CPU): seeded and reproducible, the
stated mix (50/50 kinds, 70% reuse of a resident matrix, 2000 req/s), sizes
inside the stated ranges."""
import importlib.util
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    argv = sys.argv
    sys.argv = ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = argv
    return mod


def test_stream_is_seeded_and_matches_the_stated_mix():
    b = _bench()
    specs, reqs = b.serve_stream(1500)
    specs2, reqs2 = b.serve_stream(1500)
    assert specs == specs2 and reqs == reqs2
    kinds = [specs[m][0] for _, m, _, _ in reqs]
    assert abs(kinds.count("poisson2d") / len(kinds) - 0.5) < 0.05
    new = sum(1 for r in reqs if r[3])
    assert new == len(specs)
    assert abs(1 - new / len(reqs) - 0.7) < 0.05
    rate = len(reqs) / reqs[-1][0]
    assert 1800 < rate < 2200
    for kind, n, _ in specs:
        if kind == "poisson2d":
            assert 64 <= n <= 512
        else:
            assert 1000 <= n <= 200000
    # a reused request names a matrix some earlier request brought
    seen = set()
    for _, m, _, is_new in reqs:
        assert is_new == (m not in seen)
        seen.add(m)


def test_arrivals_increase():
    b = _bench()
    _, reqs = b.serve_stream(300)
    t = np.array([r[0] for r in reqs])
    assert np.all(np.diff(t) > 0)
