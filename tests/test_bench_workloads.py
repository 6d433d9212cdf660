"""The bench's synthetic workloads are seeded and have the documented shapes (CPU only)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_cavity_batch_is_seeded_and_in_range():
    a, b = bench.cfg3_cases(), bench.cfg3_cases()
    assert a == b and len(a) == 96
    assert bench.cfg3_cases(seed=1) != a
    for n, re, u in a:
        assert 128 <= n <= 1536 and n % 64 == 0
        assert 100 <= re <= 5000 and 0.05 <= u <= 0.1
        tau = 3 * u * n / re + 0.5
        assert 0.5 < tau < 5.0  # stable BGK relaxation times
    cells = sum(n * n for n, _, _ in a)
    assert 50e6 < cells < 120e6


def test_request_stream_is_seeded_poisson():
    s1, s2 = bench.cfg4_stream(30.0, 200), bench.cfg4_stream(30.0, 200)
    assert [t for t, _ in s1] == [t for t, _ in s2] and [r for _, r in s1] == [r for _, r in s2]
    t = np.array([t for t, _ in s1])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 30.0) < 0.3 / 30.0  # mean inter-arrival time of a rate-30 stream
    kinds = {r["kind"] for _, r in s1}
    assert kinds == {"ldc", "cylinder", "tgv"}
    assert {r["storage"] for _, r in s1} == {"f32", "f16"}
    for _, r in s1:
        assert r["max_steps"] > 0 and r["n"] >= 32
        if r["kind"] == "ldc" and r.get("tol", 0) > 0:
            assert r["check_every"] > 0
