"""Maximum sizes: a domain whose device element offsets pass 2^31.

12288^2 FP32 ping-pong holds 18 planes of 12290 x 12290+ elements, about 2.7e9 in all, so every
plane past the eighth starts beyond a 32-bit signed offset. The periodic Taylor-Green start makes
every population non-zero. After two steps, the reference-order diagno sums (compute-kind,
serial order) of ping-pong and AA must equal the threaded oracle's bit for bit; any population
read or written at a wrong offset would change them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 12288


def test_domain_beyond_32bit_offsets(oracle_mod, bgk):
    o = oracle_mod.Oracle(N, N, prec=oracle_mod.SINGLE, tcase=oracle_mod.TGV, svisc=0.05, u0=0.0)
    try:
        o.step(2, threads=16)
        want = [float(x) for x in o.diagno(0)]
        want64 = o.diagno(1)
    finally:
        o.close()
    for scheme in ("pingpong", "aa"):
        with bgk.Solver(N, N, tcase="TGV", svisc=0.05, u0=0.0, init="tgv_ref", scheme=scheme) as s:
            dev_bytes, _ = s.footprint()
            if scheme == "pingpong":
                assert dev_bytes > 2 ** 31 * 4  # element offsets beyond 2^31
            s.step(2)
            assert [float(x) for x in s.diagno(2)] == want, scheme
            np.testing.assert_allclose(s.diagno(), want64, rtol=1e-12, atol=1e-15)
