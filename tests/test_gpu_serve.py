"""Serving form: continuous batching of solves that arrive while others run.

Each request must finish with the same result whether it runs alone or inside a mix of other
requests (same kernels, same arithmetic, residual checks at the same step counts)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIX = [
    dict(kind="ldc", n=128, re=100, u=0.1, storage="f32", max_steps=3000, tol=1e-7, check_every=500, keep_fields=True),
    dict(kind="cylinder", n=32, re=100, u=0.05, storage="f32", max_steps=800, keep_fields=True),
    dict(kind="tgv", n=512, re=200, u=0.02, storage="f16", max_steps=600, keep_fields=True),
    dict(kind="ldc", n=256, re=400, u=0.1, storage="f16", max_steps=1000, keep_fields=True),
    dict(kind="ldc", n=200, re=300, u=0.08, storage="f32", max_steps=700, keep_fields=True),
    dict(kind="cylinder", n=48, re=150, u=0.05, storage="f16", max_steps=500, keep_fields=True),
]


def run(bgk, reqs, stagger=0.0, max_slots=64):
    with bgk.Server(max_slots=max_slots, chunk_steps=100) as srv:
        ids = []
        for r in reqs:
            ids.append(srv.submit(**r))
            if stagger:
                time.sleep(stagger)
        srv.drain(600)
        res = {r["id"]: r for r in srv.poll()}
        out = []
        for i, rq in zip(ids, reqs):
            r = res[i]
            if rq.get("keep_fields"):
                r["fields"] = srv.fields(i, r["lx"], r["ly"])
            out.append(r)
        return out, srv.stats()


def test_alone_equals_in_mix(bgk):
    mixed, st = run(bgk, MIX, stagger=0.01)
    assert st["completed"] == len(MIX) and st["failed"] == 0
    assert st["peak_resident"] >= 2
    for rq, m in zip(MIX, mixed):
        alone, _ = run(bgk, [rq])
        a = alone[0]
        assert a["status"] == 0 and m["status"] == 0
        assert a["steps"] == m["steps"]
        assert a["diagno"] == m["diagno"] and a["draglift"] == m["draglift"]
        for fa, fm in zip(a["fields"], m["fields"]):
            assert np.array_equal(fa, fm)


def test_admission_slots_and_latency(bgk):
    reqs = [dict(kind="ldc", n=128, re=100, u=0.1, storage="f32", max_steps=400) for _ in range(12)]
    out, st = run(bgk, reqs, max_slots=3)
    assert st["completed"] == 12 and st["peak_resident"] <= 3
    assert st["p99_s"] >= st["p50_s"] > 0 and st["glups"] > 0
    assert all(r["steps"] == 400 for r in out)


def test_residual_stop_and_never_fitting_request(bgk):
    with bgk.Server(max_slots=8, chunk_steps=100, hbm_budget=64 << 20) as srv:
        big = srv.submit("ldc", 4096, 1000, 0.1, max_steps=10)          # needs > 64 MiB: rejected
        ok = srv.submit("ldc", 64, 50, 0.1, max_steps=200000, tol=1e-6, check_every=1000)
        srv.drain(300)
        res = {r["id"]: r for r in srv.poll()}
    assert res[big]["status"] == 2  # BGK_E_NOMEM
    assert res[ok]["status"] == 0 and res[ok]["steps"] < 200000 and res[ok]["residual"] < 1e-6
    assert res[ok]["steps"] % 1000 == 0
