"""Batched form: many independent cases advanced by one persistent work-list launch per step.

Every case in a batch must evolve exactly as it does alone (same kernels, same arithmetic):
results are compared bit-for-bit against the same case stepped by itself.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_cases(bgk, storage):
    cases = [
        dict(lx=128, ly=128, tcase="LDC", svisc=0.0256, u0=0.1),
        dict(lx=192, ly=192, tcase="LDC", svisc=0.05, u0=0.07),
        dict(lx=96, ly=96, tcase="LDC", svisc=0.02, u0=0.1, trick1=True),  # -DTRICK1 corners
        dict(lx=100, ly=60, tcase="LDC", svisc=0.02, u0=0.05),
        dict(lx=256, ly=64, tcase="TGV", svisc=0.04, u0=0.0, init="tgv", tgv_u0=0.02),
        dict(lx=512, ly=128, tcase="CUSTOM", svisc=0.02, u0=0.0, faces=("inflow", "outflow_zg", "wall", "wall"),
             u_inflow=0.05, inflow_profile=1, obstacle="circle", radius=16, obs_center=(128, 65)),
        dict(lx=160, ly=62, tcase="VKS", svisc=0.05, u0=0.1, radius=6),
        # backward-facing steps: their boundary rules are the fused step's own
        dict(lx=200, ly=64, tcase="BFS", svisc=0.02, u0=0.1),
        dict(lx=120, ly=50, tcase="BFS", svisc=0.03, u0=0.1),
        # Smagorinsky members: their step runs as a batched launch of its own
        dict(lx=144, ly=96, tcase="LDC", svisc=0.005, u0=0.1, les=True, cte_s=0.2),
        dict(lx=128, ly=64, tcase="TGV", svisc=0.01, u0=0.0, init="tgv", tgv_u0=0.02, les=True, cte_s=0.3),
    ]
    return [bgk.Solver(storage=storage, **c) for c in cases], cases


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_batch_equals_alone(bgk, storage):
    members, cases = make_cases(bgk, storage)
    alone = [bgk.Solver(storage=storage, **c) for c in cases]
    with bgk.Batch(storage) as b:
        for s in members:
            b.add(s)
        n, cells = b.size()
        assert n == len(cases) and cells == sum(c["lx"] * c["ly"] for c in cases)
        for chunk in (1, 40, 7, 64):
            b.step(chunk)
            for s in alone:
                s.step(chunk)
        for s, a in zip(members, alone):
            assert s.scalars()["itime"] == a.scalars()["itime"] == 112
            assert np.array_equal(s.download(), a.download())
            assert np.array_equal(s.diagno(), a.diagno())
        # a member can leave and keep stepping alone
        b.remove(members[0])
        members[0].step(3)
        alone[0].step(3)
        assert np.array_equal(members[0].download(), alone[0].download())
    for s in members + alone:
        s.close()


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_batch_long_run_with_members_joining_and_leaving(bgk, storage):
    """2000 steps of the mixed batch in chunks of graph and direct launches, with a member leaving
    halfway and another joining late (the work list rebuilt each time): every member equals the
    same case stepped alone for the same number of steps."""
    members, cases = make_cases(bgk, storage)
    alone = [bgk.Solver(storage=storage, **c) for c in cases]
    late = len(cases) - 1
    with bgk.Batch(storage) as b:
        for i, s in enumerate(members):
            if i != late:
                b.add(s)
        done = [0] * len(cases)
        for k, chunk in enumerate((500, 1, 257, 33, 200, 9, 1000)):
            if k == 3:
                b.remove(members[0])
            if k == 4:
                b.add(members[late])
            b.step(chunk)
            for i, s in enumerate(alone):
                if (i != late or k >= 4) and (i != 0 or k < 3):
                    s.step(chunk)
                    done[i] += chunk
        for i, (s, a) in enumerate(zip(members, alone)):
            assert s.scalars()["itime"] == a.scalars()["itime"] == done[i], i
            assert np.array_equal(s.download(), a.download()), cases[i]
    for s in members + alone:
        s.close()


def test_batch_member_cannot_step_alone(bgk):
    s = bgk.Solver(64, 64)
    with bgk.Batch("f32") as b:
        b.add(s)
        with pytest.raises(bgk.BgkError):
            s.step(1)
        b.step(2)
        assert s.scalars()["itime"] == 2
    s.step(1)
    s.close()


def test_batch_configs_and_tuner_give_same_result(bgk):
    """Tile shape, grid size and graph length change the schedule, never the result."""
    members, cases = make_cases(bgk, "f32")
    ref = [bgk.Solver(storage="f32", **c) for c in cases]
    with bgk.Batch("f32") as b:
        for s in members:
            b.add(s)
        done = 0
        for cfg in ((0, 2, 8), (1, 16, 32), (3, 4, 2), (2, 8, 128), (4, 0, 8), (5, 0, 32)):
            b.set_config(*cfg)
            b.step(130)
            done += 130
        done += b.tune(4)
        tile, bps, g = b.config()
        assert 0 <= tile < 6 and bps in (0, 4, 8, 16) and g in (8, 32, 128)
        for s in ref:
            s.step(done)
        for s, r in zip(members, ref):
            assert np.array_equal(s.download(), r.download())
    for s in members + ref:
        s.close()


@pytest.mark.parametrize("tile,pf", [(1, 64), (5, 608), (4, 1216)])
def test_batch_prefetch_does_not_change_results(bgk, tile, pf):
    """One block per tile with an L2 prefetch of the work-list entry pf places ahead: the same
    populations as the cases stepped alone."""
    members, cases = make_cases(bgk, "f32")
    alone = [bgk.Solver(storage="f32", **c) for c in cases]
    with bgk.Batch("f32") as b:
        for s in members:
            b.add(s)
        b.set_config(tile, 0, 8)
        b.set_prefetch(pf)
        b.step(21)
        for s in alone:
            s.step(21)
        for s, a in zip(members, alone):
            assert np.array_equal(s.download(), a.download())
    for s in members + alone:
        s.close()


def test_unsupported_members_are_rejected(bgk):
    """Two-pass handles carry a second pass the batch kernels do not (backward-facing-step and
    LES members are taken: their boundary routine and their step run as batched launches)."""
    from bgk2d_gpu_gb300 import _lib
    for kw in (dict(tcase="LDC", scheme="original"),):
        lx = kw.pop("lx", 64)
        with bgk.Solver(lx, 64, **kw) as s, bgk.Batch("f32") as b:
            with pytest.raises(bgk.BgkError) as e:
                b.add(s)
            assert e.value.code == _lib.E_UNSUPPORTED
