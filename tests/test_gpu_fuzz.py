"""Seeded random combinations against the oracle, bit for bit.

Each draw picks a case (cavity, vortex, channel, Couette, cylinder channel, periodic volume-forced
MYVERSION, backward-facing step), a precision (SINGLE, DOUBLE, MIXED2), a scheme (ping-pong, AA,
two-pass), a width and height (tiny and ragged ones included), a tile shape, the build variants
that apply (LES, NOSHIFT, TRICK1 on square cavities, FORCING_Y on forced cases) and a step count.
The GPU populations must equal the oracle's after those steps: everywhere, except obstacle
interiors under AA (never advanced there) and the solid block of the backward-facing step.
"""
import numpy as np
import pytest

from test_gpu_parity import PRECS, _bfs_fluid, assert_same

pytestmark = pytest.mark.gpu

ORACLE_CASE = {"LDC": 0, "TGV": 1, "POF": 2, "VKS": 3, "COU": 4, "BFS": 5, "MYV": 6}


def draw(rng):
    tc = str(rng.choice(["LDC", "LDC", "TGV", "POF", "COU", "VKS", "MYV", "BFS"]))
    prec = str(rng.choice(list(PRECS)))
    scheme = str(rng.choice(["pingpong", "aa", "original"]))
    if tc == "VKS":
        lx, ly = int(rng.integers(40, 131)), int(rng.integers(18, 71))
    elif tc == "BFS":
        lx, ly = int(rng.integers(40, 131)), int(rng.integers(4, 71))
    else:
        lx, ly = int(rng.integers(2, 131)), int(rng.integers(2, 71))
    okw, skw = {}, {}
    if tc == "VKS":
        r = int(rng.integers(2, min(8, ly // 2 - 3) + 1))
        okw.update(obstacle=1, radius=r)
        skw.update(radius=r)
    if tc == "TGV":
        skw.update(init="tgv_ref")
    if tc == "LDC" and rng.uniform() < 0.3:
        ly = lx = max(lx, 2)
        okw["trick1"] = skw["trick1"] = True
    if tc in ("POF", "MYV") and rng.uniform() < 0.5:
        okw["force_y"] = skw["force_y"] = True
    les = bool(rng.uniform() < 0.25)
    noshift = bool(rng.uniform() < 0.3)
    if les:
        okw.update(les=True, cte_s=0.2)
        skw.update(les=True, cte_s=0.2)
    if noshift:
        okw["noshift"] = skw["noshift"] = True
    ntile = 9 if scheme == "pingpong" else 6
    tile = int(rng.integers(0, ntile))
    svisc = float(rng.choice([0.01, 0.02, 0.05, 0.1]))
    u0 = 0.0 if tc == "TGV" else float(rng.choice([0.05, 0.1]))
    steps = int(rng.integers(1, 61))
    return dict(tc=tc, prec=prec, scheme=scheme, lx=lx, ly=ly, okw=okw, skw=skw, tile=tile, svisc=svisc, u0=u0,
                steps=steps)


@pytest.mark.parametrize("seed", range(24))
def test_random_combinations_bit_exact(oracle_mod, bgk, seed):
    rng = np.random.default_rng(1000 + seed)
    for _ in range(16):
        c = draw(rng)
        oprec, st, cp = PRECS[c["prec"]]
        o = oracle_mod.Oracle(c["lx"], c["ly"], prec=oprec, tcase=ORACLE_CASE[c["tc"]], svisc=c["svisc"], u0=c["u0"],
                              fused=c["scheme"] != "original", obs_order=oracle_mod.OBS_SNAPSHOT, **c["okw"])
        with bgk.Solver(c["lx"], c["ly"], tcase=c["tc"], svisc=c["svisc"], u0=c["u0"], storage=st, compute=cp,
                        scheme=c["scheme"], **c["skw"]) as s:
            s.set_tile(c["tile"])
            s.step(c["steps"])
            o.step(c["steps"])
            if c["tc"] == "BFS":
                got, want = _bfs_fluid(s.download(), c["lx"], c["ly"]), _bfs_fluid(o.raw(), c["lx"], c["ly"])
                assert np.array_equal(got, want), c
            else:
                try:
                    assert_same(o, s, c["scheme"])
                except AssertionError as e:
                    raise AssertionError(f"{c}: {e}") from None


@pytest.mark.parametrize("storage", ["f32", "f16"])
@pytest.mark.parametrize("seed", range(3))
def test_random_batches_equal_members_alone(bgk, storage, seed):
    """Random mixes of batch members (every case and variant a batch takes: cavities with and
    without TRICK1, vortices, channels with the force along x or y, MYVERSION, Couette, cylinder
    channels, backward-facing steps, LES members), stepped together in uneven chunks, equal the
    same cases stepped alone, bit for bit."""
    rng = np.random.default_rng(2000 + seed)
    kws = []
    for _ in range(int(rng.integers(5, 11))):
        c = draw(rng)
        skw = {k: v for k, v in c["skw"].items() if k != "noshift"}  # batches take deviations only
        kws.append(dict(lx=c["lx"], ly=c["ly"], tcase=c["tc"], svisc=c["svisc"], u0=c["u0"], **skw))
    members = [bgk.Solver(storage=storage, **kw) for kw in kws]
    alone = [bgk.Solver(storage=storage, **kw) for kw in kws]
    try:
        with bgk.Batch(storage) as b:
            for s in members:
                b.add(s)
            for chunk in (int(rng.integers(1, 20)), int(rng.integers(1, 40))):
                b.step(chunk)
                for s in alone:
                    s.step(chunk)
            for kw, s, a in zip(kws, members, alone):
                assert np.array_equal(s.download(), a.download()), kw
    finally:
        for s in members + alone:
            s.close()
