"""Ping-pong step with the source rows staged in shared memory by bulk async copies (tile
configurations 6, 7, 8).  It must give the same populations as the register-vector kernel: bit
for bit against the oracle in FP32/FP64/MIXED2, and bit for bit against tile configuration 5 in
the 16-bit kinds (same arithmetic, same stochastic-rounding words)."""
import numpy as np
import pytest

from test_gpu_parity import CASES, assert_same, make_pair

pytestmark = pytest.mark.gpu

STAGED = [6, 7, 8]


@pytest.mark.parametrize("cfg", STAGED)
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", list(CASES))
def test_staged_bit_exact_vs_oracle(oracle_mod, bgk, case, prec, cfg):
    o, s = make_pair(oracle_mod, bgk, case, prec, "pingpong")
    with s:
        s.set_tile(cfg)
        for n in (1, 2, 40, 75):          # direct launches and graph replays
            s.step(n)
            o.step(n)
            assert_same(o, s, "pingpong")
        s.sync()


@pytest.mark.parametrize("lx,ly", [(2, 2), (9, 5), (65, 33), (520, 3), (1030, 33), (257, 129)])
def test_staged_ragged_sizes(oracle_mod, bgk, lx, ly):
    """Widths that end inside a vector, a band or the row padding, and stripes of 1-2 rows."""
    o = oracle_mod.Oracle(lx, ly, prec=0, tcase=0, svisc=0.05, u0=0.1)
    with bgk.Solver(lx, ly, tcase="LDC", svisc=0.05, u0=0.1) as s:
        for cfg in STAGED:
            s.set_tile(cfg)
            s.step(3)
            o.step(3)
            assert_same(o, s, "pingpong")
        s.sync()


@pytest.mark.parametrize("storage", ["f16", "bf16"])
@pytest.mark.parametrize("case", ["ldc", "tgv", "vks"])
def test_staged_16bit_identical_to_vector_kernel(bgk, storage, case):
    tc, lx, ly, svisc, u0, _, skw = CASES[case]
    lx, ly = 4 * lx + 3, 3 * ly
    skw = dict(skw)
    if case == "tgv":
        skw["init"] = "tgv"
    out = []
    for cfg in (5, 6, 8):
        with bgk.Solver(lx, ly, tcase=tc, svisc=svisc, u0=u0, storage=storage, **skw) as s:
            s.set_tile(cfg)
            s.step(61)
            out.append(s.download())
    for k in (1, 2):
        g = out[k][:, 1:ly + 1, 1:lx + 1]
        r = out[0][:, 1:ly + 1, 1:lx + 1]
        assert np.array_equal(g, r), f"cfg {(5, 6, 8)[k]}: {int(np.sum(g != r))} populations differ"


def test_staged_tuner_may_pick_it(bgk):
    """The autotuner times the staged configurations too; whichever wins, the result is exact."""
    with bgk.Solver(1024, 512, tcase="LDC", svisc=0.05, u0=0.1, storage="f16") as s:
        cfg, run = s.tune(4)
        # 6 register-vector shapes x 3 prefetch distances + 3 staged shapes, 6 steps each
        assert 0 <= cfg <= 8 and run == (6 * 3 + 3) * 6
        assert s.prefetch() == 0 or cfg < 6
        s.step(10)
        s.sync()


@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
def test_staged_les_bit_exact(oracle_mod, bgk, prec):
    """The eddy-viscosity collision through the staged kernel (a staged configuration of an LES
    handle), on a cavity and on a channel with a cylinder."""
    oprec, st, cp = {"single": (0, "f32", "f32"), "double": (1, "f64", "f64"), "mixed2": (2, "f32", "f64")}[prec]
    for tc, otc, lx, ly, kw, okw in (("LDC", 0, 200, 90, {}, {}),
                                     ("VKS", 3, 160, 62, {"radius": 6}, {"obstacle": 1, "radius": 6})):
        o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=otc, svisc=0.01, u0=0.1, les=True, cte_s=0.2,
                              obs_order=oracle_mod.OBS_SNAPSHOT, **okw)
        with bgk.Solver(lx, ly, tcase=tc, svisc=0.01, u0=0.1, storage=st, compute=cp, les=True, cte_s=0.2,
                        **kw) as s:
            s.set_tile(7)
            s.step(50)
            o.step(50)
            assert_same(o, s, "pingpong")


def test_staged_wait_timeout_reports_status(oracle_mod, bgk, monkeypatch):
    """A staged row that never completes (the test hook declares 16 bytes more than the copies
    bring): every wait gives up after 0.5 s, the step reports BGK_E_TIMEOUT at the next
    synchronisation, the handle stays failed, and the context stays usable for new handles."""
    from bgk2d_gpu_gb300 import _lib
    monkeypatch.setenv("BGK_FAULT_INJECT_STALL", "1")
    s = bgk.Solver(1024, 256, tcase="LDC", svisc=0.05, u0=0.1)
    monkeypatch.delenv("BGK_FAULT_INJECT_STALL")
    try:
        s.set_tile(6)
        s.step(1)
        with pytest.raises(bgk.BgkError) as e:
            s.sync()
        assert e.value.code == _lib.E_TIMEOUT
        with pytest.raises(bgk.BgkError):
            s.step(1)
    finally:
        s.close()
    o = oracle_mod.Oracle(200, 90, prec=0, tcase=0, svisc=0.05, u0=0.1)
    with bgk.Solver(200, 90, tcase="LDC", svisc=0.05, u0=0.1) as t:
        t.set_tile(6)
        t.step(5)
        o.step(5)
        assert_same(o, t, "pingpong")
