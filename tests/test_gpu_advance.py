"""bgk_advance_host (upload, n steps, download in one call) against the three calls in sequence.

The pipelined path cuts the rows into bands and runs upload, steps and download of different
bands in the same launches.  Its result must be the sequential one bit for bit: the populations
written to the host, the state left on the device, and the steps that follow.  Cases cover the
boundary kinds the pipeline takes (walls, moving lid, periodic x, inflow/outflow with a
cylinder), the kinds it hands to the sequential path (periodic y, backward-facing step, AA),
every storage kind, run lengths on both sides of the 32-step split, padded rows, band heights
from one row up, and `out` aliasing `in`.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    "ldc": dict(tcase="LDC", svisc=0.05, u0=0.1),
    "pof": dict(tcase="POF", svisc=0.08, u0=0.1),
    "cou": dict(tcase="COU", svisc=0.05, u0=0.07),
    "vks": dict(tcase="VKS", svisc=0.04, u0=0.1, obstacle="circle", radius=7),
    "tgv": dict(tcase="TGV", svisc=0.05, u0=0.0),
    "bfs": dict(tcase="BFS", svisc=0.05, u0=0.1),
}


def _pinned(torch, a, ld):
    t = torch.full((9, a.shape[1], ld), -3.0, dtype=torch.float64 if a.dtype == np.float64 else torch.float32,
                   pin_memory=True)
    t[:, :, :a.shape[2]] = torch.from_numpy(a)
    return t


def _run(bgk, torch, case, storage, lx, ly, nsteps, pad=0, scheme="pingpong", alias=False, after=3):
    kw = dict(CASES[case], storage=storage, scheme=scheme)
    ld = lx + 2 + pad
    with bgk.Solver(lx, ly, **kw) as a, bgk.Solver(lx, ly, **kw) as b:
        a.step(7)
        start = a.download()
        # sequential reference: upload, steps, download
        b.upload(start)
        b.step(nsteps)
        want = b.download()
        src = _pinned(torch, start, ld)
        dst = src if alias else _pinned(torch, np.zeros_like(start), ld)
        a.advance_host(src, dst, nsteps)
        got = dst.numpy()
        assert np.array_equal(got[:, :, :lx + 2], want), f"{case} {storage} K={nsteps}: populations differ"
        if pad:
            assert np.all(got[:, :, lx + 2:] == -3.0), "row padding was written"
        # the device state and the step parity left behind match too
        assert np.array_equal(a.download(), want)
        a.step(after)
        b.step(after)
        assert np.array_equal(a.download(), b.download())


@pytest.mark.parametrize("storage", ["f32", "f64", "f16", "bf16"])
@pytest.mark.parametrize("case", ["ldc", "vks"])
@pytest.mark.parametrize("nsteps", [1, 5, 32, 45])
def test_advance_equals_sequential(bgk, storage, case, nsteps):
    torch = pytest.importorskip("torch")
    _run(bgk, torch, case, storage, 160 if case == "vks" else 96, 70, nsteps)


@pytest.mark.parametrize("case", ["pof", "cou", "tgv", "bfs"])
def test_advance_other_boundaries(bgk, case):
    torch = pytest.importorskip("torch")
    _run(bgk, torch, case, "f32", 120 if case == "bfs" else 64, 50, 20)


@pytest.mark.parametrize("storage,extra", [("f32", dict(les=True, cte_s=0.2)), ("f16", dict(les=True, cte_s=0.2)),
                                           ("f32", dict(noshift=True)), ("f64", dict(noshift=True)),
                                           ("f64", dict(noshift=True, les=True, cte_s=0.2))])
def test_advance_collision_variants_pipelined(bgk, storage, extra):
    """Handles with the Smagorinsky collision or whole-population storage go through the same
    pipelined waves (their own kernel variant inside) and match the three calls bit for bit."""
    torch = pytest.importorskip("torch")
    lx, ly, K = 96, 70, 20
    kw = dict(tcase="LDC", svisc=0.01, u0=0.1, storage=storage, **extra)
    with bgk.Solver(lx, ly, **kw) as a, bgk.Solver(lx, ly, **kw) as b:
        a.step(7)
        start = a.download()
        b.upload(start)
        b.step(K)
        want = b.download()
        src = _pinned(torch, start, lx + 2)
        dst = _pinned(torch, np.zeros_like(start), lx + 2)
        n0 = a.launches()
        a.advance_host(src, dst, K)
        # one launch per wave: more than the K + 2 of the sequential calls
        assert a.launches() - n0 > K + 2
        assert np.array_equal(dst.numpy(), want)
        a.step(3)
        b.step(3)
        assert np.array_equal(a.download(), b.download())


def test_advance_aa_takes_the_sequential_path(bgk):
    torch = pytest.importorskip("torch")
    _run(bgk, torch, "ldc", "f32", 64, 40, 9, scheme="aa")


@pytest.mark.parametrize("rows", ["1", "3", "16"])
def test_advance_band_heights_padding_and_alias(bgk, rows, monkeypatch):
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("BGK_PIPE_ROWS", rows)
    monkeypatch.setenv("BGK_PIPE_XFER", "3")
    _run(bgk, torch, "ldc", "f32", 130, 67, 12, pad=5)
    _run(bgk, torch, "vks", "f64", 150, 45, 7, alias=True)
    _run(bgk, torch, "vks", "f16", 200, 61, 40, alias=True)


def test_advance_unevenly_spaced_planes(bgk):
    """Nine separate page-locked planes (not one allocation), as a driver may pass them."""
    torch = pytest.importorskip("torch")
    lx, ly, K = 90, 52, 9
    kw = dict(tcase="LDC", svisc=0.05, u0=0.1)
    with bgk.Solver(lx, ly, **kw) as a, bgk.Solver(lx, ly, **kw) as b:
        a.step(5)
        start = a.download()
        b.upload(start)
        b.step(K)
        want = b.download()
        src = [torch.from_numpy(start[q].copy()).pin_memory() for q in range(9)]
        dst = [torch.zeros((ly + 2, lx + 2), dtype=torch.float32).pin_memory() for _ in range(9)]
        import ctypes
        pin = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in src])
        pout = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in dst])
        assert a._L.bgk_advance_host(a._h, pin, pout, lx + 2, K) == 0
        got = np.stack([t.numpy() for t in dst])
        assert np.array_equal(got, want)


def test_advance_pageable_arrays(bgk):
    """numpy (pageable) arrays take the staging copies; same result."""
    lx, ly = 80, 48
    with bgk.Solver(lx, ly, tcase="LDC", svisc=0.05, u0=0.1) as a, bgk.Solver(lx, ly, tcase="LDC", svisc=0.05, u0=0.1) as b:
        a.step(4)
        start = a.download()
        b.upload(start)
        b.step(10)
        out = np.zeros_like(start)
        a.advance_host(start, out, 10)
        assert np.array_equal(out, b.download())


def test_advance_rejects_bad_arguments(bgk):
    torch = pytest.importorskip("torch")
    with bgk.Solver(32, 24, tcase="LDC", svisc=0.05, u0=0.1) as s:
        buf = torch.zeros((9, 26, 34), dtype=torch.float32, pin_memory=True)
        import ctypes
        p = s._host_ptrs(buf)
        L = s._L
        assert L.bgk_advance_host(s._h, p, p, 33, 4) == bgk._lib.E_INVALID   # ld < lx + 2
        assert L.bgk_advance_host(s._h, p, p, 34, -1) == bgk._lib.E_INVALID  # negative step count
        null = (ctypes.c_void_p * 9)()
        assert L.bgk_advance_host(s._h, null, p, 34, 4) == bgk._lib.E_INVALID
        s.step(2)  # the handle still works
        assert np.isfinite(s.download()).all()


@pytest.mark.skipif(os.environ.get("BGK_LARGE_TESTS") == "0", reason="large case disabled")
def test_advance_large_cavity(bgk):
    """4096^2 FP32 cavity, 20 steps (the bench's end-to-end workload), against the sequential calls."""
    torch = pytest.importorskip("torch")
    n = 4096
    with bgk.Solver(n, n, tcase="LDC", svisc=0.04096, u0=0.1) as a:
        a.step(3)
        start = torch.empty((9, n + 2, n + 2), dtype=torch.float32, pin_memory=True)
        L = a._L
        assert L.bgk_download(a._h, a._host_ptrs(start), n + 2) == 0
        out = torch.empty_like(start).pin_memory()
        a.advance_host(start, out, 20)
        got = out.numpy().copy()
        assert L.bgk_upload(a._h, a._host_ptrs(start), n + 2) == 0
        a.step(20)
        want = torch.empty_like(start).pin_memory()
        assert L.bgk_download(a._h, a._host_ptrs(want), n + 2) == 0
        assert np.array_equal(got, want.numpy())
