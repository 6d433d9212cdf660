"""The product's host-side case setup against the oracle, on the CPU.

bgk_create runs csrc/bgk_setup.h on the host before it allocates anything. tests/setup_host/
compiles that header, unchanged, into a small library that makes no CUDA call. Its results are
compared bit for bit with the oracle's restatement for each precision and case:
- omega, fgrad, u00, u0 (SRC/hencol.F90:30-50, SRC/build.bcond.F90:47-56);
- obstacle masks and bounding boxes (SRC/build.obs.F90:49-205);
- the initial populations (SRC/init.F90:83-137)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SINGLE, DOUBLE, MIXED2 = 0, 1, 2
LDC, TGV, POF, VKS, COU = 0, 1, 2, 3, 4
PRECS = [SINGLE, DOUBLE, MIXED2]


@pytest.fixture(scope="module")
def hostlib(tmp_path_factory):
    from bgk2d_gpu_gb300 import build
    so = str(tmp_path_factory.mktemp("setup") / "libsetup_host.so")
    cmd = [build.nvcc()] + build.ARCH + ["-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                                         "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                                         os.path.join(ROOT, "tests", "setup_host", "setup_host.cu"), "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    ip = ctypes.POINTER(ctypes.c_int32)
    dp = ctypes.POINTER(ctypes.c_double)
    L.host_setup.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 2 + [ctypes.c_int] * 5 + [dp, ip, ip]
    L.host_setup.restype = ctypes.c_int
    L.host_init.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p]
    L.host_init.restype = None
    return L


def product_setup(L, l, m, tcase, svisc, u0, prec, obstacle=0, radius=16, centre=(-1, -1)):
    sc = np.zeros(4)
    mask = np.zeros(l * m, dtype=np.int32)
    bb = np.zeros(5, dtype=np.int32)
    rc = L.host_setup(l, m, tcase, svisc, u0, prec, obstacle, radius, centre[0], centre[1],
                      sc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                      mask.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                      bb.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    assert rc == 0
    return sc, mask.reshape(m, l), bb


CASES = [  # l, m, tcase, svisc, u0, obstacle, radius, centre
    (64, 48, LDC, 0.0384, 0.1, 0, 16, (-1, -1)),
    (32, 24, POF, 0.1, 0.1, 0, 16, (-1, -1)),
    (40, 30, COU, 0.05, 0.07, 0, 16, (-1, -1)),
    (48, 40, TGV, 1 / 30, 0.0, 0, 16, (-1, -1)),
    (160, 62, VKS, 0.05, 0.1, 1, 8, (-1, -1)),
    (120, 50, VKS, 0.02, 0.1, 1, 11, (37, 26)),
    (96, 64, LDC, 0.05, 0.1, 2, 9, (40, 30)),
    (96, 64, LDC, 0.05, 0.1, 3, 13, (-1, -1)),
]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", CASES)
def test_scalars_masks_and_boxes(hostlib, oracle_mod, prec, case):
    O = oracle_mod
    l, m, tcase, svisc, u0, obstacle, radius, centre = case
    o = O.Oracle(l, m, prec=prec, tcase=tcase, svisc=svisc, u0=u0, obstacle=obstacle, radius=radius,
                 obs_icoord=centre[0], obs_jcoord=centre[1])
    want = o.scalars()
    want_mask, want_bb = o.obs()
    o.close()
    if prec == SINGLE:  # namelist values are read in the compute kind
        svisc, u0 = float(np.float32(svisc)), float(np.float32(u0))
    sc, mask, bb = product_setup(hostlib, l, m, tcase, svisc, u0, prec, obstacle, radius, centre)
    assert sc.tolist() == [want["omega"], want["fgrad"], want["u00"], want["u0"]]
    assert np.array_equal(mask, want_mask)
    if obstacle:
        assert mask.sum() > 0 and bb.tolist() == want_bb.tolist()


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("tcase,vortex", [(LDC, 0), (TGV, 1)])
def test_initial_state(hostlib, oracle_mod, prec, tcase, vortex):
    O = oracle_mod
    l, m = 37, 29
    o = O.Oracle(l, m, prec=prec, tcase=tcase, svisc=0.05, u0=0.0 if tcase == TGV else 0.1)
    want = o.raw()
    o.close()
    got = np.empty(want.shape, dtype=want.dtype)
    hostlib.host_init(l, m, vortex, prec, got.ctypes.data_as(ctypes.c_void_p))
    itype = np.uint64 if want.dtype == np.float64 else np.uint32
    assert np.array_equal(got.view(itype), want.view(itype))  # bit for bit, signs of zero included
    if vortex:
        assert np.abs(want).max() > 0
