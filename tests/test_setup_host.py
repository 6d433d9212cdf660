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
    L.host_init.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p]
    L.host_init.restype = None
    L.host_trick1.argtypes = [ctypes.c_int] * 3
    L.host_trick1.restype = ctypes.c_int
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


@pytest.mark.parametrize("noshift", [0, 1])
@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("tcase,vortex", [(LDC, 0), (TGV, 1)])
def test_initial_state(hostlib, oracle_mod, prec, tcase, vortex, noshift):
    O = oracle_mod
    l, m = 37, 29
    o = O.Oracle(l, m, prec=prec, tcase=tcase, svisc=0.05, u0=0.0 if tcase == TGV else 0.1, noshift=bool(noshift))
    want = o.raw()
    o.close()
    got = np.empty(want.shape, dtype=want.dtype)
    hostlib.host_init(l, m, vortex, prec, noshift, got.ctypes.data_as(ctypes.c_void_p))
    itype = np.uint64 if want.dtype == np.float64 else np.uint32
    assert np.array_equal(got.view(itype), want.view(itype))  # bit for bit, signs of zero included
    if vortex or noshift:
        assert np.abs(want).max() > 0


MASK_CASES = [  # l, m, shape (1 circle, 2 square, 3 half circle), radius, centre (-1: 2l/5, m/2)
    (160, 62, 1, 6, (-1, -1)), (200, 90, 1, 16, (-1, -1)), (97, 61, 1, 11, (40, 30)), (64, 64, 1, 1, (5, 60)),
    (64, 48, 1, 9, (11, 38)), (120, 80, 2, 7, (-1, -1)), (50, 40, 2, 4, (45, 6)), (128, 96, 3, 13, (-1, -1)),
    (80, 64, 3, 20, (30, 20)),
]


@pytest.mark.parametrize("case", MASK_CASES)
def test_obstacle_mask_against_direct_formula(hostlib, case):
    """The obstacle builder against the shape written directly as array expressions over the grid
    (SRC/build.obs.F90:49-80 square |i - ic|, |j - jc| <= r; 81-116 half circle from row m/2;
    174-205 circle (ic - i)^2 + (jc - j)^2 <= r^2 with integer i, j, ic, jc and R = radius),
    sharing no code with either builder; the bounding box and count follow from the mask.  Boxes
    one cell from the walls are the closest the product accepts (a mask touching row or column 1
    or the last one is rejected)."""
    l, m, shape, r, (ic, jc) = case
    _, mask, bb = product_setup(hostlib, l, m, LDC, 0.05, 0.1, SINGLE, shape, r, (ic, jc))
    ic = 2 * l // 5 if ic < 0 else ic
    jc = m // 2 if jc < 0 else jc
    J, I = np.mgrid[1:m + 1, 1:l + 1]
    if shape == 2:
        want = (np.abs(I - ic) <= r) & (np.abs(J - jc) <= r)
    else:
        want = (ic - I) ** 2 + (jc - J) ** 2 <= r * r
        if shape == 3:
            want &= J >= m // 2
    assert np.array_equal(mask.astype(bool), want)
    jj, ii = np.nonzero(want)
    assert bb.tolist() == [ii.min() + 1, ii.max() + 1, jj.min() + 1, jj.max() + 1, int(want.sum())]


@pytest.mark.parametrize("r", [1, 2, 3, 6, 10, 16, 25])
def test_circle_count_is_the_lattice_point_count(hostlib, r):
    """A circle away from the walls covers exactly the lattice points with dx^2 + dy^2 <= r^2:
    sum over dy of 2 isqrt(r^2 - dy^2) + 1 (5, 13, 29, 113, 317, 797, 1961 for the radii here)."""
    import math
    n = 2 * r + 9
    _, mask, bb = product_setup(hostlib, n, n, LDC, 0.05, 0.1, DOUBLE, 1, r, (n // 2, n // 2))
    count = sum(2 * math.isqrt(r * r - dy * dy) + 1 for dy in range(-r, r + 1))
    assert int(mask.sum()) == count == bb[4]
    assert bb.tolist()[:4] == [n // 2 - r, n // 2 + r, n // 2 - r, n // 2 + r]


def test_trick1_accepts_only_the_square_cavity(hostlib, oracle_mod):
    """bgk_case_desc.trick1 turns on the corner rule for a square lid-driven cavity and is refused
    elsewhere, as the oracle (and SRC/check_case.F90:173-178) refuses it."""
    assert hostlib.host_trick1(64, 64, LDC) == 1
    for l, m, tc in ((64, 48, LDC), (64, 64, COU), (64, 64, TGV), (64, 64, POF)):
        assert hostlib.host_trick1(l, m, tc) == -1
        with pytest.raises(ValueError):
            oracle_mod.Oracle(l, m, tcase=tc, trick1=True)
