"""The integer IEEE binary64 add and multiply of csrc/bgk_softfp64.h against the host's own
double arithmetic (round to nearest even), bit for bit, on the CPU.

Wherever the integer path reports that it applies, its bits must equal the hardware result; it
must apply to every pair of normal operands with a normal result (and to zeros), so that the
FP64 collision takes it for all the values a simulation produces."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def sfp(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("sfp") / "libsoftfp.so")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                        os.path.join(ROOT, "tests", "softfp", "softfp_host.cpp"), "-o", so],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    P = np.ctypeslib.ndpointer
    for f in (L.soft_add_n, L.soft_mul_n):
        f.argtypes = [P(np.uint64), P(np.uint64), P(np.uint64), P(np.uint8), ctypes.c_int64]
        f.restype = None
    return L


def run(L, fn, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)
    b = np.ascontiguousarray(b, dtype=np.float64).view(np.uint64)
    r = np.zeros_like(a)
    ok = np.zeros(a.shape, dtype=np.uint8)
    getattr(L, fn)(a, b, r, ok, a.size)
    return r.view(np.float64), ok.astype(bool)


def operands(rng, n, espan):
    """Random normal doubles: random sign and significand, exponents within +-espan."""
    mant = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    e = (1023 + rng.integers(-espan, espan + 1, n)).astype(np.uint64)
    sign = rng.integers(0, 2, n).astype(np.uint64) << np.uint64(63)
    return (sign | (e << np.uint64(52)) | mant).view(np.float64)


def check(L, fn, a, b):
    with np.errstate(all="ignore"):
        want = a + b if fn == "soft_add_n" else a * b
    got, ok = run(L, fn, a, b)
    normal = np.isfinite(want) & ((want == 0) | (np.abs(want) >= np.finfo(np.float64).tiny))
    normal &= np.isfinite(a) & np.isfinite(b)
    normal &= ((a == 0) | (np.abs(a) >= np.finfo(np.float64).tiny)) & ((b == 0) | (np.abs(b) >= np.finfo(np.float64).tiny))
    assert np.array_equal(got[ok].view(np.uint64), want[ok].view(np.uint64)), fn
    assert ok[normal].all(), (fn, int((~ok[normal]).sum()))


@pytest.mark.parametrize("espan", [0, 1, 3, 60, 70, 600])
def test_add_random(sfp, espan):
    rng = np.random.default_rng(espan)
    n = 400000
    a, b = operands(rng, n, espan), operands(rng, n, espan)
    check(sfp, "soft_add_n", a, b)
    check(sfp, "soft_add_n", a, -a * (1 + rng.integers(-3, 4, n) * 2.0 ** -52))  # near cancellation


@pytest.mark.parametrize("espan", [0, 5, 300, 520])
def test_mul_random(sfp, espan):
    rng = np.random.default_rng(100 + espan)
    n = 400000
    check(sfp, "soft_mul_n", operands(rng, n, espan), operands(rng, n, espan))


def test_exponent_gaps_and_ties(sfp):
    """Every exponent difference 0..70 for the sum (shifts, sticky bit, one-bit normalisation),
    and products of integers whose exact value sits on or next to a rounding tie."""
    rng = np.random.default_rng(7)
    a = operands(rng, 71 * 2000, 0)
    d = np.repeat(np.arange(71), 2000)
    b = operands(rng, 71 * 2000, 0) * np.ldexp(1.0, -d)
    check(sfp, "soft_add_n", a, b)
    check(sfp, "soft_add_n", a, -b)
    k = rng.integers(1, 1 << 30, 200000).astype(np.float64)
    m = (2.0 ** 53 - rng.integers(1, 1 << 20, 200000)).astype(np.float64)
    check(sfp, "soft_mul_n", k, m)
    check(sfp, "soft_mul_n", m, m)
    check(sfp, "soft_add_n", m, k)


def test_zeros_and_fallbacks(sfp):
    z = np.array([0.0, -0.0, 0.0, -0.0, 1.5, -2.25, 0.0, 3.0])
    w = np.array([0.0, -0.0, -0.0, 0.0, -0.0, 0.0, -7.0, -3.0])
    check(sfp, "soft_add_n", z, w)
    check(sfp, "soft_mul_n", z, w)
    got, ok = run(sfp, "soft_add_n", np.array([-0.0]), np.array([-0.0]))
    assert ok[0] and np.signbit(got[0])
    got, ok = run(sfp, "soft_add_n", np.array([3.0]), np.array([-3.0]))
    assert ok[0] and got[0] == 0 and not np.signbit(got[0])
    # subnormal operands and results, overflow, infinities and NaN go to the hardware
    tiny = np.finfo(np.float64).tiny
    for fn, a, b in (("soft_mul_n", tiny, 0.5), ("soft_mul_n", 1e300, 1e10), ("soft_add_n", np.inf, 1.0),
                     ("soft_add_n", tiny / 4, 1.0), ("soft_mul_n", np.nan, 2.0), ("soft_add_n", tiny, -tiny * 0.75)):
        _, ok = run(sfp, fn, np.array([a]), np.array([b]))
        assert not ok[0], (fn, a, b)


@pytest.mark.gpu
def test_device_build_matches_the_gpus_dadd_and_dmul(tmp_path):
    """The same header compiled for sm_103a: on the GPU its sums and products equal the GPU's own
    DADD and DMUL (and the host's) wherever the integer path applies, and it applies to every
    normal case."""
    from bgk2d_gpu_gb300 import build
    so = str(tmp_path / "libsoftfp_dev.so")
    r = subprocess.run([build.nvcc()] + build.ARCH + ["-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC",
                                                      os.path.join(ROOT, "tests", "softfp", "softfp_device.cu"), "-o", so],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    P = np.ctypeslib.ndpointer
    L.softfp_device_run.argtypes = [P(np.uint64), P(np.uint64), P(np.uint64), P(np.uint8), ctypes.c_int64]
    L.softfp_device_run.restype = ctypes.c_int
    rng = np.random.default_rng(11)
    parts = [(operands(rng, 200000, s), operands(rng, 200000, s)) for s in (0, 2, 60, 70, 500)]
    k = rng.integers(1, 1 << 30, 100000).astype(np.float64)
    m = (2.0 ** 53 - rng.integers(1, 1 << 20, 100000)).astype(np.float64)
    parts += [(k, m), (m, -m * (1 + 2.0 ** -52)), (np.array([0.0, -0.0, 0.0, 2.0]), np.array([-0.0, -0.0, 5.0, -2.0]))]
    a = np.concatenate([p[0] for p in parts]).view(np.uint64)
    b = np.concatenate([p[1] for p in parts]).view(np.uint64)
    out = np.zeros(4 * a.size, dtype=np.uint64)
    ok = np.zeros(2 * a.size, dtype=np.uint8)
    assert L.softfp_device_run(a, b, out, ok, a.size) == 0
    out = out.reshape(-1, 4)
    ok = ok.reshape(-1, 2).astype(bool)
    assert ok.all()  # every pair here is normal with a normal result, or zero
    assert np.array_equal(out[:, 0], out[:, 1])
    assert np.array_equal(out[:, 2], out[:, 3])
    with np.errstate(all="ignore"):
        assert np.array_equal(out[:, 0], (a.view(np.float64) + b.view(np.float64)).view(np.uint64))
        assert np.array_equal(out[:, 2], (a.view(np.float64) * b.view(np.float64)).view(np.uint64))
