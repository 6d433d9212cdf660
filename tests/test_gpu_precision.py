"""Precision form: 16-bit storage of scaled deviations (FP16, BF16) with FP32 collision,
against an FP64 run of the same Taylor-Green case, and the FP64/FP32 decay against the
analytic rate.  Velocity-field L2 errors are relative: ||u - u64||_2 / ||u64||_2."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, U0, TAU = 256, 0.02, 0.6
NU = (TAU - 0.5) / 3.0
OMEGA = 1.0 / TAU


def tgv(bgk, storage, scheme="pingpong"):
    return bgk.Solver(N, N, tcase="TGV", storage=storage, omega=OMEGA, svisc=NU, u0=0.0, init="tgv",
                      tgv_u0=U0, scheme=scheme)


def l2(u, v, u0, v0):
    return np.sqrt(np.sum((u - u0) ** 2 + (v - v0) ** 2) / np.sum(u0 ** 2 + v0 ** 2))


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
def test_16bit_storage_error_vs_fp64(bgk, scheme):
    steps = 2000
    ref = tgv(bgk, "f64")
    ref.step(steps)
    _, u0, v0 = ref.fields()
    errs = {}
    for st in ("f32", "f16", "bf16"):
        s = tgv(bgk, st, scheme)
        s.step(steps)
        _, u, v = s.fields()
        errs[st] = l2(u, v, u0, v0)
        s.close()
    ref.close()
    print("velocity L2 error vs FP64:", errs)
    assert errs["f32"] < 1e-4
    assert errs["f16"] < 1e-3
    assert errs["bf16"] < 3e-2


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_tgv_decay_rate_analytic(bgk, storage):
    """The vortex mode decays as exp(-nu (kx^2 + ky^2) t): amplitude = projection of (u, v) on the
    initial field (the 2k acoustic modes of the equilibrium start are orthogonal to it)."""
    s = tgv(bgk, storage)
    _, ui, vi = s.fields()
    t = int(round(18 * N * np.sqrt(3) / 2))  # whole periods of the 2k acoustic wave
    s.step(t)
    _, u, v = s.fields()
    amp = np.sum(u * ui + v * vi) / np.sum(ui * ui + vi * vi)
    rate = -np.log(amp) / t
    k2 = 2 * (2 * np.pi / N) ** 2
    assert abs(rate / (NU * k2) - 1) < 1e-3
    s.close()


def test_residual_decreases_to_steady_state(bgk):
    s = bgk.Solver(64, 64, tcase="LDC", svisc=0.064, u0=0.1)
    assert s.residual() == 1.0
    s.step(200)
    r1 = s.residual()
    s.step(20000)
    s.residual()
    s.step(200)
    r2 = s.residual()
    assert 0 < r2 < r1 * 1e-2 and r2 < 1e-5
    s.close()


@pytest.mark.parametrize("storage,bound", [("f16", 2e-3), ("bf16", 2e-2)])
def test_tgv_decay_rate_16bit(bgk, storage, bound):
    """The vortex mode of a 16-bit-storage run decays at the analytic rate nu (kx^2 + ky^2), with the
    same projection and window as the FP64/FP32 test above.  The 0.1% bar of that test is not met
    in 16 bits: FP16 measured 1.46e-3 (its velocity L2 error against FP64 is 5.7e-4 here, and the
    amplitude decays by 15% over the window); BF16 keeps 8 significant bits."""
    s = tgv(bgk, storage)
    _, ui, vi = s.fields()
    t = int(round(18 * N * np.sqrt(3) / 2))
    s.step(t)
    _, u, v = s.fields()
    amp = np.sum(u * ui + v * vi) / np.sum(ui * ui + vi * vi)
    rate = -np.log(amp) / t
    k2 = 2 * (2 * np.pi / N) ** 2
    err = abs(rate / (NU * k2) - 1)
    print(f"{storage}: decay rate {rate:.6e}, analytic {NU * k2:.6e}, relative error {err:.2e}")
    assert err < bound
    s.close()
