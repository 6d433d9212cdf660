"""Invalid arguments through the C ABI: each call fails with BGK_E_INVALID (or BGK_E_CUDA for a
device that does not exist), names the problem in bgk_last_error, and leaves the handle and the
process usable."""
import ctypes

import numpy as np
import pytest

from bgk2d_gpu_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lx,ly", [(0, 16), (1, 16), (16, 1), (-3, 8)])
def test_too_small_domains_are_rejected(bgk, lx, ly):
    with pytest.raises(bgk.BgkError) as e:
        bgk.Solver(lx, ly)
    assert e.value.code == _lib.E_INVALID


def test_unsupported_kind_pair_is_rejected(bgk):
    with pytest.raises(bgk.BgkError) as e:
        bgk.Solver(32, 32, storage="f16", compute="f64")
    assert e.value.code == _lib.E_INVALID


def test_missing_device_leaves_later_handles_working(bgk):
    """A failed cudaSetDevice must not leave an error behind for the next launch check."""
    with pytest.raises(bgk.BgkError) as e:
        bgk.Solver(32, 32, device=97)
    assert e.value.code == _lib.E_CUDA
    with bgk.Solver(32, 32) as s:
        s.step(5)
        assert np.isfinite(s.diagno()).all()


def test_bad_call_arguments_keep_the_handle_usable(bgk):
    with bgk.Solver(40, 30, tcase="LDC", svisc=0.05, u0=0.1) as s, \
            bgk.Solver(40, 30, tcase="LDC", svisc=0.05, u0=0.1) as ref:
        L, h = s._L, s._h
        s.step(4)
        ref.step(4)
        assert L.bgk_step(h, -1) == _lib.E_INVALID
        buf = ctypes.create_string_buffer(256)
        assert L.bgk_last_error(h, buf, 256) == 0 and b"negative" in buf.value
        assert L.bgk_step(h, 0) == 0  # no-op
        pops = s.download()
        ptrs = (ctypes.c_void_p * 9)(*[pops[q].ctypes.data for q in range(9)])
        assert L.bgk_upload(h, ptrs, 40) == _lib.E_INVALID  # ld < lx + 2
        assert L.bgk_download(h, ptrs, 41) == _lib.E_INVALID
        ptrs[3] = None
        assert L.bgk_upload(h, ptrs, 42) == _lib.E_INVALID  # a NULL plane
        out = (ctypes.c_double * 4)()
        assert L.bgk_diagno(h, 7, out) == _lib.E_INVALID
        # the state was not touched and keeps stepping like an untouched handle
        assert np.array_equal(s.download(), ref.download())
        s.step(6)
        ref.step(6)
        assert np.array_equal(s.download(), ref.download())
