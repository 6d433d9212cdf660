"""Transfers through the C ABI (bgk_upload / bgk_download, the reference's host<->device updates).

Page-locked host arrays (torch pinned) are read and written in place by the transfer kernels;
pageable ones go through a device staging buffer (one linear copy per contiguous plane, a 2D
copy for a padded one).  Both paths, with contiguous (ld = lx+2) and padded (ld = lx+2+ipad)
planes, must give the same populations, and a download never writes the padding.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptrs_torch(t):
    return (ctypes.c_void_p * 9)(*[t[q].data_ptr() for q in range(9)])


def _ptrs_np(a):
    return (ctypes.c_void_p * 9)(*[a[q].ctypes.data for q in range(9)])


@pytest.mark.parametrize("storage", ["f32", "f64", "f16"])
@pytest.mark.parametrize("pad", [0, 5])
def test_pinned_and_pageable_transfers_agree(bgk, storage, pad):
    torch = pytest.importorskip("torch")
    lx, ly = 130, 67
    ld = lx + 2 + pad
    tdt = torch.float64 if storage == "f64" else torch.float32
    ndt = np.float64 if storage == "f64" else np.float32
    with bgk.Solver(lx, ly, tcase="LDC", svisc=0.05, u0=0.1, storage=storage) as s:
        s.step(25)
        ref = s.download()  # pageable, staged
        L = s._L

        # download into page-locked buffers
        pinned = torch.full((9, ly + 2, ld), -7.0, dtype=tdt, pin_memory=True)
        assert L.bgk_download(s._h, _ptrs_torch(pinned), ld) == 0
        got = pinned.numpy()
        assert np.array_equal(got[:, :, :lx + 2], ref)
        assert np.all(got[:, :, lx + 2:] == -7.0)  # the padding is not written

        # a pageable array gives the same values
        page = np.full((9, ly + 2, ld), -7.0, dtype=ndt)
        assert L.bgk_download(s._h, _ptrs_np(page), ld) == 0
        assert np.array_equal(page, got)

        # upload a perturbed state from page-locked memory, read it back through staging
        new = ref.copy()
        new[:, 1:ly + 1, 1:lx + 1] *= 0.5
        src = torch.zeros((9, ly + 2, ld), dtype=tdt, pin_memory=True)
        src[:, :, :lx + 2] = torch.from_numpy(new)
        assert L.bgk_upload(s._h, _ptrs_torch(src), ld) == 0
        back_pinned = s.download()
        # and the same from pageable memory
        src_np = np.zeros((9, ly + 2, ld), dtype=ndt)
        src_np[:, :, :lx + 2] = new
        assert L.bgk_upload(s._h, _ptrs_np(src_np), ld) == 0
        back_page = s.download()
        assert np.array_equal(back_pinned, back_page)
        s.step(3)
        assert np.isfinite(s.download()).all()
