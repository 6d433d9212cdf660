"""bgk_diagno_noalloc: diagno sums for callers that cannot let the library allocate.

Such a caller (for example an OpenACC or OpenMP-offload Fortran build whose populations live in
device data regions owned by its compiler's runtime, or a program under a fixed device-memory
budget) passes device pointers to its own nine population arrays.  The sums use one static
device array instead of allocated scratch.  Checked here against bgk_diagno of a handle holding
the same state, on two calls in a row, at the tolerance the other reduction tests use; this
file is collected last so that a stop at its first failure has run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_copies(torch, pops):
    """Caller-owned device arrays holding the downloaded populations (reference layout)."""
    return [torch.from_numpy(np.ascontiguousarray(pops[q])).cuda() for q in range(9)]


@pytest.mark.parametrize("storage", ["f32", "f64"])
def test_noalloc_diagno_matches_handle_diagno(bgk, storage):
    torch = pytest.importorskip("torch")
    from bgk2d_gpu_gb300 import _lib
    L = _lib.load()
    lx, ly = 200, 120
    with bgk.Solver(lx, ly, tcase="LDC", svisc=0.02, u0=0.1, storage=storage) as s:
        s.step(150)
        want = s.diagno()
        pops = s.download()
    dev = _device_copies(torch, pops)
    torch.cuda.synchronize()
    ptrs = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in dev])
    code = _lib.STORE[storage]
    for call in range(2):
        out = np.zeros(4)
        rc = L.bgk_diagno_noalloc(ptrs, lx + 2, lx, ly, code, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert rc == 0, (call, rc)
        np.testing.assert_allclose(out, want, rtol=1e-12, atol=1e-15)


def test_noalloc_diagno_rejects_too_large_and_bad_arguments(bgk):
    from bgk2d_gpu_gb300 import _lib
    L = _lib.load()
    out = np.zeros(4)
    P = ctypes.POINTER(ctypes.c_double)
    fake = (ctypes.c_void_p * 9)(*([1] * 9))  # never dereferenced: the size check comes first
    rc = L.bgk_diagno_noalloc(fake, 4098 + 2, 4098, 4098, 0, out.ctypes.data_as(P))
    assert rc == _lib.E_TOOLARGE
    rc = L.bgk_diagno_noalloc(fake, 10, 64, 64, 0, out.ctypes.data_as(P))  # ld < lx + 2
    assert rc == _lib.E_INVALID
    rc = L.bgk_diagno_noalloc(fake, 66, 64, 64, 2, out.ctypes.data_as(P))  # 16-bit storage not accepted
    assert rc == _lib.E_INVALID


@pytest.mark.parametrize("lx,ly,pad", [(130, 67, 9), (1024, 1024, 0), (1000, 1000, 37)])
def test_noalloc_diagno_padded_rows_and_many_chunks(bgk, lx, ly, pad):
    """Rows longer than lx + 2 (a padded leading dimension, as ipad gives) and domains of a few
    hundred chunks, against bgk_diagno, on two calls in a row."""
    torch = pytest.importorskip("torch")
    from bgk2d_gpu_gb300 import _lib
    L = _lib.load()
    ld = lx + 2 + pad
    with bgk.Solver(lx, ly, tcase="LDC", svisc=0.05, u0=0.1) as s:
        s.step(60)
        want = s.diagno()
        pops = s.download()
    dev = torch.full((9, ly + 2, ld), 1e30, dtype=torch.float32, device="cuda")  # padding never read
    dev[:, :, :lx + 2] = torch.from_numpy(pops).cuda()
    torch.cuda.synchronize()
    ptrs = (ctypes.c_void_p * 9)(*[dev[q].data_ptr() for q in range(9)])
    for call in range(2):
        out = np.zeros(4)
        rc = L.bgk_diagno_noalloc(ptrs, ld, lx, ly, 0, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert rc == 0, (call, rc)
        np.testing.assert_allclose(out, want, rtol=1e-12, atol=1e-15)
