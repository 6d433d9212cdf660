"""The serving scheduler's host logic on the CPU.

csrc/bgk_serve.cpp is compiled unchanged against tests/serve_fake/ (a fake of the handle and batch
entry points, and of the few CUDA runtime calls it makes), where a step only counts steps. The
tests check what the scheduler itself decides: admission against the HBM budget and the slot
limit, FIFO order, residual checks at multiples of check_every, per-request statuses when a
batch fails or a result is not finite, the fields hand-over, and (under ThreadSanitizer) that
client threads and the scheduler thread share no state without a lock."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FAKE = os.path.join(ROOT, "tests", "serve_fake")
OK, E_INVALID, E_NOMEM, E_CUDA, E_NUMERIC, E_NOTFOUND = 0, 1, 2, 3, 5, 8
F32, F16 = 0, 2


@pytest.fixture(scope="module")
def srvlib(tmp_path_factory):
    from bgk2d_gpu_gb300 import _lib
    so = str(tmp_path_factory.mktemp("serve") / "libserve_fake.so")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", "-I", FAKE,
                        os.path.join(ROOT, "bgk2d_gpu_gb300", "csrc", "bgk_serve.cpp"),
                        os.path.join(FAKE, "fake_abi.cpp"), "-o", so, "-lpthread"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(so)
    P, VP, I32, I64, F64 = ctypes.POINTER, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    for name, args in {
        "bgk_server_create": [P(_lib.ServerConfig), P(VP)],
        "bgk_server_destroy": [VP],
        "bgk_server_submit": [VP, P(_lib.Request), P(I64)],
        "bgk_server_poll": [VP, P(_lib.Result), I32, P(I32)],
        "bgk_server_drain": [VP, F64],
        "bgk_server_fields": [VP, I64, P(F64), P(F64), P(F64), I64],
        "bgk_server_get_stats": [VP, P(_lib.ServerStats)],
        "fake_configure": [I32, F64],
        "fake_counts": [P(I64)],
        "fake_set_free_bytes": [I64],
    }.items():
        getattr(L, name).argtypes = args
        getattr(L, name).restype = I32 if name.startswith("bgk_") else None
    return L, _lib


class Srv:
    def __init__(self, srvlib, max_slots=8, chunk_steps=100, hbm_budget=0, fail_storage=-1, nan_u0=-1.0):
        self.L, self.lib = srvlib
        self.L.fake_configure(fail_storage, nan_u0)
        cfg = self.lib.ServerConfig(device=0, max_slots=max_slots, hbm_budget=hbm_budget,
                                    chunk_steps=chunk_steps, tile_cfg=-1)
        self.s = ctypes.c_void_p()
        assert self.L.bgk_server_create(ctypes.byref(cfg), ctypes.byref(self.s)) == OK

    def submit(self, kind=0, n=64, re=100.0, u=0.1, storage=F32, max_steps=1000, tol=0.0, check_every=0,
               keep_fields=0):
        rq = self.lib.Request(kind=kind, n=n, re=re, u=u, storage=storage, max_steps=max_steps, tol=tol,
                              check_every=check_every, keep_fields=keep_fields)
        i = ctypes.c_int64()
        assert self.L.bgk_server_submit(self.s, ctypes.byref(rq), ctypes.byref(i)) == OK
        return i.value

    def finish(self):
        assert self.L.bgk_server_drain(self.s, 60.0) == OK
        buf = (self.lib.Result * 256)()
        n = ctypes.c_int32()
        assert self.L.bgk_server_poll(self.s, buf, 256, ctypes.byref(n)) == OK
        st = self.lib.ServerStats()
        assert self.L.bgk_server_get_stats(self.s, ctypes.byref(st)) == OK
        return {buf[k].id: buf[k] for k in range(n.value)}, st

    def counts(self):
        c = (ctypes.c_int64 * 3)()
        self.L.fake_counts(c)
        return list(c)

    def close(self):
        assert self.L.bgk_server_destroy(self.s) == OK


def request_bytes(n, elem=4):
    """The scheduler's own device-byte estimate of an n x n request (bgk_serve.cpp estimate_bytes)."""
    pitch = ((n + 32) * elem + 127) // 128 * 128
    return 18 * pitch * (n + 2) + (n + 2) ** 2 * 4 + n * n * 16 + (n + 2) * ((n + 33) // 32) * 4 + (1 << 20)


def test_budget_admits_two_at_a_time(srvlib):
    s = Srv(srvlib, max_slots=64, hbm_budget=int(2.5 * request_bytes(256)))
    ids = [s.submit(n=256, max_steps=20000) for _ in range(6)]
    res, st = s.finish()
    s.close()
    assert all(res[i].status == OK and res[i].steps == 20000 for i in ids)
    assert st.peak_resident == 2 and st.completed == 6
    assert s.counts()[:2] == [0, 2]  # every handle freed; never more than two alive


def test_rejected_request_does_not_enlarge_the_budget(srvlib):
    """A request that can never fit is rejected without charging its bytes: the requests after
    it are still admitted two at a time."""
    s = Srv(srvlib, max_slots=64, hbm_budget=int(2.5 * request_bytes(256)))
    big = s.submit(n=4096, max_steps=10)
    ids = [s.submit(n=256, max_steps=20000) for _ in range(6)]
    res, st = s.finish()
    s.close()
    assert res[big].status == E_NOMEM and res[big].steps == 0
    assert all(res[i].status == OK for i in ids)
    assert st.peak_resident == 2 and st.failed == 1 and st.completed == 6
    assert s.counts()[1] == 2


def test_slot_limit_and_fifo(srvlib):
    s = Srv(srvlib, max_slots=3)
    ids = [s.submit(max_steps=5000) for _ in range(9)]
    res, st = s.finish()
    s.close()
    assert st.peak_resident <= 3 and s.counts()[1] <= 3
    admits = [res[i].t_admit for i in ids]
    assert admits == sorted(admits)  # first come, first admitted


def test_residual_checks_at_multiples_of_check_every(srvlib):
    """Residual 1/s in the fake: the first check (s = 500) sets the snapshot, s = 1000 gives
    exactly the tolerance (not below it), s = 1500 stops the request."""
    s = Srv(srvlib, chunk_steps=300)
    a = s.submit(max_steps=100000, tol=1e-3, check_every=500)
    b = s.submit(max_steps=700)  # rounds must also stop at its budget
    res, _ = s.finish()
    s.close()
    assert res[a].status == OK and res[a].steps == 1500 and res[a].residual == pytest.approx(1 / 1500)
    assert res[b].status == OK and res[b].steps == 700


def test_failed_batch_fails_only_its_requests(srvlib):
    s = Srv(srvlib, fail_storage=F16)
    good = [s.submit(storage=F32, max_steps=400) for _ in range(2)]
    bad = [s.submit(storage=F16, max_steps=400) for _ in range(2)]
    res, st = s.finish()
    s.close()
    assert all(res[i].status == OK and res[i].steps == 400 for i in good)
    assert all(res[i].status == E_CUDA for i in bad)
    assert st.completed == 2 and st.failed == 2 and s.counts()[0] == 0


def test_non_finite_result_without_residual_checks(srvlib):
    s = Srv(srvlib, nan_u0=0.0625)
    ok = s.submit(u=0.1, max_steps=300)
    blown = s.submit(u=0.0625, max_steps=300, keep_fields=1)
    res, st = s.finish()
    assert res[ok].status == OK and res[blown].status == E_NUMERIC
    z = np.zeros(64 * 64)
    p = ctypes.POINTER(ctypes.c_double)
    # a failed request keeps no fields
    assert s.L.bgk_server_fields(s.s, blown, z.ctypes.data_as(p), z.ctypes.data_as(p), z.ctypes.data_as(p),
                                 z.size) == E_NOTFOUND
    s.close()
    assert st.failed == 1


def test_fields_capacity(srvlib):
    s = Srv(srvlib)
    i = s.submit(n=64, max_steps=250, keep_fields=1)
    res, _ = s.finish()
    assert res[i].status == OK and (res[i].lx, res[i].ly) == (64, 64)
    p = ctypes.POINTER(ctypes.c_double)
    small = np.zeros(64 * 63)
    args = [small.ctypes.data_as(p)] * 3
    assert s.L.bgk_server_fields(s.s, i, *args, small.size) == E_INVALID  # kept for a retry
    rho, u, v = np.zeros(64 * 64), np.zeros(64 * 64), np.zeros(64 * 64)
    assert s.L.bgk_server_fields(s.s, i, rho.ctypes.data_as(p), u.ctypes.data_as(p), v.ctypes.data_as(p),
                                 rho.size) == OK
    assert np.all(rho == 250)
    assert s.L.bgk_server_fields(s.s, i, rho.ctypes.data_as(p), u.ctypes.data_as(p), v.ctypes.data_as(p),
                                 rho.size) == E_NOTFOUND  # handed over once
    s.close()


def test_scheduler_has_no_data_races(tmp_path):
    """tests/serve_fake/race_main.cpp under ThreadSanitizer: client threads submit, poll and read
    statistics while the scheduler thread runs rounds; no unsynchronised access is reported."""
    exe = str(tmp_path / "race")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=thread", "-I", FAKE,
                        os.path.join(FAKE, "race_main.cpp"),
                        os.path.join(ROOT, "bgk2d_gpu_gb300", "csrc", "bgk_serve.cpp"),
                        os.path.join(FAKE, "fake_abi.cpp"), "-o", exe, "-lpthread"], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no ThreadSanitizer in this toolchain: " + r.stderr.strip().splitlines()[-1][:120])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    if "unexpected memory mapping" in r.stderr or "FATAL: ThreadSanitizer" in r.stderr:
        pytest.skip("ThreadSanitizer cannot run on this kernel's memory layout")
    assert "WARNING: ThreadSanitizer" not in r.stderr, r.stderr[:4000]
    assert r.returncode == 0, (r.stdout, r.stderr[:2000])


def test_admission_sees_memory_taken_after_creation(srvlib):
    """Free HBM is read again at every admission: while another process holds the memory (the
    fake's cudaMemGetInfo reports less than a request needs beyond the 4 GiB headroom), a request
    that fits the budget waits in the queue; once the memory is back it is admitted and runs."""
    import time
    L, _ = srvlib
    s = Srv(srvlib, max_slots=64)
    need = request_bytes(256)
    try:
        L.fake_set_free_bytes((4 << 30) + need // 2)
        a = s.submit(n=256, max_steps=300)
        time.sleep(0.2)
        assert s.counts()[2] == 0  # nothing created: it does not fit in what is free now
        L.fake_set_free_bytes(64 << 30)
        res, st = s.finish()
        assert res[a].status == OK and res[a].steps == 300 and st.completed == 1
    finally:
        L.fake_set_free_bytes(64 << 30)
        s.close()
