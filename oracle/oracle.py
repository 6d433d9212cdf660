"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module,
as the checker.  The product package (bgk2d_gpu_gb300) never imports it.

The oracle restates the reference's serial step (SRC/col_MC.F90, SRC/col.F90, SRC/movef.F90,
SRC/bcond.*.F90, SRC/init.F90, SRC/hencol.F90, SRC/build.obs.F90, SRC/diagno.F90,
SRC/draglift.F90, SRC/prof_j.F90) in plain C; see bgk_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbgk_oracle.so")

SINGLE, DOUBLE, MIXED2 = 0, 1, 2
LDC, TGV, POF, VKS, COU, BFS, MYV = 0, 1, 2, 3, 4, 5, 6
OBS_NONE, OBS_CIRCLE, OBS_SQUARE, OBS_HALF_CIRCLE = 0, 1, 2, 3
OBS_SERIAL, OBS_SNAPSHOT = 0, 1

# direction order of the reference (SRC/bgk2d.F90:29-39): 01,03,05,08,10,12,14,17,19
CX = np.array([1, 1, 1, 0, -1, -1, -1, 0, 0])
CY = np.array([-1, 1, 0, 1, -1, 1, 0, -1, 0])


class _Params(ctypes.Structure):
    _fields_ = [
        ("l", ctypes.c_int), ("m", ctypes.c_int), ("prec", ctypes.c_int),
        ("tcase", ctypes.c_int), ("fused", ctypes.c_int), ("obstacle", ctypes.c_int),
        ("obs_order", ctypes.c_int), ("radius", ctypes.c_int),
        ("obs_icoord", ctypes.c_int), ("obs_jcoord", ctypes.c_int),
        ("init_v", ctypes.c_int), ("svisc", ctypes.c_double), ("u0", ctypes.c_double),
        ("les", ctypes.c_int), ("cte_s", ctypes.c_double), ("trick1", ctypes.c_int),
        ("noshift", ctypes.c_int),
        ("force_y", ctypes.c_int),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    src = [os.path.join(HERE, f) for f in ("bgk_oracle.c", "bgk_oracle_body.h", "bgk_oracle.h")]
    if force or not os.path.exists(LIB_PATH) or any(
            os.path.getmtime(f) > os.path.getmtime(LIB_PATH) for f in src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int32)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(_Params)]
        L.orc_destroy.argtypes = [P]
        L.orc_step.argtypes = [P, ctypes.c_int]
        L.orc_step_omp.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_get_pops.argtypes = [P, dp]
        L.orc_set_pops.argtypes = [P, dp]
        L.orc_get_raw.argtypes = [P, ctypes.c_void_p]
        L.orc_set_raw.argtypes = [P, ctypes.c_void_p]
        L.orc_storage_bytes.argtypes = [P]
        L.orc_storage_bytes.restype = ctypes.c_int
        L.orc_get_obs.argtypes = [P, ip, ip]
        L.orc_build_obs.argtypes = [ctypes.c_int] * 7 + [ip, ip]
        L.orc_get_scalars.argtypes = [P, dp]
        L.orc_diagno.argtypes = [P, ctypes.c_int, dp]
        L.orc_draglift.argtypes = [P, ctypes.c_int, dp]
        L.orc_prof_j.argtypes = [P, ctypes.c_int, dp, dp, dp]
        L.orc_fields.argtypes = [P, dp, dp, dp]
        fp = ctypes.POINTER(ctypes.c_float)
        L.orc_vtk.argtypes = [P, ctypes.c_int, fp, fp, fp, fp, fp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Oracle:
    """One reference run: setup (alloca/init/hencol/build_obs) then `step(n)`."""

    def __init__(self, l, m, prec=SINGLE, tcase=LDC, svisc=0.1, u0=0.1, fused=True,
                 obstacle=OBS_NONE, obs_order=OBS_SNAPSHOT, radius=16,
                 obs_icoord=-1, obs_jcoord=-1, init_v=0, les=False, cte_s=0.1, trick1=False,
                 noshift=False, force_y=False):
        self.l, self.m, self.prec, self.tcase = l, m, prec, tcase
        # namelist values are read as mykind
        if prec == SINGLE:
            svisc = float(np.float32(svisc))
            u0 = float(np.float32(u0))
            cte_s = float(np.float32(cte_s))
        p = _Params(l, m, prec, tcase, int(fused), obstacle, obs_order, radius,
                    obs_icoord, obs_jcoord, init_v, svisc, u0, int(les), cte_s, int(trick1),
                    int(noshift), int(force_y))
        self._h = lib().orc_create(ctypes.byref(p))
        if not self._h:
            raise ValueError("oracle: invalid parameters")

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def sdtype(self):
        return np.float64 if self.prec == DOUBLE else np.float32

    def step(self, n=1, threads=1):
        if threads > 1:
            lib().orc_step_omp(self._h, n, threads)
        else:
            lib().orc_step(self._h, n)

    def pops(self):
        """(9, m+2, l+2) array of the current populations a01..a19 (index [q, j, i])."""
        out = np.empty(9 * (self.l + 2) * (self.m + 2), dtype=np.float64)
        lib().orc_get_pops(self._h, _dp(out))
        return out.reshape(9, self.m + 2, self.l + 2)

    def raw(self):
        """Populations in their storage kind, (9, m+2, l+2)."""
        out = np.empty(9 * (self.l + 2) * (self.m + 2), dtype=self.sdtype)
        lib().orc_get_raw(self._h, out.ctypes.data_as(ctypes.c_void_p))
        return out.reshape(9, self.m + 2, self.l + 2)

    def set_raw(self, arr):
        a = np.ascontiguousarray(arr, dtype=self.sdtype).reshape(-1)
        assert a.size == 9 * (self.l + 2) * (self.m + 2)
        lib().orc_set_raw(self._h, a.ctypes.data_as(ctypes.c_void_p))

    def obs(self):
        mask = np.empty(self.l * self.m, dtype=np.int32)
        bb = np.empty(5, dtype=np.int32)
        lib().orc_get_obs(self._h, _ip(mask), _ip(bb))
        return mask.reshape(self.m, self.l), bb

    def scalars(self):
        out = np.empty(4, dtype=np.float64)
        lib().orc_get_scalars(self._h, _dp(out))
        return dict(omega=out[0], fgrad=out[1], u00=out[2], u0=out[3])

    def diagno(self, mode=0):
        out = np.empty(4, dtype=np.float64)
        lib().orc_diagno(self._h, mode, _dp(out))
        return out

    def draglift(self, mode=0):
        out = np.empty(2, dtype=np.float64)
        lib().orc_draglift(self._h, mode, _dp(out))
        return out

    def prof_j(self, icoord):
        u = np.empty(self.m); v = np.empty(self.m); d = np.empty(self.m)
        lib().orc_prof_j(self._h, icoord, _dp(u), _dp(v), _dp(d))
        return u, v, d

    def fields(self):
        n = self.l * self.m
        r = np.empty(n); u = np.empty(n); v = np.empty(n)
        lib().orc_fields(self._h, _dp(r), _dp(u), _dp(v))
        sh = (self.m, self.l)
        return r.reshape(sh), u.reshape(sh), v.reshape(sh)


    def vtk(self, from_ghost_row=True):
        """The VTK writers' float32 fields: u, w, rho as (m, l); vorticity, stream as (m-2, l-2)."""
        l, m = self.l, self.m
        u = np.empty(l * m, np.float32); w = np.empty_like(u); r = np.empty_like(u)
        om = np.empty((l - 2) * (m - 2), np.float32); st = np.empty_like(om)
        fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        lib().orc_vtk(self._h, int(from_ghost_row), fp(u), fp(w), fp(r), fp(om), fp(st))
        return (u.reshape(m, l), w.reshape(m, l), r.reshape(m, l), om.reshape(m - 2, l - 2),
                st.reshape(m - 2, l - 2))


def build_obs(l, m, shape, radius, icoord=-1, jcoord=-1, prec=SINGLE):
    """Mask obs(1:l,1:m) as (m, l) int32 plus (imin, imax, jmin, jmax, nobs)."""
    icoord = 2 * l // 5 if icoord < 0 else icoord
    jcoord = m // 2 if jcoord < 0 else jcoord
    mask = np.empty(l * m, dtype=np.int32)
    bb = np.empty(5, dtype=np.int32)
    lib().orc_build_obs(l, m, shape, radius, icoord, jcoord, prec, _ip(mask), _ip(bb))
    return mask.reshape(m, l), bb
