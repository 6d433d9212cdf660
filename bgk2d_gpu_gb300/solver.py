"""Host-side mirror of the reference's step interface over the C ABI.

The reference driver (SRC/bgk2d.F90:92-113) calls `boundaries`, `propagation` and
`collision(itime)` once per step and reads the populations through `diagno`, `probe`,
`prof_i`/`prof_j`, `draglift`, `vtk_*` and `save_raw`.  `Solver` offers the same calls on a
device-resident case; readers that stay host-side in the reference (probe, prof_i, prof_j,
varm) work on downloaded populations with the reference's single-step arithmetic.
"""
from __future__ import annotations

import ctypes
import re

import numpy as np

from . import _lib
from ._lib import BgkError, CaseDesc

# direction order of the reference (SRC/bgk2d.F90:29-39): 01,03,05,08,10,12,14,17,19
CX = np.array([1, 1, 1, 0, -1, -1, -1, 0, 0])
CY = np.array([-1, 1, 0, 1, -1, 1, 0, -1, 0])
WEIGHTS = np.array([1 / 36, 1 / 36, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 9, 1 / 9, 4 / 9])


def read_namelist(path: str) -> dict:
    """Parse the `&parameters` namelist of bgk.input (SRC/input.F90:44-65) into a dict,
    with the reference defaults (SRC/input.F90:51-61) for absent keys.  As in Fortran list-
    directed namelist input, names ignore case (keys are returned in lower case, e.g. `ctes`),
    `!` starts a comment, and `d`/`D` exponents are accepted."""
    text = re.sub(r"!.*", "", open(path).read())
    m = re.search(r"&parameters(.*?)/", text, flags=re.S | re.I)
    if not m:
        raise ValueError(f"{path}: no &parameters namelist")
    vals = dict(flag1=0, flag2=0, flag3=0, init_v=0, ctes=0.1, ipad=0, jpad=0, radius=16)
    for key, val in re.findall(r"(\w+)\s*=\s*([^,\s/]+)", m.group(1)):
        v = val.strip().rstrip(",").replace("d", "e").replace("D", "e")
        try:
            num = int(v)
        except ValueError:
            num = float(v)
        vals[key.strip().lower()] = num
    return vals


class Solver:
    """One device-resident BGK2D case (ping-pong or AA scheme)."""

    def __init__(self, lx, ly, tcase="LDC", svisc=0.1, u0=0.1, storage="f32", compute=None,
                 scheme="pingpong", radius=16, obstacle=None, obs_center=(-1, -1), obs_mask=None,
                 init="rest", omega=None, u_inflow=None, inflow_profile=0, faces=None,
                 wall_u=None, tgv_u0=0.02, ipad=0, jpad=0, device=0, les=False, cte_s=0.1,
                 trick1=False, noshift=False, force_y=False):
        L = _lib.load()
        d = CaseDesc()
        L.bgk_default_desc(ctypes.byref(d))
        d.lx, d.ly, d.ipad, d.jpad = int(lx), int(ly), int(ipad), int(jpad)
        if compute is None:
            compute = "f64" if storage == "f64" else "f32"
        d.storage = _lib.STORE[storage]
        d.compute = _lib.COMPUTE[compute]
        d.scheme = _lib.SCHEME[scheme]
        d.tcase = _lib.CASE[tcase]
        d.svisc = float(svisc)
        d.u0 = float(u0)
        d.omega = float(omega) if omega else 0.0
        d.u_inflow = float(u_inflow) if u_inflow else 0.0
        d.inflow_profile = int(inflow_profile)
        d.radius = int(radius)
        d.obs_icoord, d.obs_jcoord = int(obs_center[0]), int(obs_center[1])
        self._mask_keep = None
        if obs_mask is not None:
            mk = np.ascontiguousarray(obs_mask, dtype=np.int32)
            if mk.shape != (ly, lx):
                raise ValueError(f"obs_mask has shape {mk.shape}, expected (ly, lx) = {(ly, lx)}")
            self._mask_keep = mk
            d.obstacle = _lib.OBS["mask"]
            d.obs_mask = mk.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        else:
            d.obstacle = _lib.OBS[obstacle]
        d.init_v = _lib.INIT[init]
        d.tgv_u0 = float(tgv_u0)
        d.device = int(device)
        d.les = int(bool(les))
        d.cte_s = float(cte_s)
        d.trick1 = int(bool(trick1))
        d.noshift = int(bool(noshift))
        d.force_y = int(bool(force_y))
        if faces is not None:
            for i, f in enumerate(faces):
                d.faces[i] = _lib.FACE[f]
        if wall_u is not None:
            for i, (ux, uy) in enumerate(wall_u):
                d.wall_u[i][0], d.wall_u[i][1] = float(ux), float(uy)
        self.desc = d
        self.lx, self.ly = int(lx), int(ly)
        self.storage, self.compute, self.scheme, self.tcase = storage, compute, scheme, tcase
        self.hdtype = np.float64 if storage == "f64" else np.float32
        self.noshift = bool(noshift)
        self._cte1 = 0 if noshift else 1  # the host readers' cte1 (SRC/probe.F90:40-44)
        self._L = L
        h = ctypes.c_void_p()
        rc = L.bgk_create(ctypes.byref(d), ctypes.byref(h))
        if rc != 0:
            raise BgkError(rc, f"bgk_create({lx}x{ly}, {tcase}, {storage}/{compute}, {scheme})")
        self._h = h

    @classmethod
    def from_namelist(cls, path, tcase="LDC", **kw):
        """A case from a `bgk.input` namelist (lx, ly, svisc, u0, radius, ipad, jpad, cteS;
        SRC/input.F90)."""
        p = read_namelist(path)
        kw.setdefault("cte_s", p["ctes"])
        return cls(p["lx"], p["ly"], tcase=tcase, svisc=p["svisc"], u0=p["u0"],
                   radius=p.get("radius", 16), ipad=p.get("ipad", 0), jpad=p.get("jpad", 0), **kw)

    # -- lifecycle ----------------------------------------------------------------------------
    def close(self):
        """Release the device memory of the case (bgk_destroy; SRC/dealloca.F90)."""
        if getattr(self, "_h", None):
            self._L.bgk_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            buf = ctypes.create_string_buffer(512)
            self._L.bgk_last_error(self._h, buf, 512)
            raise BgkError(rc, f"{what}: {buf.value.decode()}")

    # -- the reference's step sequence (SRC/bgk2d.F90:100-102) ---------------------------------
    def boundaries(self):
        """`call boundaries` (bgk_boundaries); the fused step applies the rules."""
        self._check(self._L.bgk_boundaries(self._h), "boundaries")

    def propagation(self):
        """`call propagation` (bgk_propagation); the streaming pass of the two-pass scheme."""
        self._check(self._L.bgk_propagation(self._h), "propagation")

    def collision(self, itime=0):
        """`call collision(itime)` (bgk_collision): completes one time step."""
        self._check(self._L.bgk_collision(self._h, int(itime)), "collision")

    def step(self, n=1):
        """n full time steps, replayed from CUDA graphs (bgk_step); asynchronous."""
        self._check(self._L.bgk_step(self._h, int(n)), "step")

    def step_timed(self, n):
        """n time steps bracketed by CUDA events; returns their device time in ms."""
        ms = ctypes.c_float()
        self._check(self._L.bgk_step_timed(self._h, int(n), ctypes.byref(ms)), "step_timed")
        return ms.value

    def sync(self):
        """Wait for the case's stream; reports a failure of earlier asynchronous work."""
        self._check(self._L.bgk_sync(self._h), "sync")

    # -- populations ------------------------------------------------------------------------
    def _ptrs(self, arr):
        return (ctypes.c_void_p * 9)(*[arr[q].ctypes.data for q in range(9)])

    def download(self):
        """(9, ly+2, lx+2) host-kind array a01..a19, index [q, j, i]; ghost entries are zero."""
        out = np.zeros((9, self.ly + 2, self.lx + 2), dtype=self.hdtype)
        self._check(self._L.bgk_download(self._h, self._ptrs(out), self.lx + 2), "download")
        return out

    def upload(self, arr):
        """Set the populations from a (9, ly+2, lx+2) host-kind array laid out as `download` returns."""
        a = np.ascontiguousarray(arr, dtype=self.hdtype)
        if a.shape != (9, self.ly + 2, self.lx + 2):
            raise ValueError(f"populations have shape {a.shape}, expected {(9, self.ly + 2, self.lx + 2)}")
        self._check(self._L.bgk_upload(self._h, self._ptrs(a), self.lx + 2), "upload")

    @staticmethod
    def _host_ptrs(arr):
        if hasattr(arr, "data_ptr"):  # torch tensor (page-locked when pinned)
            return (ctypes.c_void_p * 9)(*[arr[q].data_ptr() for q in range(9)])
        return (ctypes.c_void_p * 9)(*[arr[q].ctypes.data for q in range(9)])

    def advance_host(self, src, dst, nsteps):
        """bgk_advance_host: upload `src`, run nsteps steps, download into `dst`.  Both are host
        arrays of shape (9, ly+2, ld), ld >= lx+2, numpy or torch (`dst` may be `src`); with
        page-locked (torch pinned) arrays the transfers and the steps are pipelined."""
        for a in (src, dst):
            if tuple(a.shape[:2]) != (9, self.ly + 2) or a.shape[2] < self.lx + 2:
                raise ValueError(f"host populations have shape {tuple(a.shape)}, expected (9, {self.ly + 2}, >= {self.lx + 2})")
        if src.shape[2] != dst.shape[2]:
            raise ValueError("src and dst must have the same leading dimension")
        rc = self._L.bgk_advance_host(self._h, self._host_ptrs(src), self._host_ptrs(dst), int(src.shape[2]), int(nsteps))
        self._check(rc, "advance_host")

    # -- reductions (FP64 on the device) ------------------------------------------------------
    def diagno(self, mode=0):
        """(<u>, <v>, <rho>, <|u|^2>) (SRC/diagno.F90:63-101).  mode 0: FP64 sums over all cells;
        1 (or True): fluid cells only; 2: the reference's own sums in the compute kind and order,
        the values it writes to diagno.dat."""
        out = np.zeros(4)
        self._check(self._L.bgk_diagno(self._h, int(mode),
                                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "diagno")
        return out

    def draglift(self, reference=False):
        """(drag, lift) by momentum exchange (SRC/draglift.F90); reference=True: the reference's
        own compute-kind sums in its order (the values it writes to drag.lift)."""
        out = np.zeros(2)
        fn = self._L.bgk_draglift_reference if reference else self._L.bgk_draglift
        self._check(fn(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))), "draglift")
        return out

    def residual(self):
        """Steady-state residual ||u - u_prev|| / ||u|| since the previous call (1 on the first)."""
        out = ctypes.c_double()
        self._check(self._L.bgk_residual(self._h, ctypes.byref(out)), "residual")
        return out.value

    def fields(self):
        """(rho, u, v) of the interior as (ly, lx) float64 arrays, in the diagno arithmetic."""
        n = self.lx * self.ly
        r, u, v = np.empty(n), np.empty(n), np.empty(n)
        P = ctypes.POINTER(ctypes.c_double)
        self._check(self._L.bgk_fields(self._h, r.ctypes.data_as(P), u.ctypes.data_as(P), v.ctypes.data_as(P)),
                    "fields")
        sh = (self.ly, self.lx)
        return r.reshape(sh), u.reshape(sh), v.reshape(sh)

    def obs(self):
        """Obstacle mask (ly, lx) and (imin, imax, jmin, jmax, nobs) of build_obs."""
        mask = np.zeros(self.lx * self.ly, dtype=np.int32)
        bb = np.zeros(5, dtype=np.int32)
        P = ctypes.POINTER(ctypes.c_int32)
        self._check(self._L.bgk_get_obs(self._h, mask.ctypes.data_as(P), bb.ctypes.data_as(P)), "get_obs")
        return mask.reshape(self.ly, self.lx), bb

    def scalars(self):
        """omega, fgrad, u00, u0 after build_bcond and hencol, and the step counter."""
        out = np.zeros(4)
        it = ctypes.c_int64()
        self._check(self._L.bgk_get_scalars(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            ctypes.byref(it)), "get_scalars")
        return dict(omega=out[0], fgrad=out[1], u00=out[2], u0=out[3], itime=it.value)

    def footprint(self):
        """(device bytes held, algorithmic bytes moved per lattice update)."""
        b = ctypes.c_int64()
        c = ctypes.c_int32()
        self._check(self._L.bgk_footprint(self._h, ctypes.byref(b), ctypes.byref(c)), "footprint")
        return b.value, c.value

    def set_tile(self, cfg):
        """Tile configuration of the step kernels (0-5 register vectors, 6-8 staged rows)."""
        self._check(self._L.bgk_set_tile(self._h, int(cfg)), "set_tile")

    def vtk_fields(self):
        """The VTK writers' float32 fields computed on the device: (u, w, rho) as (ly, lx) and
        (vorticity, stream) as (ly-2, lx-2) (SRC/vtk_xy.binary.F90, SRC/vtk_om.binary.F90)."""
        lx, ly = self.lx, self.ly
        u = np.empty((ly, lx), np.float32); w = np.empty_like(u); r = np.empty_like(u)
        om = np.empty((ly - 2, lx - 2), np.float32); st = np.empty_like(om)
        fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        self._check(self._L.bgk_vtk_fields(self._h, fp(u), fp(w), fp(r), fp(om), fp(st)), "vtk_fields")
        return u, w, r, om, st

    def set_prefetch(self, blocks_ahead):
        """L2 prefetch distance of the step kernels, in blocks (0: off)."""
        self._check(self._L.bgk_set_prefetch(self._h, int(blocks_ahead)), "set_prefetch")

    def prefetch(self):
        """The current L2 prefetch distance in blocks."""
        n = ctypes.c_int32()
        self._check(self._L.bgk_get_prefetch(self._h, ctypes.byref(n)), "get_prefetch")
        return n.value

    def tune(self, trial_steps=20):
        """Time real steps per tile shape (the state advances); returns (tile_cfg, steps_run)."""
        c, n = ctypes.c_int32(), ctypes.c_int32()
        self._check(self._L.bgk_tune(self._h, int(trial_steps), ctypes.byref(c), ctypes.byref(n)), "tune")
        return c.value, n.value

    def launches(self):
        """Kernels this library has launched for the case so far."""
        n = ctypes.c_int64()
        self._check(self._L.bgk_launch_count(self._h, ctypes.byref(n)), "launch_count")
        return n.value

    # -- host-side readers of downloaded populations (reference arithmetic) ------------------
    # prof_i, prof_j and varm add the stored values as they lie in the arrays, in the storage
    # kind (real(sp) under MIXED2); cte1 and everything after it are in the compute kind.
    # probe copies the values into compute-kind temporaries first (SRC/probe.F90:46-54).
    def _kind(self, a):
        """The compute kind of the reference readers for arrays `a`."""
        return np.float64 if getattr(self, "compute", None) == "f64" else a.dtype.type

    def _device_reader(self, name, n, *args):
        """One of the profile readers on the device (bgk_prof_i / _prof_j / _varm / _probe): three
        arrays of n compute-kind values."""
        out = np.zeros((3, n))
        dp = ctypes.POINTER(ctypes.c_double)
        ptrs = [out[k].ctypes.data_as(dp) for k in range(3)]
        if name == "bgk_probe":  # out[3] contiguous: the (3, 1) array
            self._check(self._L.bgk_probe(self._h, *args, ptrs[0]), "probe")
        else:
            self._check(getattr(self._L, name)(self._h, *args, *ptrs), name[4:])
        k = np.float64 if self.storage == "f64" or self.compute == "f64" else np.float32
        return tuple(out[q].astype(k) for q in range(3))  # exact: the values are of kind k

    def prof_j(self, icoord, pops=None):
        """u, v, rho along column icoord, j = 1..ly (SRC/prof_j.F90:47-67); computed on the device
        (bgk_prof_j) unless downloaded populations `pops` are given."""
        if pops is None:
            return self._device_reader("bgk_prof_j", self.ly, int(icoord))
        a = pops
        k = self._kind(a)
        c = a[:, 1:self.ly + 1, icoord]
        den = c[0] + c[1]
        for q in range(2, 8):
            den = den + c[q]
        den = (den + c[8]).astype(k) + k(self._cte1)
        u = ((c[0] - c[4]) + (c[1] - c[5]) + (c[2] - c[6])).astype(k) / den
        v = ((c[1] - c[0]) + (c[3] - c[7]) + (c[5] - c[4])).astype(k) / den
        return u, v, den

    def prof_i(self, jcoord, pops=None):
        """u, v, rho along row jcoord, i = 1..lx (SRC/prof_i.F90:47-62); on the device (bgk_prof_i)
        unless `pops` are given."""
        if pops is None:
            return self._device_reader("bgk_prof_i", self.lx, int(jcoord))
        a = pops
        k = self._kind(a)
        c = a[:, jcoord, 1:self.lx + 1]
        den = c[0] + c[1]
        for q in range(2, 9):
            den = den + c[q]
        den = den.astype(k) + k(self._cte1)
        u = (((((c[0] + c[1]) + c[2]) - c[4]) - c[5]) - c[6]).astype(k) / den
        v = (((((c[1] + c[3]) + c[5]) - c[0]) - c[4]) - c[7]).astype(k) / den
        return u, v, den

    def varm(self, pops=None):
        """Row means of u, w and rho (u_med.dat; SRC/varm.F90:49-88), see `varm`; on the device
        (bgk_varm) unless `pops` are given."""
        if pops is None:
            return self._device_reader("bgk_varm", self.ly)
        return varm(pops, self.lx, self.ly, noshift=self.noshift, kind=self._kind(pops))

    def probe(self, i0, j0, pops=None):
        """u, v, rho at one node (SRC/probe.F90:46-62); on the device (bgk_probe) unless `pops`
        are given."""
        if pops is None:
            u, v, r = self._device_reader("bgk_probe", 1, int(i0), int(j0))
            return u[0], v[0], r[0]
        a = pops
        k = self._kind(a)
        x = a[:, j0, i0].astype(k)
        rho = x[0] + x[1] + x[2] + x[3] + x[4] + x[5] + x[6] + x[7] + x[8] + k(self._cte1)
        xj = x[0] + x[1] + x[2] - x[4] - x[5] - x[6]
        yj = x[1] + x[3] + x[5] - x[0] - x[4] - x[7]
        return xj / rho, yj / rho, rho


def varm(pops, lx, ly, noshift=False, kind=None):
    """Row means over i = 1..lx of u, w and rho for j = 1..ly, as SRC/varm.F90:49-88 writes them to
    u_med.dat: per cell rho = (a01 + ... + a19) + cte1 (1, or 0 for populations stored whole,
    SRC/varm.F90:42-46), the sum in the arrays' kind and the rest in the compute kind `kind`
    (default: the arrays' kind), rhoinv = 1/rho; the sums over i run in order in the compute
    kind; the means are the sums times rvol = 1.0/float(lx), a default-real quotient.  `pops` is
    the (9, ly+2, lx+2) array of `Solver.download`."""
    k = kind or pops.dtype.type
    x = pops[:, 1:ly + 1, 1:lx + 1]
    rho = x[0] + x[1]
    for q in range(2, 9):
        rho = rho + x[q]
    rho = rho.astype(k) + k(0 if noshift else 1)
    rinv = k(1) / rho
    uu = (((((x[0] + x[1]) + x[2]) - x[4]) - x[5]) - x[6]).astype(k) * rinv
    ww = (((((x[1] + x[3]) + x[5]) - x[0]) - x[4]) - x[7]).astype(k) * rinv
    u = np.zeros(ly, dtype=k)
    w = np.zeros(ly, dtype=k)
    den = np.zeros(ly, dtype=k)
    for i in range(lx):  # the reference's i loop: one addition per cell, in order
        den = den + rho[:, i]
        u = u + uu[:, i]
        w = w + ww[:, i]
    rvol = k(np.float32(1.0) / np.float32(lx))
    return u * rvol, w * rvol, den * rvol


class Batch:
    """Independent ping-pong cases of one (storage, compute) kind advanced together: one
    persistent work-list launch per time step, replayed from CUDA graphs."""

    def __init__(self, storage="f32", compute=None, device=0):
        self._L = _lib.load()
        if compute is None:
            compute = "f64" if storage == "f64" else "f32"
        b = ctypes.c_void_p()
        rc = self._L.bgk_batch_create(_lib.STORE[storage], _lib.COMPUTE[compute], int(device), ctypes.byref(b))
        if rc != 0:
            raise BgkError(rc, "bgk_batch_create")
        self._b = b
        self.members = []

    def _check(self, rc, what):
        if rc != 0:
            raise BgkError(rc, what)

    def add(self, solver):
        """Attach a ping-pong case of the batch's kinds; it then steps only with the batch."""
        self._check(self._L.bgk_batch_add(self._b, solver._h), "batch_add")
        self.members.append(solver)

    def remove(self, solver):
        """Detach a case; it keeps its state and can step alone again."""
        self._check(self._L.bgk_batch_remove(self._b, solver._h), "batch_remove")
        self.members.remove(solver)

    def size(self):
        """(members, cells) of the batch."""
        n, c = ctypes.c_int32(), ctypes.c_int64()
        self._check(self._L.bgk_batch_size(self._b, ctypes.byref(n), ctypes.byref(c)), "batch_size")
        return n.value, c.value

    def step(self, n=1):
        """n steps of every member, one launch per step."""
        self._check(self._L.bgk_batch_step(self._b, int(n)), "batch_step")

    def step_timed(self, n):
        """n steps of every member; returns their device time in ms."""
        ms = ctypes.c_float()
        self._check(self._L.bgk_batch_step_timed(self._b, int(n), ctypes.byref(ms)), "batch_step_timed")
        return ms.value

    def sync(self):
        """Wait for the batch's stream."""
        self._check(self._L.bgk_batch_sync(self._b), "batch_sync")

    def set_config(self, tile_cfg, blocks_per_sm, graph_steps):
        """Tile shape, persistent blocks per SM (0: one block per tile) and steps per graph."""
        self._check(self._L.bgk_batch_set_config(self._b, int(tile_cfg), int(blocks_per_sm), int(graph_steps)),
                    "batch_set_config")

    def set_prefetch(self, tiles_ahead):
        """L2 prefetch of the work-list entry this many tiles ahead (one block per tile)."""
        self._check(self._L.bgk_batch_set_prefetch(self._b, int(tiles_ahead)), "batch_set_prefetch")

    def config(self):
        """(tile_cfg, blocks_per_sm, graph_steps) in use."""
        out = (ctypes.c_int32 * 3)()
        self._check(self._L.bgk_batch_get_config(self._b, out), "batch_get_config")
        return tuple(out)

    def tune(self, trial_steps=10):
        """Time real steps over tile shapes, grid sizes and graph lengths and keep the fastest;
        returns the steps run."""
        n = ctypes.c_int32()
        self._check(self._L.bgk_batch_tune(self._b, int(trial_steps), ctypes.byref(n)), "batch_tune")
        return n.value

    def launches(self):
        """Kernels this batch has launched so far."""
        n = ctypes.c_int64()
        self._check(self._L.bgk_batch_launch_count(self._b, ctypes.byref(n)), "batch_launch_count")
        return n.value

    def close(self):
        """Destroy the batch; its members can step alone again."""
        if getattr(self, "_b", None):
            self._L.bgk_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Server:
    """Continuous-batching request loop (C++ scheduler thread inside the library)."""

    def __init__(self, max_slots=64, chunk_steps=200, hbm_budget=0, tile_cfg=-1, device=0):
        self._L = _lib.load()
        cfg = _lib.ServerConfig(int(device), int(max_slots), int(hbm_budget), int(chunk_steps), int(tile_cfg))
        h = ctypes.c_void_p()
        rc = self._L.bgk_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise BgkError(rc, "bgk_server_create")
        self._s = h
        self.sizes = {}

    def submit(self, kind, n, re, u, storage="f32", max_steps=1000, tol=0.0, check_every=500, keep_fields=False):
        """Queue a request; returns its id."""
        r = _lib.Request(_lib.REQ[kind], int(n), float(re), float(u), _lib.STORE[storage], int(max_steps),
                         float(tol), int(check_every), int(bool(keep_fields)))
        i = ctypes.c_int64()
        rc = self._L.bgk_server_submit(self._s, ctypes.byref(r), ctypes.byref(i))
        if rc != 0:
            raise BgkError(rc, "bgk_server_submit")
        return i.value

    def poll(self, max_results=1024):
        """Finished results, oldest first, as dicts: id, status, steps, size, residual, diagno,
        drag/lift and the submit, admit and done times."""
        buf = (_lib.Result * max_results)()
        n = ctypes.c_int32()
        rc = self._L.bgk_server_poll(self._s, buf, int(max_results), ctypes.byref(n))
        if rc != 0:
            raise BgkError(rc, "bgk_server_poll")
        out = []
        for k in range(n.value):
            r = buf[k]
            out.append(dict(id=r.id, status=r.status, steps=r.steps, lx=r.lx, ly=r.ly, residual=r.residual,
                            diagno=list(r.diagno), draglift=list(r.draglift), t_submit=r.t_submit,
                            t_admit=r.t_admit, t_done=r.t_done))
        return out

    def drain(self, timeout_s=600.0):
        """Block until every submitted request finished, or the timeout passed."""
        rc = self._L.bgk_server_drain(self._s, float(timeout_s))
        if rc != 0:
            raise BgkError(rc, "bgk_server_drain")

    def fields(self, rid, lx, ly):
        """(rho, u, v) of a finished request that kept its fields."""
        n = lx * ly
        r, u, v = np.empty(n), np.empty(n), np.empty(n)
        P = ctypes.POINTER(ctypes.c_double)
        rc = self._L.bgk_server_fields(self._s, int(rid), r.ctypes.data_as(P), u.ctypes.data_as(P),
                                       v.ctypes.data_as(P), n)
        if rc != 0:
            raise BgkError(rc, "bgk_server_fields")
        return r.reshape(ly, lx), u.reshape(ly, lx), v.reshape(ly, lx)

    def stats(self):
        """Aggregate statistics: completed, GLUPS, p50/p99 latency, launches, rounds."""
        st = _lib.ServerStats()
        rc = self._L.bgk_server_get_stats(self._s, ctypes.byref(st))
        if rc != 0:
            raise BgkError(rc, "bgk_server_get_stats")
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def close(self):
        """Stop the serving thread and release the resident requests."""
        if getattr(self, "_s", None):
            self._L.bgk_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
