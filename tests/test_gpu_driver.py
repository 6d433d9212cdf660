"""Host driver over the C ABI: bgk.input in, the reference's text outputs and checkpoints out."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMELIST = """&parameters
lx = {lx}
ly = {ly}
svisc={svisc}
u0=0.1
itfin={itfin}
ivtim={ivtim}
isignal={isignal}
itsave={itsave}
icheck={icheck}
irestart={irestart}
init_v=0
ipad=0        /
"""


def run_driver(bgk, tmp, case="LDC", prec="single", extra=(), **kw):
    from bgk2d_gpu_gb300 import build
    exe = build.EXE_PATH
    assert os.path.exists(exe)
    p = dict(lx=64, ly=48, svisc=0.0384, itfin=300, isignal=100, itsave=150, icheck=100, irestart=0, ivtim=1000000)
    p.update(kw)
    (tmp / "bgk.input").write_text(NAMELIST.format(**p))
    r = subprocess.run([exe, "--input", str(tmp / "bgk.input"), "--case", case, "--prec", prec, "--dir", str(tmp),
                        *extra], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return p


def test_driver_outputs_match_solver(bgk, tmp_path):
    p = run_driver(bgk, tmp_path)
    rows = [ln.split() for ln in (tmp_path / "diagno.dat").read_text().splitlines()]
    assert [int(r[0]) for r in rows] == [100, 200, 300, 300]
    with bgk.Solver(p["lx"], p["ly"], tcase="LDC", svisc=p["svisc"], u0=0.1) as s:
        s.step(300)
        d = s.diagno()
        u, v, den = s.prof_j(p["lx"] // 2)
    np.testing.assert_allclose([float(x) for x in rows[-1][1:]], d, rtol=1e-5, atol=1e-12)
    text = (tmp_path / "prof_j.dat").read_text()
    assert text.count("# t=") == 5  # t=0, 100, 200, 300 and the final call
    last = text.split("# t=")[-1].strip().splitlines()[1:]
    vals = np.array([[float(x) for x in ln.split()] for ln in last])
    np.testing.assert_allclose(vals[:, 1], u, rtol=1e-5, atol=1e-11)
    assert (tmp_path / "save.00000150.bin").exists() and (tmp_path / "bgk.perf").exists()
    # bgk.perf in the reference's layout (SRC/finalize.F90:34-75)
    perf = (tmp_path / "bgk.perf").read_text().splitlines()
    assert perf[1] == " # Run info " and perf[2].split() == [str(p["lx"]), str(p["ly"])]
    mlups = [ln for ln in perf if ln.startswith(" # Mlups      ")]
    assert len(mlups) == 1 and float(mlups[0].split()[-1]) > 0
    loop = float([ln for ln in perf if ln.startswith(" # loop   time")][0].split()[3])
    coll = float([ln for ln in perf if ln.startswith(" # coll   time")][0].split()[3])
    assert 0 < coll <= loop
    # u_med.dat (SRC/varm.F90): at start-up, every icheck and once more at the end
    text = (tmp_path / "u_med.dat").read_text()
    assert [int(b.split()[0]) for b in text.split("# t=")[1:]] == [0, 100, 200, 300, 300]
    with bgk.Solver(p["lx"], p["ly"], tcase="LDC", svisc=p["svisc"], u0=0.1) as s:
        s.step(300)
        um, wm, dm = s.varm()
    last = text.split("# t=")[-1].strip().splitlines()[1:]
    vals = np.array([[float(x) for x in ln.split()] for ln in last])
    assert np.array_equal(vals[:, 0], np.arange(1, p["ly"] + 1))
    np.testing.assert_allclose(vals[:, 1], um, rtol=1e-5, atol=1e-11)
    np.testing.assert_allclose(vals[:, 2], wm, rtol=1e-5, atol=1e-11)
    np.testing.assert_allclose(vals[:, 3], dm, rtol=1e-5)  # e14.6: 6 significant digits
    # the final call writes no probe line (SRC/bgk2d.F90:122-125)
    assert len((tmp_path / "probe.dat").read_text().splitlines()) == 3


def test_checkpoint_restart_continues_exactly(bgk, tmp_path):
    a = tmp_path / "a"
    b = tmp_path / "b"
    a.mkdir()
    b.mkdir()
    run_driver(bgk, a)
    shutil.copy(a / "save.00000150.bin", b / "restore.bin")
    run_driver(bgk, b, irestart=1)
    ra = (a / "diagno.dat").read_text().splitlines()
    rb = (b / "diagno.dat").read_text().splitlines()
    assert ra[-1] == rb[-1] and ra[-2] == rb[-2]
    # Fortran unformatted sequential records: 4-byte markers around the step and 9 planes
    raw = (a / "save.00000150.bin").read_bytes()
    n = 66 * 50 * 4
    assert len(raw) == (4 + 4 + 4) + 9 * (4 + n + 4)
    assert int.from_bytes(raw[4:8], "little") == 150


def test_driver_vks_writes_drag_lift(bgk, tmp_path):
    run_driver(bgk, tmp_path, case="VKS", lx=160, ly=62, svisc=0.05, itfin=200, itsave=1000000)
    rows = [ln.split() for ln in (tmp_path / "drag.lift.dat").read_text().splitlines()]
    # at every icheck; the end-of-run output has no drag/lift (SRC/bgk2d.F90:122-125)
    assert len(rows) == 2 and all(np.isfinite(float(x)) for r in rows for x in r[1:])
    # the obstacle outputs of SRC/initialize.F90:74-80 hold the mask of build_obs
    with bgk.Solver(160, 62, tcase="VKS", svisc=0.05, u0=0.1) as s:
        mask, bbox = s.obs()
    rows = np.loadtxt(tmp_path / "obstacle.dat", dtype=np.int64)
    assert rows.shape == (160 * 62, 3)
    assert np.array_equal(rows[:, 2].reshape(62, 160), mask)
    lines = (tmp_path / "tec_ob.00000000.vtk").read_text().splitlines()
    assert lines[:4] == ["# vtk DataFile Version 2.0", "Campo", "ASCII", "DATASET RECTILINEAR_GRID"]
    k = lines.index("LOOKUP_TABLE default")
    vals = np.array([float(x) for x in lines[k + 1:]])
    assert np.array_equal(vals.reshape(62, 160), mask.astype(float)) and vals.sum() == bbox[4]


def test_driver_obstacle_shapes_and_read_file(bgk, tmp_path):
    """--obstacle square / half_circle (the -DSQUARE and -DHALF_CIRCLE builds) give the solver's
    masks and diagnostics; --obstacle read:FILE (the -DREAD build's fort.96) with the square's
    mask as records gives the square run's outputs byte for byte."""
    kw = dict(lx=160, ly=62, svisc=0.05, itfin=200, itsave=1000000)
    runs = {}
    for shape in ("square", "half_circle"):
        d = tmp_path / shape
        d.mkdir()
        run_driver(bgk, d, case="VKS", extra=("--obstacle", shape), **kw)
        with bgk.Solver(160, 62, tcase="VKS", svisc=0.05, u0=0.1, obstacle=shape) as s:
            mask, _ = s.obs()
            s.step(200)
            want = s.diagno(2)  # diagno.dat holds the reference's own compute-kind sums
        rows = np.loadtxt(d / "obstacle.dat", dtype=np.int64)
        assert np.array_equal(rows[:, 2].reshape(62, 160), mask), shape
        last = (d / "diagno.dat").read_text().splitlines()[-1].split()
        np.testing.assert_allclose([float(x) for x in last[1:]], want, rtol=1e-5, atol=1e-12)
        runs[shape] = mask
    d = tmp_path / "read"
    d.mkdir()
    with open(d / "fort.96", "w") as f:
        for j in range(62):
            for i in range(160):
                f.write(f"  {float(i + 1):.6E}  {float(j + 1):.6E}  {int(runs['square'][j, i])}\n")
    run_driver(bgk, d, case="VKS", extra=("--obstacle", f"read:{d / 'fort.96'}"), **kw)
    for name in ("diagno.dat", "drag.lift.dat", "obstacle.dat", "prof_j.dat", "probe.dat"):
        assert (d / name).read_bytes() == (tmp_path / "square" / name).read_bytes(), name


def _vtk_sections(path):
    """(header lines, {section name: float32 array}) of a legacy binary VTK file as written by
    SRC/vtk_xy.binary.F90 / vtk_om.binary.F90."""
    data = path.read_bytes()
    head = data.split(b"POINT_DATA", 1)
    lines = head[0].decode().splitlines()
    rest = b"POINT_DATA" + head[1]
    eol = rest.index(b"\n")
    npts = int(rest[10:eol])
    rest = rest[eol + 1:]
    out = {}
    while rest:
        eol = rest.index(b"\n")
        title = rest[:eol].decode().strip()
        rest = rest[eol + 1:]
        count = npts
        if title.startswith("SCALARS"):
            eol = rest.index(b"\n")
            assert rest[:eol].decode().strip() == "LOOKUP_TABLE default"
            rest = rest[eol + 1:]
        else:
            count = 3 * npts
        out[title.split()[1]] = np.frombuffer(rest[:4 * count], dtype=">f4")
        rest = rest[4 * count:]
    return lines, npts, out


def test_driver_vtk_files(bgk, tmp_path):
    """tec_xy / tec_om files at the ivtim cadence, with the reference writers' header and the
    device-computed fields (big-endian float32)."""
    p = run_driver(bgk, tmp_path, itfin=200, ivtim=100)
    lx, ly = p["lx"], p["ly"]
    lines, npts, xy = _vtk_sections(tmp_path / "tec_xy.00000200.vtk")
    assert lines[:4] == ["# vtk DataFile Version 2.0", "Campo", "BINARY", "DATASET STRUCTURED_POINTS"]
    assert lines[4] == "DIMENSIONS %10d %10d %10d" % (lx, ly, 1) and npts == lx * ly
    _, npts2, om = _vtk_sections(tmp_path / "tec_om.00000200.vtk")
    assert npts2 == (lx - 2) * (ly - 2) and (tmp_path / "tec_xy.00000100.vtk").exists()
    # the start-up field (SRC/initialize.F90:119-123): velocity only
    assert (tmp_path / "tec_xy.00000000.vtk").exists() and not (tmp_path / "tec_om.00000000.vtk").exists()
    with bgk.Solver(lx, ly, tcase="LDC", svisc=p["svisc"], u0=0.1) as s:
        s.step(200)
        u, w, r, vort, st = s.vtk_fields()
    assert np.array_equal(xy["u"], u.ravel()) and np.array_equal(xy["rho"], r.ravel())
    assert np.array_equal(xy["velocity"][1::3], w.ravel())
    assert np.array_equal(om["vorticity"], vort.ravel()) and np.array_equal(om["stream"], st.ravel())


@pytest.mark.parametrize("case,prec,extra,skw", [
    ("BFS", "single", ["--scheme", "aa"], dict(scheme="aa")),
    ("MYV", "single", ["--forcing-y", "1"], dict(force_y=True)),
    ("LDC", "double", ["--noshift", "1"], dict(noshift=True, storage="f64")),
    ("LDC", "mixed2", ["--trick1", "1"], dict(trick1=True, storage="f32", compute="f64")),
])
def test_driver_build_variants_match_solver(bgk, tmp_path, case, prec, extra, skw):
    """The driver's switches for the reference's build variants (AA scheme with the backward-facing
    step, FORCING_Y with MYVERSION, NOSHIFT, TRICK1): the files it writes hold what the library
    gives for the same case: diagno.dat, the profiles computed on the device, and a checkpoint
    that restarts exactly."""
    p = run_driver(bgk, tmp_path, case=case, prec=prec, extra=extra, lx=48, ly=48, svisc=0.02)
    with bgk.Solver(p["lx"], p["ly"], tcase=case, svisc=p["svisc"], u0=0.1, **skw) as s:
        s.step(300)
        d = s.diagno(2)
        u, v, den = s.prof_j(p["lx"] // 2)
    rows = [ln.split() for ln in (tmp_path / "diagno.dat").read_text().splitlines()]
    np.testing.assert_allclose([float(x) for x in rows[-1][1:]], d, rtol=1e-5, atol=1e-12)
    last = (tmp_path / "prof_j.dat").read_text().split("# t=")[-1].strip().splitlines()[1:]
    vals = np.array([[float(x) for x in ln.split()] for ln in last])
    np.testing.assert_allclose(vals[:, 1], u, rtol=1e-5, atol=1e-11)
    np.testing.assert_allclose(vals[:, 3], den, rtol=1e-5)
    b = tmp_path / "b"
    b.mkdir()
    shutil.copy(tmp_path / "save.00000150.bin", b / "restore.bin")
    run_driver(bgk, b, case=case, prec=prec, extra=extra, lx=48, ly=48, svisc=0.02, irestart=1)
    assert (tmp_path / "diagno.dat").read_text().splitlines()[-1] == (b / "diagno.dat").read_text().splitlines()[-1]
