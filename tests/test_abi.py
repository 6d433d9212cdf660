"""C ABI surface (no GPU needed): the library loads and exports every entry point that
include/bgk2d_gb300.h declares; the Python mirror's structs match the C layout."""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_header_symbols(bgk):
    from bgk2d_gpu_gb300 import _lib
    path = _lib.lib_path()
    L = ctypes.CDLL(path)
    names = _lib.exported_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_version_and_default_desc(bgk):
    from bgk2d_gpu_gb300 import _lib
    L = _lib.load()
    assert b"sm_103a" in L.bgk_version()
    d = _lib.CaseDesc()
    assert L.bgk_default_desc(ctypes.byref(d)) == 0
    assert (d.lx, d.ly, d.radius, d.obs_icoord) == (256, 256, 16, -1)


STRUCTS = [("bgk_case_desc", "CaseDesc"), ("bgk_request", "Request"), ("bgk_result", "Result"),
           ("bgk_server_config", "ServerConfig"), ("bgk_server_stats", "ServerStats")]


def test_every_struct_layout_matches_c():
    """Every struct that crosses the ABI: the C compiler's sizeof and the offset of every field
    equal the ctypes mirror's, and the mirror names the same fields in the same order."""
    from bgk2d_gpu_gb300 import _lib
    lines = []
    for cname, pyname in STRUCTS:
        fields = [f[0] for f in getattr(_lib, pyname)._fields_]
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    src = ('#include <stdio.h>\n#include <stddef.h>\n#include "bgk2d_gb300.h"\nint main(void){'
           + "\n".join(lines) + "return 0;}\n")
    exe = os.path.join(ROOT, "bgk2d_gpu_gb300", "_build", "struct_layout")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    r = subprocess.run(["gcc", "-x", "c", "-", "-I", os.path.join(ROOT, "include"), "-o", exe], input=src,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr  # a field the mirror names but C lacks fails here
    c = dict(ln.split() for ln in subprocess.run([exe], capture_output=True, text=True).stdout.splitlines())
    for cname, pyname in STRUCTS:
        P = getattr(_lib, pyname)
        assert int(c[cname]) == ctypes.sizeof(P), cname
        for f, *_ in P._fields_:
            assert int(c[f"{cname}.{f}"]) == getattr(P, f).offset, (cname, f)


def test_no_device_means_loud_error(bgk):
    """Without a usable GPU, creating a case fails with a CUDA status; there is no CPU path."""
    import bgk2d_gpu_gb300 as m
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(m.BgkError):
        m.Solver(32, 32)


def test_namelist_reader(tmp_path):
    from bgk2d_gpu_gb300 import read_namelist
    p = tmp_path / "bgk.input"
    p.write_text("&parameters\nlx = 4096\nly = 4096\nsvisc=0.04096\nu0=0.1\nitfin=2000\n"
                 "ivtim=500000\nisignal=5000\nitsave=1000000\nicheck=100000\nirestart=0\ninit_v=0\nipad=0        /\n")
    v = read_namelist(str(p))
    assert v["lx"] == 4096 and v["svisc"] == 0.04096 and v["radius"] == 16 and v["itfin"] == 2000


def test_mask_shape_is_checked_before_the_library():
    """A wrong-shaped obstacle mask raises ValueError on the host, before any library call."""
    import numpy as np
    import bgk2d_gpu_gb300 as m
    with pytest.raises(ValueError):
        m.Solver(32, 16, obs_mask=np.zeros((32, 16), dtype=np.int32))


@pytest.mark.parametrize("lx,ly,code", [(0, 16, 1), (16, 1, 1), (16, 65534, 9), (8, 1 << 20, 9)])
def test_create_rejects_sizes_before_touching_a_device(lx, ly, code):
    """Sizes outside the library's limits fail in bgk_create before any CUDA call:
    BGK_E_INVALID below 2 cells, BGK_E_TOOLARGE above BGK_MAX_LY = 65533 rows."""
    import bgk2d_gpu_gb300 as m
    with pytest.raises(m.BgkError) as e:
        m.Solver(lx, ly)
    assert e.value.code == code


def test_namelist_fortran_forms(tmp_path):
    """Fortran namelist input as SRC/input.F90 reads it: names in any case, `!` comments,
    commas between items, d/D exponents; absent keys take the reference defaults."""
    from bgk2d_gpu_gb300 import read_namelist
    p = tmp_path / "bgk.input"
    p.write_text("! a run\n&PARAMETERS\nLX = 512, Ly=256  ! domain\nsvisc=4.d-2\nU0=1.0D-1\n"
                 "CTES=0.2 /\n")
    v = read_namelist(str(p))
    assert (v["lx"], v["ly"], v["svisc"], v["u0"], v["ctes"]) == (512, 256, 0.04, 0.1, 0.2)
    assert v["radius"] == 16 and v["ipad"] == 0


def test_driver_reads_fortran_namelist_and_rejects_bad_options(bgk, tmp_path):
    """The C++ driver's own namelist reader (case-blind names, `!` comments, d exponents), seen
    through --check-input, which stops before any device call; bad options exit with status 2."""
    from bgk2d_gpu_gb300 import build
    p = tmp_path / "bgk.input"
    p.write_text("! a run\n&PARAMETERS\nLX = 512, Ly=256  ! domain\nsvisc=4.d-2\nU0=1.0D-1\nitfin=10\n"
                 "CTES=0.2 /\n")
    r = subprocess.run([build.EXE_PATH, "--input", str(p), "--check-input", "1", "--prec", "f16"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    v = dict(kv.split("=") for kv in r.stdout.split())
    assert (v["lx"], v["ly"], v["itfin"], v["radius"], v["prec"]) == ("512", "256", "10", "16", "f16")
    assert (float(v["svisc"]), float(v["u0"]), float(v["ctes"])) == (0.04, 0.1, 0.2)
    for args in (["--prec", "dobule"], ["--scheme", "ab"], ["--bogus", "1"], ["--input"]):
        r = subprocess.run([build.EXE_PATH, *args], capture_output=True, text=True, timeout=60)
        assert r.returncode == 2, (args, r.stderr)

def _write_fort96(path, mask, sep="  "):
    ly, lx = mask.shape
    with open(path, "w") as f:
        for j in range(ly):
            for i in range(lx):
                f.write(f"{sep}{float(i + 1):.6E}{sep}{float(j + 1):.6E}{sep}{int(mask[j, i])}\n")


def test_driver_reads_the_read_build_obstacle_file(bgk, tmp_path):
    """--obstacle read:FILE takes the mask of the reference's READ build from its fort.96 records
    (`x y obs`, i fastest, list-directed: blanks or commas), counting the cells where obs is 1;
    a short file or a non-integer obs stops the driver (status 1), an unknown shape is a bad
    option (status 2)."""
    import numpy as np
    from bgk2d_gpu_gb300 import build
    lx, ly = 12, 10
    mask = np.zeros((ly, lx), dtype=int)
    mask[3:6, 4:7] = 1
    mask[7, 2] = 2  # not 1: not an obstacle cell, as the reference's obs(i,j) == 1 tests
    (tmp_path / "bgk.input").write_text("&parameters\nlx=12\nly=10\nitfin=5 /\n")

    def check(*args):
        return subprocess.run([build.EXE_PATH, "--input", str(tmp_path / "bgk.input"), "--check-input", "1",
                               "--case", "VKS", *args], capture_output=True, text=True, timeout=60)

    for sep in ("  ", ", "):
        _write_fort96(tmp_path / "fort.96", mask, sep)
        r = check("--obstacle", f"read:{tmp_path / 'fort.96'}")
        assert r.returncode == 0, r.stderr
        v = dict(kv.split("=") for kv in r.stdout.split())
        assert (v["obstacle"], v["obs_cells"]) == ("read", "9")
    lines = (tmp_path / "fort.96").read_text().splitlines()
    (tmp_path / "short.96").write_text("\n".join(lines[:-1]) + "\n")
    assert check("--obstacle", f"read:{tmp_path / 'short.96'}").returncode == 1
    (tmp_path / "real.96").write_text("\n".join(lines[:-1] + ["  1.2E+01  1.0E+01  1.0"]) + "\n")
    assert check("--obstacle", f"read:{tmp_path / 'real.96'}").returncode == 1
    assert check("--obstacle", "hexagon").returncode == 2
    r = check("--obstacle", "half_circle")
    assert r.returncode == 0 and "obstacle=half_circle" in r.stdout
