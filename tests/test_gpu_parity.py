"""GPU parity: the CUDA step through the C ABI against the CPU oracle on the same inputs.

FP32 (SINGLE), FP64 (DOUBLE) and FP32-storage/FP64-compute (MIXED2) kernels perform one IEEE
operation per reference operation, so after any number of steps the interior populations must
be bit-identical to the oracle (which restates SRC/col_MC.F90 and SRC/bcond.*.F90).  Obstacle
interiors follow the snapshot order of SRC/bcond.obs.F90 in the ping-pong scheme and are not
advanced by the AA scheme (they never influence fluid cells), so AA comparisons mask them.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRECS = {  # name: (oracle precision, storage, compute)
    "single": (0, "f32", "f32"),
    "double": (1, "f64", "f64"),
    "mixed2": (2, "f32", "f64"),
}

# (case, lx, ly, svisc, u0, extra oracle kwargs, extra solver kwargs)
CASES = {
    "ldc": ("LDC", 70, 37, 0.05, 0.1, {}, {}),
    "tgv": ("TGV", 64, 48, 0.05, 0.0, {}, {"init": "tgv_ref"}),
    "pof": ("POF", 96, 34, 0.1, 0.1, {}, {}),
    "cou": ("COU", 80, 40, 0.1, 0.1, {}, {}),
    "vks": ("VKS", 160, 62, 0.05, 0.1, {"obstacle": 1, "radius": 6}, {"radius": 6}),
}
ORACLE_CASE = {"LDC": 0, "TGV": 1, "POF": 2, "VKS": 3, "COU": 4}


def make_pair(oracle_mod, bgk, case, prec, scheme):
    tc, lx, ly, svisc, u0, okw, skw = CASES[case]
    oprec, st, cp = PRECS[prec]
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=ORACLE_CASE[tc], svisc=svisc, u0=u0,
                          obs_order=oracle_mod.OBS_SNAPSHOT, **okw)
    s = bgk.Solver(lx, ly, tcase=tc, svisc=svisc, u0=u0, storage=st, compute=cp, scheme=scheme, **skw)
    return o, s


def interior(a, lx, ly):
    return a[:, 1:ly + 1, 1:lx + 1]


def assert_same(o, s, scheme):
    lx, ly = s.lx, s.ly
    g = interior(s.download(), lx, ly)
    r = interior(o.raw(), lx, ly)
    if scheme == "aa":
        mask, bb = o.obs()
        keep = np.broadcast_to(mask == 0, g.shape)
        g, r = g[keep], r[keep]
    bad = np.argwhere(g != r) if g.ndim == 3 else np.flatnonzero(g != r)
    assert bad.size == 0, f"{len(bad)} populations differ; first {bad[:5]}; max|d|={np.abs(g - r).max()}"


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", list(CASES))
def test_step_bit_exact(oracle_mod, bgk, case, prec, scheme):
    o, s = make_pair(oracle_mod, bgk, case, prec, scheme)
    with s:
        assert_same(o, s, scheme)          # initial state (init.F90) identical
        done = 0
        for n in (1, 2, 7, 40, 75):        # odd/even counts, direct launches and graph replays
            s.step(n)
            o.step(n)
            done += n
            assert_same(o, s, scheme)
        assert s.scalars()["itime"] == done


@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
def test_reference_call_sequence(oracle_mod, bgk, prec):
    """boundaries / propagation / collision(itime), one call each per step, as SRC/bgk2d.F90:100-102."""
    o, s = make_pair(oracle_mod, bgk, "ldc", prec, "pingpong")
    with s:
        for it in range(1, 6):
            s.boundaries()
            s.propagation()
            s.collision(it)
        o.step(5)
        assert_same(o, s, "pingpong")


@pytest.mark.parametrize("case", ["ldc", "tgv", "vks"])
@pytest.mark.parametrize("prec", ["single", "double"])
def test_diagno_and_fields(oracle_mod, bgk, case, prec):
    o, s = make_pair(oracle_mod, bgk, case, prec, "pingpong")
    with s:
        s.step(33)
        o.step(33)
        d = s.diagno()
        ref = o.diagno(1)   # same per-cell arithmetic, FP64 accumulation
        np.testing.assert_allclose(d, ref, rtol=1e-12, atol=1e-15)
        ref0 = o.diagno(0)  # the reference's own mykind accumulation
        np.testing.assert_allclose(d, ref0, rtol=1e-4 if prec == "single" else 1e-12, atol=1e-7 if prec == "single" else 1e-15)
        r, u, v = s.fields()
        rr, ru, rv = o.fields()
        assert np.array_equal(r, rr) and np.array_equal(u, ru) and np.array_equal(v, rv)


@pytest.mark.parametrize("prec", ["single", "double"])
@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
def test_draglift(oracle_mod, bgk, prec, scheme):
    o, s = make_pair(oracle_mod, bgk, "vks", prec, scheme)
    with s:
        for n in (20, 13):
            s.step(n)
            o.step(n)
            np.testing.assert_allclose(s.draglift(), o.draglift(1), rtol=1e-12, atol=1e-14)
        d = s.diagno(1)
        np.testing.assert_allclose(d, o.diagno(2), rtol=1e-12, atol=1e-15)


def test_obstacle_mask_bit_exact(oracle_mod, bgk):
    """build_obs (SRC/build.obs.F90): circle, square, half circle, custom centre."""
    for shape, name in ((1, "circle"), (2, "square"), (3, "half_circle")):
        for (lx, ly, r, c) in ((200, 80, 9, (-1, -1)), (256, 64, 16, (64, 33)), (97, 51, 5, (-1, -1))):
            ref, rbb = oracle_mod.build_obs(lx, ly, shape, r, c[0], c[1])
            with bgk.Solver(lx, ly, tcase="CUSTOM", faces=("inflow", "outflow_zg", "wall", "wall"),
                            obstacle=name, radius=r, obs_center=c, u0=0.0, svisc=0.05) as s:
                mask, bb = s.obs()
            assert np.array_equal(mask, ref), (name, lx, ly)
            assert np.array_equal(bb, rbb)


@pytest.mark.parametrize("scheme", ["pingpong", "original"])
@pytest.mark.parametrize("prec", list(PRECS))
def test_large_obstacles_every_tile_shape(oracle_mod, bgk, prec, scheme):
    """Obstacles wide enough that whole vectors and their neighbourhoods lie inside them (circle,
    square and half circle of radius 3 to 20, centred and off-centre, in the periodic cylinder
    channel), stepped with every tile shape: the populations, obstacle cells included, equal the
    oracle's (SRC/build.obs.F90, SRC/bcond.obs.F90)."""
    oprec, st, cp = PRECS[prec]
    tiles = range(9) if scheme == "pingpong" else range(6)
    for shape, name, lx, ly, r, c in ((1, "circle", 200, 90, 20, (-1, -1)), (2, "square", 181, 70, 17, (60, 33)),
                                      (3, "half_circle", 150, 64, 12, (-1, -1)), (1, "circle", 97, 40, 3, (40, 20))):
        o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=ORACLE_CASE["VKS"], svisc=0.05, u0=0.1,
                              fused=scheme != "original", obs_order=oracle_mod.OBS_SNAPSHOT, obstacle=shape, radius=r,
                              obs_icoord=c[0], obs_jcoord=c[1])
        o.step(25)
        for tile in tiles:
            with bgk.Solver(lx, ly, tcase="VKS", svisc=0.05, u0=0.1, storage=st, compute=cp, scheme=scheme,
                            obstacle=name, radius=r, obs_center=c) as s:
                s.set_tile(tile)
                s.step(25)
                try:
                    assert_same(o, s, scheme)
                except AssertionError as e:
                    raise AssertionError(f"{name} r={r} tile {tile}: {e}") from None


def test_scalars_match_hencol(oracle_mod, bgk):
    for prec in ("single", "double"):
        for case in ("ldc", "pof", "cou"):
            o, s = make_pair(oracle_mod, bgk, case, prec, "pingpong")
            with s:
                a, b = s.scalars(), o.scalars()
                for k in ("omega", "fgrad", "u00", "u0"):
                    assert a[k] == b[k], (case, prec, k, a[k], b[k])


def test_upload_download_roundtrip(oracle_mod, bgk):
    for scheme in ("pingpong", "aa"):
        o, s = make_pair(oracle_mod, bgk, "tgv", "single", scheme)
        with s:
            o.step(9)
            s.upload(o.raw())
            assert_same(o, s, scheme)
            s.step(5)
            o.step(5)
            assert_same(o, s, scheme)


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
def test_ldc_256_re100_20000_steps(oracle_mod, bgk, prec, scheme):
    """The small plain case: LDC 256^2, Re=100, 20000 steps, bit-identical to the oracle in every
    precision and in both single-buffer and two-buffer schemes, profiles included."""
    oprec, st, cp = PRECS[prec]
    o = oracle_mod.Oracle(256, 256, prec=oprec, tcase=0, svisc=0.256, u0=0.1)
    with bgk.Solver(256, 256, tcase="LDC", svisc=0.256, u0=0.1, storage=st, compute=cp, scheme=scheme) as s:
        s.step(20000)
        o.step(20000, threads=16)
        assert_same(o, s, scheme)
        u, v, d = s.prof_j(128)
        ou, ov, od = o.prof_j(128)
        assert np.array_equal(u, ou) and np.array_equal(v, ov) and np.array_equal(d, od)


@pytest.mark.parametrize("prec", ["single", "double"])
def test_4096_first_steps_bit_exact(oracle_mod, bgk, prec):
    """Full-size lid-driven cavity (4096^2, Re=10000): first steps against the threaded oracle,
    then ping-pong and AA must stay bit-identical to each other."""
    oprec, st, cp = PRECS[prec]
    o = oracle_mod.Oracle(4096, 4096, prec=oprec, tcase=0, svisc=0.04096, u0=0.1)
    a = bgk.Solver(4096, 4096, tcase="LDC", svisc=0.04096, u0=0.1, storage=st, compute=cp)
    b = bgk.Solver(4096, 4096, tcase="LDC", svisc=0.04096, u0=0.1, storage=st, compute=cp, scheme="aa")
    try:
        o.step(3, threads=16)
        a.step(3)
        b.step(3)
        assert_same(o, a, "pingpong")
        assert_same(o, b, "aa")
        a.step(97)
        b.step(97)
        ga, gb = interior(a.download(), 4096, 4096), interior(b.download(), 4096, 4096)
        assert np.array_equal(ga, gb)
        # mass: bounce-back and the lid's +-u00/6 pair conserve it
        d = a.diagno()
        assert abs(d[2] - 1.0) < (2e-6 if prec == "single" else 1e-13)
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", ["ldc", "tgv", "vks"])
def test_les_bit_exact(oracle_mod, bgk, case, prec, scheme):
    """Smagorinsky eddy viscosity (-DLES, SRC/col_MC.F90:178-248), cteS = 0.2."""
    tc, lx, ly, svisc, u0, okw, skw = CASES[case]
    oprec, st, cp = PRECS[prec]
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=ORACLE_CASE[tc], svisc=svisc / 4, u0=u0,
                          obs_order=oracle_mod.OBS_SNAPSHOT, les=True, cte_s=0.2, **okw)
    with bgk.Solver(lx, ly, tcase=tc, svisc=svisc / 4, u0=u0, storage=st, compute=cp, scheme=scheme,
                    les=True, cte_s=0.2, **skw) as s:
        for n in (1, 2, 40, 75):
            s.step(n)
            o.step(n)
            assert_same(o, s, scheme)


@pytest.mark.parametrize("scheme", ["pingpong", "aa", "original"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
def test_trick1_bit_exact(oracle_mod, bgk, prec, scheme):
    """-DTRICK1 lid-cavity boundaries (SRC/bcond.driven.F90:43-81) on a square box: the x-wall rule
    sets the two upper corner ghosts.  Bit-identical to the oracle's merged loop, and different
    from the default order."""
    n = 56
    oprec, st, cp = PRECS[prec]
    kw = dict(prec=oprec, tcase=0, svisc=0.02, u0=0.1, fused=scheme != "original")
    o = oracle_mod.Oracle(n, n, trick1=True, **kw)
    d = oracle_mod.Oracle(n, n, **kw)
    with bgk.Solver(n, n, tcase="LDC", svisc=0.02, u0=0.1, storage=st, compute=cp, scheme=scheme,
                    trick1=True) as s:
        for k in (1, 2, 40, 75):
            s.step(k)
            o.step(k)
            d.step(k)
            assert_same(o, s, scheme)
    assert not np.array_equal(interior(o.raw(), n, n), interior(d.raw(), n, n))


@pytest.mark.parametrize("tile", range(9))
def test_trick1_every_tile_and_les(oracle_mod, bgk, tile):
    """The corner rule in every ping-pong kernel shape (register tiles and the staged copies),
    alone and with the Smagorinsky collision."""
    n = 72
    for les in ((False, True) if tile == 0 else (False,)):
        o = oracle_mod.Oracle(n, n, prec=0, tcase=0, svisc=0.01, u0=0.1, trick1=True, les=les, cte_s=0.2)
        with bgk.Solver(n, n, tcase="LDC", svisc=0.01, u0=0.1, trick1=True, les=les, cte_s=0.2) as s:
            if not les:
                s.set_tile(tile)
            s.step(33)
            o.step(33)
            assert_same(o, s, "pingpong")


def test_trick1_refused_off_the_square_cavity(bgk):
    for kw in (dict(lx=64, ly=48, tcase="LDC"), dict(lx=64, ly=64, tcase="COU")):
        with pytest.raises(bgk.BgkError):
            bgk.Solver(trick1=True, **kw)


def _bfs_fluid(a, lx, ly):
    """Interior populations outside the step block x < lx/20, y < ly/2 (SRC/input.F90:74-75)."""
    sx, sy = lx // 20, ly // 2
    g = a[:, 1:ly + 1, 1:lx + 1]
    keep = np.ones((ly, lx), bool)
    keep[:sy - 1, :sx - 1] = False
    return g[:, keep]


@pytest.mark.parametrize("scheme,tile", [("pingpong", 2), ("pingpong", 6), ("aa", 2), ("aa", 5)])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
def test_bfs_bit_exact(oracle_mod, bgk, prec, scheme, tile):
    """Backward-facing step (SRC/bcond.step.F90) folded into the step's rules: equilibrium outflow,
    parabolic inflow above the step and the step's wall below it, no-slip walls, the solid block
    as obstacle cells and the five bounce-backs at its corner (step_bounce).  The solid block
    holds values nobody reads back (the reference poisons its second buffer with huge()), so the
    fluid cells are compared, in ping-pong (register and staged kernels) and AA."""
    oprec, st, cp = PRECS[prec]
    lx, ly = 200, 64
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=oracle_mod.BFS, svisc=0.02, u0=0.1)
    with bgk.Solver(lx, ly, tcase="BFS", svisc=0.02, u0=0.1, storage=st, compute=cp, scheme=scheme) as s:
        s.set_tile(tile)
        for n in (1, 2, 40, 75):
            s.step(n)
            o.step(n)
            g, r = _bfs_fluid(s.download(), lx, ly), _bfs_fluid(o.raw(), lx, ly)
            bad = np.flatnonzero(g != r)
            assert bad.size == 0, f"{bad.size} populations differ after {n}"


@pytest.mark.parametrize("tile", [2, 6])
@pytest.mark.parametrize("prec", ["single", "double"])
def test_bfs_fluid_cells_never_read_the_solid_block(oracle_mod, bgk, prec, tile):
    """The poison check of the reference's allocation (SRC/alloca.F90:133-151 fills the second
    buffer with huge()): here the whole solid block x < lx/20, y < ly/2 of the starting state
    holds the largest finite value of the storage kind.  The fluid cells stay bit-identical to
    the oracle's, which starts with zeros there, so no fluid update reads a block value."""
    oprec, st, cp = PRECS[prec]
    lx, ly = 200, 64
    sx, sy = lx // 20, ly // 2
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=oracle_mod.BFS, svisc=0.02, u0=0.1)
    with bgk.Solver(lx, ly, tcase="BFS", svisc=0.02, u0=0.1, storage=st, compute=cp) as s:
        s.set_tile(tile)
        a = s.download()
        a[:, 1:sy, 1:sx] = np.finfo(a.dtype).max
        s.upload(a)
        for n in (1, 2, 40):
            s.step(n)
            o.step(n)
            got = s.download()
            assert np.array_equal(_bfs_fluid(got, lx, ly), _bfs_fluid(o.raw(), lx, ly)), f"after {n} more steps"
            assert not np.isfinite(got[:, 1:sy - 1, 1:sx - 1]).any()  # the block itself stays poisoned


@pytest.mark.parametrize("scheme", ["pingpong", "aa", "original"])
@pytest.mark.parametrize("prec", list(PRECS))
@pytest.mark.parametrize("case", ["tgv", "pof", "cou", "vks"])
def test_long_runs_stay_bit_exact(oracle_mod, bgk, case, prec, scheme):
    """3000 steps of the vortex, channel, Couette and cylinder cases (the cylinder's wake sheds
    vortices, so any difference of rounding would grow): populations and the reference's own
    diagno sums stay identical to the oracle's."""
    o, s = make_pair(oracle_mod, bgk, case, prec, scheme)
    if scheme == "original":
        s.close()
        tc, lx, ly, svisc, u0, okw, skw = CASES[case]
        oprec, st, cp = PRECS[prec]
        o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=ORACLE_CASE[tc], svisc=svisc, u0=u0, fused=False,
                              obs_order=oracle_mod.OBS_SNAPSHOT, **okw)
        s = bgk.Solver(lx, ly, tcase=tc, svisc=svisc, u0=u0, storage=st, compute=cp, scheme=scheme, **skw)
    with s:
        s.step(3000)
        o.step(3000)
        assert_same(o, s, scheme)
        if scheme != "aa" or case != "vks":  # AA leaves obstacle interiors, which diagno sums, behind
            np.testing.assert_array_equal(s.diagno(2), o.diagno(0))


VARIANT_RUNS = {  # name: (case, lx, ly, svisc, u0, oracle and solver keywords)
    "les_cavity": ("LDC", 72, 56, 0.01, 0.1, dict(les=True, cte_s=0.2)),
    "les_cylinder": ("VKS", 160, 62, 0.02, 0.1, dict(les=True, cte_s=0.2)),
    "noshift_cavity": ("LDC", 72, 56, 0.02, 0.1, dict(noshift=True)),
    "trick1_cavity": ("LDC", 64, 64, 0.02, 0.1, dict(trick1=True)),
    "myversion_force_y": ("MYV", 64, 48, 0.05, 0.1, dict(force_y=True)),
}


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", list(PRECS))
@pytest.mark.parametrize("name", list(VARIANT_RUNS))
def test_build_variants_long_runs_stay_bit_exact(oracle_mod, bgk, name, prec, scheme):
    """3000 steps of the reference's build variants (LES on a cavity and on the cylinder's wake,
    NOSHIFT, TRICK1, MYVERSION with FORCING_Y): the populations stay identical to the oracle's."""
    tc, lx, ly, svisc, u0, kw = VARIANT_RUNS[name]
    oprec, st, cp = PRECS[prec]
    okw = dict(kw, obstacle=1, radius=6) if tc == "VKS" else dict(kw)
    skw = dict(kw, radius=6) if tc == "VKS" else dict(kw)
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase={"LDC": 0, "VKS": 3, "MYV": 6}[tc], svisc=svisc, u0=u0,
                          obs_order=oracle_mod.OBS_SNAPSHOT, **okw)
    with bgk.Solver(lx, ly, tcase=tc, svisc=svisc, u0=u0, storage=st, compute=cp, scheme=scheme, **skw) as s:
        s.step(3000)
        o.step(3000)
        assert_same(o, s, scheme)


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", ["single", "double"])
def test_bfs_long_run(oracle_mod, bgk, prec, scheme):
    """1500 steps of a backward-facing step (the flow separates behind the step and reattaches):
    the fluid cells stay bit-identical to the oracle's."""
    oprec, st, cp = PRECS[prec]
    lx, ly = 160, 40
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=oracle_mod.BFS, svisc=0.01, u0=0.1)
    with bgk.Solver(lx, ly, tcase="BFS", svisc=0.01, u0=0.1, storage=st, compute=cp, scheme=scheme) as s:
        s.step(1500)
        o.step(1500)
        assert np.array_equal(_bfs_fluid(s.download(), lx, ly), _bfs_fluid(o.raw(), lx, ly))
        u, _, _ = s.prof_j(lx // 2)
        assert np.abs(u).max() > 0.01  # the inflow has reached mid-channel


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
def test_bfs_small_steps_and_tiles(oracle_mod, bgk, scheme):
    """Backward-facing steps down to the smallest (lx = 40: stepx = 2, a one-column block; ly = 4
    and 5: stepy = 2, a one-row block), odd sizes, every tile shape of the scheme; fluid cells
    bit-exact against the oracle."""
    for lx, ly in ((40, 4), (41, 5), (60, 9), (83, 31), (140, 6)):
        for tile in range(9 if scheme == "pingpong" else 6):
            o = oracle_mod.Oracle(lx, ly, prec=0, tcase=oracle_mod.BFS, svisc=0.02, u0=0.1)
            with bgk.Solver(lx, ly, tcase="BFS", svisc=0.02, u0=0.1, scheme=scheme) as s:
                s.set_tile(tile)
                s.step(23)
                o.step(23)
                assert np.array_equal(_bfs_fluid(s.download(), lx, ly), _bfs_fluid(o.raw(), lx, ly)), (lx, ly, tile)


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_prefetch_does_not_change_results(bgk, storage, scheme):
    """The L2 prefetch only moves data earlier; populations are identical with and without it."""
    out = []
    for pf in (0, 64, 1216):
        with bgk.Solver(700, 300, tcase="LDC", svisc=0.02, u0=0.1, storage=storage, scheme=scheme) as s:
            s.set_tile(5)
            s.set_prefetch(pf)
            assert s.prefetch() == pf
            s.step(70)
            out.append(s.download())
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", ["ldc", "tgv", "vks"])
def test_vtk_fields_bit_exact(oracle_mod, bgk, case, prec, scheme):
    """The VTK writers' fields (SRC/vtk_xy.binary.F90, vtk_om.binary.F90) computed on the device,
    against the oracle's restatement; the stream function integrates from row 1 on both sides."""
    if scheme == "aa" and case == "vks":
        pytest.skip("AA keeps obstacle interiors un-advanced; their neighbours' vorticity differs")
    o, s = make_pair(oracle_mod, bgk, case, prec, scheme)
    with s:
        s.step(57)
        o.step(57)
        got = s.vtk_fields()
    want = o.vtk(from_ghost_row=False)
    for name, g, w in zip(("u", "w", "rho", "vorticity", "stream"), got, want):
        assert np.array_equal(g, w), f"{name}: {int(np.sum(g != w))} values differ, max |d| {np.abs(g - w).max()}"


@pytest.mark.parametrize("tile", [0, 1, 3, 4, 5])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", ["ldc", "pof", "vks"])
def test_aa_tile_shapes_bit_exact(oracle_mod, bgk, case, prec, tile):
    """AA steps with every tile shape, 16 or 8 bytes per thread (configurations 4, 5)."""
    o, s = make_pair(oracle_mod, bgk, case, prec, "aa")
    with s:
        s.set_tile(tile)
        for n in (1, 2, 40, 75):
            s.step(n)
            o.step(n)
            assert_same(o, s, "aa")


@pytest.mark.parametrize("tile", [4, 5])
@pytest.mark.parametrize("storage", ["f16", "bf16"])
def test_aa_16bit_half_vector_accuracy(bgk, storage, tile):
    """16-bit AA with 8 bytes per thread stays as close to FP32 as the whole-vector kernels."""
    errs = []
    for t in (0, tile):
        with bgk.Solver(300, 200, tcase="LDC", svisc=0.02, u0=0.1, storage=storage, scheme="aa") as s, \
                bgk.Solver(300, 200, tcase="LDC", svisc=0.02, u0=0.1, storage="f32", scheme="aa") as r:
            s.set_tile(t)
            s.step(400)
            r.step(400)
            _, u, v = s.fields()
            _, ur, vr = r.fields()
        errs.append(float(np.sqrt(np.sum((u - ur) ** 2 + (v - vr) ** 2) / np.sum(ur ** 2 + vr ** 2))))
    assert errs[1] < max(2 * errs[0], 1e-3), errs


@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", list(CASES))
def test_original_two_pass_bit_exact(oracle_mod, bgk, case, prec):
    """BGK_SCHEME_ORIGINAL: streaming (SRC/movef.F90) then collision (SRC/col.F90) as two kernels,
    against the oracle's ORIGINAL form (movef + col)."""
    tc, lx, ly, svisc, u0, okw, skw = CASES[case]
    oprec, st, cp = PRECS[prec]
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=ORACLE_CASE[tc], svisc=svisc, u0=u0, fused=False,
                          obs_order=oracle_mod.OBS_SNAPSHOT, **okw)
    with bgk.Solver(lx, ly, tcase=tc, svisc=svisc, u0=u0, storage=st, compute=cp, scheme="original", **skw) as s:
        for n in (1, 2, 40, 75):
            s.step(n)
            o.step(n)
            assert_same(o, s, "original")
        n0 = s.launches()
        s.step(64)
        assert s.launches() - n0 == 128  # two kernels per step


def test_original_reference_call_sequence(oracle_mod, bgk):
    """boundaries / propagation / collision(itime) split the two passes like the reference."""
    o = oracle_mod.Oracle(70, 37, prec=0, tcase=0, svisc=0.05, u0=0.1, fused=False)
    with bgk.Solver(70, 37, tcase="LDC", svisc=0.05, u0=0.1, scheme="original") as s:
        for it in range(1, 6):
            s.boundaries()
            s.propagation()
            s.collision(it)
        o.step(5)
        assert_same(o, s, "original")
        s.propagation()
        with pytest.raises(bgk.BgkError):
            s.step(1)  # half a step pending
        s.collision(6)
        s.step(3)
        o.step(4)
        assert_same(o, s, "original")


def test_original_bfs_and_les(oracle_mod, bgk):
    lx, ly = 200, 64
    o = oracle_mod.Oracle(lx, ly, prec=0, tcase=oracle_mod.BFS, svisc=0.02, u0=0.1, fused=False)
    with bgk.Solver(lx, ly, tcase="BFS", svisc=0.02, u0=0.1, scheme="original") as s:
        s.step(45)
        o.step(45)
        assert np.array_equal(_bfs_fluid(s.download(), lx, ly), _bfs_fluid(o.raw(), lx, ly))
    o = oracle_mod.Oracle(70, 37, prec=1, tcase=0, svisc=0.01, u0=0.1, fused=False, les=True, cte_s=0.2)
    with bgk.Solver(70, 37, tcase="LDC", svisc=0.01, u0=0.1, storage="f64", scheme="original", les=True,
                    cte_s=0.2) as s:
        s.step(45)
        o.step(45)
        assert_same(o, s, "original")


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", ["ldc", "tgv", "vks"])
def test_diagno_reference_order_bit_exact(oracle_mod, bgk, case, prec, scheme):
    """BGK_DIAGNO_REFERENCE: sums in the compute kind in SRC/diagno.F90's serial order, equal to the
    oracle's mykind diagno (mode 0), i.e. to the values the reference writes to diagno.dat."""
    if scheme == "aa" and case == "vks":
        pytest.skip("AA keeps obstacle interiors un-advanced; all-cell sums differ there")
    o, s = make_pair(oracle_mod, bgk, case, prec, scheme)
    with s:
        s.step(41)
        o.step(41)
        got = s.diagno(2)
    assert list(got) == list(o.diagno(0))


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
def test_draglift_reference_order_bit_exact(oracle_mod, bgk, prec, scheme):
    """bgk_draglift_reference: SRC/draglift.F90's compute-kind sums in its order (oracle mode 0)."""
    o, s = make_pair(oracle_mod, bgk, "vks", prec, scheme)
    with s:
        s.step(37)
        o.step(37)
        assert list(s.draglift(reference=True)) == list(o.draglift(0))


def test_tuning_knobs_validate(bgk):
    with bgk.Solver(64, 48) as s:
        with pytest.raises(bgk.BgkError):
            s.set_prefetch(-1)
        with pytest.raises(bgk.BgkError):
            s.set_tile(9)
    with bgk.Solver(64, 48, scheme="aa") as s:
        with pytest.raises(bgk.BgkError):
            s.set_tile(6)  # staged rows exist for ping-pong only


@pytest.mark.parametrize("scheme", ["pingpong", "aa", "original"])
@pytest.mark.parametrize("lx,ly", [(2, 2), (3, 5), (5, 3), (9, 2), (17, 7), (33, 4), (130, 3)])
def test_tiny_domains_every_tile_shape(oracle_mod, bgk, scheme, lx, ly):
    """Domains narrower than one vector, a warp or a block, and one or two tile rows, in every
    tile shape (block-row order, ragged vectors, single-vector rows)."""
    for prec in ("single", "double"):
        oprec, st, cp = PRECS[prec]
        o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=0, svisc=0.05, u0=0.1, fused=scheme != "original")
        with bgk.Solver(lx, ly, tcase="LDC", svisc=0.05, u0=0.1, storage=st, compute=cp, scheme=scheme) as s:
            for tile in range(6):
                s.set_tile(tile)
                s.step(3)
                o.step(3)
                assert_same(o, s, scheme)


@pytest.mark.parametrize("scheme", ["pingpong", "aa", "original"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case", list(CASES))
def test_noshift_bit_exact(oracle_mod, bgk, case, prec, scheme):
    """-DNOSHIFT: the arrays hold the populations f themselves (cte1/cte0 of SRC/col_MC.F90:70-75,
    SRC/col.F90:61-66, SRC/init.F90:73-77, SRC/bcond.inflow.F90:48-52, SRC/diagno.F90:42-46,
    SRC/prof_j.F90:40-44, SRC/vtk_xy.binary.F90:46-50).  Populations, the reference's diagno
    sums, the VTK fields and the prof_j reader are bit-identical to the oracle's NOSHIFT form."""
    tc, lx, ly, svisc, u0, okw, skw = CASES[case]
    oprec, st, cp = PRECS[prec]
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=ORACLE_CASE[tc], svisc=svisc, u0=u0, fused=scheme != "original",
                          obs_order=oracle_mod.OBS_SNAPSHOT, noshift=True, **okw)
    with bgk.Solver(lx, ly, tcase=tc, svisc=svisc, u0=u0, storage=st, compute=cp, scheme=scheme, noshift=True,
                    **skw) as s:
        assert_same(o, s, scheme)          # the reference's init with cte1 = 1
        for n in (1, 2, 40, 75):
            s.step(n)
            o.step(n)
            assert_same(o, s, scheme)
        if scheme == "aa" and case == "vks":
            return  # AA keeps obstacle interiors un-advanced: all-cell sums differ there
        assert list(s.diagno(2)) == list(o.diagno(0))
        u, v, d = s.prof_j(lx // 2)
        ou, ov, od = o.prof_j(lx // 2)
        assert np.array_equal(u, ou) and np.array_equal(v, ov) and np.array_equal(d, od)
        r, fu, fv = s.fields()
        rr, ru, rv = o.fields()
        assert np.array_equal(r, rr) and np.array_equal(fu, ru) and np.array_equal(fv, rv)
        for name, g, w in zip(("u", "w", "rho", "vorticity", "stream"), s.vtk_fields(), o.vtk(from_ghost_row=False)):
            assert np.array_equal(g, w), name


@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
def test_noshift_bfs_les_and_limits(oracle_mod, bgk, prec):
    """NOSHIFT with the backward-facing step (parabolic inflow and outflow equilibria with
    cte1 = 1, SRC/bcond.step.F90:49-53) and with the Smagorinsky collision; 16-bit storage and
    batches refuse it; the end-to-end call falls back to the three calls and stays exact."""
    oprec, st, cp = PRECS[prec]
    lx, ly = 200, 64
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=oracle_mod.BFS, svisc=0.02, u0=0.1, noshift=True)
    with bgk.Solver(lx, ly, tcase="BFS", svisc=0.02, u0=0.1, storage=st, compute=cp, noshift=True) as s:
        for n in (1, 40):
            s.step(n)
            o.step(n)
            assert np.array_equal(_bfs_fluid(s.download(), lx, ly), _bfs_fluid(o.raw(), lx, ly))
    for scheme in ("pingpong", "aa", "original"):
        o = oracle_mod.Oracle(70, 37, prec=oprec, tcase=0, svisc=0.01, u0=0.1, les=True, cte_s=0.2, noshift=True,
                              fused=scheme != "original")
        with bgk.Solver(70, 37, tcase="LDC", svisc=0.01, u0=0.1, storage=st, compute=cp, scheme=scheme, les=True,
                        cte_s=0.2, noshift=True) as s:
            s.step(45)
            o.step(45)
            assert_same(o, s, scheme)
    torch = pytest.importorskip("torch")
    o = oracle_mod.Oracle(96, 40, prec=oprec, tcase=0, svisc=0.02, u0=0.1, noshift=True)
    with bgk.Solver(96, 40, tcase="LDC", svisc=0.02, u0=0.1, storage=st, compute=cp, noshift=True) as s:
        a = torch.from_numpy(s.download()).pin_memory()  # page-locked: the pipelined path would apply
        b = torch.zeros_like(a).pin_memory()
        s.advance_host(a, b, 30)
        o.step(30)
        assert np.array_equal(interior(b.numpy(), 96, 40), interior(o.raw(), 96, 40))
        with bgk.Batch(st, cp) as bt:
            with pytest.raises(bgk.BgkError):
                bt.add(s)
    for st16 in ("f16", "bf16"):
        with pytest.raises(bgk.BgkError):
            bgk.Solver(64, 64, storage=st16, noshift=True)


@pytest.mark.parametrize("scheme", ["pingpong", "aa", "original"])
@pytest.mark.parametrize("prec", ["single", "double", "mixed2"])
@pytest.mark.parametrize("case,force_y", [("MYV", False), ("MYV", True), ("POF", True)])
def test_body_force_variants_bit_exact(oracle_mod, bgk, case, force_y, prec, scheme):
    """-DMYVERSION (periodic boundaries with the CHANNEL volume force, SRC/boundaries.F90:46-48,
    SRC/build.bcond.F90:39-41) and -DFORCING_Y (the force along y, SRC/col_MC.F90:268-282)."""
    lx, ly = 64, 40
    oprec, st, cp = PRECS[prec]
    otc = oracle_mod.MYV if case == "MYV" else oracle_mod.POF
    o = oracle_mod.Oracle(lx, ly, prec=oprec, tcase=otc, svisc=0.1, u0=0.1, fused=scheme != "original",
                          force_y=force_y)
    with bgk.Solver(lx, ly, tcase=case, svisc=0.1, u0=0.1, storage=st, compute=cp, scheme=scheme,
                    force_y=force_y) as s:
        for n in (1, 2, 40, 75):
            s.step(n)
            o.step(n)
            assert_same(o, s, scheme)
        assert list(s.diagno(2)) == list(o.diagno(0))
        d = s.diagno()
    # the mean flow follows the force: along x, or along y with FORCING_Y
    assert (abs(d[1]) > 100 * abs(d[0])) if force_y else (abs(d[0]) > 100 * abs(d[1]))


def test_force_y_needs_a_forced_case(bgk):
    for tc in ("LDC", "TGV", "COU"):
        with pytest.raises(bgk.BgkError):
            bgk.Solver(64, 48, tcase=tc, force_y=True)


@pytest.mark.parametrize("scheme", ["pingpong", "aa"])
@pytest.mark.parametrize("storage,compute", [("f32", "f32"), ("f64", "f64"), ("f32", "f64"), ("f16", "f32"),
                                             ("bf16", "f32")])
def test_device_profile_readers_equal_host_readers(bgk, storage, compute, scheme):
    """bgk_prof_i / bgk_prof_j / bgk_varm / bgk_probe (the readers of SRC/prof_i.F90, prof_j.F90,
    varm.F90 and probe.F90 on the device) give, bit for bit, what the host readers give on the
    downloaded populations: cavities (with NOSHIFT for the exact kinds) and a channel with a
    cylinder, after an odd and an even number of steps."""
    cases = [dict(lx=90, ly=52, tcase="LDC", svisc=0.02, u0=0.1),
             dict(lx=160, ly=62, tcase="VKS", svisc=0.05, u0=0.1, radius=6)]
    if storage in ("f32", "f64"):
        cases.append(dict(lx=70, ly=37, tcase="LDC", svisc=0.02, u0=0.1, noshift=True))
    for kw in cases:
        with bgk.Solver(storage=storage, compute=compute, scheme=scheme, **kw) as s:
            for n in (37, 2):
                s.step(n)
                a = s.download()
                for dev, host in ((s.prof_i(kw["ly"] // 3), s.prof_i(kw["ly"] // 3, pops=a)),
                                  (s.prof_j(kw["lx"] // 2), s.prof_j(kw["lx"] // 2, pops=a)),
                                  (s.varm(), s.varm(pops=a)),
                                  (s.probe(5, kw["ly"] - 2), s.probe(5, kw["ly"] - 2, pops=a))):
                    for d, h in zip(dev, host):
                        d, h = np.asarray(d), np.asarray(h)
                        assert d.dtype == h.dtype and np.array_equal(d, h), (kw, n, d, h)
        with pytest.raises(bgk.BgkError):
            s2 = bgk.Solver(storage=storage, compute=compute, scheme=scheme, **kw)
            try:
                s2.prof_i(0)
            finally:
                s2.close()
