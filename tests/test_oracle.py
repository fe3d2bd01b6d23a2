"""The oracle itself: the C restatement against the reference's own outputs.

The golden fixtures were produced by the reference's macpressuresolver{2,3}
built from its sources (tests/golden/make_golden.py). The restatement must
reproduce them bit for bit: pressure, projected velocity, the set of unknown
cells and the CG iteration count.
"""
import numpy as np
import pytest

import oracle
from golden_io import Case, case_names
from shiokaze_gb300 import scenes


@pytest.mark.parametrize("name", case_names())
def test_port_matches_reference_fixture(name):
    c = Case(name)
    pj = oracle.PortProjector(c.dim, c.nx, c.ny, c.nz, c.dx, **c.params)
    res = None
    for s in range(c.steps):
        u, v, w = c.inputs[s]
        if c.volume is not None:
            pj.set_target_volume(*c.volume[s])
        res = pj.project(c.dt, c.solid, c.fluid, u, v, w)
    pj.close()
    assert np.array_equal(res.unknown, c.out_unknown)
    assert np.array_equal(res.pressure, c.out_pressure)
    assert np.array_equal(res.u, c.out_u)
    assert np.array_equal(res.v, c.out_v)
    if c.dim == 3:
        assert np.array_equal(res.w, c.out_w)
        assert res.iterations == c.iterations


def test_known_answer_accuracy():
    """accuracytest3 (src/examples/accuracytest3-example.cpp:108-127): the
    projected pressure approximates |x-c|^2 - r^2; error shrinks ~2nd order."""
    errs = []
    for n in (16, 32):
        sc, exact = scenes.accuracy3(n, 0.25)
        r = oracle.project_scene(sc, "port", residual=1e-18, eps_fluid=1e-18)
        m = r.unknown
        errs.append(float(np.max(np.abs(r.pressure[m] - exact[m]))))
    assert errs[1] < errs[0] * 0.6, errs


def test_no_fluid_is_identity_away_from_walls():
    """No fluid anywhere: no unknowns, every fluid fraction reads 1, interior
    faces keep their velocity and wall faces are zeroed."""
    sc = scenes.liquid3(8, seed=12)
    sc.fluid[...] = np.float32(sc.band)
    r = oracle.project_scene(sc, "port")
    assert not r.unknown.any()
    assert np.array_equal(r.u[:, :, 1:-1], sc.u[:, :, 1:-1])
    assert not r.u[:, :, 0].any() and not r.u[:, :, -1].any()


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", [21, 22])
def test_port_matches_live_reference(seed):
    rng = np.random.default_rng(seed)
    n = tuple(int(x) for x in rng.integers(9, 20, 3))
    sc = scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5)))
    a = oracle.project_scene(sc, "port")
    b = oracle.project_scene(sc, "reference")
    assert np.array_equal(a.unknown, b.unknown)
    assert np.array_equal(a.pressure, b.pressure)
    assert np.array_equal(a.w, b.w)
    assert a.iterations == b.iterations


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
def test_plugin_module_loads_through_reference_loader(tmp_path):
    """The drop-in: the reference's own module loader (src/core/module.cpp:
    103-172) picks gbprojection3 / gbprojection2 by the Projection key,
    creates, configures and initializes it. (project() needs a GPU.)"""
    import subprocess
    root = oracle.HERE.rsplit("/", 1)[0]
    subprocess.check_call(["make", "-s", "-C", f"{root}/shiokaze_gb300/module", f"OUT={oracle.REF_DIR}"],
                          stdout=subprocess.DEVNULL)
    lib = oracle._ref_lib()
    for dim in (3, 2):
        log = str(tmp_path / f"load{dim}.log")
        h = lib.ref_create(dim, 16, 16, 16, 1 / 16, f"Projection=gbprojection{dim} Solver=mgpcg".encode(),
                           log.encode())
        assert h
        text = open(log).read()
        assert f"gbprojection{dim}" in text
        lib.ref_destroy(h)


def test_linsolver_module_loads_through_reference_loader(tmp_path):
    """The LinSolver drop-in: macpressuresolver3 / 2 create their linear
    solver through the reference's loader by the LinSolver key
    (include/shiokaze/linsolver/RCMatrix_solver.h:40); LinSolver=gbpcg loads
    the GPU solver module in place of pcg. (solve() needs a GPU.)"""
    import subprocess
    root = oracle.HERE.rsplit("/", 1)[0]
    subprocess.check_call(["make", "-s", "-C", f"{root}/shiokaze_gb300/module", f"OUT={oracle.REF_DIR}"],
                          stdout=subprocess.DEVNULL)
    lib = oracle._ref_lib()
    for dim in (3, 2):
        log = str(tmp_path / f"lin{dim}.log")
        h = lib.ref_create(dim, 16, 16, 16, 1 / 16, b"LinSolver=gbpcg Residual=1e-6", log.encode())
        assert h
        text = open(log).read()
        assert "gbpcg" in text and "pcg.so" not in text.replace("gbpcg.so", "")
        lib.ref_destroy(h)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("kind,n", [("liquid3", 48), ("liquid3", (40, 33, 37)), ("smoke3", 40), ("liquid2", 160),
                                    ("liquid2", (150, 97))])
def test_module_densify_matches_operator_reads(kind, n):
    """The plugin modules' dense copy of the reference's tiled arrays
    (shiokaze_gb300/module/gbarray_adapter.h: background, then the filled
    cells, then the active cells) equals reading every cell through the
    reference's operator() (include/shiokaze/array/array3.h:796-800), bit
    for bit: narrow-band level sets with flood-filled tiles, a constant
    array, and a partly active velocity component over a background."""
    sc = getattr(scenes, kind)(n, seed=5)
    vel_band = float(np.quantile(np.abs(sc.u), 0.4))
    for arr, mode, band in ((sc.solid, sc.solid_mode, sc.band), (sc.fluid, sc.fluid_mode, sc.band),
                            (sc.u, 2, vel_band), (sc.v, 2, vel_band)):
        a, b, _, _ = oracle.ref_densify_compare(arr, mode, band)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    # the narrow band leaves filled and background cells on both sides
    if kind.startswith("liquid"):
        a, _, _, _ = oracle.ref_densify_compare(sc.fluid, 0, sc.band)
        assert (a == -np.float32(sc.band)).any() and (a == np.float32(sc.band)).any()
