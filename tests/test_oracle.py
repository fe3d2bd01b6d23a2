"""The oracle itself: the C restatement against the reference's own outputs.

The golden fixtures were produced by the reference's macpressuresolver{2,3}
built from its sources (tests/golden/make_golden.py). The restatement must
reproduce them bit for bit: pressure, projected velocity, the set of unknown
cells, the faces left active and the CG iteration count.
"""
import os

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
    for a, b in zip(res.active, c.out_active):
        assert np.array_equal(a, b)
    if c.dim == 3:
        assert np.array_equal(res.w, c.out_w)
        assert res.iterations == c.iterations


def test_fixtures_deactivate_closed_faces():
    """The reference's velocity update turns closed faces off
    (macpressuresolver3.cpp:264-266): in a liquid scene the faces in the air
    are inactive after the projection, and every inactive face reads 0; in
    2D a closed wall face stays active only where the flow leaves the domain
    (macpressuresolver2.cpp:233-235)."""
    c = Case("liquid3_16")
    assert all((~a).sum() > a.size // 3 for a in c.out_active)
    for a, u in zip(c.out_active, (c.out_u, c.out_v, c.out_w)):
        assert not u[~a].any()
    c = Case("liquid2_32")
    on_wall = c.out_active[0][:, 0]
    assert on_wall.any() and not on_wall.all()


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
    oracle.build_modules(oracle.REF_DIR)
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
    oracle.build_modules(oracle.REF_DIR)
    lib = oracle._ref_lib()
    for dim in (3, 2):
        log = str(tmp_path / f"lin{dim}.log")
        h = lib.ref_create(dim, 16, 16, 16, 1 / 16, b"LinSolver=gbpcg Residual=1e-6", log.encode())
        assert h
        text = open(log).read()
        assert "gbpcg" in text and "pcg.so" not in text.replace("gbpcg.so", "")
        lib.ref_destroy(h)


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("kind,n", [("liquid3", 48), ("liquid3", (40, 33, 37)), ("smoke3", 40), ("liquid3", 64)])
def test_module_bricks_match_operator_reads(kind, n):
    """The plugin modules' bricks of the reference's tiled arrays
    (gbarray_adapter.h to_bricks: listed bricks where a cell is active or
    some cells are filled, whole-fill and background bricks by kind),
    expanded by gbp.h's rule, equal reading every cell through the
    reference's operator() bit for bit; a narrow-band level set lists only
    a fraction of its bricks (its filled interior travels as fill bricks)."""
    sc = getattr(scenes, kind)(n, seed=5)
    vel_band = float(np.quantile(np.abs(sc.u), 0.4))
    for arr, mode, band in ((sc.solid, sc.solid_mode, sc.band), (sc.fluid, sc.fluid_mode, sc.band),
                            (sc.u, 2, vel_band), (sc.w, 2, vel_band)):
        a, b, counts, _, _, _, _ = oracle.ref_bricks_compare(arr, mode, band)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    if kind == "liquid3":
        _, _, counts, _, _, _, _ = oracle.ref_bricks_compare(sc.fluid, sc.fluid_mode, sc.band)
        assert counts[1] > 0 and counts[2] > 0 and counts[0] < 0.6 * counts.sum(), counts


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


def test_advection_module_loads_through_reference_loader(tmp_path):
    """The advection drop-in: the reference's loader picks gbadvection3 by
    the Advection key (macadvection3_interface.h:39) in place of
    macadvection3, configures (MacCormack, TrimNarrowBand) and initializes
    it. (Advecting needs a GPU.)"""
    import subprocess
    if not oracle.reference_available():
        pytest.skip("reference oracle not built here")
    root = oracle.HERE.rsplit("/", 1)[0]
    oracle.build_modules(oracle.REF_DIR)
    lib = oracle._ref_lib()
    log = str(tmp_path / "adv.log")
    assert lib.ref_advect_load(16, 16, 16, 1 / 16, b"Advection=gbadvection3 MacCormack=Yes TrimNarrowBand=2",
                               log.encode()) == 1
    text = open(log).read()
    assert "gbadvection3.so" in text and "macadvection3.so" not in text


def advect_module_cases():
    for seed in (41, 42, 43, 44):
        rng = np.random.default_rng(seed)
        n = tuple(int(x) for x in rng.integers(6, 20, 3))
        sc = (scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5))) if seed % 2
              else scenes.smoke3(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
        m = (rng.random(sc.fluid.shape) > 0.4).astype(np.uint8) if seed != 42 else None
        q = rng.random(sc.fluid.shape, dtype=np.float32)
        if m is not None:
            q = np.where(m != 0, q, np.float32(0.25)).astype(np.float32)
        kw = dict(q=q, q_mask=m, q_bg=0.25 if m is not None else 0.0, maccormack=seed != 43,
                  trim_narrowband=int(rng.integers(0, 3)))
        yield seed, sc, kw


# runs in a process of its own: the reference's loader, which unloads its
# modules at exit, faults at exit when a second advection module (even one
# that does nothing) was loaded after macadvection3 had run in the process
ADVECT_MODULE_RUN = r"""
import sys
import numpy as np
import oracle
sys.path.insert(0, "tests")
from test_oracle import advect_module_cases
out = {}
for seed, sc, kw in advect_module_cases():
    r = oracle.ref_advect3(sc.u, sc.v, sc.w, sc.fluid, sc.fluid_mode, sc.band, sc.dx, sc.dt,
                           extra_kv="Advection=gbadvection3stub", **kw)
    for name, a in zip("uvwq", r[:4]):
        out[f"{seed}_{name}"] = a
np.savez(sys.argv[1], **out)
"""


def test_advection_module_boundary_matches_reference_module(tmp_path):
    """The gbadvection3 module's boundary on the CPU: linked against a
    stand-in for libgbp that runs the oracle (tests/module_stub), loaded by
    the reference's own loader in place of macadvection3 on the reference's
    own tiled arrays (narrow-band liquid level sets, masked densities, every
    velocity face active), it gives the reference module's results bit for
    bit: the dense copies, the active mask, dt and the write-back are right."""
    import os
    import shutil
    import subprocess
    import sys
    if not oracle.reference_available():
        pytest.skip("reference oracle not built here")
    root = oracle.HERE.rsplit("/", 1)[0]
    oracle.build_port()
    stub = tmp_path / "libgbp.so"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-I", f"{root}/include",
                           f"{root}/tests/module_stub/gbp_oracle_stub.c", "-o", str(stub), oracle.PORT_SO,
                           f"-Wl,-rpath,{oracle.HERE}"])
    oracle.build_modules(str(tmp_path), f"{tmp_path}/libshiokaze_gbadvection3.so",
                         ldflags=f"-shared -L{tmp_path} -lgbp -Wl,-rpath,{tmp_path}")
    shutil.copy(tmp_path / "libshiokaze_gbadvection3.so", os.path.join(oracle.REF_DIR,
                                                                      "libshiokaze_gbadvection3stub.so"))
    out = tmp_path / "module.npz"
    r = subprocess.run([sys.executable, "-c", ADVECT_MODULE_RUN, str(out)], cwd=root, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = dict(np.load(out))
    for seed, sc, kw in advect_module_cases():
        want = oracle.ref_advect3(sc.u, sc.v, sc.w, sc.fluid, sc.fluid_mode, sc.band, sc.dx, sc.dt, **kw)
        for name, a in zip("uvwq", want[:4]):
            b = got[f"{seed}_{name}"]
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (seed, name)


def advect2_module_cases():
    for seed in (51, 52, 53, 54):
        rng = np.random.default_rng(seed)
        n = tuple(int(x) for x in rng.integers(6, 48, 2))
        sc = (scenes.liquid2(n, seed=seed, noise=float(rng.uniform(0.2, 3.0))) if seed % 2
              else scenes.smoke2(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
        fl = sc.fluid[0]
        m = (rng.random(fl.shape) > 0.4).astype(np.uint8) if seed != 52 else None
        q = rng.random(fl.shape, dtype=np.float32)
        if m is not None:
            q = np.where(m != 0, q, np.float32(0.25)).astype(np.float32)
        kw = dict(q=q, q_mask=m, q_bg=0.25 if m is not None else 0.0, maccormack=seed != 53,
                  trim_narrowband=int(rng.integers(0, 3)))
        yield seed, sc, kw


ADVECT2_MODULE_RUN = r"""
import sys
import numpy as np
import oracle
sys.path.insert(0, "tests")
from test_oracle import advect2_module_cases
out = {}
for seed, sc, kw in advect2_module_cases():
    r = oracle.advect2(sc.u[0], sc.v[0], sc.fluid[0], sc.dx, sc.dt, impl="reference", fluid_mode=sc.fluid_mode,
                       band=sc.band, extra_kv="Advection=gbadvection2stub", **kw)
    for name, a in zip("uvq", r[:3]):
        out[f"{seed}_{name}"] = a
np.savez(sys.argv[1], **out)
"""


def test_advection2_module_boundary_matches_reference_module(tmp_path):
    """The gbadvection2 module (Advection=gbadvection2) on the CPU: linked
    to the oracle-backed stand-in for libgbp and loaded by the reference's
    loader in place of macadvection2, on the reference's own 2D tiled arrays,
    it gives the reference module's results bit for bit."""
    import subprocess
    import sys
    if not oracle.reference_available():
        pytest.skip("reference oracle not built here")
    root = _stub_module(tmp_path, "gbadvection2", "gbadvection2stub")
    out = tmp_path / "module2.npz"
    r = subprocess.run([sys.executable, "-c", ADVECT2_MODULE_RUN, str(out)], cwd=root, capture_output=True,
                       text=True, timeout=300, env=dict(os.environ, PYTHONPATH=root))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = dict(np.load(out))
    for seed, sc, kw in advect2_module_cases():
        want = oracle.advect2(sc.u[0], sc.v[0], sc.fluid[0], sc.dx, sc.dt, impl="reference",
                              fluid_mode=sc.fluid_mode, band=sc.band, **kw)
        for name, a in zip("uvq", want[:3]):
            b = got[f"{seed}_{name}"]
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (seed, name)


def _stub_module(tmp_path, module, installed_as):
    """Builds plugin module `module` linked against the oracle-backed
    stand-in for libgbp (tests/module_stub) and installs it beside the
    reference's modules as libshiokaze_<installed_as>.so."""
    import shutil
    import subprocess
    root = oracle.HERE.rsplit("/", 1)[0]
    oracle.build_port()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-I", f"{root}/include",
                           f"{root}/tests/module_stub/gbp_oracle_stub.c", "-o", str(tmp_path / "libgbp.so"),
                           oracle.PORT_SO, f"-Wl,-rpath,{oracle.HERE}"])
    oracle.build_modules(str(tmp_path), f"{tmp_path}/libshiokaze_{module}.so",
                         ldflags=f"-shared -L{tmp_path} -lgbp -Wl,-rpath,{tmp_path}")
    shutil.copy(tmp_path / f"libshiokaze_{module}.so", os.path.join(oracle.REF_DIR, f"libshiokaze_{installed_as}.so"))
    return root


UTILITY_MODULE_RUN = r"""
import glob, os, sys
import numpy as np
import oracle
out = {}
for p in sorted(glob.glob("tests/golden/constrain/*.npz")):
    d = dict(np.load(p))
    name = os.path.basename(p)[:-4]
    r = oracle.constrain3(d["solid"], d["u"], d["v"], d["w"], float(d["dx"]), masks=(d["mu"], d["mv"], d["mw"]),
                          impl="reference", solid_mode=int(d["solid_mode"]), band=float(d["band"]),
                          extra_kv="MacUtility=gbutility3stub")
    for c, a in zip("uvw", r):
        out[f"{name}_{c}"] = a
np.savez(sys.argv[1], **out)
"""


def test_utility_module_constrain_matches_reference_module(tmp_path):
    """The gbutility3 module (MacUtility=gbutility3) on the CPU: linked to
    the oracle-backed stand-in for libgbp and loaded by the reference's
    loader in place of macutility3, its constrain_velocity gives the
    reference module's results bit for bit on the reference's own arrays
    (the constraint fixtures: narrow-band solids, masked velocities)."""
    import subprocess
    import sys
    if not oracle.reference_available():
        pytest.skip("reference oracle not built here")
    root = _stub_module(tmp_path, "gbutility3", "gbutility3stub")
    out = tmp_path / "utility.npz"
    r = subprocess.run([sys.executable, "-c", UTILITY_MODULE_RUN, str(out)], cwd=root, capture_output=True, text=True,
                       timeout=300, env=dict(os.environ, PYTHONPATH=root))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = dict(np.load(out))
    import glob
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(root, "tests/golden/constrain/*.npz")))
    assert len(names) >= 5
    for name in names:
        d = dict(np.load(os.path.join(root, "tests/golden/constrain", name + ".npz")))
        for c in "uvw":
            assert np.array_equal(got[f"{name}_{c}"].view(np.uint32), d[f"out_{c}"].view(np.uint32)), (name, c)


# runs in a process of its own, like the other module checks: the
# replacement projection module is loaded by the reference's loader beside
# the reference's own modules
PROJECTION_MODULE_RUN = r"""
import json, sys
import numpy as np
import oracle
sys.path.insert(0, "tests")
from golden_io import Case, case_names
out = {}
for name in case_names():
    c = Case(name)
    d = np.load(f"tests/golden/{name}.npz")
    params = dict(c.params)
    volume = params.pop("volume", None)
    pj = oracle.RefProjector(c.dim, c.nx, c.ny, c.nz, c.dx, extra_kv=f"Projection=gbprojection{c.dim}stub", **params)
    for s in range(c.steps):
        u, v, w = c.inputs[s]
        if c.volume is not None:
            pj.set_target_volume(*c.volume[s])
        r = pj.project(c.dt, c.solid, c.fluid, u, v, w, int(d["solid_mode"]), int(d["fluid_mode"]),
                       float(d["band"]))
    pj.close()
    out[f"{name}/pressure"] = r.pressure
    out[f"{name}/unknown"] = r.unknown
    for comp, a, on in zip("uvw", (r.u, r.v, r.w), r.active):
        out[f"{name}/{comp}"] = a
        out[f"{name}/{comp}_on"] = on
np.savez(sys.argv[1], **out)
"""


def test_projection_modules_match_reference_modules(tmp_path):
    """gbprojection3 / gbprojection2 (Projection=gbprojection3|2) at their
    boundary, on the CPU: linked to the oracle-backed stand-in for libgbp
    and loaded by the reference's loader in place of macpressuresolver3 / 2
    on the reference's own tiled arrays, they leave the reference modules'
    output state on every golden case, bit for bit: the velocity values,
    which faces stay active (the closed faces are set_off,
    macpressuresolver3.cpp:264-266, 2D macpressuresolver2.cpp:233-235), the
    pressure values and its active cells (every unknown, :245-248), over
    warm-started and volume-corrected steps too."""
    import subprocess
    import sys
    if not oracle.reference_available():
        pytest.skip("reference oracle not built here")
    root = _stub_module(tmp_path, "gbprojection3", "gbprojection3stub")
    _stub_module(tmp_path, "gbprojection2", "gbprojection2stub")
    out = tmp_path / "projection.npz"
    r = subprocess.run([sys.executable, "-c", PROJECTION_MODULE_RUN, str(out)], cwd=root, capture_output=True,
                       text=True, timeout=600, env=dict(os.environ, PYTHONPATH=root))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = dict(np.load(out))
    names = case_names()
    assert len(names) >= 15
    for name in names:
        c = Case(name)
        assert np.array_equal(got[f"{name}/unknown"], c.out_unknown), name
        assert np.array_equal(got[f"{name}/pressure"].view(np.uint32), c.out_pressure.view(np.uint32)), name
        for comp, want, on in zip("uvw", (c.out_u, c.out_v, c.out_w), c.out_active):
            assert np.array_equal(got[f"{name}/{comp}"].view(np.uint32), want.view(np.uint32)), (name, comp)
            assert np.array_equal(got[f"{name}/{comp}_on"], on), (name, comp)


def extrapolate_module_cases():
    """Seeded liquid scenes with partly active velocities (inactive faces 0),
    one without a solid level set (only the extrapolation acts)."""
    for seed in (81, 82, 83, 84):
        rng = np.random.default_rng(seed)
        n = tuple(int(x) for x in rng.integers(8, 20, 3))
        sc = scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5)))
        if seed == 84:
            sc.solid[...] = np.float32(sc.band)
        masks, comps = [], []
        for a in (sc.u, sc.v, sc.w):
            m = (rng.random(a.shape) < rng.uniform(0.2, 0.7)).astype(np.uint8)
            masks.append(m)
            comps.append(np.where(m != 0, a, 0).astype(np.float32))
        yield seed, sc, comps, masks, int(rng.integers(1, 4))


EXTRAPOLATE_MODULE_RUN = r"""
import sys
import numpy as np
import oracle
sys.path.insert(0, "tests")
from test_oracle import extrapolate_module_cases
out = {}
for seed, sc, comps, masks, width in extrapolate_module_cases():
    r = oracle.extrapolate_constrain3(sc.solid, *comps, sc.dx, masks, width, impl="reference",
                                      solid_mode=sc.solid_mode, band=sc.band, extra_kv="MacUtility=gbutility3stub")
    for c, a, m in zip("uvw", r[:3], r[3]):
        out[f"{seed}_{c}"] = a
        out[f"{seed}_{c}_on"] = m
np.savez(sys.argv[1], **out)
"""


def test_utility_module_extrapolate_constrain_matches_reference_module(tmp_path):
    """gbutility3's extrapolate_and_constrain_velocity (the velocity grown
    over its inactive faces, then constrained; macutility3.cpp:88-92) on
    the CPU: linked to the oracle-backed stand-in for libgbp and loaded by
    the reference's loader in place of macutility3, it leaves the reference
    module's velocity values and active faces bit for bit on the
    reference's own arrays, with and without a solid level set."""
    import subprocess
    import sys
    if not oracle.reference_available():
        pytest.skip("reference oracle not built here")
    root = _stub_module(tmp_path, "gbutility3", "gbutility3stub")
    out = tmp_path / "extrapolate.npz"
    r = subprocess.run([sys.executable, "-c", EXTRAPOLATE_MODULE_RUN, str(out)], cwd=root, capture_output=True,
                       text=True, timeout=300, env=dict(os.environ, PYTHONPATH=root))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    got = dict(np.load(out))
    grew = 0
    for seed, sc, comps, masks, width in extrapolate_module_cases():
        want = oracle.extrapolate_constrain3(sc.solid, *comps, sc.dx, masks, width, impl="reference",
                                             solid_mode=sc.solid_mode, band=sc.band)
        for c, a, m, m0 in zip("uvw", want[:3], want[3], masks):
            assert np.array_equal(got[f"{seed}_{c}"].view(np.uint32), a.view(np.uint32)), (seed, c)
            assert np.array_equal(got[f"{seed}_{c}_on"], m), (seed, c)
            grew += int(m.sum()) - int(m0.sum())
    assert grew > 0


def test_extrapolate_constrain_port_matches_live_reference():
    """The oracle's composition (oracle_extrapolate3 per component, then
    oracle_constrain_velocity3) equals the reference's
    extrapolate_and_constrain_velocity bit for bit, active sets included."""
    if not oracle.reference_available():
        pytest.skip("reference oracle not built here")
    for seed, sc, comps, masks, width in extrapolate_module_cases():
        a = oracle.extrapolate_constrain3(sc.solid, *comps, sc.dx, masks, width)
        b = oracle.extrapolate_constrain3(sc.solid, *comps, sc.dx, masks, width, impl="reference",
                                          solid_mode=sc.solid_mode, band=sc.band)
        for x, y in zip(a[:3], b[:3]):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), seed
        for x, y in zip(a[3], b[3]):
            assert np.array_equal(x, y), seed
