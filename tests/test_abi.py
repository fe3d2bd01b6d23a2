"""The C ABI without a GPU: the library is built for sm_103a, loads, and
exports every function include/gbp.h declares; host-only calls behave."""
import ctypes
import os
import re

import pytest

import shiokaze_gb300 as gb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(gbp_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(gb.LIB_PATH):
        from shiokaze_gb300 import build
        build.build()
    return gb.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "gbp_project" in names and "gbp_project_device" in names
    for n in names:
        assert hasattr(lib, n), n


def test_library_targets_sm103a():
    from shiokaze_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_params_default_matches_reference_defaults(lib):
    p = gb.Params()
    lib.gbp_params_default(ctypes.byref(p))
    # src/linsolver/pcg.cpp:76-77, macpressuresolver3.cpp:296-305, macutility3.cpp:424-425
    assert p.residual == 1e-4 and p.max_iterations == 30000
    assert p.eps_fluid == 1e-2 and p.eps_solid == 1e-2
    assert p.second_order_fluid == 1 and p.second_order_solid == 1
    assert p.warm_start == 0 and p.gain == 1.0


def test_config_keys(lib):
    p = gb.make_params(Residual=1e-6, WarmStart="Yes", Solver="mgpcg", Precision="mixed")
    assert p.residual == 1e-6 and p.warm_start == 1
    assert p.solver == gb.SOLVER_MGPCG and p.precision == gb.PRECISION_MIXED
    with pytest.raises(KeyError):
        gb.make_params(NoSuchKey=1)
    # values read from a configuration file arrive as strings: integer keys
    # parse as numbers, boolean keys as yes/no
    p = gb.make_params(MGSmooth="2", MGCoarsest="8", MaxIterations="500", TileClasses="No",
                       SecondOrderAccurateFluid="false", TMAStaging=True)
    assert p.mg_smooth == 2 and p.mg_coarsest == 8 and p.max_iterations == 500
    assert p.tile_classes == 0 and p.second_order_fluid == 0 and p.tma_staging == 1
    with pytest.raises(ValueError):
        gb.make_params(WarmStart="maybe")


def test_strerror_and_bytes(lib):
    assert lib.gbp_strerror(0) == b"ok"
    assert b"max_iterations" in lib.gbp_strerror(4)
    n = lib.gbp_scene_device_bytes(3, 64, 64, 64, None)
    assert n > 64 ** 3 * 8 * 9


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    rc = lib.gbp_create(0, ctypes.byref(h))
    assert rc == 6 and not h  # GBP_ERR_NO_DEVICE


def test_advect_params_default_matches_reference_defaults(lib):
    p = gb.AdvectParams()
    lib.gbp_advect_params_default(ctypes.byref(p))
    # src/advection/macadvection3.cpp:284-288: MacCormack on, TrimNarrowBand 1
    assert p.maccormack == 1 and p.trim_narrowband == 1 and p.advect_velocity == 1
