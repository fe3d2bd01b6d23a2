"""The allocation-free projection (gbp_project_device_static) against
gbp_project_device (GPU test).

gbp_project_device_static serves callers that cannot call cudaMalloc -- a
host whose device memory comes from its own allocator or a fixed pool, a
plugin in a process that forbids more device allocations, a per-step path
that must never reach the allocator. It keeps its scratch in one static
device array instead of allocating. Called twice in a row through the C ABI,
it must give the same projection as gbp_project_device (the plain FP64 CG
path) within the tolerances the parity tests use, and it must refuse grids
beyond its stated maximum with a clear error instead of touching memory.

This file is collected last so that a run stopping at its first failure has
already run every other test; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

PRESSURE_RTOL = 1e-5      # as in test_gpu_parity.py
VELOCITY_RTOL = 1e-5


def _lib():
    import shiokaze_gb300 as gb
    lib = gb.load_library()
    vp = ctypes.c_void_p
    fn = lib.gbp_project_device_static
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                   vp, vp, vp, vp, vp, ctypes.POINTER(gb.Params), vp, ctypes.POINTER(gb.Stats), vp]
    fn.restype = ctypes.c_int
    return gb, lib, fn


def _rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-30)


@pytest.mark.parametrize("make", [lambda: scenes.liquid3((24, 20, 18), seed=2),
                                  lambda: scenes.smoke3(16, seed=3),
                                  lambda: scenes.liquid2((64, 48), seed=1)])
def test_static_matches_device_entry_point_twice(make):
    import torch
    gb, lib, static = _lib()
    sc = make()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    solid, fluid = t(sc.solid), t(sc.fluid)
    vel0 = [t(a) for a in (sc.u, sc.v, sc.w) if a is not None]

    # the existing entry point (plain FP64 CG, device arrays)
    pj = gb.projector_for(sc, Residual=1e-6)
    ref_vel = [c.clone() for c in vel0]
    ref_p = torch.zeros(sc.fluid.shape, dtype=torch.float32, device=dev)
    assert pj.project(sc.dt, tuple(ref_vel), solid, fluid, pressure_out=ref_p) == gb.GBP_OK
    torch.cuda.synchronize()
    ref_iters = pj.stats.iterations

    params = gb.make_params(Residual=1e-6)
    for call in range(2):
        vel = [c.clone() for c in vel0]
        p = torch.full(sc.fluid.shape, float("nan"), dtype=torch.float32, device=dev)
        st = gb.Stats()
        torch.cuda.synchronize()
        rc = static(sc.dim, sc.nx, sc.ny, sc.nz, sc.dx, sc.dt, solid.data_ptr(), fluid.data_ptr(),
                    vel[0].data_ptr(), vel[1].data_ptr(), vel[2].data_ptr() if sc.dim == 3 else None,
                    ctypes.byref(params), p.data_ptr(), ctypes.byref(st), ctypes.c_void_p(stream.cuda_stream))
        assert rc == gb.GBP_OK, lib.gbp_strerror(rc)
        torch.cuda.synchronize()
        assert _rel(p, ref_p) <= PRESSURE_RTOL, (call, _rel(p, ref_p))
        for got, want in zip(vel, ref_vel):
            assert _rel(got, want) <= VELOCITY_RTOL, call
        assert st.iterations == ref_iters
        assert st.unknowns == pj.stats.unknowns
    pj.close()


def test_static_rejects_grids_beyond_its_maximum():
    import torch
    gb, lib, static = _lib()
    n = 33  # 33^3 = 35937 cells > 32768
    dev = torch.device("cuda", 0)
    dummy = torch.zeros(8, dtype=torch.float32, device=dev)
    ptr = dummy.data_ptr()
    rc = static(3, n, n, n, 1.0 / n, 1.0 / 60, ptr, ptr, ptr, ptr, ptr, None, ptr, None, None)
    assert rc == 1  # GBP_ERR_INVALID_ARGUMENT
    msg = lib.gbp_strerror(rc).decode()
    assert "static scratch limit of 32768 cells" in msg, msg
