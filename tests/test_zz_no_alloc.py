"""The allocation-free projection (gbp_project_device_static) against
gbp_project_device and the oracle (GPU test).

gbp_project_device_static serves callers that cannot call cudaMalloc -- a
host whose device memory comes from its own allocator or a fixed pool, a
plugin in a process that forbids more device allocations, a per-step path
that must never reach the allocator. It keeps its scratch in one static
device array instead of allocating. Called through the C ABI, several times
in a row and with grids of different sizes sharing that array, it must give
the projection of gbp_project_device's plain FP64 CG path bit for bit (both
run the same CG kernels on the same grid of blocks, and both assemblies and
velocity updates are bit-exact with the reference), agree with the oracle
within the tolerances of the parity tests, leave the device's free memory
unchanged, and refuse grids beyond its stated maximum with a clear error
instead of touching memory.

This file is collected last so that a run stopping at its first failure has
already run every other test; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

import oracle
from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

PRESSURE_RTOL = 1e-5      # against the oracle, as in test_gpu_parity.py
VELOCITY_RTOL = 1e-5
MAX_CELLS = 32768         # GBP_STATIC_MAX_CELLS


def _lib():
    import shiokaze_gb300 as gb
    lib = gb.load_library()
    vp = ctypes.c_void_p
    fn = lib.gbp_project_device_static
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                   vp, vp, vp, vp, vp, ctypes.POINTER(gb.Params), vp, ctypes.POINTER(gb.Stats), vp]
    fn.restype = ctypes.c_int
    return gb, lib, fn


def _bits(t):
    return t.cpu().numpy().view(np.uint32)


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-30)


class _Case:
    """One scene on the device, its gbp_project_device result and the
    oracle's projection of it."""

    def __init__(self, gb, sc):
        import torch
        self.sc = sc
        self.dev = torch.device("cuda", 0)

        def t(a):
            return torch.from_numpy(np.ascontiguousarray(a)).to(self.dev)

        self.solid, self.fluid = t(sc.solid), t(sc.fluid)
        self.vel0 = [t(a) for a in (sc.u, sc.v, sc.w) if a is not None]
        pj = gb.projector_for(sc, Residual=1e-6)
        self.ref_vel = [c.clone() for c in self.vel0]
        self.ref_p = torch.zeros(sc.fluid.shape, dtype=torch.float32, device=self.dev)
        assert pj.project(sc.dt, tuple(self.ref_vel), self.solid, self.fluid, pressure_out=self.ref_p) == gb.GBP_OK
        torch.cuda.synchronize()
        self.ref_iters = pj.stats.iterations
        self.ref_unknowns = pj.stats.unknowns
        pj.close()
        self.want = oracle.project_scene(sc, "port", residual=1e-6)

    def run_static(self, gb, lib, static, out=None):
        """One call; `out` = (p, vel) device buffers to reuse (no new device
        memory from this side either), else fresh ones."""
        import torch
        sc = self.sc
        if out is None:
            vel = [c.clone() for c in self.vel0]
            p = torch.empty(sc.fluid.shape, dtype=torch.float32, device=self.dev)
        else:
            p, vel = out
            for c, c0 in zip(vel, self.vel0):
                c.copy_(c0)
        p.fill_(float("nan"))
        st = gb.Stats()
        params = gb.make_params(Residual=1e-6)
        stream = torch.cuda.current_stream(self.dev)
        torch.cuda.synchronize()
        rc = static(sc.dim, sc.nx, sc.ny, sc.nz, sc.dx, sc.dt, self.solid.data_ptr(), self.fluid.data_ptr(),
                    vel[0].data_ptr(), vel[1].data_ptr(), vel[2].data_ptr() if sc.dim == 3 else None,
                    ctypes.byref(params), p.data_ptr(), ctypes.byref(st), ctypes.c_void_p(stream.cuda_stream))
        assert rc == gb.GBP_OK, lib.gbp_strerror(rc)
        torch.cuda.synchronize()
        return p, vel, st

    def check(self, p, vel, st, what):
        # the same projection as gbp_project_device, bit for bit
        assert np.array_equal(_bits(p), _bits(self.ref_p)), what
        for got, want in zip(vel, self.ref_vel):
            assert np.array_equal(_bits(got), _bits(want)), what
        assert st.iterations == self.ref_iters and st.unknowns == self.ref_unknowns, what
        # and the reference's result, as the parity tests bound it
        w = self.want
        assert st.unknowns == int(w.unknown.sum()), what
        assert _rel(p.cpu().numpy(), w.pressure) <= PRESSURE_RTOL, (what, _rel(p.cpu().numpy(), w.pressure))
        for got, ref in zip(vel, (w.u, w.v, w.w)):
            assert _rel(got.cpu().numpy(), ref) <= VELOCITY_RTOL, what


@pytest.mark.parametrize("make", [lambda: scenes.liquid3((24, 20, 18), seed=2),
                                  lambda: scenes.smoke3(16, seed=3),
                                  lambda: scenes.liquid2((64, 48), seed=1)])
def test_static_matches_device_entry_point_twice(make):
    gb, lib, static = _lib()
    case = _Case(gb, make())
    for call in range(2):
        case.check(*case.run_static(gb, lib, static), f"call {call}")


def test_static_at_its_maximum_then_smaller_grids():
    """A grid of exactly GBP_STATIC_MAX_CELLS cells (32^3), then smaller ones
    on the same static array, which still holds the larger call's values,
    then the largest again: every call equals gbp_project_device and the
    oracle."""
    gb, lib, static = _lib()
    big = _Case(gb, scenes.liquid3(32, seed=5))
    assert big.sc.cells == MAX_CELLS
    small3 = _Case(gb, scenes.liquid3((13, 11, 9), seed=6))
    small2 = _Case(gb, scenes.liquid2((40, 24), seed=9))
    for case, what in ((big, "32^3"), (small3, "13x11x9 after 32^3"), (small2, "2D 40x24 after 3D"),
                       (big, "32^3 again")):
        case.check(*case.run_static(gb, lib, static), what)


def test_static_allocates_no_device_memory():
    """After a first call (which loads the library's module on the device),
    further calls leave the device's free memory exactly as it was."""
    import torch
    gb, lib, static = _lib()
    case = _Case(gb, scenes.liquid3((24, 20, 18), seed=2))
    p, vel, st = case.run_static(gb, lib, static)
    case.check(p, vel, st, "first call")
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        # the output buffers are reused: torch's allocator stays idle too
        case.check(*case.run_static(gb, lib, static, out=(p, vel)), "no-alloc call")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


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
