"""Bounded device waits (GPU test).

Two kinds of kernel wait on other work: the cooperative coarse-level kernels
at their grid-wide barriers, and the TMA-staged fine-level kernels on the
mbarrier of each tile's copies. Every such wait polls a bounded number of
times; one that runs out records the failure in device memory, the kernel
returns, and the solve returns GBP_ERR_CUDA with a message naming the wait,
leaving the context usable.

gbp_debug_fail_wait makes that happen without a fault: in the scene's next
solve one block leaves out its barrier arrival (or the copies of its first
tile), as a block that stopped would, so the other waits find nothing to
wait for; a short poll limit keeps the test fast. The solve after it must
run normally and give the same result, bit for bit, as a solve on a fresh
scene.
"""
import ctypes

import numpy as np
import pytest

from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

GBP_WAIT_GRID_BARRIER = 1
GBP_WAIT_TILE = 2


def _solve(gb, pj, sc):
    vel = (sc.u.copy(), sc.v.copy(), sc.w.copy())
    rc = pj.project(sc.dt, vel, sc.solid, sc.fluid)
    return rc, pj.get_pressure().copy(), vel


@pytest.mark.parametrize("what,staging,message", [
    (GBP_WAIT_GRID_BARRIER, 0, "grid barrier wait ran out"),
    (GBP_WAIT_TILE, 1, "tile wait ran out"),
])
def test_wait_runs_out_and_the_next_solve_is_normal(what, staging, message):
    import shiokaze_gb300 as gb
    lib = gb.load_library()
    lib.gbp_debug_fail_wait.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    # 128^3: the fine level qualifies for TMA staging and the 64^3 and 32^3
    # levels run in the cooperative kernels
    sc = scenes.smoke3(128, seed=3)
    cfg = dict(Residual=1e-6, Solver="mgpcg", Precision="mixed", TMAStaging=staging)

    fresh = gb.projector_for(sc, **cfg)
    rc, p_ref, v_ref = _solve(gb, fresh, sc)
    assert rc == gb.GBP_OK
    if staging:
        assert fresh.stats.tma_staged == 1
    fresh.close()

    pj = gb.projector_for(sc, **cfg)
    assert lib.gbp_debug_fail_wait(pj.scene, what, 0, 256) == gb.GBP_OK
    with pytest.raises(gb.GBPError) as err:
        _solve(gb, pj, sc)
    assert err.value.code == gb.GBP_ERR_CUDA
    assert message in str(err.value), str(err.value)

    rc, p, vel = _solve(gb, pj, sc)
    assert rc == gb.GBP_OK
    assert pj.stats.true_resid_inf <= 1.01e-6
    assert np.array_equal(p.view(np.uint32), p_ref.view(np.uint32))
    for a, b in zip(vel, v_ref):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    pj.close()


def test_fail_wait_rejects_bad_arguments():
    import shiokaze_gb300 as gb
    lib = gb.load_library()
    lib.gbp_debug_fail_wait.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    sc = scenes.smoke3(8, seed=3)
    pj = gb.projector_for(sc, Solver="mgpcg")
    for what, block, polls in ((0, 0, 10), (3, 0, 10), (1, -1, 10), (1, 0, 0), (2, 0, (1 << 24) + 1)):
        assert lib.gbp_debug_fail_wait(pj.scene, what, block, polls) == gb.GBP_ERR_INVALID_ARGUMENT
    assert lib.gbp_debug_fail_wait(None, 1, 0, 10) == gb.GBP_ERR_INVALID_ARGUMENT
    pj.close()
