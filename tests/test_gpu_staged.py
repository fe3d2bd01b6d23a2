"""TMA-staged fine-level kernels (FP32 MGPCG) against the direct-load kernels.

A fine level is staged (TMAStaging=1; the default, 0, uses the direct-load
kernels) when it is 3D with 4-plane tiles (2^21 cells or more) and nx is
a multiple of 8. The staged kernels compute each cell with the same
arithmetic as the direct-load ones; a solve differs only through
the grouping of its dot-product partials (the staged launch runs one block
per SM), so the two solves agree to the last digits and take the same
number of iterations.
"""
import numpy as np
import pytest

from gpu_util import rel_inf

pytestmark = pytest.mark.gpu


def _solve(sc, **cfg):
    import shiokaze_gb300 as gb
    pj = gb.projector_for(sc, Residual=1e-6, Solver="mgpcg", Precision="mixed", **cfg)
    u, v, w = (a.copy() for a in (sc.u, sc.v, sc.w))
    rc = pj.project(sc.dt, (u, v, w), sc.solid, sc.fluid)
    out = (rc, pj.get_pressure().copy(), (u, v, w), pj.stats.as_dict())
    pj.close()
    return out


@pytest.mark.parametrize("kind", ["liquid", "smoke"])
def test_staged_matches_direct_loads(kind):
    import shiokaze_gb300 as gb
    from shiokaze_gb300 import scenes
    shape = (136, 128, 128)  # 2.2M cells: 4-plane tiles; nx % 8 == 0
    sc = scenes.liquid3(shape, seed=31) if kind == "liquid" else scenes.smoke3(shape, seed=32)
    rc1, p1, v1, st1 = _solve(sc, TMAStaging=1)
    rc0, p0, v0, st0 = _solve(sc, TMAStaging=0)
    assert rc1 == gb.GBP_OK and rc0 == gb.GBP_OK
    assert st1["tma_staged"] == 1 and st0["tma_staged"] == 0
    assert abs(st1["iterations"] - st0["iterations"]) <= 1
    if kind == "smoke":  # pressure up to a constant
        p1 = p1 - p1.mean()
        p0 = p0 - p0.mean()
    assert rel_inf(p1, p0) < 1e-5
    for a, b in zip(v1, v0):
        assert rel_inf(a, b) < 1e-5
    assert st1["true_resid_inf"] <= 1e-6 and st0["true_resid_inf"] <= 1e-6


def test_staged_not_used_where_grid_disallows():
    from shiokaze_gb300 import scenes
    # nx not a multiple of 8: the direct-load kernels run
    sc = scenes.liquid3((132, 128, 128), seed=33)
    rc, _, _, st = _solve(sc, TMAStaging=1)
    assert st["tma_staged"] == 0
    assert st["true_resid_inf"] <= 1e-6


def test_batch_mixing_staged_and_plain_scenes():
    import torch
    import shiokaze_gb300 as gb
    from shiokaze_gb300 import scenes
    big = scenes.liquid3((136, 128, 128), seed=34)
    small = scenes.liquid3(48, seed=35)
    cfg = dict(Residual=1e-6, Solver="mgpcg", Precision="mixed", TMAStaging=1)
    dev = torch.device("cuda", 0)

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    ctx = gb.Context(0)
    pjs = [gb.projector_for(s, ctx, **cfg) for s in (big, small)]
    batch = gb.Batch(pjs, ctx, **cfg)
    vels = [tuple(d(a) for a in (s.u, s.v, s.w)) for s in (big, small)]
    ps = [torch.zeros(s.fluid.shape, dtype=torch.float32, device=dev) for s in (big, small)]
    rc = batch.project([s.dt for s in (big, small)], vels, [d(s.solid) for s in (big, small)],
                       [d(s.fluid) for s in (big, small)], ps)
    torch.cuda.synchronize()
    assert rc == gb.GBP_OK
    assert [st.tma_staged for st in batch.stats] == [1, 0]
    batch.close()
    for pj in pjs:
        pj.close()
    for s, p, vel in zip((big, small), ps, vels):
        rc1, p1, v1, _ = _solve(s, TMAStaging=0)
        assert rel_inf(p.cpu().numpy(), p1) < 1e-5
        for a, b in zip(vel, v1):
            assert rel_inf(a.cpu().numpy(), b) < 1e-5
