"""Tile classes (TileClasses=1, the default) against the kernels that read
every coupling array (TileClasses=0).

In the FP32 kernels a tile whose stencils read only couplings of one value
u uses u instead of the arrays (the same products in the same order; on
4-plane tiles (fine grids of 2^21 cells or more), with every load of a thread's
column issued first); in
both precisions a tile with no unknown writes zeros without loading, or
is skipped where its values are already 0. The solves must therefore
agree exactly: the same iteration counts and the same pressure and
velocities (up to the sign of zeros, which compare equal).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(sc, **cfg):
    import shiokaze_gb300 as gb
    pj = gb.projector_for(sc, Residual=1e-6, Solver="mgpcg", **cfg)
    vel = tuple(a.copy() for a in (sc.u, sc.v, sc.w) if a is not None)
    rc = pj.project(sc.dt, vel, sc.solid, sc.fluid)
    out = (rc, pj.get_pressure().copy(), vel, pj.stats.as_dict())
    pj.close()
    return out


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("kind,shape", [("liquid3", 96), ("smoke3", (80, 64, 72)), ("liquid3", 160),
                                        ("smoke3", (136, 128, 128)), ("liquid3", (129, 130, 127)),
                                        ("liquid2", 200)])
def test_tile_classes_change_nothing(kind, shape, precision):
    import shiokaze_gb300 as gb
    from shiokaze_gb300 import scenes
    sc = getattr(scenes, kind)(shape, seed=41)
    rc1, p1, v1, st1 = _solve(sc, Precision=precision, TileClasses=1)
    rc0, p0, v0, st0 = _solve(sc, Precision=precision, TileClasses=0)
    assert rc1 == gb.GBP_OK and rc0 == gb.GBP_OK
    assert st1["iterations"] == st0["iterations"]
    assert st1["outer_iterations"] == st0["outer_iterations"]
    assert st1["true_resid_inf"] == st0["true_resid_inf"]
    assert np.array_equal(p1, p0)
    for a, b in zip(v1, v0):
        assert np.array_equal(a, b)


def test_tile_classes_in_a_batch():
    """A batch whose scenes hold empty, uniform and mixed tiles solves as the
    same scenes alone without classes."""
    import torch
    import shiokaze_gb300 as gb
    from shiokaze_gb300 import scenes
    scs = [scenes.liquid3(64, seed=42), scenes.smoke3(48, seed=43), scenes.liquid3((40, 56, 48), seed=44)]
    cfg = dict(Residual=1e-6, Solver="mgpcg", Precision="mixed")
    dev = torch.device("cuda", 0)

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    ctx = gb.Context(0)
    pjs = [gb.projector_for(s, ctx, **cfg) for s in scs]
    batch = gb.Batch(pjs, ctx, **cfg)
    vels = [tuple(d(a) for a in (s.u, s.v, s.w)) for s in scs]
    ps = [torch.zeros(s.fluid.shape, dtype=torch.float32, device=dev) for s in scs]
    rc = batch.project([s.dt for s in scs], vels, [d(s.solid) for s in scs], [d(s.fluid) for s in scs], ps)
    torch.cuda.synchronize()
    assert rc == gb.GBP_OK
    batch.close()
    for pj in pjs:
        pj.close()
    for s, p, vel in zip(scs, ps, vels):
        _, p0, v0, _ = _solve(s, Precision="mixed", TileClasses=0)
        # a batch groups its partial sums differently from a lone solve
        assert np.max(np.abs(p.cpu().numpy() - p0)) <= 1e-5 * max(1.0, np.max(np.abs(p0)))
        for a, b in zip(vel, v0):
            assert np.max(np.abs(a.cpu().numpy() - b)) <= 1e-5 * max(1.0, np.max(np.abs(b)))
