"""Sparse arrays in bricks on the GPU (GPU tests).

gbp_bricks_expand and gbp_project_bricks take the reference's tiled arrays
(src/array/tiledarray3.cpp; a cell reads its value if active, else the fill
value if filled, else the background, include/shiokaze/array/array3.h:
796-800) as bricks of 8^3 cells and expand only the listed ones on the GPU.
The expansion must equal the dense array the bricks stand for bit for bit,
and the projection through bricks must equal gbp_project_active on that
dense array, value for value and flag for flag, on every output brick.
"""
import numpy as np
import pytest

import shiokaze_gb300 as gb
from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("shape,seed", [((19, 17, 23), 1), ((8, 8, 8), 2), ((33, 40, 9), 3), ((64, 64, 64), 4),
                                        ((1, 1, 1), 5)])
def test_bricks_expand_matches_dense(shape, seed):
    import torch
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(shape).astype(np.float32)
    for act_frac, fill_below in ((0.3, -1.0), (0.0, 0.0), (1e9, -1e9), (0.05, 10.0)):
        bricks, dense = gb.to_bricks(v, np.abs(v) < act_frac, v < fill_below, background=2.5, fill=-1.25)
        out = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
        gb.bricks_expand(shape[2], shape[1], shape[0], bricks, out)
        torch.cuda.synchronize()
        assert np.array_equal(_bits(out.cpu().numpy()), _bits(dense))


def _scene_bricks(sc, rng):
    """Bricks of a scene's arrays as the modules build them from narrow-band
    level sets (|phi| < band active, phi <= -band filled) and partly active
    velocities; returns the bricks and the dense arrays they stand for."""
    out, dense = [], []
    for a, bg in ((sc.solid, sc.band), (sc.fluid, sc.band)):
        b, d = gb.to_bricks(a, np.abs(a) < sc.band, a <= -sc.band, background=sc.band, fill=-sc.band)
        out.append(b)
        dense.append(d)
    for a in (sc.u, sc.v, sc.w):
        b, d = gb.to_bricks(a, rng.random(a.shape) < 0.7, None, background=0.0)
        out.append(b)
        dense.append(d)
    return out, dense


@pytest.mark.parametrize("kind,n,solver,precision", [("liquid3", 40, "cg", "fp64"), ("liquid3", (37, 30, 41), "mgpcg",
                                                                                   "mixed"),
                                                     ("smoke3", 32, "mgpcg", "fp64"), ("liquid3", 96, "mgpcg", "mixed")])
def test_project_bricks_matches_project_active(kind, n, solver, precision):
    rng = np.random.default_rng(7)
    sc = getattr(scenes, kind)(n, seed=3)
    bricks, dense = _scene_bricks(sc, rng)
    cfg = dict(Residual=1e-6, Solver=solver, Precision=precision)
    # the dense call on the arrays the bricks stand for
    pj = gb.projector_for(sc, **cfg)
    vel = [d.copy() for d in dense[2:]]
    rc = pj.project(sc.dt, vel, dense[0], dense[1], active_sets=True)
    assert rc == gb.GBP_OK
    want_p, want_unknown, want_on = pj.pressure.copy(), pj.unknown.copy(), [a.copy() for a in pj.active]
    pj.close()
    # every brick of the pressure, the velocity's listed bricks
    nbc = bricks[1][0].size
    out_slots = [np.arange(nbc, dtype=np.int32)] + [np.where(b[0] >= 0, b[0], -1).astype(np.int32)
                                                   for b in bricks[2:]]
    pj = gb.projector_for(sc, **cfg)
    rc, outs = pj.project_bricks(sc.dt, bricks[0], bricks[1], bricks[2:], out_slots)
    pj.close()
    assert rc == gb.GBP_OK
    for (vals, act), slots, want, want_a in zip(outs, out_slots, [want_p] + vel, [want_unknown] + want_on):
        bv = gb._brick_view(want, np.float32(0))
        ba = gb._brick_view(want_a, np.uint8(0))
        sel = slots.reshape(bv.shape[:3]) >= 0
        order = np.argsort(slots.reshape(-1)[slots.reshape(-1) >= 0])
        exp_v = bv[sel].reshape(-1, 512)[order].reshape(-1)
        exp_a = ba[sel].reshape(-1, 512)[order].reshape(-1)
        assert np.array_equal(_bits(vals), _bits(exp_v))
        assert np.array_equal(act, exp_a)


def test_bricks_reject_bad_slots():
    """A slot outside [GBP_BRICK_FILL, count) is refused on the host before
    anything reaches the GPU; so is an output slot used twice."""
    import torch
    v = np.zeros((8, 8, 16), np.float32)
    (slot, vals, bg, fill), _ = gb.to_bricks(v, np.ones(v.shape, bool))
    out = torch.zeros(v.shape, dtype=torch.float32, device="cuda")
    for bad in (2, -3):
        s = slot.copy()
        s[1] = bad
        with pytest.raises(gb.GBPError) as e:
            gb.bricks_expand(16, 8, 8, (s, vals, bg, fill), out)
        assert e.value.code == gb.GBP_ERR_INVALID_ARGUMENT
    sc = scenes.liquid3(16, seed=1)
    bricks, _ = _scene_bricks(sc, np.random.default_rng(1))
    nbc = bricks[1][0].size
    twice = np.zeros(nbc, np.int32)  # every brick to slot 0
    pj = gb.projector_for(sc, Residual=1e-6)
    with pytest.raises(gb.GBPError) as e:
        pj.project_bricks(sc.dt, bricks[0], bricks[1], bricks[2:], [twice] + [np.full(b[0].size, -1, np.int32)
                                                                             for b in bricks[2:]])
    assert e.value.code == gb.GBP_ERR_INVALID_ARGUMENT
    pj.close()
