"""Batched projection (gbp_batch_*) on the GPU.

Every kernel of the MGPCG iteration runs once per iteration for all scenes
of a batch; reductions are per scene (one partial per block and scene,
combined in a fixed order), so a scene's result in a batch differs from its
result alone only by the summation grouping: within ALONE_RTOL of |p|_inf
(ALONE_RTOL_NEUMANN after removing the mean for all-Neumann scenes), with
iteration counts within 2. Also checked against the reference's restatement.
"""
import numpy as np
import pytest

import oracle
from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

ALONE_RTOL = 1e-5
ALONE_RTOL_NEUMANN = 1e-4


def _rel(a, b, neumann, mask):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    if neumann:
        a = np.where(mask, a - a[mask].mean(), 0)
        b = np.where(mask, b - b[mask].mean(), 0)
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-30)


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")


def _run_batch(gb, scs, **cfg):
    import torch
    pjs = [gb.projector_for(sc, **cfg) for sc in scs]
    batch = gb.Batch(pjs, **cfg)
    vel = [tuple(_dev(a) for a in (sc.u, sc.v, sc.w) if a is not None) for sc in scs]
    ps = [torch.zeros(sc.fluid.shape, dtype=torch.float32, device="cuda") for sc in scs]
    rc = batch.project([sc.dt for sc in scs], vel, [_dev(sc.solid) for sc in scs], [_dev(sc.fluid) for sc in scs], ps)
    torch.cuda.synchronize()
    stats = [batch.stats[i].iterations for i in range(len(scs))]
    batch.close()
    out = [(p.cpu().numpy(), [t.cpu().numpy() for t in v]) for p, v in zip(ps, vel)]
    for pj in pjs:
        pj.close()
    return rc, out, stats


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_alone(precision):
    import shiokaze_gb300 as gb
    rng = np.random.default_rng(5)
    scs = [scenes.liquid3(int(n), seed=int(s), pool=float(f)) for n, s, f in
           zip(rng.integers(12, 40, 6), rng.integers(1, 1000, 6), rng.uniform(0.15, 0.6, 6))]
    scs.append(scenes.smoke3((20, 18, 22), seed=9))
    scs.append(scenes.liquid2((48, 40), seed=3))
    cfg = dict(Residual=1e-6, Solver="mgpcg", Precision=precision)
    rc, out, iters = _run_batch(gb, scs, **cfg)
    assert rc == gb.GBP_OK
    for sc, (p, vel), it in zip(scs, out, iters):
        rc1, alone, it1 = _run_batch(gb, [sc], **cfg)
        assert rc1 == gb.GBP_OK
        assert abs(it - it1[0]) <= 2, (sc.name, it, it1)
        neumann = sc.name.startswith("smoke")
        mask = alone[0][0] != 0
        tol = ALONE_RTOL_NEUMANN if neumann else ALONE_RTOL
        assert _rel(p, alone[0][0], neumann, mask) <= tol, sc.name
        for a, b in zip(vel, alone[0][1]):
            assert _rel(a, b, False, None) <= 10 * tol, sc.name


def test_batch_matches_oracle():
    import shiokaze_gb300 as gb
    scs = [scenes.liquid3(n, seed=n) for n in (16, 27, 33)] + [scenes.smoke3(24, seed=4)]
    rc, out, iters = _run_batch(gb, scs, Residual=1e-9, Solver="mgpcg", Precision="mixed")
    assert rc == gb.GBP_OK
    for sc, (p, vel) in zip(scs, out):
        want = oracle.project_scene(sc, "port", residual=1e-9)
        m = want.unknown
        pa, pb = p.astype(np.float64), want.pressure.astype(np.float64)
        if sc.name.startswith("smoke"):
            pa = np.where(m, pa - pa[m].mean(), 0)
            pb = np.where(m, pb - pb[m].mean(), 0)
        err = np.max(np.abs(pa - pb)) / np.max(np.abs(pb))
        assert err < 1e-5, (sc.name, err)
