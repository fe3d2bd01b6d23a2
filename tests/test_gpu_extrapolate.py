"""Extrapolation on the GPU against the reference (GPU tests).

gbp_extrapolate3(_device) replaces array_extrapolator3::extrapolate
(include/shiokaze/array/array_extrapolator3.h:36-73) as the reference's tiled
array runs it (src/array/dilate3.h:43-95), and
gbp_extrapolate_constrain_velocity3 replaces
macutility3::extrapolate_and_constrain_velocity (src/utility/
macutility3.cpp:88-92). Results must equal the reference's bit for bit: the
golden fixtures made by the reference build (tests/golden/extrapolate/), and
the oracle (pinned to those fixtures and to live reference runs) on seeded
scenes up to 128^3, for values, active sets and the activated counts.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "extrapolate")


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def util():
    import shiokaze_gb300 as gb
    return gb.MacUtility3(4, 4, 4, 0.25)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_extrapolate_matches_reference_fixture(util, path):
    d = dict(np.load(path))
    a = np.where(d["active"] != 0, d["values"], 0).astype(np.float32)
    m = d["active"].astype(np.uint8).copy()
    added = util.extrapolate(a, m, int(d["count"]))
    assert added == int(d["added"])
    assert np.array_equal(m, d["out_active"])
    assert np.array_equal(_bits(np.where(m != 0, a, 0)), _bits(d["out_values"]))


@pytest.mark.parametrize("seed", [1, 2, 3, 4, 5])
def test_extrapolate_matches_oracle_host_and_device(util, seed):
    import torch
    rng = np.random.default_rng(seed)
    d, h, w = (int(x) for x in rng.integers(1, 40, 3))
    act = (rng.random((d, h, w)) < [0.0, 0.01, 0.2, 0.6, 1.0][seed - 1]).astype(np.uint8)
    vals = np.where(act != 0, rng.normal(0, 1, (d, h, w)), 0).astype(np.float32)
    for count in (0, 1, 2, 5):
        want = oracle.extrapolate3(vals, act, count)
        a, m = vals.copy(), act.copy()
        assert util.extrapolate(a, m, count) == want[2]
        assert np.array_equal(m, want[1]) and np.array_equal(_bits(np.where(m != 0, a, 0)), _bits(want[0]))
        ta, tm = torch.from_numpy(vals.copy()).cuda(), torch.from_numpy(act.copy()).cuda()
        assert util.extrapolate(ta, tm, count) == want[2]
        torch.cuda.synchronize()
        assert np.array_equal(tm.cpu().numpy(), want[1])
        assert np.array_equal(_bits(np.where(want[1] != 0, ta.cpu().numpy(), 0)), _bits(want[0]))


def _velocity_case(seed, n, no_solid=False):
    rng = np.random.default_rng(seed)
    sc = scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5)))
    if no_solid:
        sc.solid[...] = np.float32(sc.band)
    masks, comps = [], []
    for a in (sc.u, sc.v, sc.w):
        m = (rng.random(a.shape) < rng.uniform(0.2, 0.7)).astype(np.uint8)
        masks.append(m)
        comps.append(np.where(m != 0, a, 0).astype(np.float32))
    return sc, comps, masks


@pytest.mark.parametrize("seed,n,width,no_solid", [(91, (17, 13, 19), 1, False), (92, (24, 20, 18), 3, False),
                                                   (93, (16, 16, 16), 2, True), (94, 128, 2, False)])
def test_extrapolate_constrain_matches_oracle(seed, n, width, no_solid):
    import shiokaze_gb300 as gb
    sc, comps, masks = _velocity_case(seed, n, no_solid)
    want = oracle.extrapolate_constrain3(sc.solid, *comps, sc.dx, masks, width)
    vel = [c.copy() for c in comps]
    ms = [m.copy() for m in masks]
    gb.MacUtility3(sc.nx, sc.ny, sc.nz, sc.dx).extrapolate_and_constrain_velocity(sc.solid, vel, ms, width)
    grew = 0
    for got, m, w, wm, m0 in zip(vel, ms, want[:3], want[3], masks):
        assert np.array_equal(m, wm)
        assert np.array_equal(_bits(got), _bits(w))
        grew += int(m.sum()) - int(m0.sum())
    assert grew > 0
