"""The advection oracle (oracle/advect_oracle.c) against the reference.

The fixtures in golden/advect/ were produced by the reference's own
macadvection3 (src/advection/macadvection3.cpp) built from its sources
(tests/golden/make_golden_advect.py). The C restatement must reproduce them
bit for bit: MacCormack and semi-Lagrangian, masked scalars with a
background, narrow-band trimming, traces that leave the grid, faces at rest.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from shiokaze_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "advect")


def advect_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_advect(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", advect_cases())
def test_port_matches_reference_advect_fixture(name):
    d = load_advect(name)
    u, v, w, q, _ = oracle.advect3(d["u"], d["v"], d["w"], d["fluid"], float(d["dx"]), float(d["dt"]), q=d["q"],
                                   q_mask=d["q_mask"], q_bg=float(d["q_bg"]), maccormack=bool(d["maccormack"]),
                                   trim_narrowband=int(d["trim"]))
    assert bits_equal(u, d["out_u"]) and bits_equal(v, d["out_v"]) and bits_equal(w, d["out_w"])
    assert bits_equal(q, d["out_q"])


def test_advect_fixtures_cover_the_branches():
    """The fixtures exercise what the parity claim rests on: the MacCormack
    clamp on both sides, the narrow-band fallback, the at-rest copy."""
    names = advect_cases()
    assert len(names) >= 5
    d = load_advect("liquid3_19x23x16_fast")
    assert (d["u"][:, :, :5] == 0).all()
    assert np.abs(d["u"]).max() * float(d["dt"]) / float(d["dx"]) > 2.0
    d = load_advect("smoke3_12x16x10_mask")
    assert (d["q_mask"] == 0).any() and (d["out_q"][d["q_mask"] == 0] == np.float32(d["q_bg"])).all()


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", [31, 32, 33])
def test_port_matches_live_reference_advect(seed):
    rng = np.random.default_rng(seed)
    n = tuple(int(x) for x in rng.integers(6, 22, 3))
    sc = (scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5))) if seed % 2
          else scenes.smoke3(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
    m = (rng.random(sc.fluid.shape) > rng.uniform(0.0, 0.6)).astype(np.uint8)
    q = np.where(m != 0, rng.normal(0, 1, sc.fluid.shape), 0.5).astype(np.float32)
    kw = dict(q=q, q_mask=m, q_bg=0.5, maccormack=seed != 33, trim_narrowband=int(rng.integers(0, 3)))
    a = oracle.advect3(sc.u, sc.v, sc.w, sc.fluid, sc.dx, sc.dt, **kw)
    b = oracle.advect3(sc.u, sc.v, sc.w, sc.fluid, sc.dx, sc.dt, impl="reference", fluid_mode=sc.fluid_mode,
                       band=sc.band, **kw)
    for x, y in zip(a[:4], b[:4]):
        assert bits_equal(x, y)


# ---- 2D (src/advection/macadvection2.cpp) -----------------------------------------
GOLDEN2 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "advect2")


def advect2_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN2, "*.npz")))


@pytest.mark.parametrize("name", advect2_cases())
def test_port_matches_reference_advect2_fixture(name):
    """The 2D restatement reproduces the reference's macadvection2 fixtures
    (tests/golden/make_golden_advect.py) bit for bit."""
    d = dict(np.load(os.path.join(GOLDEN2, name + ".npz")))
    u, v, q, _ = oracle.advect2(d["u"], d["v"], d["fluid"], float(d["dx"]), float(d["dt"]), q=d["q"],
                                q_mask=d["q_mask"], q_bg=float(d["q_bg"]), maccormack=bool(d["maccormack"]),
                                trim_narrowband=int(d["trim"]))
    assert bits_equal(u, d["out_u"]) and bits_equal(v, d["out_v"]) and bits_equal(q, d["out_q"])


def test_advect2_fixtures_cover_the_branches():
    names = advect2_cases()
    assert len(names) >= 5
    d = dict(np.load(os.path.join(GOLDEN2, "liquid2_37x29_fast.npz")))
    assert (d["u"][:, :5] == 0).all()
    assert np.abs(d["u"]).max() * float(d["dt"]) / float(d["dx"]) > 2.0
    d = dict(np.load(os.path.join(GOLDEN2, "smoke2_33x45_mask.npz")))
    assert (d["q_mask"] == 0).any() and (d["out_q"][d["q_mask"] == 0] == np.float32(d["q_bg"])).all()


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", [41, 42, 43, 44])
def test_port_matches_live_reference_advect2(seed):
    rng = np.random.default_rng(seed)
    n = tuple(int(x) for x in rng.integers(6, 60, 2))
    sc = (scenes.liquid2(n, seed=seed, noise=float(rng.uniform(0.2, 3.0))) if seed % 2
          else scenes.smoke2(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
    fl = sc.fluid[0]
    m = (rng.random(fl.shape) > rng.uniform(0.0, 0.6)).astype(np.uint8)
    q = np.where(m != 0, rng.normal(0, 1, fl.shape), 0.5).astype(np.float32)
    kw = dict(q=q, q_mask=m, q_bg=0.5, maccormack=seed != 43, trim_narrowband=int(rng.integers(0, 3)))
    a = oracle.advect2(sc.u[0], sc.v[0], fl, sc.dx, sc.dt, **kw)
    b = oracle.advect2(sc.u[0], sc.v[0], fl, sc.dx, sc.dt, impl="reference", fluid_mode=sc.fluid_mode,
                       band=sc.band, **kw)
    for x, y in zip(a[:3], b[:3]):
        assert bits_equal(x, y)
