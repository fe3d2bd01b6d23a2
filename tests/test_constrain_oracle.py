"""The velocity-constraint oracle (oracle_constrain_velocity3 in
oracle/advect_oracle.c) against the reference.

The fixtures in golden/constrain/ were produced by the reference's own
macutility3::constrain_velocity (src/utility/macutility3.cpp:61-86) built
from its sources (tests/golden/make_golden_constrain.py). The restatement
must reproduce them bit for bit: faces inside a solid sphere, cylinder and
box wall, masked (narrow-band) velocities, a grid spacing that is not a
power of two, and a scene without solid (left alone).
"""
import glob
import os

import numpy as np
import pytest

import oracle
from shiokaze_gb300 import scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "constrain")


def constrain_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_constrain(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name", constrain_cases())
def test_port_matches_reference_constrain_fixture(name):
    d = load_constrain(name)
    out = oracle.constrain3(d["solid"], d["u"], d["v"], d["w"], float(d["dx"]), masks=(d["mu"], d["mv"], d["mw"]))
    for a, key in zip(out, ("out_u", "out_v", "out_w")):
        assert bits_equal(a, d[key])


def test_constrain_fixtures_cover_the_branches():
    names = constrain_cases()
    assert len(names) >= 5
    changed = {n: sum(int((load_constrain(n)[f"out_{c}"] != load_constrain(n)[c]).sum()) for c in "uvw")
               for n in names}
    assert changed["nosolid_8"] == 0 and all(changed[n] > 100 for n in names if n != "nosolid_8")
    d = load_constrain("liquid3_20x14x17_masked")
    assert (d["mu"] == 0).any()
    d = load_constrain("container_18x13x11")
    assert (d["out_u"][:, :, 0] >= 0).all() and (d["out_u"][:, :, -1] <= 0).all()


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", [51, 52, 53])
def test_port_matches_live_reference_constrain(seed):
    rng = np.random.default_rng(seed)
    n = tuple(int(x) for x in rng.integers(5, 20, 3))
    sc = (scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5))) if seed % 2
          else scenes.smoke3(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
    vel = tuple(a * np.float32(rng.uniform(0.5, 10)) for a in (sc.u, sc.v, sc.w))
    masks = (None, None, None)
    if seed == 53:
        masks = tuple((rng.random(a.shape) > 0.3).astype(np.uint8) for a in vel)
        vel = tuple(np.where(m != 0, a, np.float32(0)).astype(np.float32) for a, m in zip(vel, masks))
    a = oracle.constrain3(sc.solid, *vel, sc.dx, masks=masks)
    b = oracle.constrain3(sc.solid, *vel, sc.dx, masks=masks, impl="reference", solid_mode=sc.solid_mode,
                          band=sc.band)
    for x, y in zip(a, b):
        assert bits_equal(x, y)
