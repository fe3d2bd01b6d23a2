"""GPU parity of the solid constraint of the velocity
(gbp_constrain_velocity3 / _device, the drop-in for the reference's
macutility3::constrain_velocity, src/utility/macutility3.cpp:61-86), bit
for bit:

  * the golden fixtures in golden/constrain/ (made by the reference build):
    solid sphere, cylinder and box wall, masked (narrow-band) velocities, a
    grid spacing that is not a power of two, no solid;
  * seeded random scenes against the oracle, including solids whose values
    lie close to 0 (the sign test then needs the interpolant itself);
  * 128^3 against the oracle;
  * 256^3 smoke: the constraint is idempotent, and the host-array call
    equals the device-array call (size-independent properties).
"""
import glob
import os

import numpy as np
import pytest

import oracle
import shiokaze_gb300 as gb
from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "constrain")


def bits_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def gpu_constrain(solid, u, v, w, dx, masks=None):
    nz, ny, nx = (d - 1 for d in solid.shape)
    out = tuple(np.array(a, dtype=np.float32, order="C") for a in (u, v, w))
    gb.MacUtility3(nx, ny, nz, dx).constrain_velocity(solid, out, masks=masks)
    return out


@pytest.mark.parametrize("name", sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))))
def test_constrain_matches_reference_fixture(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    out = gpu_constrain(d["solid"], d["u"], d["v"], d["w"], float(d["dx"]), masks=(d["mu"], d["mv"], d["mw"]))
    for a, key in zip(out, ("out_u", "out_v", "out_w")):
        assert bits_equal(a, d[key])


@pytest.mark.parametrize("seed", range(10))
def test_constrain_matches_oracle_random(seed):
    rng = np.random.default_rng(seed)
    n = tuple(int(x) for x in rng.integers(2, 20, 3))
    sc = (scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5))) if seed % 2
          else scenes.smoke3(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
    dx = sc.dx if seed % 3 else float(rng.uniform(0.01, 0.2))
    solid = sc.solid
    if seed % 5 == 0:
        solid = (solid * np.float32(rng.uniform(1e-6, 1e-3))).astype(np.float32)
    vel = tuple(a * np.float32(rng.uniform(0.5, 10)) for a in (sc.u, sc.v, sc.w))
    masks = None
    if seed % 4 == 1:
        masks = tuple((rng.random(a.shape) > 0.3).astype(np.uint8) for a in vel)
        vel = tuple(np.where(m != 0, a, np.float32(0)).astype(np.float32) for a, m in zip(vel, masks))
    want = oracle.constrain3(solid, *vel, dx, masks=masks or (None, None, None))
    got = gpu_constrain(solid, *vel, dx, masks=masks)
    for a, b in zip(got, want):
        assert bits_equal(a, b)


def test_constrain_liquid_128_matches_oracle():
    sc = scenes.liquid3(128, seed=2)
    want = oracle.constrain3(sc.solid, sc.u, sc.v, sc.w, sc.dx)
    got = gpu_constrain(sc.solid, sc.u, sc.v, sc.w, sc.dx)
    for a, b in zip(got, want):
        assert bits_equal(a, b)


def test_constrain_256_changes_only_solid_and_wall_faces():
    """256^3 smoke (solid cylinder), size-independent properties: the
    host-array call equals the device-array call; a face changes only if
    it lies on a wall or one of its four solid nodes is negative (the
    interpolated solid can be negative only then); no face on a wall lets
    the velocity out."""
    torch = pytest.importorskip("torch")
    sc = scenes.smoke3(256, seed=3)
    n = 256
    util = gb.MacUtility3(sc.nx, sc.ny, sc.nz, sc.dx)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sc.u, sc.v, sc.w)]
    solid = torch.from_numpy(np.ascontiguousarray(sc.solid)).cuda()
    util.constrain_velocity(solid, tuple(dev))
    out = [t.cpu().numpy() for t in dev]
    host = tuple(a.copy() for a in (sc.u, sc.v, sc.w))
    util.constrain_velocity(sc.solid, host)
    for a, b in zip(host, out):
        assert bits_equal(a, b)
    neg = sc.solid < 0  # nodal (z, y, x)
    # the four nodes of each face: x-faces span (y, z), y-faces (x, z), z-faces (x, y)
    near = [neg[:-1, :-1, :] | neg[1:, :-1, :] | neg[:-1, 1:, :] | neg[1:, 1:, :],
            neg[:-1, :, :-1] | neg[1:, :, :-1] | neg[:-1, :, 1:] | neg[1:, :, 1:],
            neg[:, :-1, :-1] | neg[:, 1:, :-1] | neg[:, :-1, 1:] | neg[:, 1:, 1:]]
    walls = []
    for d, a in enumerate(out):
        wall = np.zeros(a.shape, bool)
        idx = [slice(None)] * 3
        idx[2 - d] = 0
        wall[tuple(idx)] = True
        lo = a[tuple(idx)]
        idx[2 - d] = n
        wall[tuple(idx)] = True
        hi = a[tuple(idx)]
        assert (lo >= 0).all() and (hi <= 0).all()
        walls.append(wall)
    changed = 0
    for a, b, nr, wl in zip(out, (sc.u, sc.v, sc.w), near, walls):
        ch = a.view(np.uint32) != b.view(np.uint32)
        assert not (ch & ~nr & ~wl).any()
        changed += int((ch & nr).sum())
    assert changed > 1000
