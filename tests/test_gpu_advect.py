"""GPU parity of the MAC advection step (gbp_advect3 / gbp_advect3_device,
the drop-in for the reference's macadvection3 module) against the
reference's own outputs and the oracle, bit for bit.

  * the golden fixtures in golden/advect/ (made by the reference build):
    MacCormack and semi-Lagrangian, masked scalars with a background,
    narrow-band trimming, traces that leave the grid, faces at rest;
  * seeded random scenes against the oracle restatement, including a
    grid spacing that is not a power of two;
  * 128^3 smoke (the 3D workloads' scale) against the oracle;
  * 256^3: a uniform flow of exactly one cell per step translates the
    scalar by one cell (a size-independent property), and the host-array
    call equals the device-array call.
"""
import glob
import os

import numpy as np
import pytest

import oracle
import shiokaze_gb300 as gb
from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "advect")


def bits_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def bits_equal_nan(a, b):
    """Bit-equal except that any NaN equals any NaN: the GPU writes the
    canonical NaN where a CPU propagates an input NaN's payload."""
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape or not np.array_equal(np.isnan(a), np.isnan(b)):
        return False
    keep = ~np.isnan(a)
    return np.array_equal(a.view(np.uint32)[keep], b.view(np.uint32)[keep])


def gpu_step(u, v, w, fluid, dx, dt, q=None, q_mask=None, q_bg=0.0, maccormack=True, trim_narrowband=1):
    nz, ny, nx = fluid.shape
    adv = gb.MacAdvection3(nx, ny, nz, dx, MacCormack=maccormack, TrimNarrowBand=trim_narrowband)
    uo, vo, wo = (np.array(a, dtype=np.float32, order="C") for a in (u, v, w))
    qo = None if q is None else np.array(q, dtype=np.float32, order="C")
    adv.advect_step((uo, vo, wo), fluid, dt, scalar=qo, mask=q_mask, background=q_bg)
    return uo, vo, wo, qo


@pytest.mark.parametrize("name", sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))))
def test_advect_matches_reference_fixture(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    u, v, w, q = gpu_step(d["u"], d["v"], d["w"], d["fluid"], float(d["dx"]), float(d["dt"]), q=d["q"],
                          q_mask=d["q_mask"], q_bg=float(d["q_bg"]), maccormack=bool(d["maccormack"]),
                          trim_narrowband=int(d["trim"]))
    assert bits_equal(u, d["out_u"]) and bits_equal(v, d["out_v"]) and bits_equal(w, d["out_w"])
    assert bits_equal(q, d["out_q"])


def random_case(seed):
    rng = np.random.default_rng(seed)
    n = tuple(int(x) for x in rng.integers(2, 24, 3))
    sc = (scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5))) if seed % 2
          else scenes.smoke3(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
    dx = sc.dx if seed % 3 else float(rng.uniform(0.01, 0.2))
    m = (rng.random(sc.fluid.shape) > rng.uniform(0.0, 0.6)).astype(np.uint8) if seed % 4 else None
    q = rng.normal(0, 1, sc.fluid.shape).astype(np.float32)
    u, v, w = (a * np.float32(rng.uniform(0.5, 30)) for a in (sc.u, sc.v, sc.w))
    if seed % 5 == 0:
        for a in (u, v, w):
            a[:, :, :2] = 0.0
    kw = dict(q=q, q_mask=m, q_bg=float(rng.normal()), maccormack=seed % 7 != 3,
              trim_narrowband=int(rng.integers(0, 3)))
    return (u, v, w, sc.fluid, dx, sc.dt), kw


@pytest.mark.parametrize("seed", range(12))
def test_advect_matches_oracle_random(seed):
    args, kw = random_case(seed)
    want = oracle.advect3(*args, **kw)
    got = gpu_step(*args, **kw)
    for a, b in zip(got, want[:4]):
        assert bits_equal(a, b)


@pytest.mark.parametrize("seed", range(8))
def test_narrow_band_test_near_its_limit(seed):
    """Level sets within a hair of the trimming limit, and non-finite
    values: the kernels decide most narrow-band tests from the corners'
    range and must agree with the interpolant wherever it is close."""
    rng = np.random.default_rng(100 + seed)
    n = tuple(int(x) for x in rng.integers(2, 14, 3))
    sc = scenes.smoke3(n, seed=seed, sigma=float(rng.uniform(0.5, 3.0)))
    trim = int(rng.integers(0, 3))
    limit = -sc.dx * trim
    scale = float(10.0 ** rng.uniform(-12, -3)) * sc.dx
    fluid = (limit + rng.normal(0, 1, sc.fluid.shape) * scale).astype(np.float32)
    if seed % 3 == 0:
        fluid.flat[rng.integers(0, fluid.size, 3)] = [np.nan, np.inf, -np.inf]
    if seed % 4 == 1:
        fluid[...] = np.float32(limit)
    q = rng.normal(0, 1, sc.fluid.shape).astype(np.float32)
    if seed % 4 == 2:
        q.flat[rng.integers(0, q.size, 2)] = [np.inf, np.nan]
    u, v, w = (a * np.float32(rng.uniform(0.5, 20)) for a in (sc.u, sc.v, sc.w))
    kw = dict(q=q, q_mask=None, q_bg=0.0, maccormack=True, trim_narrowband=trim)
    want = oracle.advect3(u, v, w, fluid, sc.dx, sc.dt, **kw)
    got = gpu_step(u, v, w, fluid, sc.dx, sc.dt, **kw)
    for a, b in zip(got, want[:4]):
        assert bits_equal_nan(a, b)


def test_scalar_and_vector_calls_equal_the_step():
    """advect_scalar then advect_vector (the reference's two calls) equal the
    combined step, and a NULL mask equals an all-ones mask."""
    args, kw = random_case(20)
    u, v, w, fluid, dx, dt = args
    want = gpu_step(*args, **kw)
    nz, ny, nx = fluid.shape
    adv = gb.MacAdvection3(nx, ny, nz, dx, MacCormack=kw["maccormack"], TrimNarrowBand=kw["trim_narrowband"])
    uo, vo, wo = (a.copy() for a in (u, v, w))
    q = kw["q"].copy()
    adv.advect_scalar(q, (uo, vo, wo), fluid, dt, mask=kw["q_mask"], background=kw["q_bg"])
    adv.advect_vector((uo, vo, wo), (uo, vo, wo), fluid, dt)
    for a, b in zip((uo, vo, wo, q), want):
        assert bits_equal(a, b)
    kw2 = dict(kw, q_mask=None)
    a = gpu_step(*args, **kw2)
    b = gpu_step(*args, **dict(kw, q_mask=np.ones(fluid.shape, np.uint8)))
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_advect_smoke_128_matches_oracle():
    sc = scenes.smoke3(128, seed=3)
    q = np.random.default_rng(7).random(sc.fluid.shape, dtype=np.float32)
    want = oracle.advect3(sc.u, sc.v, sc.w, sc.fluid, sc.dx, sc.dt, q=q)
    got = gpu_step(sc.u, sc.v, sc.w, sc.fluid, sc.dx, sc.dt, q=q)
    for a, b in zip(got, want[:4]):
        assert bits_equal(a, b)


def test_advect_256_uniform_flow_translates_by_one_cell():
    torch = pytest.importorskip("torch")
    n = 256
    dx = 1.0 / n
    dt = dx  # u = 1: dt*u/dx is exactly one cell
    rng = np.random.default_rng(5)
    q = rng.random((n, n, n), dtype=np.float32)
    u = np.ones((n, n, n + 1), np.float32)
    v = np.zeros((n, n + 1, n), np.float32)
    w = np.zeros((n + 1, n, n), np.float32)
    fluid = np.full((n, n, n), -1.0, np.float32)  # all fluid, outside the narrow band: the limiter applies
    dev = [torch.from_numpy(a).cuda() for a in (u, v, w, fluid, q)]
    adv = gb.MacAdvection3(n, n, n, dx)
    adv.advect_step(tuple(dev[:3]), dev[3], dt, scalar=dev[4])
    torch.cuda.synchronize()
    qo = dev[4].cpu().numpy()
    assert np.array_equal(qo[:, :, 1:n - 1], q[:, :, 0:n - 2])
    assert np.array_equal(qo[:, :, 0], q[:, :, 0])
    assert np.array_equal(dev[0].cpu().numpy(), u)
    assert not dev[1].any().item() and not dev[2].any().item()
    # the host-array call gives the same bits as the device-array call
    uh, vh, wh, qh = u.copy(), v.copy(), w.copy(), q.copy()
    adv.advect_step((uh, vh, wh), fluid, dt, scalar=qh)
    assert bits_equal(qh, qo) and bits_equal(uh, dev[0].cpu().numpy())


def test_advect_rejects_bad_arguments():
    ctx = gb.default_context()
    lib = ctx.lib
    a = np.zeros(64, np.float32)
    fp = a.ctypes.data_as(gb.ctypes.POINTER(gb.ctypes.c_float))
    p = gb.AdvectParams()
    lib.gbp_advect_params_default(gb.ctypes.byref(p))
    # a grid edge of one cell, a non-positive dx, and nothing to advect
    assert lib.gbp_advect3(ctx.handle, 1, 4, 4, 0.25, 0.1, gb.ctypes.byref(p), fp, fp, fp, fp, None, None, 0.0) == 1
    assert lib.gbp_advect3(ctx.handle, 2, 2, 2, 0.0, 0.1, gb.ctypes.byref(p), fp, fp, fp, fp, None, None, 0.0) == 1
    p.advect_velocity = 0
    assert lib.gbp_advect3(ctx.handle, 2, 2, 2, 0.5, 0.1, gb.ctypes.byref(p), fp, fp, fp, fp, None, None, 0.0) == 1
    assert b"nothing to advect" in lib.gbp_strerror(1)
