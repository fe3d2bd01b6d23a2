"""Generates the golden fixtures in this directory from the reference itself.

Each case runs the reference's own ``macpressuresolver{2,3}::project``
(compiled from its sources by ``oracle/ref/Makefile``, driven through its
module loader by ``oracle/ref/ref_harness.cpp``) on a small seeded scene and
stores inputs, settings and outputs in ``<case>.npz``:

  dim, shape (nx, ny, nz), dx, dt, params (JSON of the projector settings),
  solid, fluid, u, v[, w]         inputs (dense, x fastest)
  solid_mode, fluid_mode, band    how the harness built the sparse arrays
  steps                           number of project() calls (warm start)
  out_pressure, out_u, out_v[, out_w], out_unknown    after the last call
  out_u_on, out_v_on[, out_w_on]  faces still active after the last call
                                  (the velocity update deactivates closed faces)
  iterations, reresid             the reference's CG report (3D only)

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden.py [--reference /path/to/shiokaze]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from shiokaze_gb300 import scenes  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def next_velocity(res, sc, rng):
    """Synthetic step between projections: projected u + dt*g + N(0, 0.05^2)."""
    u = (res.u + rng.normal(0, 0.05, res.u.shape)).astype(np.float32)
    v = (res.v + sc.dt * scenes.GRAVITY + rng.normal(0, 0.05, res.v.shape)).astype(np.float32)
    w = None if res.w is None else (res.w + rng.normal(0, 0.05, res.w.shape)).astype(np.float32)
    return u, v, w


def isolated_cells3(n=10):
    """A pool plus a lone fluid cell and a two-cell pocket in the air: the
    lone cell is not an unknown (mark_body needs a fluid neighbour)."""
    sc = scenes.liquid3(n, seed=11, pool=0.3)
    b = np.float32(sc.band)
    f = sc.fluid
    # air around each drop stays inside the band so the flood fill is bounded
    f[6:9, 6:9, 1:4] = 0.5 * b
    f[7, 7, 2] = -0.5 * b           # lone cell
    f[6:9, 1:4, 5:9] = 0.5 * b
    f[7, 2, 6] = -0.5 * b           # pocket of two cells
    f[7, 2, 7] = -0.25 * b
    sc.name = "isolated3"
    return sc


CASES = {
    # name: (scene factory, params, steps)
    "liquid3_16": (lambda: scenes.liquid3(16, seed=2), {}, 1),
    "liquid3_20x28x18": (lambda: scenes.liquid3((20, 28, 18), seed=7), {}, 1),
    "liquid3_12_tight": (lambda: scenes.liquid3(12, seed=8), {"residual": 1e-12}, 1),
    "liquid3_12_firstorder": (lambda: scenes.liquid3(12, seed=9),
                              {"second_order_fluid": False, "second_order_solid": False}, 1),
    "liquid3_12_maxiter": (lambda: scenes.liquid3(12, seed=10), {"max_iterations": 5}, 1),
    "liquid3_12_warm": (lambda: scenes.liquid3(12, seed=13), {"warm_start": True}, 3),
    "smoke3_16": (lambda: scenes.smoke3(16, seed=3), {}, 1),
    "smoke3_12x16x10": (lambda: scenes.smoke3((12, 16, 10), seed=14), {}, 1),
    "liquid2_32": (lambda: scenes.liquid2(32, seed=1), {}, 1),
    "liquid2_40x24": (lambda: scenes.liquid2((40, 24), seed=9), {}, 1),
    "isolated3": (isolated_cells3, {}, 1),
    "liquid3_16_tension": (lambda: scenes.liquid3(16, seed=21), {"surface_tension": 0.05}, 1),
    "liquid2_32_tension": (lambda: scenes.liquid2(32, seed=22), {"surface_tension": 0.02}, 1),
    # volume correction: (current, target) volumes set before each step; two
    # steps so that the controller's integral term carries over
    "liquid3_12_volume": (lambda: scenes.liquid3(12, seed=23),
                          {"gain": 1.0, "volume": [[0.30, 0.32], [0.31, 0.32]]}, 2),
    # No case without fluid: the reference then assembles an empty system and
    # pcg_solver.h:62-63 takes abs_max of an empty vector, which crashes.
    "accuracy3_16": (lambda: scenes.accuracy3(16, 0.25)[0], {"residual": 1e-18, "eps_fluid": 1e-18}, 1),
}


def check_realizable(sc):
    """The dense level sets must survive the reference's narrow-band storage
    (set inside the band, flood fill) unchanged."""
    lib = oracle._ref_lib()
    for arr, mode, shp in ((sc.solid, sc.solid_mode, (sc.nx + 1, sc.ny + 1, sc.nz + 1)),
                           (sc.fluid, sc.fluid_mode, (sc.nx, sc.ny, sc.nz))):
        if sc.dim == 2:
            shp = (shp[0], shp[1], 1)
        a = np.ascontiguousarray(arr, np.float32)
        back = np.zeros_like(a)
        lib.ref_levelset_roundtrip(sc.dim, shp[0], shp[1], shp[2], oracle._ptr(a), mode, sc.band, oracle._ptr(back))
        if not np.array_equal(a, back):
            raise ValueError(f"{sc.name}: level set does not survive narrow-band storage")


def make_case(name, factory, params, steps):
    sc = factory()
    check_realizable(sc)
    params = dict(params)
    volume = params.pop("volume", None)
    pj = oracle.RefProjector(sc.dim, sc.nx, sc.ny, sc.nz, sc.dx, **params)
    rng = np.random.default_rng(1000 + len(name))
    u, v, w = sc.u, sc.v, sc.w
    inputs = []
    res = None
    for s in range(steps):
        inputs.append((u, v, w))
        if volume is not None:
            pj.set_target_volume(*volume[s])
        res = pj.project(sc.dt, sc.solid, sc.fluid, u, v, w, sc.solid_mode, sc.fluid_mode, sc.band)
        if s + 1 < steps:
            u, v, w = next_velocity(res, sc, rng)
    pj.close()
    out = dict(dim=sc.dim, shape=np.array([sc.nx, sc.ny, sc.nz]), dx=sc.dx, dt=sc.dt, params=json.dumps(params),
               solid=sc.solid, fluid=sc.fluid, solid_mode=sc.solid_mode, fluid_mode=sc.fluid_mode, band=sc.band,
               steps=steps, out_pressure=res.pressure, out_u=res.u, out_v=res.v, out_unknown=res.unknown,
               iterations=res.iterations, reresid=res.reresid)
    if volume is not None:
        out["volume"] = np.array(volume, np.float64)
    for s, (uu, vv, ww) in enumerate(inputs):
        out[f"u{s}"] = uu
        out[f"v{s}"] = vv
        if ww is not None:
            out[f"w{s}"] = ww
    if res.w is not None:
        out["out_w"] = res.w
    for c, a in zip("uvw", res.active):
        out[f"out_{c}_on"] = a.astype(np.uint8)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if not oracle.build_reference(a.reference):
        sys.exit("reference sources not found; cannot generate fixtures")
    for name, (factory, params, steps) in CASES.items():
        if a.only and name != a.only:
            continue
        res = make_case(name, factory, params, steps)
        print(f"{name}: unknowns={int(res.unknown.sum())} iterations={res.iterations} reresid={res.reresid:.3e}")


if __name__ == "__main__":
    main()
