"""Generates the advection fixtures in golden/advect/ from the reference itself.

Each case runs the reference's own ``macadvection3`` (compiled from its
sources by ``oracle/ref/Makefile``, loaded by name through its module loader
by ``oracle/ref/ref_harness.cpp``) in macsmoke3::idle's order: the scalar q
advected by the velocity, then the velocity by itself. Stored per case in
``advect/<case>.npz``:

  shape (nx, ny, nz), dx, dt, maccormack, trim        settings
  u, v, w, fluid, q, q_mask, q_bg                     inputs (dense, x fastest;
                                                      q_mask all ones = all active)
  fluid_mode, band                                    how the harness built fluid
  out_u, out_v, out_w, out_q                          the reference's outputs

The 2D cases (``advect2/<case>.npz``, arrays y, x, no w) run the
reference's ``macadvection2`` in macsmoke2's order the same way.

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden_advect.py [--2d-only]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from shiokaze_gb300 import scenes  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "advect")


def cases():
    rng = np.random.default_rng(11)
    sc = scenes.smoke3(16, seed=3)
    yield "smoke3_16", sc, rng.random(sc.fluid.shape, dtype=np.float32), None, 0.0, True, 1
    sc = scenes.smoke3((12, 16, 10), seed=4, sigma=2.0)
    m = (rng.random(sc.fluid.shape) > 0.4).astype(np.uint8)
    yield "smoke3_12x16x10_mask", sc, rng.random(sc.fluid.shape, dtype=np.float32), m, 0.25, True, 1
    sc = scenes.smoke3(16, seed=5)
    yield "smoke3_16_semilagrangian", sc, rng.random(sc.fluid.shape, dtype=np.float32), None, 0.0, False, 1
    sc = scenes.liquid3(16, seed=2)
    m = (sc.fluid < sc.band).astype(np.uint8)
    yield "liquid3_16_band", sc, rng.random(sc.fluid.shape, dtype=np.float32), m, 0.0, True, 1
    # traces that leave the grid (CFL ~ 4), faces and cells at rest, -0.0
    sc = scenes.liquid3((19, 23, 16), seed=9)
    for a in (sc.u, sc.v, sc.w):
        a *= 40.0
        a[:, :, :5] = 0.0
        a[:3] = -0.0
    m = (rng.random(sc.fluid.shape) > 0.5).astype(np.uint8)
    yield "liquid3_19x23x16_fast", sc, rng.random(sc.fluid.shape, dtype=np.float32), m, 0.0, True, 2


OUT2 = os.path.join(os.path.dirname(os.path.abspath(__file__)), "advect2")


def cases2():
    """2D cases for the reference's macadvection2 (arrays y, x)."""
    rng = np.random.default_rng(12)
    sc = scenes.smoke2((40, 32), seed=3)
    yield "smoke2_40x32", sc, rng.random(sc.fluid.shape[1:], dtype=np.float32), None, 0.0, True, 1
    sc = scenes.smoke2((33, 45), seed=4, sigma=2.0)
    m = (rng.random(sc.fluid.shape[1:]) > 0.4).astype(np.uint8)
    yield "smoke2_33x45_mask", sc, rng.random(sc.fluid.shape[1:], dtype=np.float32), m, 0.25, True, 1
    sc = scenes.smoke2(32, seed=5)
    yield "smoke2_32_semilagrangian", sc, rng.random(sc.fluid.shape[1:], dtype=np.float32), None, 0.0, False, 1
    sc = scenes.liquid2(48, seed=2, noise=1.0)
    m = (sc.fluid[0] < sc.band).astype(np.uint8)
    yield "liquid2_48_band", sc, rng.random(sc.fluid.shape[1:], dtype=np.float32), m, 0.0, True, 1
    # traces that leave the grid (CFL ~ 4), faces and cells at rest, -0.0
    sc = scenes.liquid2((37, 29), seed=9, noise=1.0)
    for a in (sc.u, sc.v):
        a *= 15.0
        a[:, :, :5] = 0.0
        a[:, :3] = -0.0
    m = (rng.random(sc.fluid.shape[1:]) > 0.5).astype(np.uint8)
    yield "liquid2_37x29_fast", sc, rng.random(sc.fluid.shape[1:], dtype=np.float32), m, 0.0, True, 2


def main():
    if oracle.build_reference() is None:
        sys.exit("the reference sources are needed (oracle/ref/Makefile)")
    os.makedirs(OUT2, exist_ok=True)
    for name, sc, q, m, bg, mac, trim in cases2():
        q = q.astype(np.float32)
        if m is not None:
            q = np.where(m != 0, q, np.float32(bg)).astype(np.float32)
        u2, v2, fl2 = sc.u[0], sc.v[0], sc.fluid[0]
        u, v, qo, _ = oracle.advect2(u2, v2, fl2, sc.dx, sc.dt, q=q, q_mask=m, q_bg=bg, maccormack=mac,
                                     trim_narrowband=trim, impl="reference", fluid_mode=sc.fluid_mode, band=sc.band)
        ny, nx = fl2.shape
        np.savez_compressed(
            os.path.join(OUT2, name + ".npz"), shape=np.array([nx, ny]), dx=sc.dx, dt=sc.dt, maccormack=mac,
            trim=trim, u=u2, v=v2, fluid=fl2, fluid_mode=sc.fluid_mode, band=sc.band, q=q,
            q_mask=np.ones(fl2.shape, np.uint8) if m is None else m, q_bg=np.float32(bg), out_u=u, out_v=v,
            out_q=qo)
        print(name, "written")
    if "--2d-only" in sys.argv:
        return
    os.makedirs(OUT, exist_ok=True)
    for name, sc, q, m, bg, mac, trim in cases():
        q = q.astype(np.float32)
        if m is not None:
            q = np.where(m != 0, q, np.float32(bg)).astype(np.float32)
        u, v, w, qo, _ = oracle.advect3(sc.u, sc.v, sc.w, sc.fluid, sc.dx, sc.dt, q=q, q_mask=m, q_bg=bg,
                                         maccormack=mac, trim_narrowband=trim, impl="reference",
                                         fluid_mode=sc.fluid_mode, band=sc.band)
        nz, ny, nx = sc.fluid.shape
        np.savez_compressed(
            os.path.join(OUT, name + ".npz"), shape=np.array([nx, ny, nz]), dx=sc.dx, dt=sc.dt, maccormack=mac,
            trim=trim, u=sc.u, v=sc.v, w=sc.w, fluid=sc.fluid, fluid_mode=sc.fluid_mode, band=sc.band, q=q,
            q_mask=np.ones(sc.fluid.shape, np.uint8) if m is None else m, q_bg=np.float32(bg), out_u=u, out_v=v,
            out_w=w, out_q=qo)
        print(name, "written")


if __name__ == "__main__":
    main()
