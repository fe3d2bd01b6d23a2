"""Generates the velocity-constraint fixtures in golden/constrain/ from the
reference itself.

Each case runs the reference's own ``macutility3::constrain_velocity``
(src/utility/macutility3.cpp:61-86; compiled from its sources by
``oracle/ref/Makefile``, loaded by name through its module loader by
``oracle/ref/ref_harness.cpp``). Stored per case in ``constrain/<case>.npz``:

  shape (nx, ny, nz), dx                         settings
  solid, solid_mode, band                        nodal solid level set and how the harness built it
  u, v, w, mu, mv, mw                            face velocities and their active masks (dense, x fastest;
                                                 inactive faces hold 0, the velocity's background)
  out_u, out_v, out_w                            the reference's outputs

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden_constrain.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from shiokaze_gb300 import scenes  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "constrain")


def container(n, seed):
    """A solid box wall: the solid occupies everything outside [0.1, 0.9]^3
    (a non-power-of-two grid spacing), velocities N(0, 1)."""
    nx, ny, nz = n
    dx = 1.0 / max(n)
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(m + 1) * dx for m in (nz, ny, nx)), indexing="ij")
    solid = scenes.clamp_band(np.minimum.reduce([x - 0.1, 0.9 - x, y - 0.1, 0.9 - y, z - 0.1, 0.9 - z]), dx)
    u = rng.normal(0, 1, (nz, ny, nx + 1)).astype(np.float32)
    v = rng.normal(0, 1, (nz, ny + 1, nx)).astype(np.float32)
    w = rng.normal(0, 1, (nz + 1, ny, nx)).astype(np.float32)
    return solid, dx, u, v, w


def cases():
    rng = np.random.default_rng(13)
    sc = scenes.liquid3(16, seed=2)
    yield "liquid3_16", sc.solid, sc.solid_mode, sc.band, sc.dx, (sc.u, sc.v, sc.w), (None, None, None)
    sc = scenes.liquid3((20, 14, 17), seed=6)
    vel = tuple(a * np.float32(5.0) for a in (sc.u, sc.v, sc.w))
    masks = tuple((rng.random(a.shape) > 0.4).astype(np.uint8) for a in vel)
    vel = tuple(np.where(m != 0, a, np.float32(0)).astype(np.float32) for a, m in zip(vel, masks))
    yield "liquid3_20x14x17_masked", sc.solid, sc.solid_mode, sc.band, sc.dx, vel, masks
    solid, dx, u, v, w = container((18, 13, 11), seed=7)
    yield "container_18x13x11", solid, 0, scenes.band_of(dx), dx, (u, v, w), (None, None, None)
    sc = scenes.smoke3((12, 16, 10), seed=4, sigma=2.0)
    yield "smoke3_12x16x10", sc.solid, sc.solid_mode, sc.band, sc.dx, (sc.u, sc.v, sc.w), (None, None, None)
    solid = np.full((9, 9, 9), 0.5, np.float32)  # no solid: the reference leaves the velocity alone
    sc = scenes.smoke3(8, seed=5)
    yield "nosolid_8", solid, 1, 0.0, sc.dx, (sc.u, sc.v, sc.w), (None, None, None)


def main():
    if oracle.build_reference() is None:
        sys.exit("the reference sources are needed (oracle/ref/Makefile)")
    os.makedirs(OUT, exist_ok=True)
    for name, solid, mode, band, dx, vel, masks in cases():
        out = oracle.constrain3(solid, *vel, dx, masks=masks, impl="reference", solid_mode=mode, band=band)
        nz, ny, nx = (d - 1 for d in solid.shape)
        ones = [np.ones(a.shape, np.uint8) for a in vel]
        ms = [o if m is None else m for m, o in zip(masks, ones)]
        np.savez_compressed(os.path.join(OUT, name + ".npz"), shape=np.array([nx, ny, nz]), dx=dx, solid=solid,
                            solid_mode=mode, band=band, u=vel[0], v=vel[1], w=vel[2], mu=ms[0], mv=ms[1], mw=ms[2],
                            out_u=out[0], out_v=out[1], out_w=out[2])
        changed = sum(int((a != b).sum()) for a, b in zip(out, vel))
        print(name, "written,", changed, "faces changed")


if __name__ == "__main__":
    main()
