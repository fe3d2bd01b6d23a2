"""Generates the extrapolation fixtures in golden/extrapolate/ from the
reference itself: array_extrapolator3::extrapolate
(include/shiokaze/array/array_extrapolator3.h:36-73, on the reference's
tiled array3 built from its sources, oracle/ref/ref_harness.cpp), the first
half of the liquid solver's velocity extension (src/liquid/macliquid3.cpp:
309-319). Stored per case in ``extrapolate/<case>.npz``: values, active
(dense, x fastest; values 0 where inactive), count, and the reference's
out_values (read back through operator()), out_active, added.

Run from the repository root where the reference sources exist:
    python tests/golden/make_golden_extrapolate.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from shiokaze_gb300 import scenes  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "extrapolate")


def cases():
    # the x velocity of a liquid scene, active on faces next to fluid (as after
    # a projection), extended by the liquid solver's width
    sc = scenes.liquid3(16, seed=2)
    fl = sc.fluid < 0
    act = np.zeros(sc.u.shape, bool)
    act[:, :, 1:] |= fl
    act[:, :, :-1] |= fl
    yield "liquid3_16_u", sc.u, act, 3
    rng = np.random.default_rng(17)
    vals = rng.normal(0, 1, (9, 13, 11)).astype(np.float32)
    yield "sparse_11x13x9", vals, rng.random(vals.shape) < 0.05, 4
    vals = rng.normal(0, 1, (6, 5, 7)).astype(np.float32)
    yield "dense_7x5x6", vals, rng.random(vals.shape) < 0.6, 1
    vals = rng.normal(0, 1, (8, 8, 8)).astype(np.float32)
    one = np.zeros(vals.shape, bool)
    one[3, 4, 5] = True
    yield "single_8", vals, one, 5


def main():
    if oracle.build_reference() is None:
        sys.exit("the reference sources are needed (oracle/ref/Makefile)")
    os.makedirs(OUT, exist_ok=True)
    for name, vals, act, count in cases():
        act = act.astype(np.uint8)
        vals = np.where(act != 0, vals, np.float32(0)).astype(np.float32)
        out, out_act, added = oracle.extrapolate3(vals, act, count, impl="reference")
        np.savez_compressed(os.path.join(OUT, name + ".npz"), values=vals, active=act, count=count, out_values=out,
                            out_active=out_act, added=added)
        print(name, "written,", added, "cells activated")


if __name__ == "__main__":
    main()
