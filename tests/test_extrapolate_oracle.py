"""The extrapolation oracle (oracle_extrapolate3 in oracle/advect_oracle.c)
against the reference: array_extrapolator3::extrapolate
(include/shiokaze/array/array_extrapolator3.h:36-73) as the reference's
tiled array runs it (dilate3.h). The fixtures in golden/extrapolate/ were
made by the reference build (tests/golden/make_golden_extrapolate.py); the
restatement must reproduce the values bit for bit, the active set and the
count of activated cells. This is the oracle for the extrapolation half of
the liquid solver's velocity extension (src/liquid/macliquid3.cpp:309-319);
the GPU side of that step is not built.
"""
import glob
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "extrapolate")


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_port_matches_reference_extrapolate_fixture(path):
    d = dict(np.load(path))
    out, act, added = oracle.extrapolate3(d["values"], d["active"], int(d["count"]))
    assert np.array_equal(out.view(np.uint32), d["out_values"].view(np.uint32))
    assert np.array_equal(act, d["out_active"]) and added == int(d["added"])


def test_extrapolate_fixtures_cover_the_cases():
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    assert len(names) >= 4
    d = dict(np.load(os.path.join(GOLDEN, "single_8.npz")))
    # one active cell spreads as a diamond of radius `count` (6-neighbour rounds)
    assert int(d["out_active"].sum()) == 1 + int(d["added"]) and int(d["count"]) == 5


@pytest.mark.skipif(not oracle.reference_available(), reason="reference oracle not built here")
@pytest.mark.parametrize("seed", [61, 62, 63, 64])
def test_port_matches_live_reference_extrapolate(seed):
    rng = np.random.default_rng(seed)
    d, h, w = (int(x) for x in rng.integers(2, 20, 3))
    vals = rng.normal(0, 1, (d, h, w)).astype(np.float32)
    act = (rng.random((d, h, w)) < rng.uniform(0.02, 0.5)).astype(np.uint8)
    vals = np.where(act != 0, vals, np.float32(0)).astype(np.float32)
    count = int(rng.integers(1, 5))
    a = oracle.extrapolate3(vals, act, count)
    b = oracle.extrapolate3(vals, act, count, impl="reference")
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    assert np.array_equal(a[1], b[1]) and a[2] == b[2]
