"""The advection and solid-constraint kernels' per-element code on the CPU.

tests/kernel_host/advect_host_harness.cpp compiles the same source the CUDA
kernels call (shiokaze_gb300/csrc/advect_core.cuh) with g++ and runs it in
the kernels' launch order. It must reproduce the reference's fixtures and the
oracle bit for bit: a check of the kernels' arithmetic and indexing that
needs no GPU (the GPU runs of the same cases are in test_gpu_advect.py and
test_gpu_constrain.py).
"""
import ctypes
import glob
import os
import subprocess

import numpy as np
import pytest

import oracle
from shiokaze_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
FP = ctypes.POINTER(ctypes.c_float)
U8 = ctypes.POINTER(ctypes.c_ubyte)


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("kernel_host") / "libadvect_host.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                           os.path.join(ROOT, "shiokaze_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "kernel_host", "advect_host_harness.cpp"), "-o", so])
    lib = ctypes.CDLL(so)
    lib.host_advect3.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 2 + [ctypes.c_int] * 2 + [FP] * 5 + \
        [U8, ctypes.c_float]
    lib.host_constrain3.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] + [FP] * 4 + [U8] * 3
    return lib


def _u8(m):
    return None if m is None else np.ascontiguousarray(m, dtype=np.uint8).ctypes.data_as(U8)


def host_advect(lib, u, v, w, fluid, dx, dt, q=None, q_mask=None, q_bg=0.0, maccormack=True, trim_narrowband=1):
    nz, ny, nx = fluid.shape
    uo, vo, wo = (np.array(a, dtype=np.float32, order="C") for a in (u, v, w))
    fl = np.ascontiguousarray(fluid, dtype=np.float32)
    qo = None if q is None else np.array(q, dtype=np.float32, order="C")
    qm = None if q_mask is None else np.ascontiguousarray(q_mask, dtype=np.uint8)
    lib.host_advect3(nx, ny, nz, dx, dt, int(maccormack), int(trim_narrowband), uo.ctypes.data_as(FP),
                     vo.ctypes.data_as(FP), wo.ctypes.data_as(FP), fl.ctypes.data_as(FP),
                     None if qo is None else qo.ctypes.data_as(FP), _u8(qm), q_bg)
    return uo, vo, wo, qo


def host_constrain(lib, solid, u, v, w, dx, masks=(None, None, None)):
    nz, ny, nx = (d - 1 for d in solid.shape)
    out = tuple(np.array(a, dtype=np.float32, order="C") for a in (u, v, w))
    sl = np.ascontiguousarray(solid, dtype=np.float32)
    ms = [None if m is None else np.ascontiguousarray(m, dtype=np.uint8) for m in masks]
    lib.host_constrain3(nx, ny, nz, dx, sl.ctypes.data_as(FP), *(a.ctypes.data_as(FP) for a in out),
                        *(None if m is None else m.ctypes.data_as(U8) for m in ms))
    return out


def bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "advect", "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_advect_kernel_code_matches_reference_fixture(host, path):
    d = dict(np.load(path))
    out = host_advect(host, d["u"], d["v"], d["w"], d["fluid"], float(d["dx"]), float(d["dt"]), q=d["q"],
                      q_mask=d["q_mask"], q_bg=float(d["q_bg"]), maccormack=bool(d["maccormack"]),
                      trim_narrowband=int(d["trim"]))
    for a, key in zip(out, ("out_u", "out_v", "out_w", "out_q")):
        assert bits_equal(a, d[key])


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "constrain", "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_constrain_kernel_code_matches_reference_fixture(host, path):
    d = dict(np.load(path))
    out = host_constrain(host, d["solid"], d["u"], d["v"], d["w"], float(d["dx"]), (d["mu"], d["mv"], d["mw"]))
    for a, key in zip(out, ("out_u", "out_v", "out_w")):
        assert bits_equal(a, d[key])


@pytest.mark.parametrize("seed", range(8))
def test_kernel_code_matches_oracle_random(host, seed):
    """Random scenes, a grid spacing that is not a power of two, masks,
    faces at rest, level sets within a hair of the narrow-band limit."""
    rng = np.random.default_rng(seed)
    n = tuple(int(x) for x in rng.integers(2, 16, 3))
    sc = (scenes.liquid3(n, seed=seed, pool=float(rng.uniform(0.2, 0.5))) if seed % 2
          else scenes.smoke3(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
    dx = sc.dx if seed % 3 else float(rng.uniform(0.01, 0.2))
    m = (rng.random(sc.fluid.shape) > rng.uniform(0.0, 0.6)).astype(np.uint8) if seed % 4 else None
    q = rng.normal(0, 1, sc.fluid.shape).astype(np.float32)
    u, v, w = (a * np.float32(rng.uniform(0.5, 30)) for a in (sc.u, sc.v, sc.w))
    if seed % 5 == 0:
        for a in (u, v, w):
            a[:, :, :2] = 0.0
    trim = int(rng.integers(0, 3))
    fluid = sc.fluid
    if seed % 3 == 2:
        fluid = (-dx * trim + rng.normal(0, 1, sc.fluid.shape) * 1e-7 * dx).astype(np.float32)
    kw = dict(q=q, q_mask=m, q_bg=float(rng.normal()), maccormack=seed % 7 != 3, trim_narrowband=trim)
    want = oracle.advect3(u, v, w, fluid, dx, sc.dt, **kw)
    got = host_advect(host, u, v, w, fluid, dx, sc.dt, **kw)
    for a, b in zip(got, want[:4]):
        assert bits_equal(a, b)
    solid = sc.solid if seed % 2 else (sc.solid * np.float32(1e-4)).astype(np.float32)
    want = oracle.constrain3(solid, u, v, w, dx)
    got = host_constrain(host, solid, u, v, w, dx)
    for a, b in zip(got, want):
        assert bits_equal(a, b)


def test_integer_double_to_float_conversion_is_exact(tmp_path):
    """gbp_convert.cuh's d2f_rn (double -> float from integer instructions,
    used by kernels that narrow FP64 values) equals the hardware conversion
    (round to nearest, ties to even) bit for bit: random doubles of every
    exponent, floats and the points halfway between neighbouring floats with
    the doubles on either side, the edges of the float range (largest
    finite, the overflow to infinity, the smallest normal and subnormals),
    zeros, infinities and NaN."""
    so = str(tmp_path / "libconvert_host.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I",
                           os.path.join(ROOT, "shiokaze_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "kernel_host", "convert_host_harness.cpp"), "-o", so])
    lib = ctypes.CDLL(so)
    lib.host_d2f.argtypes = [ctypes.POINTER(ctypes.c_double), FP, ctypes.c_longlong]
    rng = np.random.default_rng(5)
    bits = rng.integers(0, 1 << 63, 1 << 20, dtype=np.uint64) | (rng.integers(0, 2, 1 << 20, dtype=np.uint64) << 63)
    a = bits.view(np.float64)
    f = rng.standard_normal(1 << 18).astype(np.float32)
    fd = f.astype(np.float64)
    half = (fd + np.nextafter(f, np.float32(np.inf)).astype(np.float64)) / 2
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 3.4028234663852886e38, 3.4028235677973366e38,
                        3.4028235677973362e38, 3.402823567797337e38, 1.1754943508222875e-38, 1.1754942e-38,
                        1e-45, 1.401298464324817e-45, 7e-46, 1e-300, 1e300, -1e300, 0.5, 1.5, 2.5],
                       dtype=np.float64)
    x = np.ascontiguousarray(np.concatenate([a, fd, half, np.nextafter(half, np.inf), np.nextafter(half, -np.inf),
                                             special]))
    out = np.zeros(x.shape, np.float32)
    lib.host_d2f(x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), out.ctypes.data_as(FP), x.size)
    with np.errstate(over="ignore"):
        want = x.astype(np.float32)
    same = (out.view(np.uint32) == want.view(np.uint32)) | (np.isnan(want) & np.isnan(out))
    assert same.all(), x[~same][:8]
