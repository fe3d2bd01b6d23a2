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
    lib.host_advect2.argtypes = [ctypes.c_int] * 2 + [ctypes.c_double] * 2 + [ctypes.c_int] * 2 + [FP] * 4 + \
        [U8, ctypes.c_float]
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


def host_advect2(lib, u, v, fluid, dx, dt, q=None, q_mask=None, q_bg=0.0, maccormack=True, trim_narrowband=1):
    ny, nx = fluid.shape
    uo, vo = (np.array(a, dtype=np.float32, order="C") for a in (u, v))
    fl = np.ascontiguousarray(fluid, dtype=np.float32)
    qo = None if q is None else np.array(q, dtype=np.float32, order="C")
    qm = None if q_mask is None else np.ascontiguousarray(q_mask, dtype=np.uint8)
    lib.host_advect2(nx, ny, dx, dt, int(maccormack), int(trim_narrowband), uo.ctypes.data_as(FP),
                     vo.ctypes.data_as(FP), fl.ctypes.data_as(FP), None if qo is None else qo.ctypes.data_as(FP),
                     _u8(qm), q_bg)
    return uo, vo, qo


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "advect2", "*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_advect2_kernel_code_matches_reference_fixture(host, path):
    """The 2D passes (advect_core.cuh face_forward2 ... cell_backward2)
    reproduce the reference's macadvection2 fixtures bit for bit."""
    d = dict(np.load(path))
    out = host_advect2(host, d["u"], d["v"], d["fluid"], float(d["dx"]), float(d["dt"]), q=d["q"],
                       q_mask=d["q_mask"], q_bg=float(d["q_bg"]), maccormack=bool(d["maccormack"]),
                       trim_narrowband=int(d["trim"]))
    for a, key in zip(out, ("out_u", "out_v", "out_q")):
        assert bits_equal(a, d[key])


@pytest.mark.parametrize("seed", range(6))
def test_advect2_kernel_code_matches_oracle_random(host, seed):
    rng = np.random.default_rng(100 + seed)
    n = tuple(int(x) for x in rng.integers(2, 40, 2))
    sc = (scenes.liquid2(n, seed=seed, noise=float(rng.uniform(0.2, 3.0))) if seed % 2
          else scenes.smoke2(n, seed=seed, sigma=float(rng.uniform(0.5, 4.0))))
    dx = sc.dx if seed % 3 else float(rng.uniform(0.01, 0.2))
    fl = sc.fluid[0]
    m = (rng.random(fl.shape) > rng.uniform(0.0, 0.6)).astype(np.uint8) if seed % 4 else None
    q = rng.normal(0, 1, fl.shape).astype(np.float32)
    u, v = (a[0] * np.float32(rng.uniform(0.5, 30)) for a in (sc.u, sc.v))
    if seed % 5 == 0:
        u[:, :2] = 0.0
        v[:, :2] = 0.0
    trim = int(rng.integers(0, 3))
    kw = dict(q=q, q_mask=m, q_bg=float(rng.normal()), maccormack=seed % 7 != 3, trim_narrowband=trim)
    want = oracle.advect2(u, v, fl, dx, sc.dt, **kw)
    got = host_advect2(host, u, v, fl, dx, sc.dt, **kw)
    for a, b in zip(got, want[:3]):
        assert bits_equal(a, b)


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
    used by kernels that narrow FP64 values) and f2d_exact (float -> double)
    equal the hardware conversions, and nonzero_bits / positive_bits the FP64
    comparisons d != 0 and d > 0; d2f_rn equals the hardware conversion
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
    # f2d_exact: float -> double from integer instructions equals the cast
    lib.host_f2d.argtypes = [FP, ctypes.POINTER(ctypes.c_double), ctypes.c_longlong]
    fl = np.concatenate([rng.integers(0, 1 << 32, 1 << 20, dtype=np.uint64).astype(np.uint32).view(np.float32),
                         np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-40, 3.4e38], np.float32)])
    fl = np.ascontiguousarray(fl)
    d = np.zeros(fl.shape, np.float64)
    lib.host_f2d(fl.ctypes.data_as(FP), d.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), fl.size)
    wd = fl.astype(np.float64)
    same = (d.view(np.uint64) == wd.view(np.uint64)) | (np.isnan(wd) & np.isnan(d))
    assert same.all()
    # the integer tests for d != 0 and d > 0
    U8P = ctypes.POINTER(ctypes.c_ubyte)
    lib.host_bits_tests.argtypes = [ctypes.POINTER(ctypes.c_double), U8P, U8P, ctypes.c_longlong]
    nz = np.zeros(x.size, np.uint8)
    po = np.zeros(x.size, np.uint8)
    lib.host_bits_tests(x.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nz.ctypes.data_as(U8P),
                        po.ctypes.data_as(U8P), x.size)
    with np.errstate(invalid="ignore"):
        assert np.array_equal(nz != 0, x != 0.0) and np.array_equal(po != 0, x > 0.0)
    # split_lo: the low float of a double against its float rounding
    lib.host_split.argtypes = [ctypes.POINTER(ctypes.c_double), FP, FP, ctypes.c_longlong]
    fin = np.isfinite(x) & (np.abs(x) < 3.0e38)
    xs = np.ascontiguousarray(np.concatenate([x[fin], rng.standard_normal(1 << 18) * np.exp2(rng.integers(-60, 60, 1 << 18)),
                                              (fd * (1 + 2.0 ** -30)), 1.0 / 3.0 * np.exp2(np.arange(-90, 90.0))]))
    hi = np.zeros(xs.size, np.float32)
    lo = np.zeros(xs.size, np.float32)
    lib.host_split(xs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), hi.ctypes.data_as(FP), lo.ctypes.data_as(FP),
                   xs.size)
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        want = (xs - hi.astype(np.float64)).astype(np.float32)
    ok = (lo.view(np.uint32) == want.view(np.uint32)) | (np.isnan(want) & np.isnan(lo))
    assert ok.all(), (xs[~ok][:4], lo[~ok][:4], want[~ok][:4])
    rel = np.abs(hi.astype(np.float64) + lo.astype(np.float64) - xs)[np.abs(xs) > 1e-30]
    assert (rel <= 2.0 ** -47 * np.abs(xs[np.abs(xs) > 1e-30])).all()


def test_float_float_dot_error_bound(tmp_path):
    """gbp_floatfloat.cuh's add_product (the FP32 inner solve's dot products
    and norms, one thread's partial) is within gamma_n^2 sum |a_i b_i| of the
    exact dot product (gamma_n = n u / (1 - n u), u = 2^-24), plus the one
    FP64 rounding of hi + lo; add (the coarsening's sums of at most 27
    terms) rounds the exact sum correctly or within one float ulp. The exact
    values come from math.fsum of the products, each exact in FP64. The
    cases: random vectors, sums that cancel to a tiny fraction of sum |a b|,
    terms spread over 60 binary orders, and n up to 2^20 terms (a thread
    sums about cells / resident threads terms: 72 at 256^3)."""
    import math
    so = str(tmp_path / "libff_host.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                           os.path.join(ROOT, "shiokaze_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "kernel_host", "floatfloat_host_harness.cpp"), "-o", so])
    lib = ctypes.CDLL(so)
    lib.host_ff_dot.argtypes = [FP, FP, ctypes.c_longlong]
    lib.host_ff_dot.restype = ctypes.c_double
    lib.host_ff_sum.argtypes = [FP, ctypes.c_longlong]
    lib.host_ff_sum.restype = ctypes.c_float
    rng = np.random.default_rng(11)
    u = 2.0 ** -24
    worst = 0.0
    for n in (1, 7, 72, 1000, 1 << 14, 1 << 20):
        for kind in ("normal", "cancel", "spread", "square"):
            a = rng.standard_normal(n).astype(np.float32)
            b = rng.standard_normal(n).astype(np.float32)
            if kind == "cancel" and n > 1:
                h = n // 2
                a[h:2 * h], b[h:2 * h] = a[:h], -b[:h]
                b[:h] *= np.float32(1 + 2 ** -20)
            elif kind == "spread":
                a *= np.exp2(rng.integers(-30, 30, n)).astype(np.float32)
            elif kind == "square":
                b = a
            a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
            prod = a.astype(np.float64) * b.astype(np.float64)
            exact = math.fsum(prod)
            got = lib.host_ff_dot(a.ctypes.data_as(FP), b.ctypes.data_as(FP), n)
            g = n * u / (1 - n * u)
            bound = g * g * float(np.abs(prod).sum()) + 2.0 ** -53 * abs(exact)
            err = abs(got - exact)
            assert err <= bound, (n, kind, err, bound)
            if bound > 0:
                worst = max(worst, err / bound)
    for n in (2, 8, 27):
        for _ in range(2000):
            x = (rng.standard_normal(n) * np.exp2(rng.integers(-12, 12, n))).astype(np.float32)
            exact = math.fsum(x.astype(np.float64))
            got = lib.host_ff_sum(np.ascontiguousarray(x).ctypes.data_as(FP), n)
            lo = np.nextafter(np.float32(exact), np.float32(-np.inf))
            hi = np.nextafter(np.float32(exact), np.float32(np.inf))
            assert lo <= got <= hi, (x, got, exact)
    print(f"largest dot error / bound: {worst:.3g}")


@pytest.fixture(scope="module")
def exact_lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("exact_host") / "libexact_host.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
                           os.path.join(ROOT, "shiokaze_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "kernel_host", "exact_host_harness.cpp"), "-o", so])
    lib = ctypes.CDLL(so)
    U32 = ctypes.POINTER(ctypes.c_uint)
    I32 = ctypes.POINTER(ctypes.c_int)
    DP = ctypes.POINTER(ctypes.c_double)
    lib.host_exact_sum.argtypes = [FP, U32, I32, ctypes.c_int, ctypes.c_longlong, DP, U8]
    lib.host_mul_round.argtypes = [ctypes.c_double, ctypes.c_int, FP, ctypes.c_longlong, FP, U8]
    return lib


def _sequential_sum(f, neg, n, k):
    """0 + t_0 + t_1 + ... in FP64, t_i = +-f_i 2^k, one rounding per addition."""
    s = np.zeros(f.shape[0])
    for i in range(6):
        t = np.ldexp(f[:, i].astype(np.float64), k)
        t = np.where((neg >> i) & 1, -t, t)
        s = np.where(i < n, s + t, s)
    return s


def test_exact_sum_equals_sequential_fp64(exact_lib):
    """gbp_exact.cuh's exact_sum (the assembly's right-hand side: six face
    fluxes u/dx added in FP64 in the reference's face order) equals the
    sequential FP64 sum bit for bit wherever it decides, and decides for
    terms within a few binary orders of each other (the common case); terms
    far apart, cancellation, zeros of both signs, 1..6 terms."""
    rng = np.random.default_rng(21)
    rows = 1 << 18
    f = rng.standard_normal((rows, 6)).astype(np.float32)
    scale = rng.integers(0, 4, rows)
    f *= np.exp2(rng.integers(-40, 40, (rows, 6)) * (scale[:, None] == 3)).astype(np.float32)
    f[rows // 8: rows // 4, 3] = -f[rows // 8: rows // 4, 0]          # exact cancellation
    f[rows // 4: rows // 3, :] = np.float32(0.0)                      # all zeros
    f[rows // 4: rows // 3: 2, 2] = np.float32(-0.0)
    # near-equal terms of full 24-bit significands
    f[rows // 3: rows // 2] = (1.0 + 2.0 ** -23 * rng.integers(0, 4, (rows // 2 - rows // 3, 6))).astype(np.float32)
    neg = rng.integers(0, 64, rows).astype(np.uint32)
    n = rng.integers(1, 7, rows).astype(np.int32)
    n[: rows // 2] = 6
    for k in (0, 7, -3):
        out = np.zeros(rows)
        ok = np.zeros(rows, np.uint8)
        fa = np.ascontiguousarray(f)
        exact_lib.host_exact_sum(fa.ctypes.data_as(FP), neg.ctypes.data_as(ctypes.POINTER(ctypes.c_uint)),
                                 n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), k, rows,
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ok.ctypes.data_as(U8))
        want = _sequential_sum(f, neg, n, k)
        sel = ok != 0
        assert np.array_equal(out[sel].view(np.uint64), want[sel].view(np.uint64))
        near = scale != 3
        assert sel[near].mean() > 0.999, sel[near].mean()


def test_mul_round_equals_fp64_product(exact_lib):
    """gbp_exact.cuh's mul_round (the velocity update's dt dp / dx with dx a
    power of two) equals (float)((dt * (double)dp) * 2^s) bit for bit
    wherever it decides, and decides for every normal result: random
    time steps and pressure differences over every float exponent, the
    products whose 77-bit significand lies halfway between two doubles or
    whose double lies halfway between two floats (both tie rules), zeros of
    both signs, subnormals and the float overflow edge."""
    rng = np.random.default_rng(22)
    n = 1 << 20
    f = (rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n))).astype(np.float32)
    f[:64] = [0.0, -0.0, 1e-45, -1e-40, np.float32(3.4e38), 1.0, -1.0, 0.5] * 8
    # significands with few bits: products land on ties of both roundings
    f[64:4096] = (rng.integers(1, 1 << 12, 4032) * np.exp2(rng.integers(-20, 0, 4032))).astype(np.float32)
    for a in (0.01, 1.0 / 3.0, 0.004, -0.0125, 1.0 + 2 ** -30 + 2 ** -52, 3.0, 1e-3 * (1 + 2 ** -29),
              float(rng.uniform(1e-4, 1e-1)), 1.5 * 2 ** -29):
        for s in (0, 7, 9, -2, 100):
            out = np.zeros(n, np.float32)
            ok = np.zeros(n, np.uint8)
            exact_lib.host_mul_round(a, s, f.ctypes.data_as(FP), n, out.ctypes.data_as(FP), ok.ctypes.data_as(U8))
            with np.errstate(over="ignore", under="ignore"):
                want = (np.ldexp(np.float64(a) * f.astype(np.float64), s)).astype(np.float32)
            sel = ok != 0
            assert np.array_equal(out[sel].view(np.uint32), want[sel].view(np.uint32)), (a, s)
            normal = (np.abs(want) >= np.finfo(np.float32).tiny) & np.isfinite(want) & (np.abs(f) >= np.finfo(np.float32).tiny)
            assert sel[normal].all(), (a, s, f[normal & ~sel][:4])
