"""The oracle: CPU projections the GPU module is checked against.

TEST INFRASTRUCTURE. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` import this package; the shipped module
never does.

Two implementations sit behind the same Python call:

* ``port``: ``oracle/gbp_oracle.c``, a dense C restatement of the reference's
  ``macpressuresolver{2,3}::project`` (built to ``oracle/liboracle.so``);
* ``reference``: the reference itself, compiled from its own sources by
  ``oracle/ref/Makefile`` into ``oracle/_ref/`` and driven through its module
  loader by ``oracle/ref/ref_harness.cpp``. It can only be built where the
  reference sources are present.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import tempfile
import time
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libref_harness.so")


def build_port(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("gbp_oracle.c", "advect_oracle.c")]
    if force or not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < max(map(os.path.getmtime, srcs)):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", *srcs, "-o",
                               PORT_SO, "-lm"])
    return PORT_SO


def build_reference(ref_dir: str | None = None, jobs: int = 8) -> str | None:
    """Compile the reference from its sources in `ref_dir` (default: the
    SHIOKAZE_REFERENCE environment variable); returns the harness path, or
    None where neither names a Shiokaze source tree and nothing was built
    before."""
    ref_dir = ref_dir or os.environ.get("SHIOKAZE_REFERENCE")
    if not ref_dir or not os.path.isdir(os.path.join(ref_dir, "src", "projection")):
        return REF_SO if os.path.exists(REF_SO) else None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={ref_dir}", f"-j{jobs}"],
                          stdout=subprocess.DEVNULL)
    with open(os.path.join(REF_DIR, "SOURCES"), "w") as f:
        f.write(os.path.abspath(ref_dir) + "\n")
    return REF_SO


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def reference_sources() -> str | None:
    """The Shiokaze source tree the reference build was made from (its
    headers also build the plugin modules), or None."""
    try:
        with open(os.path.join(REF_DIR, "SOURCES")) as f:
            path = f.read().strip()
        return path if os.path.isdir(path) else None
    except OSError:
        return None


def build_modules(out: str, *targets: str, ldflags: str | None = None) -> None:
    """Builds the plugin modules (shiokaze_gb300/module/Makefile) into `out`
    against the headers of the reference build's source tree."""
    src = reference_sources()
    if not src:
        raise RuntimeError("reference sources unknown: build the reference first (oracle.build_reference)")
    cmd = ["make", "-s", "-C", os.path.join(os.path.dirname(HERE), "shiokaze_gb300", "module"), f"SHIOKAZE={src}",
           f"OUT={out}"]
    if ldflags is not None:
        cmd += ["-B", f"LDFLAGS={ldflags}"]
    subprocess.check_call(cmd + list(targets), stdout=subprocess.DEVNULL)


class _Params(ctypes.Structure):
    _fields_ = [("residual", ctypes.c_double), ("max_iterations", ctypes.c_int), ("warm_start", ctypes.c_int),
                ("eps_fluid", ctypes.c_double), ("eps_solid", ctypes.c_double),
                ("second_order_fluid", ctypes.c_int), ("second_order_solid", ctypes.c_int),
                ("gain", ctypes.c_double), ("surface_tension", ctypes.c_double)]


class _Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("reresid", ctypes.c_double),
                ("unknowns", ctypes.c_longlong), ("b_inf", ctypes.c_double)]


@dataclass
class Result:
    pressure: np.ndarray
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray | None
    unknown: np.ndarray  # bool per cell
    iterations: int
    reresid: float
    ms: float = 0.0
    index: np.ndarray | None = None
    # per face component, 1 where the projection leaves the face active, 0
    # where the reference deactivates it (set_off); None if not asked for
    active: tuple | None = None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t=ctypes.c_float):
    return a.ctypes.data_as(ctypes.POINTER(t)) if a is not None else None


_port = None


def _port_lib():
    global _port
    if _port is None:
        lib = ctypes.CDLL(build_port())
        lib.oracle_create.restype = ctypes.c_void_p
        lib.oracle_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        lib.oracle_destroy.argtypes = [ctypes.c_void_p]
        lib.oracle_set_target_volume.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        lp = ctypes.POINTER(ctypes.c_longlong)
        lib.oracle_set_threads.argtypes = [ctypes.c_int]
        lib.oracle_project.argtypes = [ctypes.c_void_p, ctypes.c_double, fp, fp, fp, fp, fp,
                                       ctypes.POINTER(_Params), fp, lp, ctypes.POINTER(_Stats)]
        u8 = ctypes.POINTER(ctypes.c_ubyte)
        lib.oracle_project_active.argtypes = [ctypes.c_void_p, ctypes.c_double, fp, fp, fp, fp, fp,
                                              ctypes.POINTER(_Params), fp, lp, ctypes.POINTER(_Stats), u8, u8, u8]
        lib.oracle_assemble.argtypes = [ctypes.c_void_p, ctypes.c_double, fp, fp, fp, fp, fp,
                                        ctypes.POINTER(_Params), dp, dp, dp, dp, dp, lp]
        lib.oracle_face_fractions.argtypes = [ctypes.c_void_p, fp, fp, ctypes.POINTER(_Params), fp, fp, fp, fp, fp,
                                              fp]
        lib.oracle_advect3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, fp, fp, fp, fp, fp, ctypes.POINTER(ctypes.c_ubyte),
                                       ctypes.c_float]
        lib.oracle_advect2.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_int, fp, fp, fp, fp, ctypes.POINTER(ctypes.c_ubyte), ctypes.c_float]
        u8 = ctypes.POINTER(ctypes.c_ubyte)
        lib.oracle_extrapolate3.restype = ctypes.c_longlong
        lib.oracle_extrapolate3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, u8, ctypes.c_int]
        lib.oracle_constrain_velocity3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, fp, fp,
                                                   fp, fp, u8, u8, u8]
        _port = lib
    return _port


def set_threads(n: int | None = None) -> int:
    """Threads for the element-wise loops of the oracle's CG (matrix-vector
    product, vector updates, maximum norm); its dot products stay serial in
    index order, so results are bit-identical for every count. None: all
    host cores. Returns the count set."""
    n = int(n or os.cpu_count() or 1)
    _port_lib().oracle_set_threads(n)
    return n


def make_params(residual=1e-6, max_iterations=30000, warm_start=False, eps_fluid=1e-2, eps_solid=1e-2,
                second_order_fluid=True, second_order_solid=True, gain=1.0, surface_tension=0.0):
    return _Params(residual, max_iterations, int(warm_start), eps_fluid, eps_solid, int(second_order_fluid),
                   int(second_order_solid), gain, surface_tension)


class PortProjector:
    """The C restatement, one context per scene shape (holds warm-start state)."""

    def __init__(self, dim, nx, ny, nz, dx, **params):
        self.lib = _port_lib()
        self.dim, self.nx, self.ny, self.nz, self.dx = dim, nx, ny, (nz if dim == 3 else 1), dx
        self.params = make_params(**params)
        self.ctx = self.lib.oracle_create(dim, nx, ny, self.nz, dx)

    def close(self):
        if self.ctx:
            self.lib.oracle_destroy(self.ctx)
            self.ctx = None

    __del__ = close

    def set_target_volume(self, current, target):
        self.lib.oracle_set_target_volume(self.ctx, current, target)

    def project(self, dt, solid, fluid, u, v, w=None) -> Result:
        u, v = _f32(u).copy(), _f32(v).copy()
        w = _f32(w).copy() if w is not None else None
        solid, fluid = _f32(solid), _f32(fluid)
        p = np.zeros(fluid.shape, np.float32)
        idx = np.zeros(fluid.shape, np.int64)
        st = _Stats()
        on = [np.zeros(a.shape, np.uint8) for a in (u, v, w) if a is not None]
        u8 = ctypes.c_ubyte
        self.lib.oracle_project_active(self.ctx, dt, _ptr(solid), _ptr(fluid), _ptr(u), _ptr(v), _ptr(w),
                                       ctypes.byref(self.params), _ptr(p), _ptr(idx, ctypes.c_longlong),
                                       ctypes.byref(st), *[_ptr(a, u8) for a in on],
                                       *([None] if w is None else []))
        return Result(p, u, v, w, idx >= 0, st.iterations, st.reresid, index=idx,
                      active=tuple(a.astype(bool) for a in on))

    def face_fractions(self, solid, fluid):
        """Open area and fluid fraction of every face (float32, shaped like
        the velocity components), as the projection computes them
        (macutility3.cpp:94-194 with this projector's eps and order flags)."""
        solid, fluid = _f32(solid), _f32(fluid)
        shapes = ([(self.nz, self.ny, self.nx + 1), (self.nz, self.ny + 1, self.nx), (self.nz + 1, self.ny, self.nx)]
                  if self.dim == 3 else [(self.ny, self.nx + 1), (self.ny + 1, self.nx)])
        area = [np.zeros(sh, np.float32) for sh in shapes]
        rho = [np.zeros(sh, np.float32) for sh in shapes]
        pa = [_ptr(a) for a in area] + [None] * (3 - self.dim)
        pr = [_ptr(a) for a in rho] + [None] * (3 - self.dim)
        self.lib.oracle_face_fractions(self.ctx, _ptr(solid), _ptr(fluid), ctypes.byref(self.params), *pa, *pr)
        return area, rho

    def assemble(self, dt, solid, fluid, u, v, w=None):
        solid, fluid, u, v = _f32(solid), _f32(fluid), _f32(u), _f32(v)
        w = _f32(w) if w is not None else None
        shp = fluid.shape
        out = [np.zeros(shp, np.float64) for _ in range(5)]
        idx = np.zeros(shp, np.int64)
        dp = ctypes.c_double
        self.lib.oracle_assemble(self.ctx, dt, _ptr(solid), _ptr(fluid), _ptr(u), _ptr(v), _ptr(w),
                                 ctypes.byref(self.params), *[_ptr(o, dp) for o in out],
                                 _ptr(idx, ctypes.c_longlong))
        diag, cpx, cpy, cpz, b = out
        return {"diag": diag, "cpx": cpx, "cpy": cpy, "cpz": cpz, "b": b, "index": idx}


_ref = None


def _ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise RuntimeError("reference oracle not built (oracle/ref/Makefile needs the reference sources)")
        lib = ctypes.CDLL(REF_SO, mode=ctypes.RTLD_GLOBAL)
        fp = ctypes.POINTER(ctypes.c_float)
        lib.ref_create.restype = ctypes.c_void_p
        lib.ref_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_char_p, ctypes.c_char_p]
        lib.ref_destroy.argtypes = [ctypes.c_void_p]
        lib.ref_set_target_volume.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        lib.ref_project.restype = ctypes.c_double
        u8p = ctypes.POINTER(ctypes.c_ubyte)
        lib.ref_project.argtypes = [ctypes.c_void_p, ctypes.c_double, fp, ctypes.c_int, ctypes.c_float, fp,
                                    ctypes.c_int, ctypes.c_float, fp, fp, fp, ctypes.c_double, fp,
                                    u8p, u8p, u8p, u8p, ctypes.c_char_p]
        lib.ref_levelset_roundtrip.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp,
                                               ctypes.c_int, ctypes.c_float, fp]
        dp = ctypes.POINTER(ctypes.c_double)
        lib.ref_advect_load.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_char_p,
                                        ctypes.c_char_p]
        lib.ref_advect2.restype = ctypes.c_double
        lib.ref_advect2.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_char_p,
                                    fp, fp, fp, ctypes.c_int, ctypes.c_float, fp, ctypes.POINTER(ctypes.c_ubyte),
                                    ctypes.c_float, ctypes.c_char_p]
        lib.ref_advect2_load.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_char_p,
                                         ctypes.c_char_p]
        lib.ref_advect3.restype = ctypes.c_double
        lib.ref_advect3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_char_p, fp, fp, fp, fp, ctypes.c_int, ctypes.c_float, fp,
                                    ctypes.POINTER(ctypes.c_ubyte), ctypes.c_float, ctypes.c_char_p]
        u8 = ctypes.POINTER(ctypes.c_ubyte)
        lib.ref_extrapolate3.restype = ctypes.c_longlong
        lib.ref_extrapolate3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, u8, ctypes.c_int]
        lib.ref_constrain3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_char_p,
                                       fp, ctypes.c_int, ctypes.c_float, fp, fp, fp, u8, u8, u8, ctypes.c_char_p]
        lib.ref_extrapolate_constrain3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                   ctypes.c_char_p, fp, ctypes.c_int, ctypes.c_float, fp, fp, fp,
                                                   u8, u8, u8, ctypes.c_int, ctypes.c_char_p]
        lib.ref_densify_compare.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int,
                                            ctypes.c_float, ctypes.c_int, fp, fp, dp, dp]
        lib.ref_bricks_compare.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, ctypes.c_int, ctypes.c_float,
                                           fp, fp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int),
                                           fp, fp]
        _ref = lib
    return _ref


def ref_densify_compare(values: np.ndarray, mode: int, band: float, reps: int = 1):
    """The plugin modules' dense copy of a reference array (gbarray_adapter.h)
    and a read of every cell through the reference's operator(), for an array
    built from `values` (z, y, x or y, x; x fastest) as a narrow-band level set
    (mode 0), a constant (mode 1) or a partly active velocity component with
    background `band` (mode 2). Returns (adapter, lookup, ms_adapter,
    ms_lookup), the times the best of `reps`."""
    lib = _ref_lib()
    v = np.ascontiguousarray(values, dtype=np.float32)
    dim = v.ndim
    sx, sy, sz = (v.shape[2], v.shape[1], v.shape[0]) if dim == 3 else (v.shape[1], v.shape[0], 1)
    fp = ctypes.POINTER(ctypes.c_float)
    a, b = np.empty_like(v), np.empty_like(v)
    ma, ml = ctypes.c_double(), ctypes.c_double()
    lib.ref_densify_compare(dim, sx, sy, sz, v.ctypes.data_as(fp), mode, band, reps, a.ctypes.data_as(fp),
                            b.ctypes.data_as(fp), ctypes.byref(ma), ctypes.byref(ml))
    return a, b, ma.value, ml.value


def ref_bricks_compare(values: np.ndarray, mode: int, band: float):
    """The plugin modules' bricks (gbarray_adapter.h to_bricks) of a 3D
    reference array built as in ref_densify_compare. Returns (expanded,
    lookup, counts, slot, listed_values, background, fill): the bricks
    expanded by gbp.h's rule, operator()'s reads, the (listed, fill,
    background) brick counts, and the bricks themselves."""
    lib = _ref_lib()
    v = np.ascontiguousarray(values, dtype=np.float32)
    sz, sy, sx = v.shape
    nb = ((sx + 7) // 8) * ((sy + 7) // 8) * ((sz + 7) // 8)
    fp = ctypes.POINTER(ctypes.c_float)
    a, b = np.empty_like(v), np.empty_like(v)
    counts = np.zeros(3, np.int64)
    slot = np.zeros(nb, np.int32)
    vals = np.zeros(nb * 512, np.float32)
    bgf = np.zeros(2, np.float32)
    lib.ref_bricks_compare(sx, sy, sz, v.ctypes.data_as(fp), mode, ctypes.c_float(band), a.ctypes.data_as(fp),
                           b.ctypes.data_as(fp), counts.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                           slot.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), vals.ctypes.data_as(fp),
                           bgf.ctypes.data_as(fp))
    return a, b, counts, slot, vals[: int(counts[0]) * 512].copy(), float(bgf[0]), float(bgf[1])


def advect3(u, v, w, fluid, dx, dt, q=None, q_mask=None, q_bg=0.0, maccormack=True, trim_narrowband=1,
            impl="port", fluid_mode=0, band=0.0):
    """macsmoke3's advection step (the scalar q, if given, by the velocity,
    then the velocity by itself) on dense 3D arrays (z, y, x), by the C
    restatement (impl "port") or the reference's own module ("reference";
    fluid_mode / band say how it builds its fluid array). Returns (u, v, w,
    q, ms) as new arrays."""
    if impl == "reference":
        return ref_advect3(u, v, w, fluid, fluid_mode, band, dx, dt, q=q, q_mask=q_mask, q_bg=q_bg,
                           maccormack=maccormack, trim_narrowband=trim_narrowband)
    lib = _port_lib()
    fp = ctypes.POINTER(ctypes.c_float)
    nz, ny, nx = fluid.shape
    uo, vo, wo = (np.array(a, dtype=np.float32, order="C") for a in (u, v, w))
    fl = np.ascontiguousarray(fluid, dtype=np.float32)
    qo = None if q is None else np.array(q, dtype=np.float32, order="C")
    qm = None if q_mask is None else np.ascontiguousarray(q_mask, dtype=np.uint8)
    t0 = time.perf_counter()
    rc = lib.oracle_advect3(nx, ny, nz, dx, dt, int(maccormack), int(trim_narrowband), uo.ctypes.data_as(fp),
                            vo.ctypes.data_as(fp), wo.ctypes.data_as(fp), fl.ctypes.data_as(fp),
                            None if qo is None else qo.ctypes.data_as(fp),
                            None if qm is None else qm.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), q_bg)
    ms = 1000.0 * (time.perf_counter() - t0)
    if rc:
        raise ValueError("oracle_advect3: grid too small")
    return uo, vo, wo, qo, ms


def advect2(u, v, fluid, dx, dt, q=None, q_mask=None, q_bg=0.0, maccormack=True, trim_narrowband=1, impl="port",
            fluid_mode=0, band=0.0, extra_kv=""):
    """macsmoke2's advection step on dense 2D arrays (y, x): the scalar q (if
    given) by the velocity, then the velocity by itself, by the C
    restatement ("port") or the reference's own macadvection2
    ("reference"; fluid_mode / band say how it builds its fluid array,
    extra_kv adds configuration). Returns (u, v, q, ms) as new arrays."""
    fp = ctypes.POINTER(ctypes.c_float)
    ny, nx = fluid.shape
    uo, vo = (np.array(a, dtype=np.float32, order="C") for a in (u, v))
    fl = np.ascontiguousarray(fluid, dtype=np.float32)
    qo = None if q is None else np.array(q, dtype=np.float32, order="C")
    qm = None if q_mask is None else np.ascontiguousarray(q_mask, dtype=np.uint8)
    qp = None if qo is None else qo.ctypes.data_as(fp)
    if impl == "reference":
        lib = _ref_lib()
        kv = f"MacCormack={'Yes' if maccormack else 'No'} TrimNarrowBand={int(trim_narrowband)} {extra_kv}".strip()
        log = tempfile.NamedTemporaryFile(prefix="ref_advect_", suffix=".log", delete=False).name
        try:
            ms = lib.ref_advect2(nx, ny, dx, dt, kv.encode(), uo.ctypes.data_as(fp), vo.ctypes.data_as(fp),
                                 fl.ctypes.data_as(fp), fluid_mode, band, qp, _u8p(qm), q_bg, log.encode())
        finally:
            os.unlink(log)
        return uo, vo, qo, ms
    lib = _port_lib()
    t0 = time.perf_counter()
    rc = lib.oracle_advect2(nx, ny, dx, dt, int(maccormack), int(trim_narrowband), uo.ctypes.data_as(fp),
                            vo.ctypes.data_as(fp), fl.ctypes.data_as(fp), qp, _u8p(qm), q_bg)
    ms = 1000.0 * (time.perf_counter() - t0)
    if rc:
        raise ValueError("oracle_advect2: grid too small")
    return uo, vo, qo, ms


def _u8p(m):
    return None if m is None else m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))


def constrain3(solid, u, v, w, dx, masks=(None, None, None), impl="port", solid_mode=0, band=0.0, extra_kv=""):
    """macutility3::constrain_velocity (src/utility/macutility3.cpp:61-86)
    on dense 3D arrays (z, y, x): solid nodal, u, v, w faces (holding the
    velocity's background, 0, on inactive faces), updated where the
    component's mask is nonzero (all faces for None). By the C restatement
    ("port") or the reference's own macutility3 ("reference"; solid_mode /
    band say how it builds its solid array; extra_kv adds configuration,
    MacUtility=<module> loads another module). Returns new (u, v, w)."""
    fp = ctypes.POINTER(ctypes.c_float)
    nz, ny, nx = (d - 1 for d in solid.shape)
    uo, vo, wo = (np.array(a, dtype=np.float32, order="C") for a in (u, v, w))
    sl = np.ascontiguousarray(solid, dtype=np.float32)
    ms = [None if m is None else np.ascontiguousarray(m, dtype=np.uint8) for m in masks]
    if impl == "reference":
        lib = _ref_lib()
        log = tempfile.NamedTemporaryFile(prefix="ref_constrain_", suffix=".log", delete=False).name
        try:
            lib.ref_constrain3(nx, ny, nz, dx, extra_kv.encode(), sl.ctypes.data_as(fp), solid_mode, band, uo.ctypes.data_as(fp),
                               vo.ctypes.data_as(fp), wo.ctypes.data_as(fp), *[_u8p(m) for m in ms], log.encode())
        finally:
            os.unlink(log)
    else:
        rc = _port_lib().oracle_constrain_velocity3(nx, ny, nz, dx, sl.ctypes.data_as(fp), uo.ctypes.data_as(fp),
                                                    vo.ctypes.data_as(fp), wo.ctypes.data_as(fp),
                                                    *[_u8p(m) for m in ms])
        if rc:
            raise ValueError("oracle_constrain_velocity3: grid too small")
    return uo, vo, wo


def extrapolate_constrain3(solid, u, v, w, dx, masks, width, impl="port", solid_mode=0, band=0.0, extra_kv=""):
    """macutility3::extrapolate_and_constrain_velocity: each velocity
    component extrapolated `width` rounds over its active faces (masks),
    then the solid constraint over the grown sets. Inactive faces hold 0.
    Returns (u, v, w, masks). port: oracle_extrapolate3 per component, then
    oracle_constrain_velocity3; reference: the reference's module through
    its loader (extra_kv may select another MacUtility module)."""
    comps = [np.array(a, dtype=np.float32, order="C") for a in (u, v, w)]
    ms = [np.array(m, dtype=np.uint8, order="C") for m in masks]
    sl = np.ascontiguousarray(solid, dtype=np.float32)
    nz, ny, nx = (d - 1 for d in sl.shape)
    u8 = ctypes.c_ubyte
    if impl == "reference":
        lib = _ref_lib()
        log = tempfile.NamedTemporaryFile(prefix="ref_extc_", suffix=".log", delete=False).name
        try:
            lib.ref_extrapolate_constrain3(nx, ny, nz, dx, extra_kv.encode(), _ptr(sl), solid_mode, band,
                                           *[_ptr(c) for c in comps], *[_ptr(m, u8) for m in ms], int(width),
                                           log.encode())
        finally:
            os.unlink(log)
        return comps[0], comps[1], comps[2], tuple(ms)
    lib = _port_lib()
    for c, m in zip(comps, ms):
        d, h, wd = c.shape
        lib.oracle_extrapolate3(wd, h, d, _ptr(c), _ptr(m, u8), int(width))
    lib.oracle_constrain_velocity3(nx, ny, nz, dx, _ptr(sl), *[_ptr(c) for c in comps], *[_ptr(m, u8) for m in ms])
    return comps[0], comps[1], comps[2], tuple(ms)


def extrapolate3(values, active, count=1, impl="port"):
    """array_extrapolator3::extrapolate (include/shiokaze/array/
    array_extrapolator3.h:36-73) on a dense 3D array (z, y, x) with an
    active mask: `count` rounds of activating every inactive neighbour of an
    active cell with the float mean of its active neighbours. By the C
    restatement ("port") or the reference's own code ("reference"). Returns
    (values as read back, 0 on inactive cells; active; cells activated)."""
    d, h, w = values.shape
    a = np.array(values, dtype=np.float32, order="C")
    m = np.array(active, dtype=np.uint8, order="C")
    lib = _ref_lib() if impl == "reference" else _port_lib()
    fn = lib.ref_extrapolate3 if impl == "reference" else lib.oracle_extrapolate3
    added = fn(w, h, d, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
               int(count))
    a = np.where(m != 0, a, np.float32(0)).astype(np.float32)  # inactive cells read the background, 0
    return a, m, int(added)


def ref_advect3(u, v, w, fluid, fluid_mode, band, dx, dt, q=None, q_mask=None, q_bg=0.0, maccormack=True,
                trim_narrowband=1, extra_kv=""):
    """The reference's own macadvection3 on dense 3D arrays (arrays z, y, x;
    every velocity face active): the scalar q (if given; active where q_mask,
    all if None) advected by the velocity, then the velocity by itself, as
    macsmoke3::idle does. extra_kv adds configuration (Advection=<module>
    loads another module through the reference's loader). Returns (u, v, w,
    q, ms) as new arrays."""
    lib = _ref_lib()
    fp = ctypes.POINTER(ctypes.c_float)
    nz, ny, nx = fluid.shape
    uo, vo, wo = (np.array(a, dtype=np.float32, order="C") for a in (u, v, w))
    fl = np.ascontiguousarray(fluid, dtype=np.float32)
    qo = None if q is None else np.array(q, dtype=np.float32, order="C")
    qm = None if q_mask is None else np.ascontiguousarray(q_mask, dtype=np.uint8)
    kv = f"MacCormack={'Yes' if maccormack else 'No'} TrimNarrowBand={int(trim_narrowband)} {extra_kv}".strip()
    log = tempfile.NamedTemporaryFile(prefix="ref_advect_", suffix=".log", delete=False).name
    try:
        ms = lib.ref_advect3(nx, ny, nz, dx, dt, kv.encode(), uo.ctypes.data_as(fp), vo.ctypes.data_as(fp),
                             wo.ctypes.data_as(fp), fl.ctypes.data_as(fp), fluid_mode, band,
                             None if qo is None else qo.ctypes.data_as(fp),
                             None if qm is None else qm.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), q_bg,
                             log.encode())
    finally:
        os.unlink(log)
    return uo, vo, wo, qo, ms


_ITER_RE = re.compile(r"Took (\d+) iterations, Reresid=([0-9][0-9.eE+\-]*[0-9]|nan|inf)")


class RefProjector:
    """The reference's own macpressuresolver{2,3}, loaded by name."""

    def __init__(self, dim, nx, ny, nz, dx, residual=1e-6, max_iterations=30000, warm_start=False, eps_fluid=1e-2,
                 eps_solid=1e-2, second_order_fluid=True, second_order_solid=True, gain=1.0, surface_tension=0.0,
                 threads=None, extra_kv=""):
        self.lib = _ref_lib()
        self.surface_tension = float(surface_tension)  # project()'s argument, not a configuration key
        self.dim, self.nx, self.ny, self.nz, self.dx = dim, nx, ny, (nz if dim == 3 else 1), dx
        kv = (f"Residual={residual!r} MaxIterations={max_iterations} WarmStart={'Yes' if warm_start else 'No'} "
              f"EpsFluid={eps_fluid!r} EpsSolid={eps_solid!r} "
              f"SecondOrderAccurateFluid={'Yes' if second_order_fluid else 'No'} "
              f"SecondOrderAccurateSolid={'Yes' if second_order_solid else 'No'} Gain={gain!r}")
        if threads:
            kv += f" Threads={threads}"
        if extra_kv:
            kv += " " + extra_kv
        self._log = tempfile.NamedTemporaryFile(prefix="ref_project_", suffix=".log", delete=False).name
        self.ctx = self.lib.ref_create(dim, nx, ny, self.nz, dx, kv.encode(), self._log.encode())

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.ref_destroy(self.ctx)
            self.ctx = None
            try:
                os.unlink(self._log)
            except OSError:
                pass

    __del__ = close

    def set_target_volume(self, current, target):
        self.lib.ref_set_target_volume(self.ctx, current, target)

    def project(self, dt, solid, fluid, u, v, w=None, solid_mode=0, fluid_mode=0, band=None) -> Result:
        if band is None:
            band = float(np.float32(np.sqrt(3.0) * self.dx))
        u, v = _f32(u).copy(), _f32(v).copy()
        w = _f32(w).copy() if w is not None else None
        solid, fluid = _f32(solid), _f32(fluid)
        p = np.zeros(fluid.shape, np.float32)
        act = np.zeros(fluid.shape, np.uint8)
        on = [None if a is None else np.zeros(a.shape, np.uint8) for a in (u, v, w)]
        open(self._log, "w").close()
        u8 = ctypes.c_ubyte
        ms = self.lib.ref_project(self.ctx, dt, _ptr(solid), solid_mode, band, _ptr(fluid), fluid_mode, band,
                                  _ptr(u), _ptr(v), _ptr(w), self.surface_tension, _ptr(p),
                                  _ptr(act, u8), *[_ptr(a, u8) for a in on], self._log.encode())
        with open(self._log, errors="replace") as f:
            log = f.read()
        m = _ITER_RE.findall(log)
        iters, rr = (int(m[-1][0]), float(m[-1][1])) if m else (-1, float("nan"))
        return Result(p, u, v, w, act.astype(bool), iters, rr, ms=ms,
                      active=tuple(a.astype(bool) for a in on if a is not None))


def divergence(area, velocity, dx, unknown):
    """max over the unknown cells of |sum over faces of sgn area u / dx| (the
    discrete divergence the projection removes: the right-hand side of its
    system with the sign flipped, macpressuresolver3.cpp:190-197), in FP64."""
    div = np.zeros(unknown.shape, np.float64)
    for d in range(len(velocity)):
        f = area[d].astype(np.float64) * velocity[d].astype(np.float64).reshape(area[d].shape)
        f = f.reshape(f.shape[:0] + (1,) * (unknown.ndim - f.ndim) + f.shape)
        nd = f.ndim
        ax = nd - 1 - d  # numpy axis of direction d (arrays are (z,) y, x, x fastest)
        hi = [slice(None)] * nd
        lo = [slice(None)] * nd
        hi[ax] = slice(1, None)
        lo[ax] = slice(None, -1)
        div += f[tuple(hi)] - f[tuple(lo)]
    div /= dx
    return float(np.max(np.abs(div[unknown]))) if unknown.any() else 0.0


def project_scene(scene, impl="port", **params) -> Result:
    """One projection of a ``shiokaze_gb300.scenes.Scene`` on the CPU."""
    if impl == "port":
        pj = PortProjector(scene.dim, scene.nx, scene.ny, scene.nz, scene.dx, **params)
        try:
            return pj.project(scene.dt, scene.solid, scene.fluid, scene.u, scene.v, scene.w)
        finally:
            pj.close()
    pj = RefProjector(scene.dim, scene.nx, scene.ny, scene.nz, scene.dx, **params)
    try:
        return pj.project(scene.dt, scene.solid, scene.fluid, scene.u, scene.v, scene.w, scene.solid_mode,
                          scene.fluid_mode, scene.band)
    finally:
        pj.close()
