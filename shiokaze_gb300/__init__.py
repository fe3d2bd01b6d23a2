"""GB300 pressure projection for Shiokaze scenes.

Python mirror of the reference's projection plugin interface
(``include/shiokaze/projection/macproject3_interface.h:38-99``,
``macproject2_interface.h``), on top of the C ABI in ``include/gbp.h``
(``libgbp.so``, hand-written sm_103a CUDA kernels):

    proj = MacProject3(nx, ny, nz, dx, Residual=1e-6)     # initialize(shape, dx)
    proj.project(dt, (u, v, w), solid, fluid)             # in place on u, v, w
    p = proj.get_pressure()

Configuration keys are the reference's (``Residual``, ``MaxIterations``,
``WarmStart``, ``EpsFluid``, ``EpsSolid``, ``SecondOrderAccurateFluid``,
``SecondOrderAccurateSolid``, ``Gain``) plus this module's own
(``Solver`` = "cg" | "mgpcg", ``Precision`` = "fp64" | "mixed",
``MGSmooth``, ``MGCoarsest``, ``InnerTolerance``, ``IterationsPerSync``,
``TMAStaging``, ``TileClasses``), and
``SurfaceTension``, the value the reference passes as project()'s
surface_tension argument.

Arrays may be numpy arrays (host; copied in and out by the call) or torch
CUDA tensors (device; used in place). There is no CPU fallback: without the
built library every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbp.so")

# status codes of include/gbp.h
GBP_OK = 0
GBP_ERR_INVALID_ARGUMENT = 1
GBP_ERR_CUDA = 2
GBP_ERR_OUT_OF_MEMORY = 3
GBP_ERR_NOT_CONVERGED = 4
GBP_ERR_NAN = 5
GBP_ERR_NO_DEVICE = 6
GBP_ERR_BUDGET = 7
GBP_ERR_TIMEOUT = 8
SOLVER_CG, SOLVER_MGPCG = 0, 1
PRECISION_FP64, PRECISION_MIXED = 0, 1


class Params(ctypes.Structure):
    _fields_ = [("residual", ctypes.c_double), ("max_iterations", ctypes.c_int), ("warm_start", ctypes.c_int),
                ("eps_fluid", ctypes.c_double), ("eps_solid", ctypes.c_double),
                ("second_order_fluid", ctypes.c_int), ("second_order_solid", ctypes.c_int),
                ("gain", ctypes.c_double), ("solver", ctypes.c_int), ("precision", ctypes.c_int),
                ("mg_smooth", ctypes.c_int), ("mg_coarsest", ctypes.c_int), ("inner_tolerance", ctypes.c_double),
                ("iterations_per_sync", ctypes.c_int), ("surface_tension", ctypes.c_double),
                ("tma_staging", ctypes.c_int), ("tile_classes", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("outer_iterations", ctypes.c_int), ("converged", ctypes.c_int),
                ("reresid", ctypes.c_double), ("true_resid_inf", ctypes.c_double),
                ("true_resid_l2", ctypes.c_double), ("b_inf", ctypes.c_double), ("unknowns", ctypes.c_longlong),
                ("ms_assemble", ctypes.c_float), ("ms_solve", ctypes.c_float), ("ms_update", ctypes.c_float),
                ("ms_total", ctypes.c_float), ("tma_staged", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class CsrStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("reresid", ctypes.c_double),
                ("ms_solve", ctypes.c_float), ("ms_total", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdvectParams(ctypes.Structure):
    _fields_ = [("maccormack", ctypes.c_int), ("trim_narrowband", ctypes.c_int), ("advect_velocity", ctypes.c_int)]


class Bricks(ctypes.Structure):
    """gbp_bricks: a sparse 3D array in bricks of 8^3 cells (include/gbp.h)."""
    _fields_ = [("background", ctypes.c_float), ("fill", ctypes.c_float), ("slot", ctypes.POINTER(ctypes.c_int)),
                ("count", ctypes.c_longlong), ("values", ctypes.POINTER(ctypes.c_float))]


class BricksOut(ctypes.Structure):
    """gbp_bricks_out: the bricks an output is copied back for."""
    _fields_ = [("slot", ctypes.POINTER(ctypes.c_int)), ("count", ctypes.c_longlong),
                ("values", ctypes.POINTER(ctypes.c_float)), ("active", ctypes.POINTER(ctypes.c_ubyte))]


BRICK = 8
BRICK_CELLS = 512
BRICK_BACKGROUND = -1
BRICK_FILL = -2


def _brick_view(a, fill_value=0):
    """(nbz, nby, nbx, 8, 8, 8) view of a 3D array padded to whole bricks."""
    nz, ny, nx = a.shape
    pz, py, px = (-nz) % 8, (-ny) % 8, (-nx) % 8
    p = np.pad(a, ((0, pz), (0, py), (0, px)), constant_values=fill_value)
    nbz, nby, nbx = p.shape[0] // 8, p.shape[1] // 8, p.shape[2] // 8
    return p.reshape(nbz, 8, nby, 8, nbx, 8).transpose(0, 2, 4, 1, 3, 5)


def to_bricks(values, active, filled=None, background=0.0, fill=0.0):
    """The bricks of a sparse 3D array given densely (z, y, x): cells where
    ``active`` read ``values``, other ``filled`` cells read ``fill``, the
    rest ``background`` (the reference's tiled-array rule). A brick with an
    active cell or some but not all cells filled is listed; one with every
    cell filled and none active is BRICK_FILL; the rest BRICK_BACKGROUND
    (the plugin modules' rule, gbarray_adapter.h). Returns (slot,
    listed_values, background, fill) and the dense array those bricks
    stand for."""
    values = np.asarray(values, np.float32)
    active = np.asarray(active, bool)
    filled = np.zeros_like(active) if filled is None else np.asarray(filled, bool)
    dense = np.where(active, values, np.where(filled, np.float32(fill), np.float32(background))).astype(np.float32)
    inside = _brick_view(np.ones(values.shape, bool), False)
    na = _brick_view(active, False).sum(axis=(3, 4, 5))
    nf = _brick_view(filled, False).sum(axis=(3, 4, 5))
    cells = inside.sum(axis=(3, 4, 5))
    listed = (na > 0) | ((nf > 0) & (nf < cells))
    slot = np.full(na.shape, BRICK_BACKGROUND, np.int32)
    slot[(na == 0) & (nf == cells)] = BRICK_FILL
    slot[listed] = np.arange(int(listed.sum()), dtype=np.int32)
    bv = _brick_view(dense, np.float32(background))
    listed_values = np.ascontiguousarray(bv[listed].reshape(-1), dtype=np.float32)
    return (np.ascontiguousarray(slot.reshape(-1)), listed_values, float(background), float(fill)), dense


def _bricks_struct(b):
    slot, vals, bg, fill = b
    return Bricks(bg, fill, slot.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(vals) // BRICK_CELLS,
                  vals.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))


def bricks_expand(nx, ny, nz, bricks, dense, context: "Context | None" = None, stream=None):
    """gbp_bricks_expand: ``dense`` (a contiguous float32 torch CUDA tensor
    of nz*ny*nx) receives the cell values of ``bricks`` (as to_bricks
    returns them)."""
    ctx = context or default_context()
    b = _bricks_struct(bricks)
    check(load_library().gbp_bricks_expand(ctx.handle, nx, ny, nz, ctypes.byref(b), dense.data_ptr(),
                                           ctypes.c_void_p(stream) if stream else None))


class GBPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gbp error {code}: {msg}")
        self.code = code


_lib = None
EXPORTED = ["gbp_params_default", "gbp_create", "gbp_destroy", "gbp_scene_create", "gbp_scene_destroy",
            "gbp_scene_device_bytes", "gbp_scene_set_target_volume", "gbp_project", "gbp_project_device",
            "gbp_debug_assemble", "gbp_bench_kernel", "gbp_launch_count", "gbp_strerror", "gbp_batch_create",
            "gbp_batch_destroy", "gbp_batch_project_device", "gbp_project_active", "gbp_project_bricks",
            "gbp_bricks_expand"]


def library_path() -> str:
    return LIB_PATH


def load_library():
    """Loads libgbp.so (building it first if sources are newer is the
    caller's job: ``python -m shiokaze_gb300.build``). Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run `python -m shiokaze_gb300.build` "
                          "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    vp, fp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double)
    lib.gbp_params_default.argtypes = [ctypes.POINTER(Params)]
    lib.gbp_params_default.restype = None
    lib.gbp_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
    lib.gbp_destroy.argtypes = [vp]
    lib.gbp_destroy.restype = None
    lib.gbp_scene_create.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.POINTER(vp)]
    lib.gbp_scene_destroy.argtypes = [vp]
    lib.gbp_scene_destroy.restype = None
    lib.gbp_scene_device_bytes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(Params)]
    lib.gbp_scene_device_bytes.restype = ctypes.c_size_t
    lib.gbp_scene_set_target_volume.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    lib.gbp_project.argtypes = [vp, ctypes.c_double, fp, fp, fp, fp, fp, ctypes.POINTER(Params), fp,
                                ctypes.POINTER(Stats)]
    u8p = ctypes.POINTER(ctypes.c_ubyte)
    lib.gbp_project_active.argtypes = [vp, ctypes.c_double, fp, fp, fp, fp, fp, ctypes.POINTER(Params), fp,
                                       ctypes.POINTER(Stats), u8p, u8p, u8p, u8p]
    lib.gbp_project_device.argtypes = [vp, ctypes.c_double, vp, vp, vp, vp, vp, ctypes.POINTER(Params), vp,
                                       ctypes.POINTER(Stats), vp]
    lib.gbp_debug_assemble.argtypes = [vp, ctypes.c_double, fp, fp, fp, fp, fp, ctypes.POINTER(Params), dp, dp, dp,
                                       dp, dp]
    lib.gbp_bench_kernel.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, ctypes.POINTER(ctypes.c_float),
                                     ctypes.POINTER(ctypes.c_double)]
    lib.gbp_batch_create.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp)]
    lib.gbp_batch_destroy.argtypes = [vp]
    lib.gbp_batch_destroy.restype = None
    pp = ctypes.POINTER(vp)
    lib.gbp_batch_project_device.argtypes = [vp, ctypes.POINTER(ctypes.c_double), pp, pp, pp, pp, pp,
                                             ctypes.POINTER(Params), pp, ctypes.POINTER(Stats), vp]
    lp = ctypes.POINTER(ctypes.c_longlong)
    lib.gbp_csr_cg.argtypes = [vp, ctypes.c_longlong, lp, lp, dp, dp, dp, ctypes.c_double, ctypes.c_int,
                               ctypes.POINTER(CsrStats)]
    lib.gbp_advect_params_default.argtypes = [ctypes.POINTER(AdvectParams)]
    lib.gbp_advect_params_default.restype = None
    u8p = ctypes.POINTER(ctypes.c_ubyte)
    lib.gbp_advect3.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                ctypes.POINTER(AdvectParams), fp, fp, fp, fp, fp, u8p, ctypes.c_float]
    lib.gbp_advect3_device.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, ctypes.POINTER(AdvectParams), vp, vp, vp, vp, vp, vp,
                                       ctypes.c_float, vp]
    lib.gbp_advect2.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                ctypes.POINTER(AdvectParams), fp, fp, fp, fp, u8p, ctypes.c_float]
    lib.gbp_advect2_device.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                       ctypes.POINTER(AdvectParams), vp, vp, vp, vp, vp, ctypes.c_float, vp]
    lib.gbp_constrain_velocity3.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, fp, fp, fp,
                                            fp, u8p, u8p, u8p]
    lib.gbp_constrain_velocity3_device.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, vp,
                                                   vp, vp, vp, vp, vp, vp, vp]
    lib.gbp_extrapolate3.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, u8p, ctypes.c_int, lp]
    lib.gbp_extrapolate3_device.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, lp,
                                            vp]
    lib.gbp_extrapolate_constrain_velocity3.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                        ctypes.c_double, fp, fp, fp, fp, u8p, u8p, u8p, ctypes.c_int]
    lib.gbp_bricks_expand.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Bricks), vp, vp]
    bp, bo = ctypes.POINTER(Bricks), ctypes.POINTER(BricksOut)
    lib.gbp_project_bricks.argtypes = [vp, ctypes.c_double, bp, bp, bp, bp, bp, ctypes.POINTER(Params), bo, bo, bo, bo,
                                       ctypes.POINTER(Stats)]
    lib.gbp_launch_count.argtypes = [vp]
    lib.gbp_launch_count.restype = ctypes.c_longlong
    lib.gbp_strerror.argtypes = [ctypes.c_int]
    lib.gbp_strerror.restype = ctypes.c_char_p
    _lib = lib
    return lib


def check(rc: int, allow=(GBP_OK,)):
    if rc not in allow:
        raise GBPError(rc, load_library().gbp_strerror(rc).decode())
    return rc


def _flag(val) -> int:
    """A boolean key's value: bool, int, or the strings yes/no, true/false, 1/0."""
    if isinstance(val, str):
        low = val.strip().lower()
        if low in ("yes", "true", "1"):
            return 1
        if low in ("no", "false", "0"):
            return 0
        raise ValueError(f"not a boolean value: {val!r}")
    return 1 if val else 0


_KEYMAP = {
    "Residual": ("residual", float), "MaxIterations": ("max_iterations", int), "WarmStart": ("warm_start", _flag),
    "EpsFluid": ("eps_fluid", float), "EpsSolid": ("eps_solid", float),
    "SecondOrderAccurateFluid": ("second_order_fluid", _flag),
    "SecondOrderAccurateSolid": ("second_order_solid", _flag),
    "Gain": ("gain", float), "MGSmooth": ("mg_smooth", int), "MGCoarsest": ("mg_coarsest", int),
    "InnerTolerance": ("inner_tolerance", float), "IterationsPerSync": ("iterations_per_sync", int),
    "SurfaceTension": ("surface_tension", float), "TMAStaging": ("tma_staging", _flag),
    "TileClasses": ("tile_classes", _flag),
}


def make_params(**keys) -> Params:
    """Params from the reference's configuration keys (see module docstring)."""
    p = Params()
    load_library().gbp_params_default(ctypes.byref(p))
    for k, val in keys.items():
        if k == "Solver":
            p.solver = {"cg": SOLVER_CG, "pcg": SOLVER_CG, "mgpcg": SOLVER_MGPCG}[str(val).lower()]
        elif k == "Precision":
            p.precision = {"fp64": PRECISION_FP64, "mixed": PRECISION_MIXED}[str(val).lower()]
        elif k in _KEYMAP:
            name, conv = _KEYMAP[k]
            setattr(p, name, conv(val))
        else:
            raise KeyError(f"unknown configuration key {k}")
    return p


class Context:
    """A CUDA device context (stream, events) of libgbp."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        self.handle = ctypes.c_void_p()
        check(self.lib.gbp_create(device, ctypes.byref(self.handle)))

    def close(self):
        if self.handle:
            self.lib.gbp_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def launches(self) -> int:
        return int(self.lib.gbp_launch_count(self.handle))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def csr_cg(indptr, indices, data, b, residual=1e-4, max_iterations=30000, context: Context | None = None):
    """Solves A x = b for A in compressed rows (indptr, indices, data: the
    row pointers, column indices and values of a symmetric positive
    (semi)definite matrix) with the reference's LinSolver "pcg" algorithm
    (plain FP64 CG from x = 0, stop at |r|_inf <= residual |b|_inf) on the
    GPU. Returns (x, status, stats)."""
    ctx = context or default_context()
    lib = ctx.lib
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    ix = np.ascontiguousarray(indices, dtype=np.int64)
    va = np.ascontiguousarray(data, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    n = bb.shape[0]
    assert ip.shape[0] == n + 1, "indptr must have n + 1 entries"
    x = np.zeros(n, np.float64)
    st = CsrStats()
    lp = ctypes.POINTER(ctypes.c_longlong)
    dpp = ctypes.POINTER(ctypes.c_double)
    rc = lib.gbp_csr_cg(ctx.handle, n, ip.ctypes.data_as(lp), ix.ctypes.data_as(lp), va.ctypes.data_as(dpp),
                        bb.ctypes.data_as(dpp), x.ctypes.data_as(dpp), residual, max_iterations, ctypes.byref(st))
    check(rc, (GBP_OK, GBP_ERR_NOT_CONVERGED, GBP_ERR_NAN))
    return x, rc, st.as_dict()


def _host_f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class _MacProject:
    dim = 3

    def __init__(self, nx, ny, nz, dx, context: Context | None = None, **config):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self.nx, self.ny, self.nz = nx, ny, (nz if self.dim == 3 else 1)
        self.dx = dx
        self.config = dict(config)
        self.params = make_params(**self.config)
        self.scene = ctypes.c_void_p()
        check(self.lib.gbp_scene_create(self.ctx.handle, self.dim, nx, ny, self.nz, dx, ctypes.byref(self.scene)))
        self.pressure = None
        self.stats = Stats()
        # active sets of the last host call made with active_sets=True: the
        # unknown cells (the pressure's active cells in the reference) and,
        # per face component, the faces the velocity update leaves active
        self.unknown = None
        self.active = None

    def configure(self, **config):
        """Sets configuration keys (merged with the ones already set)."""
        self.config.update(config)
        self.params = make_params(**self.config)
        return self

    def close(self):
        if self.scene:
            self.lib.gbp_scene_destroy(self.scene)
            self.scene = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_target_volume(self, current_volume: float, target_volume: float):
        check(self.lib.gbp_scene_set_target_volume(self.scene, current_volume, target_volume))

    def get_pressure(self):
        return self.pressure

    def device_bytes(self) -> int:
        return int(self.lib.gbp_scene_device_bytes(self.dim, self.nx, self.ny, self.nz, ctypes.byref(self.params)))

    def project(self, dt, velocity, solid, fluid, pressure_out=None, stream=None, active_sets=False):
        """Projects ``velocity`` (tuple of face arrays) in place. numpy arrays
        go through the host call; torch CUDA tensors through the device call.
        Returns the status code (GBP_OK, or GBP_ERR_NOT_CONVERGED /
        GBP_ERR_NAN, after which the last iterate was still applied, as in
        the reference). With ``active_sets`` (host arrays) the call also
        fills ``self.unknown`` and ``self.active`` (gbp_project_active)."""
        comps = list(velocity) + [None] * (3 - len(velocity))
        u, v, w = comps[0], comps[1], comps[2] if self.dim == 3 else None
        if _is_torch_cuda(u):
            import torch
            if pressure_out is None:
                if self.pressure is None or not _is_torch_cuda(self.pressure):
                    self.pressure = torch.empty((self.nz, self.ny, self.nx) if self.dim == 3 else (self.ny, self.nx),
                                                dtype=torch.float32, device=u.device)
                pressure_out = self.pressure
            else:
                self.pressure = pressure_out
            for t in (u, v, w, solid, fluid, pressure_out):
                if t is not None:
                    assert t.dtype == torch.float32 and t.is_contiguous(), "device arrays must be contiguous float32"
            st = stream if stream is not None else torch.cuda.current_stream(u.device).cuda_stream
            rc = self.lib.gbp_project_device(self.scene, dt, solid.data_ptr(), fluid.data_ptr(), u.data_ptr(),
                                             v.data_ptr(), w.data_ptr() if w is not None else None, ctypes.byref(self.params),
                                             pressure_out.data_ptr(), ctypes.byref(self.stats), ctypes.c_void_p(st))
            return check(rc, (GBP_OK, GBP_ERR_NOT_CONVERGED, GBP_ERR_NAN))
        arrs = []
        for a in (u, v, w):
            if a is None:
                arrs.append((None, None))
            else:
                if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                    raise TypeError("host velocity components must be contiguous float32 numpy arrays (updated in place)")
                arrs.append((a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        solid_a, solid_p = _host_f32(solid)
        fluid_a, fluid_p = _host_f32(fluid)
        if self.pressure is None or not isinstance(self.pressure, np.ndarray):
            self.pressure = np.zeros(fluid_a.shape, np.float32)
        pp = self.pressure.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        if active_sets:
            self.unknown = np.zeros(fluid_a.shape, np.uint8)
            self.active = tuple(np.zeros(a.shape, np.uint8) for a, _ in arrs if a is not None)
            u8 = ctypes.POINTER(ctypes.c_ubyte)
            mp = [m.ctypes.data_as(u8) for m in (self.unknown,) + self.active] + [None] * (3 - self.dim)
            rc = self.lib.gbp_project_active(self.scene, dt, solid_p, fluid_p, arrs[0][1], arrs[1][1], arrs[2][1],
                                             ctypes.byref(self.params), pp, ctypes.byref(self.stats), *mp)
        else:
            rc = self.lib.gbp_project(self.scene, dt, solid_p, fluid_p, arrs[0][1], arrs[1][1], arrs[2][1],
                                      ctypes.byref(self.params), pp, ctypes.byref(self.stats))
        return check(rc, (GBP_OK, GBP_ERR_NOT_CONVERGED, GBP_ERR_NAN))

    def project_bricks(self, dt, solid, fluid, velocity, out_slots, outputs=None):
        """gbp_project_bricks (3D): inputs as to_bricks returns them (solid
        nodes, fluid cells, the three face components); out_slots: slot per
        brick (-1 = not copied out) for the pressure and u, v, w. Returns
        the status and, per output, (values, active) of its listed bricks;
        `outputs`, the list a previous call returned for the same slots, is
        written again instead of new arrays (as a caller keeps its buffers)."""
        ins = [_bricks_struct(b) for b in (solid, fluid) + tuple(velocity)]
        outs, keep = [], []
        for n, sl in enumerate(out_slots):
            sl = np.ascontiguousarray(sl, np.int32)
            count = int((sl >= 0).sum())
            if outputs is not None and outputs[n][0].size == count * BRICK_CELLS:
                vals, act = outputs[n]
            else:
                vals = np.zeros(count * BRICK_CELLS, np.float32)
                act = np.zeros(count * BRICK_CELLS, np.uint8)
            keep.append((sl, vals, act))
            outs.append(BricksOut(sl.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), count,
                                  vals.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                  act.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))))
        rc = self.lib.gbp_project_bricks(self.scene, dt, *[ctypes.byref(b) for b in ins], ctypes.byref(self.params),
                                         *[ctypes.byref(o) for o in outs], ctypes.byref(self.stats))
        return check(rc, (GBP_OK, GBP_ERR_NOT_CONVERGED, GBP_ERR_NAN)), [(v, a) for _, v, a in keep]

    def bench_kernel(self, which: int, reps: int = 20, stream=None):
        """Mean ms per launch and algorithmic bytes per launch of one kernel."""
        ms, nbytes = ctypes.c_float(), ctypes.c_double()
        check(self.lib.gbp_bench_kernel(self.scene, which, reps, ctypes.c_void_p(stream) if stream else None,
                                        ctypes.byref(ms), ctypes.byref(nbytes)))
        return float(ms.value), float(nbytes.value)

    def debug_assemble(self, dt, velocity, solid, fluid):
        """Operator and right-hand side as assembled on the device."""
        comps = list(velocity) + [None] * (3 - len(velocity))
        u, up = _host_f32(comps[0])
        v, vp = _host_f32(comps[1])
        w, wp = (None, None) if self.dim == 2 else _host_f32(comps[2])
        s, sp = _host_f32(solid)
        f, fp = _host_f32(fluid)
        out = [np.zeros(f.shape, np.float64) for _ in range(5)]
        ptrs = [o.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for o in out]
        if self.dim == 2:
            ptrs[3] = None
        check(self.lib.gbp_debug_assemble(self.scene, dt, sp, fp, up, vp, wp, ctypes.byref(self.params), *ptrs))
        return dict(zip(["diag", "cpx", "cpy", "cpz", "b"], out))


def _is_torch_cuda(a) -> bool:
    return type(a).__module__.startswith("torch") and getattr(a, "is_cuda", False)


class MacProject3(_MacProject):
    """macproject3_interface on the GPU (3D)."""
    dim = 3


class MacProject2(_MacProject):
    """macproject2_interface on the GPU (2D)."""
    dim = 2

    def __init__(self, nx, ny, dx, context: Context | None = None, **config):
        super().__init__(nx, ny, 1, dx, context, **config)


class Batch:
    """Many scenes projected together (gbp_batch_*): one launch per kernel
    per iteration for all of them. Each projector keeps its own state (warm
    start, volume correction); configuration comes from `config` and must
    select Solver="mgpcg"."""

    def __init__(self, projectors, context: Context | None = None, **config):
        self.ctx = context or projectors[0].ctx
        self.lib = self.ctx.lib
        self.projectors = list(projectors)
        self.config = dict(config)
        self.config.setdefault("Solver", "mgpcg")
        self.params = make_params(**self.config)
        n = len(self.projectors)
        arr = (ctypes.c_void_p * n)(*[pj.scene.value for pj in self.projectors])
        self.handle = ctypes.c_void_p()
        check(self.lib.gbp_batch_create(self.ctx.handle, n, arr, ctypes.byref(self.handle)))
        self.stats = (Stats * n)()

    def close(self):
        if self.handle:
            self.lib.gbp_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def project(self, dts, velocities, solids, fluids, pressures, stream=None):
        """Device (torch CUDA) arrays, one entry per scene; velocities are
        tuples (u, v[, w]) updated in place; pressures are outputs."""
        import torch
        n = len(self.projectors)
        V = ctypes.c_void_p

        def ptrs(items):
            return (V * n)(*[None if t is None else t.data_ptr() for t in items])
        u = ptrs([vel[0] for vel in velocities])
        v = ptrs([vel[1] for vel in velocities])
        w = ptrs([vel[2] if len(vel) > 2 else None for vel in velocities])
        dt = (ctypes.c_double * n)(*dts)
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        rc = self.lib.gbp_batch_project_device(self.handle, dt, ptrs(solids), ptrs(fluids), u, v, w,
                                               ctypes.byref(self.params), ptrs(pressures), self.stats, V(st))
        return check(rc, (GBP_OK, GBP_ERR_NOT_CONVERGED, GBP_ERR_NAN))


class MacAdvection3:
    """macadvection3_interface on the GPU
    (``include/shiokaze/advection/macadvection3_interface.h:36-88``, the
    reference's ``macadvection3`` module, ``src/advection/macadvection3.cpp``,
    with bilinear interpolation). Configuration keys: ``MacCormack``
    (default yes) and ``TrimNarrowBand`` (default 1); ``WENO`` is not
    available. Results equal the reference's bit for bit.

    Arrays are dense (z, y, x) float32: numpy arrays (copied in and out by
    the call) or torch CUDA tensors (used in place). Every velocity face is
    active; a scalar's inactive cells (``mask`` == 0) read and are written
    as ``background``."""

    def __init__(self, nx, ny, nz, dx, context: Context | None = None, **config):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self.nx, self.ny, self.nz, self.dx = nx, ny, nz, dx
        self.params = AdvectParams()
        self.lib.gbp_advect_params_default(ctypes.byref(self.params))
        self.configure(**config)

    def configure(self, **config):
        for k, val in config.items():
            if k == "MacCormack":
                self.params.maccormack = _flag(val)
            elif k == "TrimNarrowBand":
                self.params.trim_narrowband = int(val)
            elif k == "WENO":
                if _flag(val):
                    raise ValueError("WENO interpolation is not available")
            else:
                raise KeyError(f"unknown configuration key {k}")
        return self

    def advect_scalar(self, scalar, velocity, fluid, dt, mask=None, background=0.0, stream=None):
        """Carries the cell ``scalar`` (in place) by ``velocity`` (u, v, w)
        (advect_scalar, macadvection3.cpp:38-45)."""
        self._run(velocity, fluid, dt, scalar, mask, background, False, stream)

    def advect_vector(self, u, velocity, fluid, dt, stream=None):
        """Carries the face arrays ``u`` (in place). As in the reference
        (advect_u, macadvection3.cpp:136-180), the trace uses the full
        velocity of ``u`` itself; ``velocity`` is accepted for the
        interface's sake and must hold the same values when it differs from
        ``u`` (macsmoke3 passes a copy of u)."""
        self._run(u, fluid, dt, None, None, 0.0, True, stream)

    def advect_step(self, velocity, fluid, dt, scalar=None, mask=None, background=0.0, stream=None):
        """macsmoke3::idle's advection (src/smoke/macsmoke3.cpp:270-281):
        the scalar, if given, by the velocity, then the velocity by itself,
        in one call."""
        self._run(velocity, fluid, dt, scalar, mask, background, True, stream)

    def _run(self, velocity, fluid, dt, q, mask, bg, do_velocity, stream):
        u, v, w = velocity
        p = AdvectParams(self.params.maccormack, self.params.trim_narrowband, 1 if do_velocity else 0)
        if _is_torch_cuda(u):
            import torch
            for t in (u, v, w, fluid, q):
                if t is not None:
                    assert t.dtype == torch.float32 and t.is_contiguous(), "device arrays must be contiguous float32"
            if mask is not None:
                assert mask.dtype == torch.uint8 and mask.is_contiguous(), "mask must be contiguous uint8"
            st = stream if stream is not None else torch.cuda.current_stream(u.device).cuda_stream
            rc = self.lib.gbp_advect3_device(self.ctx.handle, self.nx, self.ny, self.nz, self.dx, dt, ctypes.byref(p),
                                             u.data_ptr(), v.data_ptr(), w.data_ptr(), fluid.data_ptr(),
                                             q.data_ptr() if q is not None else None,
                                             mask.data_ptr() if mask is not None else None, bg, ctypes.c_void_p(st))
            check(rc)
            return
        ptrs = []
        for a in (u, v, w) + ((q,) if q is not None else ()):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                raise TypeError("host arrays must be contiguous float32 numpy arrays (updated in place)")
            ptrs.append(a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        fa, fptr = _host_f32(fluid)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        rc = self.lib.gbp_advect3(self.ctx.handle, self.nx, self.ny, self.nz, self.dx, dt, ctypes.byref(p), ptrs[0],
                                  ptrs[1], ptrs[2], fptr, ptrs[3] if q is not None else None,
                                  None if m is None else m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), bg)
        check(rc)


class MacAdvection2(MacAdvection3):
    """macadvection2_interface on the GPU
    (``include/shiokaze/advection/macadvection2_interface.h:38-85``, the
    reference's ``macadvection2`` module, ``src/advection/macadvection2.cpp``,
    bilinear). Arrays dense (y, x) float32; otherwise as MacAdvection3.
    ``velocity`` is (u, v)."""

    def __init__(self, nx, ny, dx, context: Context | None = None, **config):
        super().__init__(nx, ny, 1, dx, context, **config)

    def _run(self, velocity, fluid, dt, q, mask, bg, do_velocity, stream):
        u, v = velocity[0], velocity[1]
        p = AdvectParams(self.params.maccormack, self.params.trim_narrowband, 1 if do_velocity else 0)
        if _is_torch_cuda(u):
            import torch
            for t in (u, v, fluid, q):
                if t is not None:
                    assert t.dtype == torch.float32 and t.is_contiguous(), "device arrays must be contiguous float32"
            if mask is not None:
                assert mask.dtype == torch.uint8 and mask.is_contiguous(), "mask must be contiguous uint8"
            st = stream if stream is not None else torch.cuda.current_stream(u.device).cuda_stream
            rc = self.lib.gbp_advect2_device(self.ctx.handle, self.nx, self.ny, self.dx, dt, ctypes.byref(p),
                                             u.data_ptr(), v.data_ptr(), fluid.data_ptr(),
                                             q.data_ptr() if q is not None else None,
                                             mask.data_ptr() if mask is not None else None, bg, ctypes.c_void_p(st))
            check(rc)
            return
        ptrs = []
        for a in (u, v) + ((q,) if q is not None else ()):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                raise TypeError("host arrays must be contiguous float32 numpy arrays (updated in place)")
            ptrs.append(a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        fa, fptr = _host_f32(fluid)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        rc = self.lib.gbp_advect2(self.ctx.handle, self.nx, self.ny, self.dx, dt, ctypes.byref(p), ptrs[0], ptrs[1],
                                  fptr, ptrs[2] if q is not None else None,
                                  None if m is None else m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), bg)
        check(rc)


class MacUtility3:
    """macutility3_interface::constrain_velocity on the GPU
    (``src/utility/macutility3.cpp:61-86``): the velocity's component into
    the solid removed at faces inside it, no outflow through the walls.
    Results equal the reference's bit for bit. Arrays are dense (z, y, x)
    float32, numpy (copied in and out) or torch CUDA tensors (in place);
    ``masks`` are the three components' active faces (uint8, None: all),
    inactive faces holding 0."""

    def __init__(self, nx, ny, nz, dx, context: Context | None = None):
        self.ctx = context or default_context()
        self.lib = self.ctx.lib
        self.nx, self.ny, self.nz, self.dx = nx, ny, nz, dx

    def _check_sizes(self, solid, velocity, masks):
        """Every array must hold exactly its grid's element count: the call
        hands raw pointers to the library, so a wrong shape would be read or
        written out of bounds."""
        nx, ny, nz = self.nx, self.ny, self.nz
        faces = ((nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1))
        size = (lambda a: a.numel()) if _is_torch_cuda(velocity[0]) else (lambda a: np.asarray(a).size)
        if size(solid) != (nx + 1) * (ny + 1) * (nz + 1):
            raise ValueError(f"solid holds {size(solid)} values, expected {(nx + 1) * (ny + 1) * (nz + 1)} (nodal)")
        for d, (a, m) in enumerate(zip(velocity, masks)):
            if size(a) != faces[d]:
                raise ValueError(f"velocity component {d} holds {size(a)} values, expected {faces[d]}")
            if m is not None:
                n = m.numel() if _is_torch_cuda(m) else np.asarray(m).size
                if n != faces[d]:
                    raise ValueError(f"mask of component {d} holds {n} values, expected {faces[d]}")

    def constrain_velocity(self, solid, velocity, masks=None, stream=None):
        u, v, w = velocity
        masks = masks or (None, None, None)
        self._check_sizes(solid, velocity, masks)
        if _is_torch_cuda(u):
            import torch
            for t in (u, v, w, solid):
                assert t.dtype == torch.float32 and t.is_contiguous(), "device arrays must be contiguous float32"
            st = stream if stream is not None else torch.cuda.current_stream(u.device).cuda_stream
            # masks may be numpy, copied to the device here by a synchronous
            # copy (complete before the call), or uint8 CUDA tensors
            masks = [None if m is None else (m if _is_torch_cuda(m) else torch.from_numpy(
                np.ascontiguousarray(m, dtype=np.uint8)).to(u.device)) for m in masks]
            for m in masks:
                if m is not None:
                    assert m.dtype == torch.uint8 and m.is_contiguous(), "masks must be contiguous uint8"
            mp = [None if m is None else m.data_ptr() for m in masks]
            check(self.lib.gbp_constrain_velocity3_device(self.ctx.handle, self.nx, self.ny, self.nz, self.dx,
                                                          solid.data_ptr(), u.data_ptr(), v.data_ptr(), w.data_ptr(),
                                                          *mp, ctypes.c_void_p(st)))
            return
        ptrs = []
        for a in (u, v, w):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                raise TypeError("host arrays must be contiguous float32 numpy arrays (updated in place)")
            ptrs.append(a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        sa, sp = _host_f32(solid)
        ms = [None if m is None else np.ascontiguousarray(m, dtype=np.uint8) for m in masks]
        mp = [None if m is None else m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)) for m in ms]
        check(self.lib.gbp_constrain_velocity3(self.ctx.handle, self.nx, self.ny, self.nz, self.dx, sp, *ptrs, *mp))

    def extrapolate(self, values, active, count, stream=None):
        """array_extrapolator3::extrapolate (array_extrapolator3.h:36-73) of
        one array (z, y, x) with its active mask (uint8), both in place:
        `count` rounds, each activating every inactive neighbour of an active
        cell with the float mean of its active neighbours. numpy arrays go
        through the host call, torch CUDA tensors through the device call.
        Returns the number of cells activated (the reference's count)."""
        d, h, w = values.shape
        added = ctypes.c_longlong(0)
        if _is_torch_cuda(values):
            import torch
            assert values.dtype == torch.float32 and values.is_contiguous(), "values: contiguous float32"
            assert active.dtype == torch.uint8 and active.is_contiguous() and active.numel() == values.numel()
            st = stream if stream is not None else torch.cuda.current_stream(values.device).cuda_stream
            check(self.lib.gbp_extrapolate3_device(self.ctx.handle, w, h, d, values.data_ptr(), active.data_ptr(),
                                                   int(count), ctypes.byref(added), ctypes.c_void_p(st)))
            return added.value
        if not (isinstance(values, np.ndarray) and values.dtype == np.float32 and values.flags.c_contiguous):
            raise TypeError("values must be a contiguous float32 numpy array (updated in place)")
        if not (isinstance(active, np.ndarray) and active.dtype == np.uint8 and active.flags.c_contiguous
                and active.size == values.size):
            raise TypeError("active must be a contiguous uint8 numpy array of the same size (updated in place)")
        check(self.lib.gbp_extrapolate3(self.ctx.handle, w, h, d, values.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                        active.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), int(count),
                                        ctypes.byref(added)))
        return added.value

    def extrapolate_and_constrain_velocity(self, solid, velocity, masks, width):
        """macutility3::extrapolate_and_constrain_velocity
        (src/utility/macutility3.cpp:88-92) on host arrays, in place: each
        component grown `width` rounds over its inactive faces (masks: uint8
        active faces, updated to the grown sets; inactive faces hold 0),
        then the solid constraint over the grown sets."""
        self._check_sizes(solid, velocity, masks)
        ptrs = []
        for a in velocity:
            if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous):
                raise TypeError("host arrays must be contiguous float32 numpy arrays (updated in place)")
            ptrs.append(a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        for m in masks:
            if not (isinstance(m, np.ndarray) and m.dtype == np.uint8 and m.flags.c_contiguous):
                raise TypeError("masks must be contiguous uint8 numpy arrays (updated in place)")
        sa, sp = _host_f32(solid)
        mp = [m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)) for m in masks]
        check(self.lib.gbp_extrapolate_constrain_velocity3(self.ctx.handle, self.nx, self.ny, self.nz, self.dx, sp,
                                                           *ptrs, *mp, int(width)))


def projector_for(scene, context: Context | None = None, **config):
    """A projector shaped for a ``shiokaze_gb300.scenes.Scene``."""
    if scene.dim == 3:
        return MacProject3(scene.nx, scene.ny, scene.nz, scene.dx, context, **config)
    return MacProject2(scene.nx, scene.ny, scene.dx, context, **config)
