"""Seeded synthetic scenes for the pressure projection.

Each scene is the dense input of one ``project(dt, velocity, solid, fluid)``
call (``include/shiokaze/projection/macproject3_interface.h:67-72``):

* ``solid``: nodal level set, shape ``(nz+1, ny+1, nx+1)`` (x fastest), as the
  liquid scene allocates it (``src/liquid/macliquid3.cpp:116``);
* ``fluid``: cell-centred level set, shape ``(nz, ny, nx)``;
* ``u, v, w``: MAC face velocities, shapes ``(nz, ny, nx+1)``,
  ``(nz, ny+1, nx)``, ``(nz+1, ny, nx)``.

Level sets are given as the reference reads them through its narrow-band
arrays: a value is kept where ``|phi| < sqrt(3) dx`` and replaced by
``+-float(sqrt(3) dx)`` elsewhere (``src/utility/macutility3.cpp:343-373``:
values are stored only inside the band, the array is a level set of that
half-width and is flood filled). Positions follow ``include/shiokaze/math/vec.h``:
cell ``(i+1/2) dx``, node ``i dx``, face ``d`` at ``i_d dx`` on axis ``d`` and
``+dx/2`` on the others. Smoke scenes use a fluid that is ``-1`` everywhere
with no band, as ``src/smoke/macsmoke3.cpp:106`` builds it.

The reference publishes no benchmark inputs; these generators stand in with
the shapes, sizes and value distributions of the workloads the module is
measured on.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

GRAVITY = -9.8


@dataclass
class Scene:
    dim: int
    nx: int
    ny: int
    nz: int
    dx: float
    dt: float
    solid: np.ndarray
    fluid: np.ndarray
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray | None
    solid_mode: int = 0  # 0: narrow-band level set, 1: constant array
    fluid_mode: int = 0
    band: float = 0.0
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    def copy(self) -> "Scene":
        return Scene(self.dim, self.nx, self.ny, self.nz, self.dx, self.dt, self.solid.copy(), self.fluid.copy(),
                     self.u.copy(), self.v.copy(), None if self.w is None else self.w.copy(), self.solid_mode,
                     self.fluid_mode, self.band, self.name, dict(self.meta))


def band_of(dx: float) -> float:
    return float(np.float32(math.sqrt(3.0) * dx))


def clamp_band(phi: np.ndarray, dx: float) -> np.ndarray:
    """Dense view of a narrow-band level set: exact inside the band (double
    compare against sqrt(3) dx, then stored as float), +-band outside."""
    half = math.sqrt(3.0) * dx
    b = np.float32(half)
    out = np.where(np.abs(phi) < half, phi.astype(np.float32), np.where(phi < 0, -b, b))
    return out.astype(np.float32)


def _grid(shape_zyx, dx, offs):
    """Coordinates (x, y, z) of a dense grid; offs = per-axis offset in cells."""
    nz, ny, nx = shape_zyx
    x = (np.arange(nx, dtype=np.float64) + offs[0]) * dx
    y = (np.arange(ny, dtype=np.float64) + offs[1]) * dx
    z = (np.arange(nz, dtype=np.float64) + offs[2]) * dx
    return x[None, None, :], y[None, :, None], z[:, None, None]


def _sphere(x, y, z, c, r):
    return np.sqrt((x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2) - r


def liquid3(n: int | tuple, seed: int = 2, pool: float = 0.35, drop_c=(0.5, 0.75, 0.5), drop_r: float = 0.18,
            solid_c=(0.5, 0.2, 0.5), solid_r: float = 0.12, sigma: float = 0.2, dt: float = 1.0 / 60.0,
            dtype_noise: str = "normal") -> Scene:
    """3D liquid: solid sphere, pool y<pool unioned with a drop; box walls.
    The fluid is max(liquid, -(solid+dx)) at cell centres, the convention of
    the reference's scene setup (src/utility/macutility3.cpp:351-358)."""
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    dx = 1.0 / max(nx, ny, nz)
    xn, yn, zn = _grid((nz + 1, ny + 1, nx + 1), dx, (0.0, 0.0, 0.0))
    solid_phi = _sphere(xn, yn, zn, solid_c, solid_r)
    xc, yc, zc = _grid((nz, ny, nx), dx, (0.5, 0.5, 0.5))
    liquid = np.minimum(yc - pool + 0 * xc + 0 * zc, _sphere(xc, yc, zc, drop_c, drop_r))
    solid_at_c = _sphere(xc, yc, zc, solid_c, solid_r) + dx
    fluid_phi = np.maximum(liquid, -solid_at_c)
    rng = np.random.default_rng(seed)
    g = GRAVITY * dt
    if dtype_noise == "normal":
        u = rng.normal(0.0, sigma, size=(nz, ny, nx + 1))
        v = rng.normal(0.0, sigma, size=(nz, ny + 1, nx)) + g
        w = rng.normal(0.0, sigma, size=(nz + 1, ny, nx))
    else:
        u = rng.uniform(-sigma, sigma, size=(nz, ny, nx + 1))
        v = rng.uniform(-sigma, sigma, size=(nz, ny + 1, nx)) + g
        w = rng.uniform(-sigma, sigma, size=(nz + 1, ny, nx))
    return Scene(3, nx, ny, nz, dx, dt, clamp_band(np.broadcast_to(solid_phi, (nz + 1, ny + 1, nx + 1)), dx),
                 clamp_band(np.broadcast_to(fluid_phi, (nz, ny, nx)), dx), u.astype(np.float32),
                 v.astype(np.float32), w.astype(np.float32), 0, 0, band_of(dx), f"liquid3_{nx}x{ny}x{nz}",
                 {"seed": seed, "pool": pool})


def smoke3(n: int | tuple, seed: int = 3, cyl_c=(0.5, 0.5), cyl_r: float = 0.1, sigma: float = 1.0,
           dt: float = 1.0 / 60.0) -> Scene:
    """3D smoke: every cell is fluid (constant -1, no band), Neumann box walls,
    a solid cylinder along z; face velocities N(0, sigma^2)."""
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    dx = 1.0 / max(nx, ny, nz)
    xn, yn, zn = _grid((nz + 1, ny + 1, nx + 1), dx, (0.0, 0.0, 0.0))
    solid_phi = np.sqrt((xn - cyl_c[0]) ** 2 + (yn - cyl_c[1]) ** 2) - cyl_r + 0 * zn
    fluid = np.full((nz, ny, nx), -1.0, dtype=np.float32)
    rng = np.random.default_rng(seed)
    u = rng.normal(0.0, sigma, size=(nz, ny, nx + 1)).astype(np.float32)
    v = rng.normal(0.0, sigma, size=(nz, ny + 1, nx)).astype(np.float32)
    w = rng.normal(0.0, sigma, size=(nz + 1, ny, nx)).astype(np.float32)
    return Scene(3, nx, ny, nz, dx, dt, clamp_band(np.broadcast_to(solid_phi, (nz + 1, ny + 1, nx + 1)), dx),
                 fluid, u, v, w, 0, 1, band_of(dx), f"smoke3_{nx}x{ny}x{nz}", {"seed": seed})


def liquid2(n: int | tuple = 128, seed: int = 1, pool: float = 0.3, drop_c=(0.5, 0.7), drop_r: float = 0.15,
            noise: float = 0.1, dt: float = 1.0 / 60.0) -> Scene:
    """2D liquid: pool y<pool unioned with a circle; no interior solid (walls
    come from the domain boundary); u,v ~ U[-noise, noise], v += g dt."""
    nx, ny = (n, n) if isinstance(n, int) else n
    dx = 1.0 / max(nx, ny)
    b = np.float32(math.sqrt(3.0) * dx)
    solid = np.full((1, ny + 1, nx + 1), b, dtype=np.float32)
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    X, Y = x[None, :], y[:, None]
    liquid = np.minimum(Y - pool + 0 * X, np.sqrt((X - drop_c[0]) ** 2 + (Y - drop_c[1]) ** 2) - drop_r)
    rng = np.random.default_rng(seed)
    u = rng.uniform(-noise, noise, size=(1, ny, nx + 1))
    v = rng.uniform(-noise, noise, size=(1, ny + 1, nx)) + GRAVITY * dt
    return Scene(2, nx, ny, 1, dx, dt, solid, clamp_band(liquid, dx).reshape(1, ny, nx), u.astype(np.float32),
                 v.astype(np.float32), None, 0, 0, band_of(dx), f"liquid2_{nx}x{ny}", {"seed": seed})


def smoke2(n: int | tuple = 128, seed: int = 3, circ_c=(0.5, 0.5), circ_r: float = 0.1, sigma: float = 1.0,
           dt: float = 1.0 / 60.0) -> Scene:
    """2D smoke: every cell fluid (constant -1, no band, as src/smoke/
    macsmoke2.cpp:97 builds it), a solid circle, face velocities
    N(0, sigma^2)."""
    nx, ny = (n, n) if isinstance(n, int) else n
    dx = 1.0 / max(nx, ny)
    xn = np.arange(nx + 1) * dx
    yn = np.arange(ny + 1) * dx
    solid_phi = np.sqrt((xn[None, :] - circ_c[0]) ** 2 + (yn[:, None] - circ_c[1]) ** 2) - circ_r
    rng = np.random.default_rng(seed)
    u = rng.normal(0.0, sigma, size=(1, ny, nx + 1)).astype(np.float32)
    v = rng.normal(0.0, sigma, size=(1, ny + 1, nx)).astype(np.float32)
    return Scene(2, nx, ny, 1, dx, dt, clamp_band(solid_phi, dx).reshape(1, ny + 1, nx + 1),
                 np.full((1, ny, nx), -1.0, dtype=np.float32), u, v, None, 0, 1, band_of(dx), f"smoke2_{nx}x{ny}",
                 {"seed": seed})


def batch_liquid3(count: int = 64, seed: int = 4, edge_lo: int = 32, edge_hi: int = 160) -> list[Scene]:
    """Batch of independent 3D liquid scenes: edge log-uniform in
    [edge_lo, edge_hi] (cubic), fluid fraction ~ U[0.1, 0.6] set by the pool
    height (the drop keeps its size relative to the domain)."""
    rng = np.random.default_rng(seed)
    scenes = []
    for s in range(count):
        edge = int(round(math.exp(rng.uniform(math.log(edge_lo), math.log(edge_hi)))))
        frac = rng.uniform(0.1, 0.6)
        # the drop (r=0.18) holds ~0.024 of the volume; the pool makes up the rest
        pool = float(np.clip(frac - 0.02, 0.05, 0.9))
        sc = liquid3(edge, seed=int(rng.integers(1 << 30)), pool=pool)
        sc.name = f"batch{s}_{edge}"
        sc.meta["fluid_fraction_target"] = frac
        scenes.append(sc)
    return scenes


def accuracy3(n: int, r: float = 0.25) -> tuple[Scene, np.ndarray]:
    """Known-answer case of src/examples/accuracytest3-example.cpp:68-108:
    fluid = |x-c| - r in a band of 2 dx, u = grad |x-c|^2, dt = 1, no solid.
    Returns the scene and the analytic pressure |x-c|^2 - r^2 at cells."""
    nx = ny = nz = n
    dx = 1.0 / n
    c = (0.5, 0.5, 0.5)
    xc, yc, zc = _grid((nz, ny, nx), dx, (0.5, 0.5, 0.5))
    d = np.broadcast_to(_sphere(xc, yc, zc, c, r), (nz, ny, nx))
    band = 2.0 * dx
    fl = np.where(np.abs(d) < band, d.astype(np.float32), np.where(d < 0, -np.float32(band), np.float32(band)))
    xu, yu, zu = _grid((nz, ny, nx + 1), dx, (0.0, 0.5, 0.5))
    xv, yv, zv = _grid((nz, ny + 1, nx), dx, (0.5, 0.0, 0.5))
    xw, yw, zw = _grid((nz + 1, ny, nx), dx, (0.5, 0.5, 0.0))
    u = np.broadcast_to(2.0 * (xu - c[0]) + 0 * yu + 0 * zu, (nz, ny, nx + 1)).astype(np.float32)
    v = np.broadcast_to(2.0 * (yv - c[1]) + 0 * xv + 0 * zv, (nz, ny + 1, nx)).astype(np.float32)
    w = np.broadcast_to(2.0 * (zw - c[2]) + 0 * xw + 0 * yw, (nz + 1, ny, nx)).astype(np.float32)
    solid = np.full((nz + 1, ny + 1, nx + 1), 1.0, dtype=np.float32)
    exact = np.broadcast_to((xc - c[0]) ** 2 + (yc - c[1]) ** 2 + (zc - c[2]) ** 2 - r * r, (nz, ny, nx))
    sc = Scene(3, nx, ny, nz, dx, 1.0, solid, fl.astype(np.float32), u, v, w, 1, 0, float(np.float32(band)),
               f"accuracy3_{n}", {"r": r})
    return sc, np.ascontiguousarray(exact)


def config_scene(index: int, scale: float = 1.0) -> Scene:
    """The single-scene workloads by number: 1 = 2D liquid 128^2,
    2 = 3D liquid 128^3, 3 = 3D smoke 256^3. scale shrinks them for tests."""
    if index == 1:
        return liquid2(max(8, int(round(128 * scale))))
    if index == 2:
        return liquid3(max(8, int(round(128 * scale))))
    if index == 3:
        return smoke3(max(8, int(round(256 * scale))))
    raise ValueError(f"no single-scene workload {index}")
