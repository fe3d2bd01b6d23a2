"""Parity at the workloads' full sizes (GPU tests).

The parity tests elsewhere run small scenes and the golden fixtures; these
run the benchmark workloads themselves against the oracle (the C
restatement of the reference, pinned bit for bit to the reference's build;
its CG runs its element-wise loops on every host core and its dot products
serially in the reference's order, bit-identical to one thread):

* the 2D liquid scene at 128^2 (plain CG, FP64 and mixed MGPCG);
* the 3D smoke scene at 256^3 (mixed and FP64 MGPCG, plain CG), one oracle
  solve shared by the session;
* the 64 seeded liquid scenes of the batched workload (edges 32..160),
  solved in one batch, mixed and FP64.

Criteria (Residual 1e-6 on both sides): the unknown cells equal the
oracle's exactly; pressure within the stated tolerance of |p_oracle|_inf
(after removing each side's mean over the unknowns on the all-Neumann
smoke scene, whose pressure is defined up to a constant); velocity within
10x that of |u_oracle|_inf; the divergence left after projection (max over
the unknowns of |sum sgn area u / dx|, relative to its value before) at
most twice the oracle's own, or 2e-6. A plain CG on both sides differs only
by summation order (CG_RTOL); MGPCG follows another Krylov sequence and
differs by up to the solve error (MG_RTOL_*). The accuracy the solve must
meet is the relative residual itself: every path's true FP64 residual and
its divergence after projection are at most 1e-6 (times float rounding).
"""
import numpy as np
import pytest

import oracle
from shiokaze_gb300 import scenes

pytestmark = pytest.mark.gpu

# At Residual 1e-6 two different Krylov solves differ by up to about
# cond(A) x 1e-6 (cond grows as n^2): MGPCG measured 3.7e-4 from the oracle
# on the 256^3 smoke scene, 2e-5 on the 128^3 liquid one.
CG_RTOL = 1e-4
MG_RTOL_LIQUID = 1e-4
MG_RTOL_NEUMANN = 1e-3


def _pressure_err(p, want, unknown, neumann):
    a = p[unknown].astype(np.float64)
    b = want[unknown].astype(np.float64)
    if neumann:
        a -= a.mean()
        b -= b.mean()
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-30)


def _vel_err(vel, want):
    ref = [a for a in (want.u, want.v, want.w) if a is not None]
    den = max(float(np.max(np.abs(a))) for a in ref)
    return max(float(np.max(np.abs(g.astype(np.float64) - r.astype(np.float64)))) for g, r in zip(vel, ref)) / den


class _Divergence:
    def __init__(self, sc, want):
        pj = oracle.PortProjector(sc.dim, sc.nx, sc.ny, sc.nz, sc.dx, residual=1e-6)
        self.area, _ = pj.face_fractions(sc.solid, sc.fluid)
        pj.close()
        self.sc, self.unknown = sc, want.unknown
        vin = tuple(a for a in (sc.u, sc.v, sc.w) if a is not None)
        self.before = oracle.divergence(self.area, vin, sc.dx, self.unknown)
        self.oracle = self(tuple(a for a in (want.u, want.v, want.w) if a is not None))

    def __call__(self, vel):
        return oracle.divergence(self.area, vel, self.sc.dx, self.unknown) / self.before


def _project(gb, sc, **cfg):
    pj = gb.projector_for(sc, **cfg)
    vel = tuple(a.copy() for a in (sc.u, sc.v, sc.w) if a is not None)
    rc = pj.project(sc.dt, vel, sc.solid, sc.fluid)
    st = pj.stats.as_dict()
    p = pj.get_pressure().copy()
    pj.close()
    return rc, p, vel, st


def _check(sc, want, div, p, vel, st, rtol, neumann, what):
    assert st["unknowns"] == int(want.unknown.sum()), what
    assert not p[~want.unknown].any(), what
    e_p = _pressure_err(p, want.pressure, want.unknown, neumann)
    e_u = _vel_err(vel, want)
    d = div(vel)
    print(f"{what}: iterations {st['iterations']} (oracle {want.iterations}) pressure {e_p:.2e} "
          f"velocity {e_u:.2e} divergence {d:.2e} (oracle {div.oracle:.2e})")
    assert e_p <= rtol, (what, e_p)
    assert e_u <= 10 * rtol, (what, e_u)
    assert d <= max(2 * div.oracle, 2e-6), (what, d, div.oracle)


@pytest.fixture(scope="module")
def gb():
    import shiokaze_gb300 as gb
    gb.load_library()
    oracle.set_threads(None)
    return gb


@pytest.fixture(scope="session")
def smoke256():
    """The 256^3 smoke workload and its oracle projection (one solve)."""
    oracle.set_threads(None)
    sc = scenes.smoke3(256, seed=3)
    want = oracle.project_scene(sc, "port", residual=1e-6)
    return sc, want, _Divergence(sc, want)


def test_liquid2_128_full_size(gb):
    sc = scenes.liquid2(128, seed=1)
    want = oracle.project_scene(sc, "port", residual=1e-6)
    div = _Divergence(sc, want)
    for solver, precision, rtol in (("cg", "fp64", CG_RTOL), ("mgpcg", "fp64", MG_RTOL_LIQUID),
                                    ("mgpcg", "mixed", MG_RTOL_LIQUID)):
        rc, p, vel, st = _project(gb, sc, Residual=1e-6, Solver=solver, Precision=precision)
        assert rc == gb.GBP_OK
        _check(sc, want, div, p, vel, st, rtol, False, f"2D 128^2 {solver}/{precision}")


@pytest.mark.parametrize("solver,precision", [("mgpcg", "mixed"), ("mgpcg", "fp64"), ("cg", "fp64")])
def test_smoke3_256_full_size(gb, smoke256, solver, precision):
    sc, want, div = smoke256
    rc, p, vel, st = _project(gb, sc, Residual=1e-6, Solver=solver, Precision=precision)
    assert rc == gb.GBP_OK
    assert st["true_resid_inf"] <= 1.01e-6
    rtol = CG_RTOL if solver == "cg" else MG_RTOL_NEUMANN
    _check(sc, want, div, p, vel, st, rtol, True, f"smoke 256^3 {solver}/{precision}")


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch64_full_size(gb, precision):
    """The batched workload: 64 liquid scenes, edges log-uniform in
    [32, 160], one batched solve, each scene against its own oracle solve."""
    import torch
    scs = scenes.batch_liquid3(64, seed=4)
    cfg = dict(Residual=1e-6, Solver="mgpcg", Precision=precision)
    pjs = [gb.projector_for(sc, **cfg) for sc in scs]
    batch = gb.Batch(pjs, **cfg)

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")

    vel = [tuple(dev(a) for a in (sc.u, sc.v, sc.w)) for sc in scs]
    ps = [torch.zeros(sc.fluid.shape, dtype=torch.float32, device="cuda") for sc in scs]
    rc = batch.project([sc.dt for sc in scs], vel, [dev(sc.solid) for sc in scs], [dev(sc.fluid) for sc in scs], ps)
    torch.cuda.synchronize()
    assert rc == gb.GBP_OK
    stats = [batch.stats[i] for i in range(len(scs))]
    worst = 0.0
    for sc, p, v, st in zip(scs, ps, vel, stats):
        want = oracle.project_scene(sc, "port", residual=1e-6)
        div = _Divergence(sc, want)
        s = {"unknowns": st.unknowns, "iterations": st.iterations}
        hp, hv = p.cpu().numpy(), tuple(t.cpu().numpy() for t in v)
        _check(sc, want, div, hp, hv, s, MG_RTOL_LIQUID, False, f"batch {sc.name} {precision}")
        assert st.true_resid_inf <= 1.01e-6, sc.name
        worst = max(worst, _pressure_err(hp, want.pressure, want.unknown, False))
    print(f"batch of 64 ({precision}): worst pressure difference {worst:.2e}")
    batch.close()
    for pj in pjs:
        pj.close()
