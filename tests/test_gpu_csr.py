"""The LinSolver drop-in on the GPU (gbp_csr_cg, the engine of the gbpcg
plugin module that replaces the reference's pcg, src/linsolver/pcg.cpp).

* The pressure systems of the golden fixtures, assembled by the oracle and
  numbered as the reference numbers its unknowns, solve to the reference's
  own pressures (within the plain-CG tolerances of the projection parity
  tests: the two CG runs differ only in summation order) with the
  reference's iteration count within 10 % (+-3).
* A random symmetric positive definite matrix in compressed rows solves to
  a reference CG restated in numpy (pcg_solver.h:246-295), and the
  argument checks turn malformed rows into errors before any device work.
"""
import numpy as np
import pytest

import oracle
from golden_io import Case, case_names

pytestmark = pytest.mark.gpu

PRESSURE_RTOL = 1e-5


def _csr_from_assembly(A):
    """The reference's matrix: one row per unknown (its tile-major index),
    the off-diagonals of the in-grid fluid neighbours in the order +x, -x,
    +y, -y, +z, -z, then the diagonal (macpressuresolver3.cpp:163-199)."""
    idx = A["index"]
    shape = idx.shape
    dim = len(shape)
    n = int(idx.max()) + 1
    cells = np.argwhere(idx >= 0)
    order = np.argsort(idx[idx >= 0])
    cells = cells[order]
    cp = [A["cpz"], A["cpy"], A["cpx"]] if dim == 3 else [A["cpy"], A["cpx"]]
    rows, cols, vals = [], [], []
    indptr = np.zeros(n + 1, np.int64)
    for r, cell in enumerate(cells):
        cell = tuple(int(v) for v in cell)
        for ax in (dim - 1, dim - 2) + ((0,) if dim == 3 else ()):
            for plus in (True, False):
                q = list(cell)
                q[ax] += 1 if plus else -1
                if q[ax] < 0 or q[ax] >= shape[ax]:
                    continue
                q = tuple(q)
                if idx[q] < 0:
                    continue
                w = cp[ax][cell] if plus else cp[ax][q]
                if w == 0:
                    continue
                cols.append(int(idx[q]))
                vals.append(-float(w))
        cols.append(r)
        vals.append(float(A["diag"][cell]))
        indptr[r + 1] = len(cols)
    b = np.array([A["b"][tuple(int(v) for v in c)] for c in cells], np.float64)
    return indptr, np.array(cols, np.int64), np.array(vals, np.float64), b, cells


def _plain_cases():
    out = []
    for name in case_names():
        c = Case(name)
        if c.steps == 1 and not c.params.get("warm_start") and c.volume is None and not c.params.get("surface_tension"):
            out.append(name)
    return out


@pytest.mark.parametrize("name", _plain_cases())
def test_csr_cg_reproduces_reference_pressure(name):
    import shiokaze_gb300 as gb
    c = Case(name)
    u, v, w = c.inputs[0]
    params = {k: v_ for k, v_ in c.params.items() if k != "warm_start"}
    port = oracle.PortProjector(c.dim, c.nx, c.ny, c.nz, c.dx, **params)
    A = port.assemble(c.dt, c.solid, c.fluid, u, v, w)
    port.close()
    if not np.any(A["index"] >= 0):
        pytest.skip("no unknown")
    indptr, cols, vals, b, cells = _csr_from_assembly(A)
    # the fixtures' defaults: Residual 1e-6 (oracle.RefProjector)
    max_it = params.get("max_iterations", 30000)
    x, rc, st = gb.csr_cg(indptr, cols, vals, b, residual=params.get("residual", 1e-6), max_iterations=max_it)
    p = np.zeros(A["index"].shape, np.float32)
    for r, cell in enumerate(cells):
        p[tuple(int(v_) for v_ in cell)] = np.float32(x[r])
    want = c.out_pressure
    assert np.max(np.abs(p - want)) <= PRESSURE_RTOL * max(1e-30, np.max(np.abs(want)))
    if c.iterations >= 0:  # (the 2D fixtures carry no count)
        assert abs(st["iterations"] - c.iterations) <= max(3, 0.1 * c.iterations)
    if c.iterations < max_it:
        assert rc == gb.GBP_OK and st["converged"] == 1


def _numpy_cg(indptr, cols, vals, b, residual, max_it):
    """pcg_solver.h:246-295 with the identity preconditioner, serial sums."""
    n = len(b)
    def mul(s):
        z = np.zeros(n)
        for r in range(n):
            acc = 0.0
            for e in range(indptr[r], indptr[r + 1]):
                acc += vals[e] * s[cols[e]]
            z[r] = acc
        return z
    x = np.zeros(n)
    r = b.copy()
    res0 = np.max(np.abs(r))
    if res0 == 0:
        return x, 0
    tol = max(residual, 1e-30) * res0
    s = r.copy()
    rho = float(r @ r)
    for it in range(max_it):
        z = mul(s)
        alpha = rho / float(s @ z)
        x += alpha * s
        r -= alpha * z
        if np.max(np.abs(r)) <= tol:
            return x, it + 1
        rho_new = float(r @ r)
        s = r + (rho_new / rho) * s
        rho = rho_new
    return x, max_it


def test_csr_cg_random_spd_matrix():
    import shiokaze_gb300 as gb
    rng = np.random.default_rng(7)
    n = 300
    # a weighted graph Laplacian plus a positive diagonal: SPD
    edges = {}
    for i in range(n):
        for _ in range(3):
            j = int(rng.integers(0, n))
            if j != i:
                edges[(min(i, j), max(i, j))] = float(rng.uniform(0.1, 2.0))
    rows = [dict() for _ in range(n)]
    for (i, j), wgt in edges.items():
        rows[i][j] = rows[i].get(j, 0.0) - wgt
        rows[j][i] = rows[j].get(i, 0.0) - wgt
        rows[i][i] = rows[i].get(i, 0.0) + wgt
        rows[j][j] = rows[j].get(j, 0.0) + wgt
    for i in range(n):
        rows[i][i] = rows[i].get(i, 0.0) + 0.05
    indptr = np.zeros(n + 1, np.int64)
    cols, vals = [], []
    for i in range(n):
        for j, val in sorted(rows[i].items()):
            cols.append(j)
            vals.append(val)
        indptr[i + 1] = len(cols)
    cols, vals = np.array(cols, np.int64), np.array(vals)
    b = rng.normal(size=n)
    x_ref, it_ref = _numpy_cg(indptr, cols, vals, b, 1e-10, 2000)
    x, rc, st = gb.csr_cg(indptr, cols, vals, b, residual=1e-10, max_iterations=2000)
    assert rc == gb.GBP_OK
    assert np.max(np.abs(x - x_ref)) <= 1e-7 * np.max(np.abs(x_ref))
    assert abs(st["iterations"] - it_ref) <= max(3, 0.1 * it_ref)
    # the same system capped at 5 iterations: not converged, the iterate kept
    x5, rc5, st5 = gb.csr_cg(indptr, cols, vals, b, residual=1e-10, max_iterations=5)
    assert rc5 == gb.GBP_ERR_NOT_CONVERGED and st5["iterations"] == 5 and st5["converged"] == 0
    x5_ref, _ = _numpy_cg(indptr, cols, vals, b, 1e-10, 5)
    assert np.max(np.abs(x5 - x5_ref)) <= 1e-9 * max(1.0, np.max(np.abs(x5_ref)))


def test_csr_cg_edge_cases():
    import shiokaze_gb300 as gb
    indptr = np.array([0, 2, 4], np.int64)
    cols = np.array([0, 1, 0, 1], np.int64)
    vals = np.array([2.0, -1.0, -1.0, 2.0])
    # b = 0: x = 0 at once, as pcg_solver.h:253-256
    x, rc, st = gb.csr_cg(indptr, cols, vals, np.zeros(2))
    assert rc == gb.GBP_OK and st["iterations"] == 0 and np.all(x == 0)
    # an empty system
    x, rc, st = gb.csr_cg(np.zeros(1, np.int64), np.zeros(0, np.int64), np.zeros(0), np.zeros(0))
    assert rc == gb.GBP_OK and x.shape == (0,)
    # malformed rows are rejected on the host
    with pytest.raises(gb.GBPError):
        gb.csr_cg(indptr, np.array([0, 5, 0, 1], np.int64), vals, np.ones(2))
    with pytest.raises(gb.GBPError):
        gb.csr_cg(np.array([0, 3, 2], np.int64), cols, vals, np.ones(2))
