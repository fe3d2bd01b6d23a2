"""Continuous-batching server (GPU test).

Requests arrive while others run, are admitted at the next tick, and every
tick projects all active scenes in one batched call; each scene's state
(warm-start pressure, hierarchy, velocity) stays on the device between its
steps. Each request's result must be the same alone and in the mix within
the stated tolerance: SERVE_RTOL of |p|_inf for liquids, SERVE_RTOL_NEUMANN
after removing the mean for smoke (pressure up to a constant), and the same
on velocities relative to |u|_inf.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SERVE_RTOL = 1e-5
SERVE_RTOL_NEUMANN = 1e-4


def _rel(a, b, neumann):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    if neumann:
        m = b != 0
        a = np.where(m, a - a[m].mean(), 0)
        b = np.where(m, b - b[m].mean(), 0)
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-30)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_served_results_equal_alone(precision):
    from shiokaze_gb300.serving import ProjectionServer, Request, simulate_alone
    # three requests arrive together (they must share ticks), one later
    reqs = [Request(0, 0.0, "liquid", 24, 5, 11), Request(1, 0.0, "smoke", 16, 4, 12),
            Request(2, 0.0, "liquid", 32, 6, 13), Request(3, 0.2, "liquid", 20, 3, 14)]
    final = {}

    def rec(rid, step, p, vel):
        final[rid] = (p.clone(), tuple(t.clone() for t in vel))
    srv = ProjectionServer(budget_bytes=8e9, max_active=3, precision=precision, record=rec)
    done, out = srv.serve(reqs)
    assert out["requests"] == 4 and out["solves"] == sum(r.steps for r in reqs)
    assert out["max_batch"] >= 2          # work overlapped on the device
    assert out["batch_rebuilds"] >= 2     # the batch changed as requests came and went
    for r in reqs:
        p_alone, v_alone = simulate_alone(r, precision)
        p_mix, v_mix = final[r.rid]
        neumann = r.kind == "smoke"
        tol = SERVE_RTOL_NEUMANN if neumann else SERVE_RTOL
        assert _rel(p_mix, p_alone, neumann) <= tol, (r, _rel(p_mix, p_alone, neumann))
        for a, b in zip(v_mix, v_alone):
            assert _rel(a, b, False) <= 10 * tol, r


def test_admission_respects_budget():
    from shiokaze_gb300.serving import ProjectionServer, Request
    srv = ProjectionServer(budget_bytes=1.0e8, max_active=8, precision="mixed")
    reqs = [Request(i, 0.0, "liquid", 32, 2, 100 + i) for i in range(4)]
    one = srv.scene_bytes(reqs[0])
    done, out = srv.serve(reqs)
    assert out["requests"] == 4
    assert out["peak_bytes"] <= 1.0e8
    assert out["max_batch"] <= int(1.0e8 // one)
