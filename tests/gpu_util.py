"""Helpers shared by the GPU tests: run the CUDA library through its C ABI."""
import numpy as np

import shiokaze_gb300 as gb
from golden_io import Case

CONFIG_KEYS = {"residual": "Residual", "max_iterations": "MaxIterations", "warm_start": "WarmStart",
               "eps_fluid": "EpsFluid", "eps_solid": "EpsSolid", "second_order_fluid": "SecondOrderAccurateFluid",
               "second_order_solid": "SecondOrderAccurateSolid", "gain": "Gain",
               "surface_tension": "SurfaceTension"}


def config_from(params: dict, **extra):
    cfg = {"Residual": 1e-6}
    for k, v in params.items():
        cfg[CONFIG_KEYS[k]] = v
    cfg.update(extra)
    return cfg


def run_case_gpu(c: Case, **extra):
    """All project() steps of a golden case on the GPU (host-array call)."""
    pj = gb.projector_for(c, **config_from(c.params, **extra))
    out = None
    statuses = []
    for s in range(c.steps):
        u, v, w = (None if a is None else a.copy() for a in c.inputs[s])
        vel = (u, v, w) if c.dim == 3 else (u, v)
        if c.volume is not None:
            pj.set_target_volume(*c.volume[s])
        statuses.append(pj.project(c.dt, vel, c.solid, c.fluid))
        out = (u, v, w)
    p = pj.get_pressure().copy()
    stats = pj.stats.as_dict()
    pj.close()
    return p, out, stats, statuses


def rel_inf(a, b):
    den = max(float(np.max(np.abs(b))), 1e-30)
    return float(np.max(np.abs(a.astype(np.float64) - b.astype(np.float64)))) / den
