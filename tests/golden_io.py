"""Loading the golden fixtures made by tests/golden/make_golden.py."""
import glob
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def case_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


class Case:
    def __init__(self, name):
        d = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.name = name
        self.dim = int(d["dim"])
        self.nx, self.ny, self.nz = (int(x) for x in d["shape"])
        self.dx = float(d["dx"])
        self.dt = float(d["dt"])
        self.params = json.loads(str(d["params"]))
        self.solid = d["solid"]
        self.fluid = d["fluid"]
        self.steps = int(d["steps"])
        self.inputs = [(d[f"u{s}"], d[f"v{s}"], d[f"w{s}"] if f"w{s}" in d else None) for s in range(self.steps)]
        self.out_pressure = d["out_pressure"]
        self.out_u = d["out_u"]
        self.out_v = d["out_v"]
        self.out_w = d["out_w"] if "out_w" in d else None
        self.out_unknown = d["out_unknown"].astype(bool)
        # faces the reference's velocity update leaves active (closed faces are set_off)
        self.out_active = tuple(d[f"out_{c}_on"].astype(bool) for c in "uvw"[:self.dim])
        self.iterations = int(d["iterations"])
        self.reresid = float(d["reresid"])
        # (current, target) volumes set before each step, if the case has them
        self.volume = d["volume"] if "volume" in d else None
