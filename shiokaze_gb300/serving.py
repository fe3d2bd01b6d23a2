"""Continuous-batching projection server.

Requests are whole simulations: a scene (3D liquid or smoke, one grid edge)
advanced for a number of time steps, each step one projection. The server
keeps every admitted scene resident on the device -- its level sets and
velocity, its projector (operator, multigrid hierarchy, warm-start
pressure) -- and on every tick advances all active scenes by one step with
ONE batched projection (gbp_batch_*): scenes at different step counts and of
different sizes share the same launches. Requests that arrive while others
run are admitted at the next tick when a slot and device memory are free
(admission against an HBM budget); finished scenes leave and free theirs.

Between projections a scene's velocity is advanced by a synthetic step
u <- projected u + dt g + N(0, noise^2) (advection is outside the projection
module); the level sets stay fixed, and warm start uses the previous
pressure, as the reference's WarmStart option does
(src/projection/macpressuresolver3.cpp:221-242).

Latency of a step = completion time - the time the step became ready (the
request's arrival for its first step, the previous step's completion after
that); reported as p50/p99 over all steps of all requests.
"""
from __future__ import annotations

import heapq
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import scenes as scn

GRAVITY = -9.8


@dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start
    kind: str               # "liquid" or "smoke"
    edge: int
    steps: int = 50
    seed: int = 0
    scene: object = None    # the request's input arrays (made by make_scene if absent)


@dataclass
class Active:
    req: Request
    scene: object
    projector: object
    solid: object
    fluid: object
    vel: tuple
    pressure: object
    nbytes: int
    step: int = 0
    ready: float = 0.0
    rng: object = None
    finish: float = 0.0
    latencies: list = field(default_factory=list)


def poisson_requests(n: int, rate: float, seed: int = 5, edges=(32, 64, 96, 128, 192, 256), liquid_share=0.7,
                     steps: int = 50) -> list[Request]:
    """n requests with exponential inter-arrival times (rate per second),
    70 % liquid / 30 % smoke, edges uniform over `edges`."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        kind = "liquid" if rng.uniform() < liquid_share else "smoke"
        out.append(Request(i, t, kind, int(rng.choice(edges)), steps, int(rng.integers(1 << 30))))
    return out


def make_scene(req: Request):
    if req.scene is not None:
        return req.scene
    if req.kind == "liquid":
        return scn.liquid3(req.edge, seed=req.seed)
    return scn.smoke3(req.edge, seed=req.seed)


class ProjectionServer:
    """Continuous batching of projection requests on one GPU."""

    def __init__(self, budget_bytes: float = 150e9, max_active: int = 64, precision: str = "mixed",
                 residual: float = 1e-6, noise: float = 0.05, device: int = 0, record=None):
        import torch
        import shiokaze_gb300 as gb
        self.gb = gb
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.ctx = gb.Context(device)
        self.budget = budget_bytes
        self.max_active = max_active
        self.cfg = dict(Residual=residual, Solver="mgpcg", Precision=precision, WarmStart=1)
        self.noise = noise
        self.stream = torch.cuda.Stream(device=self.dev)
        self.record = record  # optional callback(rid, step, pressure, vel) after each step
        self.active: list[Active] = []
        self.used = 0
        self._batch = None
        self._batch_key = None
        self.stats = {"ticks": 0, "solves": 0, "batch_sizes": [], "rebuilds": 0, "peak_bytes": 0,
                      "admission_waits": 0}

    # ---- admission ------------------------------------------------------------
    def scene_bytes(self, req: Request) -> int:
        import ctypes
        n = req.edge
        p = self.gb.make_params(**self.cfg)
        state = int(self.gb.load_library().gbp_scene_device_bytes(3, n, n, n, ctypes.byref(p)))
        inputs = 4 * ((n + 1) ** 3 + n ** 3 + 3 * (n + 1) * n * n + n ** 3)
        return state + inputs

    def try_admit(self, req: Request, now: float) -> bool:
        nbytes = self.scene_bytes(req)
        if len(self.active) >= self.max_active or self.used + nbytes > self.budget:
            return False
        torch = self.torch
        sc = make_scene(req)

        def dev(a):
            return torch.from_numpy(np.ascontiguousarray(a)).to(self.dev)
        pj = self.gb.projector_for(sc, self.ctx, **self.cfg)
        vel = tuple(dev(a) for a in (sc.u, sc.v, sc.w))
        act = Active(req, sc, pj, dev(sc.solid), dev(sc.fluid), vel,
                     torch.zeros(sc.fluid.shape, dtype=torch.float32, device=self.dev), nbytes, ready=now,
                     rng=torch.Generator(device=self.dev).manual_seed(req.seed))
        self.active.append(act)
        self.used += nbytes
        self.stats["peak_bytes"] = max(self.stats["peak_bytes"], self.used)
        return True

    # ---- one tick: one batched step of every active scene ------------------------------
    def _batch_for(self):
        key = tuple(a.req.rid for a in self.active)
        if key != self._batch_key:
            if self._batch is not None:
                self._batch.close()
            self._batch = self.gb.Batch([a.projector for a in self.active], self.ctx, **self.cfg)
            self._batch_key = key
            self.stats["rebuilds"] += 1
        return self._batch

    def _advance_velocity(self, a: Active):
        """Synthetic step between projections: u += dt g (v) + N(0, noise^2)."""
        torch = self.torch
        dt = a.scene.dt
        for d, t in enumerate(a.vel):
            t.add_(torch.randn(t.shape, generator=a.rng, device=self.dev, dtype=torch.float32), alpha=self.noise)
            if d == 1:
                t.add_(dt * GRAVITY)

    def tick(self, clock):
        torch = self.torch
        with torch.cuda.stream(self.stream):
            for a in self.active:
                if a.step > 0:
                    self._advance_velocity(a)
            batch = self._batch_for()
            rc = batch.project([a.scene.dt for a in self.active], [a.vel for a in self.active],
                               [a.solid for a in self.active], [a.fluid for a in self.active],
                               [a.pressure for a in self.active], stream=self.stream.cuda_stream)
        if rc not in (self.gb.GBP_OK,):
            raise RuntimeError(f"batched projection returned {rc}")
        now = clock()
        self.stats["ticks"] += 1
        self.stats["solves"] += len(self.active)
        self.stats["batch_sizes"].append(len(self.active))
        finished = []
        for a in self.active:
            a.latencies.append(now - a.ready)
            a.ready = now
            if self.record is not None:
                self.record(a.req.rid, a.step, a.pressure, a.vel)
            a.step += 1
            if a.step >= a.req.steps:
                a.finish = now
                finished.append(a)
        for a in finished:
            self.active.remove(a)
            self.used -= a.nbytes
            a.projector.close()
        return finished

    # ---- the request loop ------------------------------------------------------------
    def serve(self, requests: list[Request], time_scale: float = 1.0):
        """Runs until every request is done; arrivals are replayed in real
        time (scaled). A request's input arrays exist when it arrives: the
        synthetic ones are made before the clock starts. Returns per-request
        records and the server stats."""
        for r in requests:
            r.scene = make_scene(r)
        pending = [(r.arrival * time_scale, r.rid, r) for r in requests]
        heapq.heapify(pending)
        waiting: list[Request] = []
        done = []
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731
        while pending or waiting or self.active:
            now = clock()
            while pending and pending[0][0] <= now:
                _, _, r = heapq.heappop(pending)
                r.arrival = r.arrival * time_scale
                waiting.append(r)
            still = []
            for r in waiting:
                if not self.try_admit(r, r.arrival):
                    still.append(r)
                    self.stats["admission_waits"] += 1
            waiting = still
            if not self.active:
                if pending:
                    time.sleep(max(0.0, min(pending[0][0] - clock(), 0.05)))
                continue
            done.extend(self.tick(clock))
        wall = clock()
        if self._batch is not None:
            self._batch.close()
            self._batch = None
        lat = np.array([x for a in done for x in a.latencies]) * 1e3
        req_lat = np.array([a.finish - a.req.arrival for a in done])
        out = {
            "requests": len(done), "solves": self.stats["solves"], "wall_s": wall,
            "solves_per_s": self.stats["solves"] / wall if wall > 0 else 0.0,
            "step_latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}
            if len(lat) else None,
            "request_latency_s": {"p50": float(np.percentile(req_lat, 50)), "p99": float(np.percentile(req_lat, 99))}
            if len(req_lat) else None,
            "ticks": self.stats["ticks"], "mean_batch": float(np.mean(self.stats["batch_sizes"]))
            if self.stats["batch_sizes"] else 0.0,
            "max_batch": int(max(self.stats["batch_sizes"])) if self.stats["batch_sizes"] else 0,
            "batch_rebuilds": self.stats["rebuilds"], "peak_bytes": self.stats["peak_bytes"],
            "admission_waits": self.stats["admission_waits"],
        }
        return done, out


def simulate_alone(req: Request, precision: str = "mixed", residual: float = 1e-6, noise: float = 0.05,
                   device: int = 0, record=None):
    """The same simulation as the server runs for `req`, with the scene
    projected on its own (single-scene call) at every step."""
    import torch
    import shiokaze_gb300 as gb
    dev = torch.device("cuda", device)
    sc = make_scene(req)
    cfg = dict(Residual=residual, Solver="mgpcg", Precision=precision, WarmStart=1)
    pj = gb.projector_for(sc, **cfg)

    def d(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    vel = tuple(d(a) for a in (sc.u, sc.v, sc.w))
    solid, fluid = d(sc.solid), d(sc.fluid)
    p = torch.zeros(sc.fluid.shape, dtype=torch.float32, device=dev)
    rng = torch.Generator(device=dev).manual_seed(req.seed)
    for step in range(req.steps):
        if step > 0:
            for k, t in enumerate(vel):
                t.add_(torch.randn(t.shape, generator=rng, device=dev, dtype=torch.float32), alpha=noise)
                if k == 1:
                    t.add_(sc.dt * GRAVITY)
        rc = pj.project(sc.dt, vel, solid, fluid, pressure_out=p)
        if rc != gb.GBP_OK:
            raise RuntimeError(f"projection returned {rc}")
        if record is not None:
            record(req.rid, step, p, vel)
    torch.cuda.synchronize()
    pj.close()
    return p, vel
