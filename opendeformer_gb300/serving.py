"""Serving many simulation scenes on one GPU: the host mirror of od_server_*.

Step requests (one implicit Newmark step of one scene, with that request's
time step, gravity direction and surface load) arrive over time.  Scenes stay
resident on the device (mesh, element data, matrices, sliced FP32 system,
integrator state) while the memory budget allows; a scene that must make room
is evicted least-recently-used first, its state kept in a host checkpoint and
restored when it is admitted again.  Every tick steps all resident scenes
that have a pending request in one batched step (continuous batching at step
granularity): requests that arrive while a tick runs join the next one.
Admission runs on a host worker thread inside the library while ticks run on
the device; a newly admitted scene joins the tick after it is built.  The
reference has no serving layer; each scene still advances exactly as
Scene.step would.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass
from typing import Callable

import numpy as np

from . import api


@dataclass
class SceneSpec:
    """How to build a scene: build() returns (X, tets, facets, cdofs,
    load_facets); the load facets take each request's surface load."""
    build: Callable[[], tuple]
    material: api.Material
    newton_iters: int = 1
    tol: float = 1e-6
    max_iter: int = 5000
    precond: str = "block_jacobi"
    rayleigh: tuple = (0.01, 0.001)
    precision: str = "mixed"


@dataclass
class StepRequest:
    scene: int
    arrival: float          # seconds, on the server's clock (Server.now())
    dt: float
    gravity: tuple          # unit direction of gravity
    traction: float         # Pa, on the scene's load facets, along -y
    done: float | None = None
    status: int | None = None
    pcg_iterations: int = 0
    ticket: int = 0


class Server:
    """od_server: admission by device-memory budget, LRU eviction, one
    batched step per tick.  budget_bytes: memory the resident scenes may use
    (default: the device's free memory at creation less reserve_bytes).
    batched=False steps each tick's requests one scene at a time instead (the
    plain path, for comparison; the scenes' precision is their spec's).
    admission_thread: host threads that build admitted scenes while ticks
    run (True: half the host's cores, at most 8); False or 0 builds them
    inside the tick."""

    def __init__(self, ctx: api.Context, budget_bytes: int | None = None, reserve_bytes: int = 4 << 30,
                 max_batch: int | None = None, batched: bool = True, admission_thread: int | bool = True):
        self.ctx = ctx
        self.batched = batched
        if admission_thread is True:   # default: several builders in parallel
            import os
            admission_thread = max(1, min(8, (os.cpu_count() or 2) // 2))
        cfg = api.od_server_config(int(budget_bytes or 0), int(reserve_bytes), int(max_batch or 0), int(batched),
                                   int(admission_thread))
        self._L = api.load_library()
        self.h = api._vp()
        api._check(self._L.od_server_create(ctx.h, C.byref(cfg), C.byref(self.h)), "od_server_create")
        self._reqs: dict[int, StepRequest] = {}
        self._rho: list[float] = []
        self._nodes: list[int] = []
        self._n_scenes = 0
        self._res = (api.od_step_result * 1)()

    # -- registry, clock and queue
    def add_scene(self, spec: SceneSpec) -> int:
        X, tets, facets, cdofs, load_facets = spec.build()
        X = np.ascontiguousarray(X, dtype=np.float64)
        tets = np.ascontiguousarray(tets, dtype=np.int32)
        facets = np.ascontiguousarray(facets, dtype=np.int32)
        cdofs = np.ascontiguousarray(cdofs, dtype=np.int32)
        load_facets = np.ascontiguousarray(load_facets, dtype=np.int32)
        integ = api.NewmarkIntegrator(0.25, 0.5, spec.rayleigh[0], spec.rayleigh[1], 1 / 60,
                                      api.CGSolver(spec.tol, spec.max_iter, api.Preconditioner(spec.precond),
                                                   precision=spec.precision), spec.newton_iters)
        ip = C.POINTER(C.c_int)
        cs = api.od_scene_spec(X.shape[0], X.ctypes.data_as(api._dp), tets.shape[0], tets.ctypes.data_as(ip),
                               facets.shape[0], facets.ctypes.data_as(ip), cdofs.size, cdofs.ctypes.data_as(ip),
                               load_facets.size, load_facets.ctypes.data_as(ip), spec.material.to_c(),
                               integ.to_c())
        sid = C.c_int(0)
        api._check(self._L.od_server_add_scene(self.h, C.byref(cs), C.byref(sid)), "od_server_add_scene")
        self._n_scenes += 1
        self._rho.append(float(spec.material.density))
        self._nodes.append(int(X.shape[0]))
        return sid.value

    def displacements(self, sid: int) -> np.ndarray:
        """Mesh displacement of a scene (admitted first if it is evicted)."""
        h = api._vp()
        api._check(self._L.od_server_get_scene(self.h, int(sid), C.byref(h)), "od_server_get_scene")
        u = np.zeros((self._nodes[sid], 3))
        api._check(self._L.od_scene_get_displacements(h, u.ctypes.data_as(api._dp)), "get_displacements")
        return u

    def now(self) -> float:
        t = C.c_double(0.0)
        api._check(self._L.od_server_now(self.h, C.byref(t)), "od_server_now")
        return t.value

    def submit(self, req: StepRequest):
        g = np.asarray(req.gravity, dtype=np.float64) * (9.8 * self._rho[req.scene])
        r = api.od_step_request(int(req.scene), float(req.dt), (C.c_double * 3)(*g),
                                (C.c_double * 3)(0.0, -float(req.traction), 0.0), float(req.arrival))
        t = C.c_longlong(0)
        api._check(self._L.od_server_submit(self.h, C.byref(r), C.byref(t)), "od_server_submit")
        req.ticket = t.value
        self._reqs[t.value] = req

    def pending(self) -> int:
        n = C.c_longlong(0)
        api._check(self._L.od_server_pending(self.h, C.byref(n)), "od_server_pending")
        return n.value

    def warm(self, scene_ids) -> int:
        ids = np.ascontiguousarray(list(scene_ids), dtype=np.int32)
        n = C.c_int(0)
        api._check(self._L.od_server_warm(self.h, ids.size, ids.ctypes.data_as(C.POINTER(C.c_int)), C.byref(n)),
                   "od_server_warm")
        return n.value

    # -- one tick
    def tick(self) -> list[StepRequest]:
        """Steps every resident scene with a pending request (the oldest
        request of each); returns the completed requests.  When the step
        fails as a call, its requests (with that status) are in self.failed
        and ODError is raised."""
        if len(self._res) < self._n_scenes:
            self._res = (api.od_step_result * max(1, self._n_scenes))()
        n = C.c_int(0)
        rc = self._L.od_server_tick(self.h, len(self._res), self._res, C.byref(n))
        out = []
        for k in range(n.value):
            r = self._res[k]
            req = self._reqs.pop(r.ticket)
            req.done = r.done
            req.status = r.status
            req.pcg_iterations = r.pcg_iterations
            out.append(req)
        self.failed = out if rc != api.OD_OK else []   # a failed tick's requests, with its status
        api._check(rc, "od_server_tick")
        return out

    @property
    def stats(self) -> dict:
        s = api.od_server_stats()
        api._check(self._L.od_server_get_stats(self.h, C.byref(s)), "od_server_get_stats")
        return {name: getattr(s, name) for name, _ in s._fields_}

    def close(self):
        if self.h:
            self._L.od_server_destroy(self.h)
            self.h = api._vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def wall_clock_loop(server: Server, arrivals, window_s: float, make_request) -> tuple[list, float, int]:
    """Feeds requests to the server at their arrival times (seconds from the
    start, on the server clock) and ticks it until window_s; returns the
    completed requests, the elapsed time and the requests still pending."""
    t0 = server.now()
    nxt, done = 0, []
    while True:
        now = server.now() - t0
        while nxt < len(arrivals) and arrivals[nxt] <= now:
            req = make_request(nxt)
            req.arrival = t0 + arrivals[nxt]
            server.submit(req)
            nxt += 1
        if now >= window_s:
            break
        out = server.tick()
        if out:
            done += out
        elif nxt < len(arrivals):
            time.sleep(max(0.0, min(0.001, arrivals[nxt] - now)))
    return done, server.now() - t0, server.pending()
