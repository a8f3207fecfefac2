"""Serving many simulation scenes on one GPU.

Step requests (one implicit Newmark step of one scene, with that request's
time step, gravity direction and surface load) arrive over time.  Scenes stay
resident on the device (mesh, element data, matrices, sliced FP32 system,
integrator state) while the memory budget allows; a scene that must make room
is evicted least-recently-used first, its state kept in a host checkpoint
(od_scene_save) and restored on its next request (od_scene_load).  Every tick
steps all scenes that have a pending request and fit in memory together, in
one od_batch step (continuous batching at step granularity): requests that
arrive while a tick runs join the next one.  The reference has no serving
layer; each scene still advances exactly as Scene.step would.
"""
from __future__ import annotations

import time
from collections import OrderedDict, deque
from dataclasses import dataclass, field
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
    arrival: float          # seconds, on the server's clock
    dt: float
    gravity: tuple          # unit direction of gravity
    traction: float         # Pa, on the scene's load facets, along -y
    done: float | None = None
    status: int | None = None
    pcg_iterations: int = 0


@dataclass
class _Slot:
    spec: SceneSpec
    mesh: tuple | None = None       # host arrays (built once)
    scene: api.Scene | None = None
    blob: bytes | None = None       # checkpoint while evicted
    bytes: int = 0                  # device bytes while resident (or the last residency)
    queue: deque = field(default_factory=deque)


class Server:
    """Admission by device-memory budget, LRU eviction, one batched step per
    tick.  budget_bytes: memory the resident scenes may use (default: the
    device's free memory at creation less reserve_bytes).  batched=False
    steps the tick's requests one scene at a time with Scene.step instead
    (the plain path, for comparison; the scenes' precision is their spec's)."""

    def __init__(self, ctx: api.Context, budget_bytes: int | None = None, reserve_bytes: int = 4 << 30,
                 max_batch: int | None = None, clock: Callable[[], float] = time.perf_counter,
                 batched: bool = True):
        self.ctx = ctx
        self.batched = batched
        if budget_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info(ctx.device)
            budget_bytes = max(0, free - reserve_bytes)
        self.budget = int(budget_bytes)
        self.max_batch = max_batch
        self.clock = clock
        self.slots: list[_Slot] = []
        self.resident: "OrderedDict[int, None]" = OrderedDict()   # LRU order, most recent last
        self.used = 0
        self.bytes_per_tet = 2600.0   # first estimate; raised to the largest measured ratio
        self.stats = {"ticks": 0, "steps": 0, "admissions": 0, "restores": 0, "evictions": 0, "deferred": 0,
                      "s_admit": 0.0, "s_loads": 0.0, "s_batch_create": 0.0, "s_step": 0.0, "s_other": 0.0}

    # -- registry and queue
    def add_scene(self, spec: SceneSpec) -> int:
        self.slots.append(_Slot(spec))
        return len(self.slots) - 1

    def submit(self, req: StepRequest):
        self.slots[req.scene].queue.append(req)

    def pending(self) -> int:
        return sum(len(s.queue) for s in self.slots)

    # -- residency
    def _estimate(self, slot: _Slot) -> int:
        if slot.bytes:
            return slot.bytes
        return int(self.bytes_per_tet * slot.mesh[1].shape[0])

    def _evict_one(self, keep: set) -> bool:
        for sid in self.resident:
            if sid in keep:
                continue
            slot = self.slots[sid]
            slot.blob = slot.scene.save()
            slot.scene.close()
            slot.scene = None
            self.used -= slot.bytes
            del self.resident[sid]
            self.stats["evictions"] += 1
            return True
        return False

    def _admit(self, sid: int, keep: set) -> bool:
        slot = self.slots[sid]
        if slot.scene is not None:
            self.resident.move_to_end(sid)
            return True
        if slot.mesh is None:
            slot.mesh = slot.spec.build()
        need = self._estimate(slot)
        while self.used + need > self.budget:
            if not self._evict_one(keep):
                return False
        X, tets, facets, cdofs, _ = slot.mesh
        sc = api.Scene(self.ctx, X, tets, facets, cdofs, slot.spec.material)
        self._integrator(slot, sc, 1 / 60)
        if slot.blob is not None:
            sc.load(slot.blob)
            slot.blob = None
            self.stats["restores"] += 1
        slot.scene = sc
        slot.bytes = need
        self.used += need
        self.resident[sid] = None
        self.stats["admissions"] += 1
        return True

    @staticmethod
    def _integrator(slot, sc, dt, setup=True):
        sp = slot.spec
        integ = api.NewmarkIntegrator(0.25, 0.5, sp.rayleigh[0], sp.rayleigh[1], dt,
                                      api.CGSolver(sp.tol, sp.max_iter, api.Preconditioner(sp.precond),
                                                   precision=sp.precision), sp.newton_iters)
        if setup:
            sc.setup_integrator(integ)
        else:
            sc.update_integrator(integ)

    # -- one tick
    def tick(self) -> list[StepRequest]:
        """Admit and step every scene with a pending request (the oldest
        request of each scene) that fits; returns the completed requests."""
        now = self.clock()
        heads = [(s.queue[0].arrival, sid) for sid, s in enumerate(self.slots) if s.queue and
                 s.queue[0].arrival <= now]
        heads.sort()
        if self.max_batch:
            heads = heads[: self.max_batch]
        chosen = [sid for _, sid in heads]
        keep = set(chosen)
        batch_ids = []
        t0 = time.perf_counter()
        for sid in chosen:
            if self._admit(sid, keep):
                batch_ids.append(sid)
            else:
                self.stats["deferred"] += 1
        t1 = time.perf_counter()
        self.stats["s_admit"] += t1 - t0
        if not batch_ids:
            return []
        reqs = []
        for sid in batch_ids:
            slot = self.slots[sid]
            req = slot.queue.popleft()
            self._integrator(slot, slot.scene, req.dt, setup=False)
            rho = slot.spec.material.density
            g = np.asarray(req.gravity, dtype=np.float64) * (9.8 * rho)
            load_facets = slot.mesh[4]
            tr = [([0.0, -req.traction, 0.0], load_facets)] if req.traction and len(load_facets) else []
            slot.scene.set_loads(body=g, tractions=tr)
            reqs.append(req)
        t2 = time.perf_counter()
        self.stats["s_loads"] += t2 - t1
        if self.batched:
            batch = api.Batch(self.ctx, [self.slots[sid].scene for sid in batch_ids])
            t3 = time.perf_counter()
            self.stats["s_batch_create"] += t3 - t2
            try:
                st = batch.step(1)
            finally:
                batch.close()
        else:
            t3 = t2
            st = [self.slots[sid].scene.step(1) for sid in batch_ids]
        t4 = time.perf_counter()
        self.stats["s_step"] += t4 - t3
        t = self.clock()
        for req, s in zip(reqs, st):
            req.done = t
            req.status = s.status
            req.pcg_iterations = s.pcg_iterations
        for sid in batch_ids:   # device bytes now include the scene's FP32 system
            slot = self.slots[sid]
            real = int(slot.scene.info_now().device_bytes)
            self.used += real - slot.bytes
            slot.bytes = real
            self.bytes_per_tet = max(self.bytes_per_tet, real / slot.mesh[1].shape[0])
        while self.used > self.budget and self._evict_one(set()):   # an estimate fell short
            pass
        self.stats["s_other"] += time.perf_counter() - t4
        self.stats["ticks"] += 1
        self.stats["steps"] += len(reqs)
        return reqs

    def warm(self, scene_ids) -> int:
        """Make scenes resident (in order) while they fit; returns how many."""
        n = 0
        for sid in scene_ids:
            slot = self.slots[sid]
            if slot.scene is not None:
                continue
            if slot.mesh is None:
                slot.mesh = slot.spec.build()
            if self.used + self._estimate(slot) > self.budget:
                break
            self._admit(sid, set())
            n += 1
        return n

    def close(self):
        for slot in self.slots:
            if slot.scene is not None:
                slot.scene.close()
                slot.scene = None
        self.resident.clear()
        self.used = 0
