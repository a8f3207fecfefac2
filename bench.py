"""Benchmark of the implicit FEM time step on GB300.

Default workload (the configuration the headline metric is quoted on): a
64x16x16-cube grid of 0.05 m cubes split into 6 tets each (98,304 tets,
18,785 nodes), seeded jitter 0.15 h, invertible Neo-Hookean (mu = 3.4e4 Pa,
lambda = 3.1e5 Pa, rho = 1000), x = 0 face fixed, the opposite face loaded by
a 500 Pa traction along -y scaled by sin(2 pi 2 t), implicit Newmark
(beta 1/4, gamma 1/2, dt 1/120 s, Rayleigh 0.01 / 0.001) with 3 Newton
iterations per step, block-Jacobi PCG at relative tolerance 1e-8.  A "step"
is one Newmark step.  Synthetic seeded mesh (the reference ships no data).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  --impl reference times the reference's own CPU code
(oracle/_ref, compiled from the reference sources) on the same workload;
the reference has no block-Jacobi, so it runs its Jacobi PCG.

Beside the headline the line carries two more workloads (skipped with
--no-tiers): "precision_tier", the 2.6M-tet Neo-Hookean block with
prescribed top displacements solved with the FP64 and with the mixed-precision
PCG (steps/s of both, the displacement error between them, and the HBM
roofline of the FP32 SpMV phase measured inside the solve), and
"batched_tier", 512 uneven scenes stepped one by one with the FP64 solver and
together through od_batch with the mixed solver; "serving_tier", Poisson step
requests over a pool of scenes; "sweep_tier", the headline step preconditioned
by the reference's incomplete LDL^T and by its threshold incomplete Cholesky,
beside the reference's CPU code for each; "ic0_tier", the headline step with
the IC(0)-preconditioned PCG (the configuration's second preconditioner)
beside the oracle's CPU restatement of it; "relabel_tier", the step and the
triangular sweeps on the generator's node order, a shuffled order and the
shuffle relabeled by od_mesh_relabel.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from opendeformer_gb300 import meshgen  # noqa: E402

NH_MU, NH_LAMBDA = 3.4e4, 3.1e5
NH_E = NH_MU * (3 * NH_LAMBDA + 2 * NH_MU) / (NH_LAMBDA + NH_MU)
NH_NU = NH_LAMBDA / (2 * (NH_LAMBDA + NH_MU))

WORKLOADS = {
    "beam98k_nh_newmark": dict(mesh=lambda: meshgen.beam_98k(), material=("neohookean", 1000.0, NH_E, NH_NU, 0.1),
                               dt=1 / 120, newton=3, alpha_m=0.01, beta_k=0.001, traction=500.0,
                               freq=2.0, body=None, tol=1e-8),
    "cantilever3000_corot_newmark": dict(mesh=lambda: meshgen.cantilever_3000(),
                                         material=("corotational", 1000.0, 1e5, 0.45, 0.1), dt=1 / 60, newton=1,
                                         alpha_m=0.01, beta_k=0.001, traction=0.0, freq=0.0,
                                         body=(0.0, 0.0, -9800.0), tol=1e-8),
}
L2_FLUSH_BYTES = 256 << 20


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def traction_groups(g, amp):
    return [([0.0, -amp, 0.0], g.face_facets(0, 1))] if amp else []


def spmv_bytes(info):
    """Algorithmic bytes of one full-BSR FP64 SpMV launch (values + column
    indices + row pointers + x read once + y written once)."""
    nb = (info.dofs + 2) // 3
    return info.num_full_blocks * (9 * 8 + 4) + (nb + 1) * 4 + 2 * 3 * nb * 8


def pcg_iteration_bytes(info, precond):
    """Algorithmic bytes of one PCG iteration: the SpMV, the x/r/z update with
    the preconditioner apply, and the direction update (each array once)."""
    n = 3 * ((info.dofs + 2) // 3)
    pre = {"block_jacobi": 3 * n * 8, "jacobi": n * 8}.get(precond, 0)
    return spmv_bytes(info) + (16 + 8 + 8 + 16 + 8) * n + pre + (16 + 8) * n


def pcg_iteration_fmas(info, precond):
    """FP64 multiply-adds of one PCG iteration: 9 per stored block (SpMV), 9
    per block row (block-Jacobi) or 1 per DOF (Jacobi), and 6 per DOF for
    x, r, p and the three dot products."""
    nb = (info.dofs + 2) // 3
    pre = {"block_jacobi": 9 * nb, "jacobi": 3 * nb}.get(precond, 0)
    return 9 * info.num_full_blocks + pre + 6 * 3 * nb


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profiles(workload, kernel, field=None):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary, or
    with field="fp64_pipe_pct" that capture's FP64 pipe activity (a
    "fp64_pipe_pct=<value>" entry on the same line)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3 and parts[0] == workload and parts[1] == kernel:
                if field is None:
                    return float(parts[2])
                for p in parts[3:]:
                    if p.startswith(field + "="):
                        return float(p.split("=", 1)[1])
                return None
    return None


def cpu_reference_sample(wl, max_seconds=15.0, max_steps=8):
    """The reference's CPU Newmark (reference material, SpMDV, CGSolver with its
    Jacobi preconditioner) on the same workload; a bounded sample."""
    from oracle import build_ref, reforacle
    if not reforacle.available():
        build_ref.build()
    g = wl["mesh"]()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    kind, rho, E, nu, thr = wl["material"]
    s = reforacle.RefScene(g.X, g.tets, g.facets, cd, kind, rho, E, nu, thr)
    s.nm_setup(wl["dt"], wl["alpha_m"], wl["beta_k"], newton=wl["newton"], tol=wl["tol"], maxit=5000,
               precond="jacobi")
    steps, t_used = 0, 0.0
    t = 0.0
    while steps < max_steps and t_used < max_seconds:
        t += wl["dt"]
        scale = math.sin(2 * math.pi * wl["freq"] * t) if wl["freq"] else 1.0
        t0 = time.perf_counter()
        s.loads(body=wl["body"], tractions=[(np.array(tr) * scale, fac) for tr, fac in
                                            traction_groups(g, wl["traction"])])
        s.nm_apply_loads()
        s.nm_step(1)
        t_used += time.perf_counter() - t0
        steps += 1
    return steps, t_used


def run_reference(args, wl):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    from oracle import build_ref, reforacle
    if not reforacle.available():
        if build_ref.build() is None:
            print(json.dumps({"impl": "reference", "unavailable": "reference sources not present to build oracle/_ref"}))
            return 0
    g = wl["mesh"]()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    kind, rho, E, nu, thr = wl["material"]
    s = reforacle.RefScene(g.X, g.tets, g.facets, cd, kind, rho, E, nu, thr)
    s.nm_setup(wl["dt"], wl["alpha_m"], wl["beta_k"], newton=wl["newton"], tol=wl["tol"], maxit=5000,
               precond="jacobi")
    t = 0.0
    groups = traction_groups(g, wl["traction"])

    def one():
        nonlocal t
        t += wl["dt"]
        scale = math.sin(2 * math.pi * wl["freq"] * t) if wl["freq"] else 1.0
        s.loads(body=wl["body"], tractions=[(np.array(tr) * scale, fac) for tr, fac in groups])
        s.nm_apply_loads()
        return s.nm_step(1)

    for _ in range(args.warmup):
        one()
    t0 = time.perf_counter()
    iters = 0
    for _ in range(args.steps):
        iters += one()
    el = time.perf_counter() - t0
    v = args.steps / el
    line = {"metric": "newmark_steps_per_s", "value": v, "unit": "steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": args.workload, "n_tets": g.n_tets, "precond": "jacobi (reference)",
                       "pcg_iterations_per_step": iters / args.steps},
            "cpu_baseline": {"value": v, "unit": "steps/s", "cores": 1, "kind": "reference",
                             "sample": f"{args.steps} Newmark steps after {args.warmup} warm-up, single thread "
                                       "(the reference has no threading)"},
            "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _rel(a, b):
    return float(np.abs(a - b).max() / max(1e-300, np.abs(b).max()))


def headline_parity(args, wl, api, ctx, steps=5):
    """Displacements of the headline workload after `steps` steps from rest
    (a fresh scene, same solver) against the oracle's restatement of the same
    steps (test infrastructure, run in the CPU-baseline leg)."""
    from oracle import restated as O
    g = wl["mesh"]()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    kind, rho, E, nu, thr = wl["material"]
    s = api.Scene(ctx, g.X, g.tets, g.facets, cd, api.Material(kind, rho, E, nu, thr))
    s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"],
                                             api.CGSolver(wl["tol"], 5000, api.Preconditioner(args.precond),
                                                          precision=args.precision), wl["newton"]))
    groups = traction_groups(g, wl["traction"])
    s.set_loads(body=wl["body"], tractions=groups)
    if wl["freq"]:
        s.set_traction_schedule(wl["freq"])
    st = s.step(steps)
    ug = s.displacements()
    s.close()
    o = O.OracleScene(g.X, g.tets, g.facets, cd, kind, rho, E, nu, thr)
    o.integrator_setup(wl["dt"], wl["alpha_m"], wl["beta_k"], newton=wl["newton"], tol=wl["tol"], maxit=5000,
                       precond=args.precond)
    t, t0 = 0.0, time.perf_counter()
    for _ in range(steps):
        t += wl["dt"]
        scale = math.sin(2 * math.pi * wl["freq"] * t) if wl["freq"] else 1.0
        o.set_fext(o.loads(body=wl["body"], tractions=[(np.array(tr) * scale, fac) for tr, fac in groups]))
        o.nm_step(1)
    uo = o.displacements()
    o.close()
    return {"headline_rel_err": _rel(ug, uo), "steps": steps, "status": st.status,
            "bound": 1e-8 if args.precision == "fp64" else 1e-6,
            "oracle": f"restatement ({args.precond} PCG), single thread, {time.perf_counter() - t0:.1f} s",
            "rule": "max |u_gpu - u_oracle| / max |u_oracle| over all nodes, fresh scene from rest"}


def _cpu_batch_worker(job):
    """One oracle process of the batched CPU baseline: steps instances of
    the batched workload (one Newmark step each, FP64 block-Jacobi PCG,
    the oracle's restatement) until its time budget is used."""
    idx, budget = job
    from oracle import restated as O
    insts = meshgen.batch_instances(512)
    tets = scenes = 0
    step_s = 0.0
    t_end = time.perf_counter() + budget
    for i in idx:
        if time.perf_counter() > t_end:
            break
        inst = insts[i]
        g = meshgen.instance_grid(inst)
        cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
        kind = "corotational" if inst["kind"] == "corotational" else "neohookean"
        o = O.OracleScene(g.X, g.tets, g.facets, cd, kind, 1000.0, inst["E"], inst["nu"], 0.1)
        o.integrator_setup(1 / 60, 0.01, 0.001, newton=1, tol=1e-8, maxit=5000, precond="block_jacobi")
        o.set_fext(o.loads(body=[0.0, 0.0, -9800.0]))
        t0 = time.perf_counter()
        o.nm_step(1)
        step_s += time.perf_counter() - t0
        o.close()
        tets += g.n_tets
        scenes += 1
    return tets, scenes, step_s


def _cpu_serving_worker(job):
    """One oracle process of the serving CPU baseline: serves sampled step
    requests of the serving workload back to back (scene, time step, gravity
    direction and surface load drawn as the requests are; FP64 block-Jacobi
    PCG at 1e-6, the oracle's restatement), until its time budget is used;
    scene construction is not counted (a CPU server keeps scenes resident)."""
    seed, pool_n, budget = job
    from oracle import restated as O
    pool = meshgen.serving_pool(4096)[:pool_n]
    rng = np.random.default_rng(seed)
    reqs = 0
    step_s = 0.0
    t_end = time.perf_counter() + budget
    while time.perf_counter() < t_end:
        inst = pool[int(rng.integers(len(pool)))]
        dt = float(rng.uniform(1 / 120, 1 / 30))
        gdir = rng.normal(size=3)
        gdir /= np.linalg.norm(gdir)
        trac = float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0))))
        g = meshgen.pool_grid(inst)
        cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
        o = O.OracleScene(g.X, g.tets, g.facets, cd, inst["kind"], 1000.0, inst["E"], inst["nu"], 0.1)
        o.integrator_setup(dt, 0.01, 0.001, newton=1, tol=1e-6, maxit=5000, precond="block_jacobi")
        o.set_fext(o.loads(body=gdir * 9800.0, tractions=[([0.0, -trac, 0.0], g.face_facets(0, 1))]))
        t0 = time.perf_counter()
        o.nm_step(1)
        step_s += time.perf_counter() - t0
        o.close()
        reqs += 1
    return reqs, step_s


def cpu_processes():
    return max(1, os.cpu_count() or 1)


def cpu_pool_map(fn, jobs):
    """Runs the oracle workers in spawned processes (never forked from a
    process that holds a CUDA context): at most one process per host core,
    each with single-threaded BLAS, the jobs spread over them in order."""
    import multiprocessing as mp
    procs = max(1, min(len(jobs), cpu_processes()))
    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
    os.environ.update({k: "1" for k in saved})   # inherited by the spawned workers
    try:
        with mp.get_context("spawn").Pool(procs) as pool:
            return pool.map(fn, jobs, chunksize=max(1, len(jobs) // (4 * procs)))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def host_cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def precision_tier(args, api, ctx):
    """Mixed-precision large solve: 128x64x64 cubes x 5 tets (2,621,440 tets,
    longest side 1 m, jitter 0.2 h), invertible Neo-Hookean (mu 3.4e4,
    lambda 3.1e5), bottom face fixed, a seeded 20% of the top-face nodes
    prescribed to -0.05 height along z; Newmark dt 1/120 s, Rayleigh
    0.01 / 0.001, one Newton iteration, block-Jacobi PCG to 1e-10.  The
    same steps run with the FP64 solver and the mixed one (FP32 sliced SpMV
    and preconditioner, compensated dots summed in FP64, FP64 refinement)."""
    nz = args.precision_nz
    g = meshgen.block_2m6() if nz == 64 else meshgen.tet_grid(128, 64, nz, h=1.0 / 128, jitter=0.20, seed=4,
                                                              tets_per_cube=5)
    bottom, top = g.face_nodes(2, 0), g.face_nodes(2, 1)
    rng = np.random.default_rng(4)
    presc = np.sort(rng.choice(top, size=int(0.2 * top.size), replace=False))
    cd = meshgen.constrained_dofs_for_nodes(np.concatenate([bottom, presc]))
    u0 = np.zeros((g.n_nodes, 3))
    u0[presc, 2] = -0.05 * g.dims[2] * g.h
    mat = api.InvertibleNeoHookeanMaterial(1000.0, NH_E, NH_NU, 0.1)
    out, res, first = {}, {}, {}
    warm, steps = 2, args.tier_steps
    # mixed: the inner SpMV streams the lower triangle (transposed products by
    # reductions); mixed_full: both triangles (OD_GB300_MIXED_SPMV=full)
    # mixed_ic0: the IC(0) preconditioner (FP64 factor, FP32 sweeps) in the
    # mixed solve
    variants = [v for v in args.precision_variants.split(",") if v]
    for prec in variants:
        if prec == "mixed_full":
            os.environ["OD_GB300_MIXED_SPMV"] = "full"
        pc = api.IC0Preconditioner() if prec == "mixed_ic0" else api.BlockJacobiPreconditioner()
        s = api.Scene(ctx, g.X, g.tets, g.facets, cd, mat)
        s.set_displacements(u0)
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 120,
                                                 api.CGSolver(1e-10, 20000, pc, precision=prec.split("_")[0]), 1))
        for w in range(warm):
            s.step(1)
            if w == 0:
                first[prec] = s.displacements()   # after the first step from rest (oracle check)
        os.environ.pop("OD_GB300_MIXED_SPMV", None)
        ms, it = [], 0
        for _ in range(steps):
            st = s.step(1)
            if st.status != 0:
                raise RuntimeError(f"precision tier: {prec} step status {st.status}")
            ms.append(st.device_ms)
            it += st.pcg_iterations
        out[prec] = s.displacements()
        # one more step with the device-side phase timers on (kept out of the timed steps)
        ctx.reset_counters()
        ctx.set_profiling(True)
        s.step(1)
        ctx.set_profiling(False)
        c = ctx.counters()
        res[prec] = {"steps_per_s": 1000.0 / statistics.mean(ms), "ms_per_step": statistics.mean(ms),
                     "pcg_iterations_per_step": it / steps, "mix": (c.mix_spmv_bytes, c.mix_spmv_ms,
                                                                    c.mix_iterations, c.mix_spmv_work_ms)}
        s.close()
        del s
    peak, peak_kind = peaks()
    if not {"fp64", "mixed"} <= set(res):
        return {"workload": f"block128x64x{nz}_nh_prescribed_newmark", "variants": res}
    nbytes, sms, nit, wms = res["mixed"].pop("mix")
    res["fp64"].pop("mix")
    if "mixed_ic0" in res:
        res["mixed_ic0"].pop("mix")
    if "mixed_full" in res:
        fb, fs, fi, fw = res["mixed_full"].pop("mix")
        res["mixed_full"]["spmv_phase"] = {"bytes": fb, "ms": fw, "phases": fi,
                                           "achieved_gbs": fb / (fw * 1e-3) / 1e9 if fw else None,
                                           "us_per_phase_with_sum": 1000.0 * fs / max(1, fi)}
    spmv_gbs = nbytes / (wms * 1e-3) / 1e9 if wms else None
    phase_gbs = nbytes / (sms * 1e-3) / 1e9 if sms else None
    oracle = None
    if not args.no_cpu_baseline and nz == 64:
        # the oracle's restatement of the first step (FP64, same solver settings,
        # one thread): the error bound of the precision form is against it
        try:
            from oracle import restated as O
            o = O.OracleScene(g.X, g.tets, g.facets, cd, "neohookean", 1000.0, NH_E, NH_NU, 0.1)
            o.set_displacements(u0)
            o.integrator_setup(1 / 120, 0.01, 0.001, newton=1, tol=1e-10, maxit=20000, precond="block_jacobi")
            t0 = time.perf_counter()
            its = o.nm_step(1)
            secs = time.perf_counter() - t0
            uo = o.displacements()
            o.close()
            oracle = {"rel_err_mixed_vs_oracle": _rel(first["mixed"], uo),
                      "rel_err_fp64_vs_oracle": _rel(first["fp64"], uo), "bound": 1e-6,
                      "step": "first Newmark step from rest (fresh scenes)",
                      "cpu_baseline": {"value": 1.0 / secs, "unit": "steps/s", "cores": 1, "kind": "port",
                                       "sample": f"the first step ({its} PCG iterations, {secs:.1f} s), the "
                                                 "oracle's FP64 restatement with block-Jacobi, one thread; "
                                                 "later steps cost about the same"}}
        except Exception as exc:
            oracle = {"error": str(exc)}
    return {"workload": "block2m6_nh_prescribed_newmark" if nz == 64 else f"block128x64x{nz}_nh_prescribed_newmark",
            "n_tets": g.n_tets, "dofs": 3 * g.n_nodes - len(cd),
            "newton_iters": 1, "tol": 1e-10, "precond": "block_jacobi", "warmup": warm, "steps": steps,
            "fp64": res["fp64"], "mixed": res["mixed"], "mixed_full": res.get("mixed_full"),
            "mixed_ic0": {**res["mixed_ic0"], "rel_err_vs_fp64": _rel(out["mixed_ic0"], out["fp64"]),
                          "speedup_vs_fp64": res["mixed_ic0"]["steps_per_s"] / res["fp64"]["steps_per_s"],
                          "precond": "IC(0): FP64 factor (colour order), FP32 sweeps and SpMV, multi-kernel inner PCG"}
            if "mixed_ic0" in res else None,
            "speedup_mixed_vs_fp64": res["mixed"]["steps_per_s"] / res["fp64"]["steps_per_s"],
            "speedup_mixed_full_vs_fp64": res["mixed_full"]["steps_per_s"] / res["fp64"]["steps_per_s"]
            if "mixed_full" in res else None,
            "rel_err_mixed_full_vs_fp64": _rel(out["mixed_full"], out["fp64"]) if "mixed_full" in res else None,
            "rel_err_mixed_vs_fp64": _rel(out["mixed"], out["fp64"]),
            "oracle": oracle,
            "spmv_roofline": {"kernel": "pcg32_ring_kernel SpMV phase (sliced FP32 matrix streamed by "
                                        "cp.async.bulk), from the phase start to the moment the last CTA "
                                        "finished it, timed on the device inside the real solve",
                              "bound": "hbm", "achieved": spmv_gbs, "peak": peak, "unit": "GB/s",
                              "frac": spmv_gbs / peak if spmv_gbs else None, "peak_source": peak_kind,
                              "algorithmic_bytes": nbytes, "phase_ms": wms, "phases": nit,
                              "with_grid_sum": {"achieved": phase_gbs, "frac": phase_gbs / peak if phase_gbs else None,
                                                "phase_ms": sms},
                              "us_per_phase_with_sum": 1000.0 * sms / max(1, nit),
                              "bytes_rule": "stored 3x3 blocks x 40 B (9 FP32 values + int32 column; the lower "
                                            "triangle with the diagonal) + 24 B per block row (own p read, q "
                                            "written); the transposed products go to L2 as reductions"}}


def sweep_tier(args, api, ctx):
    """The headline beam workload (98,304 tets, Newmark, 3 Newton iterations,
    tolerance 1e-8) preconditioned by the reference's two factored
    preconditioners, InLDLTPreconditioner(0.1, 0.01) and
    InCholeskyPreconditioner(0.01, 0): each factor is remade on the host for
    every solve as the reference does (bit-identical to it), the two
    triangular sweeps of every apply run on the device.  Wall time per step
    (the host factorisations are inside it), the apply's device time from a
    profiled step, and the reference's own CPU code on the same step."""
    wl = WORKLOADS["beam98k_nh_newmark"]
    g = wl["mesh"]()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    kind, rho, E, nu, thr = wl["material"]
    peak, peak_kind = peaks()
    result = {"workload": "beam98k_nh_newmark", "n_tets": g.n_tets}
    for name, prec, ref_args in (("ic", api.InCholeskyPreconditioner(0.01, 0.0), ("ic", 0.01, 0.0)),
                                 ("ldlt", api.InLDLTPreconditioner(0.1, 0.01), ("ldlt", 0.1, 0.01))):
        s = api.Scene(ctx, g.X, g.tets, g.facets, cd, api.Material(kind, rho, E, nu, thr))
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"],
                                                 api.CGSolver(wl["tol"], 5000, prec), wl["newton"]))
        s.set_loads(body=wl["body"], tractions=traction_groups(g, wl["traction"]))
        s.set_traction_schedule(wl["freq"])
        s.step(1)
        steps = max(2, min(args.tier_steps, 4))
        ctx.reset_counters()
        walls, it, solves = [], 0, 0
        for _ in range(steps):
            t0 = time.perf_counter()
            st = s.step(1)
            walls.append(time.perf_counter() - t0)
            if st.status != 0:
                raise RuntimeError(f"sweep tier ({name}): step status {st.status}")
            it += st.pcg_iterations
            solves += st.solves
        c = ctx.counters()
        factor_ms = c.sweep_factor_ms / max(1, c.sweep_factors)
        ctx.reset_counters()
        ctx.set_profiling(True)
        s.step(1)
        ctx.set_profiling(False)
        p = ctx.counters()
        s.close()
        apply_ms = p.sweep_apply_ms / max(1, p.sweep_applies)
        gbs = p.sweep_apply_bytes / (p.sweep_apply_ms * 1e-3) / 1e9 if p.sweep_apply_ms else None
        wall = statistics.mean(walls)
        label = {"ldlt": "InLDLTPreconditioner", "ic": "InCholeskyPreconditioner"}[name]
        out = {"precond": f"{label}({ref_args[1]}, {ref_args[2]})", "steps": steps, "wall_ms_per_step": 1000 * wall, "steps_per_s": 1.0 / wall,
               "pcg_iterations_per_step": it / steps, "solves_per_step": solves / steps,
               "factor_ms_per_solve": factor_ms, "factor_nnz": c.sweep_nnz,
               "apply": {"kernel": f"sweep_apply_kernel<{1 if name == 'ic' else 0}> (forward and backward sweeps, "
                                   "one cooperative launch)",
                         "bound": "latency: dependency chain", "levels": p.sweep_levels, "avg_launch_ms": apply_ms,
                         "us_per_level": 1000.0 * apply_ms / max(1, p.sweep_levels), "launches": p.sweep_applies,
                         "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak if gbs else None,
                         "peak_source": peak_kind,
                         "bytes_rule": "L entries x 12 B (value + index) per sweep + 7 x 8 B per row"},
               "share_of_step": {"host_factor": factor_ms * solves / steps / (1000 * wall)}}
        if not args.no_cpu_baseline:
            try:
                from oracle import build_ref, reforacle
                if not reforacle.available():
                    build_ref.build()
                r = reforacle.RefScene(g.X, g.tets, g.facets, cd, kind, rho, E, nu, thr)
                r.nm_setup(wl["dt"], wl["alpha_m"], wl["beta_k"], newton=wl["newton"], tol=wl["tol"], maxit=5000,
                           precond=ref_args[0], eps=ref_args[1], relax=ref_args[2])
                t, n_ref, used = 0.0, 0, 0.0
                while n_ref < 2:
                    t += wl["dt"]
                    scale = math.sin(2 * math.pi * wl["freq"] * t)
                    t0 = time.perf_counter()
                    r.loads(body=wl["body"], tractions=[(np.array(tr) * scale, fac) for tr, fac in
                                                        traction_groups(g, wl["traction"])])
                    r.nm_apply_loads()
                    r.nm_step(1)
                    used += time.perf_counter() - t0
                    n_ref += 1
                out["cpu_reference"] = {"steps_per_s": n_ref / used, "cores": 1, "kind": "reference",
                                        "sample": f"{n_ref} Newmark steps, reference code with the same "
                                                  "preconditioner, single thread"}
                out["speedup_vs_cpu_reference"] = out["steps_per_s"] / out["cpu_reference"]["steps_per_s"]
            except Exception as exc:
                out["cpu_reference"] = {"error": str(exc)}
        result[name] = out
    return result


def ic0_tier(args, api, ctx):
    """The headline beam workload with the IC(0)-preconditioned PCG: the
    shifted IC(0) factor of every solve and the two triangular sweeps of
    every apply on the device, each one cooperative launch.  The factor's
    blocks go in colour order (greedy colouring of the block graph: as many
    dependency levels per sweep as colours); the natural DOF order is timed
    beside it.  Device time per step, PCG iterations, the apply's time per
    dependency level from a profiled step, and the oracle's CPU restatement
    of the same step (the reference has no IC(0); single thread, two steps)."""
    wl = WORKLOADS["beam98k_nh_newmark"]
    g = wl["mesh"]()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    kind, rho, E, nu, thr = wl["material"]

    def run(order):
        if order == "natural":
            os.environ["OD_GB300_IC0_ORDER"] = "natural"
        try:
            s = api.Scene(ctx, g.X, g.tets, g.facets, cd, api.Material(kind, rho, E, nu, thr))
            s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"],
                                                     api.CGSolver(wl["tol"], 5000, api.IC0Preconditioner()),
                                                     wl["newton"]))
            s.set_loads(body=wl["body"], tractions=traction_groups(g, wl["traction"]))
            s.set_traction_schedule(wl["freq"])
            for _ in range(3):
                s.step(1)
        finally:
            os.environ.pop("OD_GB300_IC0_ORDER", None)
        steps = max(3, args.tier_steps)
        ms, it, solves = [], 0, 0
        for _ in range(steps):
            st = s.step(1)
            if st.status != 0:
                raise RuntimeError(f"ic0 tier: step status {st.status}")
            ms.append(st.device_ms)
            it += st.pcg_iterations
            solves += st.solves
        ctx.reset_counters()
        ctx.set_profiling(True)
        s.step(1)
        ctx.set_profiling(False)
        p = ctx.counters()
        s.close()
        apply_ms = p.sweep_apply_ms / max(1, p.sweep_applies)
        return {"steps": steps, "ms_per_step": statistics.mean(ms), "steps_per_s": 1000.0 / statistics.mean(ms),
                "pcg_iterations_per_step": it / steps, "solves_per_step": solves / steps,
                "apply": {"kernel": "sweep_apply_kernel<1> over row triples (one cooperative launch)",
                          "levels": p.sweep_levels, "avg_launch_ms": apply_ms,
                          "us_per_level": 1000.0 * apply_ms / max(1, p.sweep_levels), "launches": p.sweep_applies}}

    colour = run("colour")
    out = {"workload": "beam98k_nh_newmark", "n_tets": g.n_tets,
           "precond": "IC0Preconditioner (shifted IC(0), blocks in colour order)", **colour,
           "natural_order": run("natural"),
           "factor_kernel": "ic0_factor_coop_kernel (warp per row, rows by level, one cooperative launch)"}
    if not args.no_cpu_baseline:
        try:
            from oracle import restated as O
            o = O.OracleScene(g.X, g.tets, g.facets, cd, kind, rho, E, nu, thr)
            o.integrator_setup(wl["dt"], wl["alpha_m"], wl["beta_k"], newton=wl["newton"], tol=wl["tol"],
                               maxit=5000, precond="ic0")
            t, n_cpu, used = 0.0, 0, 0.0
            while n_cpu < 2:
                t += wl["dt"]
                scale = math.sin(2 * math.pi * wl["freq"] * t)
                t0 = time.perf_counter()
                o.set_fext(o.loads(body=wl["body"], tractions=[(np.array(tr) * scale, fac) for tr, fac in
                                                               traction_groups(g, wl["traction"])]))
                o.nm_step(1)
                used += time.perf_counter() - t0
                n_cpu += 1
            o.close()
            out["cpu_port"] = {"steps_per_s": n_cpu / used, "cores": 1, "kind": "port",
                               "sample": f"{n_cpu} Newmark steps, the oracle's restatement with IC(0), single thread"}
            out["speedup_vs_cpu_port"] = out["steps_per_s"] / out["cpu_port"]["steps_per_s"]
        except Exception as exc:
            out["cpu_port"] = {"error": str(exc)}
    return out


def relabel_tier(args, api, ctx):
    """Node order on the headline beam step: the generator's order, a seeded
    random shuffle of the node ids, and the shuffle relabeled by
    od_mesh_relabel (MeshRelabeler's Gibbs-Poole-Stockmeyer pass).  Per
    order: element colours, the FP64 block-Jacobi step (device ms), and the
    dependency depth and device time of one apply of the reference's IC
    factor (0.01, 0) of the step's system -- bandwidth-reducing orders help
    the SpMV but lengthen the triangular sweeps' chains."""
    wl = WORKLOADS["beam98k_nh_newmark"]
    g = wl["mesh"]()
    kind, rho, E, nu, thr = wl["material"]
    mat = api.Material(kind, rho, E, nu, thr)
    perm = np.random.default_rng(1).permutation(g.n_nodes)
    Xs = np.empty_like(g.X)
    Xs[perm] = g.X
    ts = perm[g.tets].astype(np.int32)
    fs = perm[g.facets].astype(np.int32)
    cds = meshgen.constrained_dofs_for_nodes(perm[g.face_nodes(0, 0)])
    load = np.where(np.isin(fs, perm[g.face_nodes(0, 1)]).all(axis=1))[0]
    t0 = time.perf_counter()
    Xr, tr, fr, cdr, _ = api.relabel_mesh(Xs, ts, fs, cds)
    relabel_s = time.perf_counter() - t0
    cases = {"generator": (g.X, g.tets, g.facets, meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0)),
                           g.face_facets(0, 1)),
             "shuffled": (Xs, ts, fs, cds, load), "relabeled": (Xr, tr, fr, cdr, load)}
    out = {"workload": "beam98k_nh_newmark", "relabel_host_s": relabel_s}
    for name, (X, T, F, C, L) in cases.items():
        s = api.Scene(ctx, X, T, F, C, mat)
        s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"],
                                                 api.CGSolver(wl["tol"], 5000, api.BlockJacobiPreconditioner()),
                                                 wl["newton"]))
        s.set_loads(tractions=[([0.0, -wl["traction"], 0.0], L)])
        s.set_traction_schedule(wl["freq"])
        for _ in range(3):
            s.step(1)
        ms = [s.step(1).device_ms for _ in range(max(5, args.tier_steps))]
        vals, _ = s.evaluate()
        h = wl["dt"]
        A = (1 + h * wl["alpha_m"]) * s.mass() + (h * h + h * wl["beta_k"]) * vals
        s.ic_factor(A, 1e-2, 0.0)
        levels = ctx.counters().sweep_levels
        r = np.random.default_rng(2).normal(size=s.dofs)
        ctx.set_profiling(True)
        ctx.reset_counters()
        s.ic_apply(r)
        apply_ms = ctx.counters().sweep_apply_ms
        ctx.set_profiling(False)
        out[name] = {"colours": s.info.num_colors, "fp64_step_ms": statistics.median(ms),
                     "ic_sweep_levels": levels, "ic_apply_ms": apply_ms}
        s.close()
    return out


def modal_tier(args, api, ctx):
    """Modal linear Newmark (intergrator/linearNewmark.cpp) on the headline
    beam: Hooke stiffness with the beam material's E and nu, consistent
    mass, 16 modes; Newmark beta 1/4, gamma 1/2, Rayleigh 0.01 / 0.001,
    dt 1/120 s, the beam's 500 Pa traction held constant.  Setup on the GPU
    (Hooke assembly, thick-restart Lanczos on K^-1 M with FP64 block-Jacobi
    PCG applies) against the reference's setup algorithm on one host core
    (ARPACK shift-invert at 0 with a SuperLU factorisation, through scipy's
    eigsh, on the compiled reference's K and M).  Steps end to end as the
    reference's loop runs them: runOneTimeStep and
    updateMeshVerticesDisplacements (the full-order field to the host) per
    step, against the restated steps with numpy on the host."""
    wl = WORKLOADS["beam98k_nh_newmark"]
    g = wl["mesh"]()
    _, rho, E, nu, thr = wl["material"]
    r = args.modal_modes
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    s = api.Scene(ctx, g.X, g.tets, g.facets, cd, api.Material("corotational", rho, E, nu, thr))
    s.set_loads(tractions=[([0.0, -wl["traction"], 0.0], g.face_facets(0, 1))])
    ctx.synchronize()
    t0 = time.perf_counter()
    m = api.LinearNewmark(s, r, 0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"], youngs=E, poisson=nu)
    setup_s = time.perf_counter() - t0
    info = m.info
    lam, phi = m.modes()
    m.setExternalVirtualWork()
    u = np.zeros((g.n_nodes, 3))
    L = api.load_library()
    for _ in range(3):
        m.runOneTimeStep()
        L.od_modal_get_displacements(m.h, api._d(u))
    n_steps = max(200, 40 * args.tier_steps)
    t0 = time.perf_counter()
    for _ in range(n_steps):
        api._check(L.od_modal_step(m.h, 1), "od_modal_step")
        api._check(L.od_modal_get_displacements(m.h, api._d(u)), "od_modal_get_displacements")
    gpu_step_s = (time.perf_counter() - t0) / n_steps
    out = {"workload": "beam98k_hooke_modal16", "n_modes": r, "dofs": s.dofs, "krylov": info.krylov,
           "lanczos_applies": info.lanczos_steps, "restarts": info.restarts,
           "pcg_iterations_per_apply": info.pcg_iterations / max(1, info.lanczos_steps),
           "max_residual": info.max_residual, "gpu_setup_s": setup_s,
           "lambda_first_last": [float(lam[0]), float(lam[-1])],
           "gpu_steps_per_s_e2e": 1.0 / gpu_step_s,
           "e2e_note": "per step: od_modal_step + od_modal_get_displacements (the 3 x 18,785 field, pageable "
                       "host buffer)"}
    fext = s.external_forces()
    m.close()
    if not args.no_cpu_baseline:
        try:
            from oracle import modal as MO
            from oracle import reforacle as R
            if not R.available():
                raise RuntimeError("compiled reference not available")
            rs = R.RefScene(g.X, g.tets, g.facets, cd, "corotational", rho, E, nu, thr)
            K, M = MO.reference_matrices(rs, E, nu)
            os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
            t0 = time.perf_counter()
            lam_ref, phi_ref = MO.modes(K, M, r)
            cpu_setup = time.perf_counter() - t0
            o = MO.LinearNewmarkOracle(lam_ref, phi_ref, 0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"])
            o.set_external(fext)
            nc = 50
            t0 = time.perf_counter()
            for _ in range(nc):
                o.step(1)
                MO.to_nodes(o.full_order(), g.n_nodes, cd)
            cpu_step_s = (time.perf_counter() - t0) / nc
            # parity: the same 50 + (3 + n_steps) steps on the GPU modes
            m = api.LinearNewmark(s, r, 0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"], youngs=E, poisson=nu)
            m.setExternalVirtualWork()
            m.runOneTimeStep(nc)
            gpu_u = m.displacements()
            m.close()
            ref_u = MO.to_nodes(o.full_order(), g.n_nodes, cd)
            out.update({
                "cpu_baseline": {"value": 1.0 / cpu_setup, "unit": "setups/s", "cores": 1, "kind": "reference",
                                 "sample": f"ARPACK shift-invert at 0 with SuperLU (scipy eigsh, the algorithm "
                                           f"and libraries EigenSolver links) on the compiled reference's Hooke K "
                                           f"and mass: {cpu_setup:.1f} s for {r} modes of {s.dofs} DOFs; steps: "
                                           f"the restated LinearNewmark step + full-order field in numpy, "
                                           f"{nc} steps"},
                "cpu_setup_s": cpu_setup, "cpu_steps_per_s": 1.0 / cpu_step_s,
                "speedup_setup": cpu_setup / setup_s, "speedup_steps_e2e": cpu_step_s / gpu_step_s,
                "lambda_max_rel_err_vs_arpack": float(np.abs(lam / lam_ref - 1.0).max()),
                "u_rel_err_vs_oracle_after_50_steps": float(np.abs(gpu_u - ref_u).max() / np.abs(ref_u).max())})
        except Exception as exc:
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {exc}"}
    s.close()
    return out


def batched_tier(args, api, ctx):
    """Batched uneven instances: 512 jittered grids (per-axis cube counts
    log-uniform in [4, 40], 6 tets per cube), corotational / Neo-Hookean
    with per-instance E and nu, x = 0 fixed, gravity; Newmark dt 1/60 s,
    Rayleigh 0.01 / 0.001, one Newton iteration, block-Jacobi PCG to 1e-8.
    Plain FP64 path: every scene stepped alone with the FP64 solver; batched
    path: one od_batch step for all scenes with the mixed solver.  Under N
    ranks every rank steps its shard of the scenes (opendeformer_gb300.
    sharding: by tet count, no exchange) and the batch step time is the
    slowest rank's."""
    from opendeformer_gb300 import sharding
    rank, world, _ = env_rank()
    all_insts = meshgen.batch_instances(512)
    ids = list(range(len(all_insts)))
    if world > 1:
        ids = sharding.my_shard([6 * int(np.prod(i["dims"])) for i in all_insts], rank, world)
    insts = [all_insts[i] for i in ids]
    scenes = []
    for inst in insts:
        g = meshgen.instance_grid(inst)
        cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
        kind = "corotational" if inst["kind"] == "corotational" else "neohookean"
        s = api.Scene(ctx, g.X, g.tets, g.facets, cd, api.Material(kind, 1000.0, inst["E"], inst["nu"], 0.1))
        s.set_loads(body=(0.0, 0.0, -9800.0))
        scenes.append(s)

    def setup(prec):
        for s in scenes:
            s.setup_integrator(api.NewmarkIntegrator(0.25, 0.5, 0.01, 0.001, 1 / 60,
                                                     api.CGSolver(1e-8, 5000, api.BlockJacobiPreconditioner(),
                                                                  precision=prec), 1))
    warm, steps = 1, 3
    setup("fp64")
    for _ in range(warm):
        for s in scenes:
            s.step(1)
    t0 = time.perf_counter()
    fp_ms = 0.0
    for _ in range(steps):
        for s in scenes:
            st = s.step(1)
            fp_ms += st.device_ms
            if st.status != 0:
                raise RuntimeError(f"batched tier: FP64 step status {st.status}")
    fp_wall = (time.perf_counter() - t0) / steps
    u64 = [s.displacements() for s in scenes]
    setup("mixed")
    b = api.Batch(ctx, scenes)
    for _ in range(warm):
        b.step(1)
    lat = []
    for _ in range(steps):
        st = b.step(1)
        if any(x.status != 0 for x in st):
            raise RuntimeError("batched tier: batch step failed")
        lat.append(st[0].device_ms)
    ub = [s.displacements() for s in scenes]
    err = max(_rel(a, c) for a, c in zip(ub, u64))
    # autotuner (tile shapes of the inner solve), then steps with the tuned
    # shapes between two runs of steps with the defaults
    default_shape = b.tuning()
    tune = b.autotune(repeats=1)
    tuned = {"choice": {k: tune[k] for k in ("piece_steps", "consumer_warps", "slice_cost")},
             "solve_ms_default": tune.get("default_ms"), "solve_ms_tuned": tune.get("best_ms"),
             "candidates": tune.get("candidates"), "key": tune["key"]}
    def timed(n):
        out = []
        for _ in range(n):
            st = b.step(1)
            if any(x.status != 0 for x in st):
                raise RuntimeError("batched tier: batch step failed")
            out.append(st[0].device_ms)
        return statistics.mean(out)
    t_tuned = timed(steps)
    b.set_tuning(default_shape["piece_steps"], default_shape["slice_cost"], default_shape["consumer_warps"])
    t_default = timed(steps)
    tuned.update({"default": default_shape, "ms_per_step_tuned": t_tuned, "ms_per_step_default_after": t_default,
                  "ms_per_step_default_before": statistics.mean(lat),
                  "gain": 0.5 * (t_default + statistics.mean(lat)) / t_tuned})
    n_tets = sum(s.n_tets for s in scenes)
    b.close()
    for s in scenes:
        s.close()
    bms = statistics.mean(lat)
    if world > 1:   # the job's batch step ends with the slowest rank's shard
        import torch
        import torch.distributed as dist
        t = torch.tensor([bms, fp_wall], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        bms, fp_wall = float(t[0]), float(t[1])
        n = torch.tensor([n_tets], dtype=torch.float64, device="cuda")
        dist.all_reduce(n)
        n_tets = int(n.item())
    lat.sort()
    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        cpu = batched_cpu_baseline(len(all_insts), n_tets)
    return {"workload": "batch512_uneven_newmark", "cpu_baseline": cpu, "ranks": world, "autotune": tuned,
            "sharding": "scenes by tet count (greedy, no exchange)" if world > 1 else None,
            "speedup_batched_vs_cpu": (1000.0 / bms) / cpu["value"] if cpu and cpu.get("value") else None, "instances": len(scenes), "n_tets_total": n_tets,
            "newton_iters": 1, "tol": 1e-8, "precond": "block_jacobi", "warmup": warm, "steps": steps,
            "fp64_alone": {"batch_steps_per_s": 1.0 / fp_wall, "wall_ms_per_step": 1000.0 * fp_wall,
                           "device_ms_per_step": fp_ms / steps},
            "batched_mixed": {"batch_steps_per_s": 1000.0 / bms, "scene_steps_per_s": 1000.0 * len(scenes) / bms,
                              "ms_per_step": bms, "p50_ms": lat[len(lat) // 2],
                              "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
            "speedup_batched_mixed_vs_fp64_alone": fp_wall * 1000.0 / bms,
            "max_rel_err_vs_fp64": err}


def batched_cpu_baseline(n_inst, n_tets, budget=20.0):
    """P = host cores oracle processes, each owning a shard of the batch's
    instances, step them one by one for a bounded time; the batch's CPU
    throughput is extrapolated by tets (work per scene step ~ its tets)."""
    P = cpu_processes()
    order = np.random.default_rng(11).permutation(n_inst)
    jobs = [([int(i) for i in order[w::P]], budget) for w in range(P)]
    t0 = time.perf_counter()
    res = cpu_pool_map(_cpu_batch_worker, jobs)
    rate = sum(t / s for t, _, s in res if s > 0)   # tets stepped per second, all processes
    scenes = sum(n for _, n, _ in res)
    sampled = sum(t for t, _, _ in res)
    return {"value": rate / n_tets if rate else None, "unit": "batch steps/s", "cores": P, "kind": "port",
            "cpu": host_cpu_model(),
            "sample": f"{scenes} of the {n_inst} instances stepped once ({sampled / 1e6:.2f}M tets) by {P} "
                      f"single-threaded oracle processes (FP64 block-Jacobi PCG, the oracle's restatement) in "
                      f"{budget:.0f} s each; batch steps/s = summed tets per second / the batch's {n_tets} "
                      f"tets (extrapolated), wall {time.perf_counter() - t0:.0f} s"}


def serving_cpu_baseline(pool_n, budget=20.0):
    """P = host cores oracle processes serve sampled requests of the serving
    workload back to back: the CPU server's capacity in steps/s."""
    P = cpu_processes()
    jobs = [(100 + w, pool_n, budget) for w in range(P)]
    t0 = time.perf_counter()
    res = cpu_pool_map(_cpu_serving_worker, jobs)
    cap = sum(n / s for n, s in res if s > 0)
    n = sum(r for r, _ in res)
    return {"value": cap, "unit": "steps/s", "cores": P, "kind": "port", "cpu": host_cpu_model(),
            "sample": f"{n} requests (scene, dt, gravity, load drawn as the workload's) served back to back by "
                      f"{P} single-threaded oracle processes (FP64 block-Jacobi PCG at 1e-6, the oracle's "
                      f"restatement), {budget:.0f} s each, scene construction not counted; capacity = summed "
                      f"requests per second of stepping, wall {time.perf_counter() - t0:.0f} s"}


def _pool_mesh(inst):
    g = meshgen.pool_grid(inst)
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    return (g.X, g.tets, g.facets, cd, g.face_facets(0, 1))


def serving_tier(args, api, ctx):
    """Serving: Poisson arrivals of step requests over a pool of scenes whose
    sizes are log-uniform in [1e3, 2e5] tets (random aspect ratios 1-8),
    corotational / Neo-Hookean; per request a time step (uniform 1/120 to
    1/30 s), a gravity direction and a 10-1000 Pa surface load (log-uniform);
    PCG at 1e-6; admission by a device-memory budget smaller than the pool
    (half of its resident size), LRU eviction, scenes built by the library's
    admission thread while ticks run.  The pool is the first
    args.serving_pool scenes of the 4096-scene pool.  The batched server
    (one od_batch step per tick, mixed solver) and the plain path (each
    request stepped alone with the FP64 solver) serve the same arrival
    sequence at the configured rate, which saturates both: their completed
    steps per second are the capacities.  The batched server then serves a
    rate of half its capacity, where p50/p99 are service latencies."""
    from opendeformer_gb300 import serving
    pool = meshgen.serving_pool(4096)[: args.serving_pool]
    n_tets = sum(6 * int(np.prod(p["dims"])) for p in pool)
    budget = int(args.serving_budget_frac * 2600 * n_tets)
    t0 = time.perf_counter()
    meshes = cpu_pool_map(_pool_mesh, pool) if len(pool) > 32 else [_pool_mesh(p) for p in pool]
    mesh_s = time.perf_counter() - t0

    def requests(rate, window, seed):
        rng = np.random.default_rng(seed)
        arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * window * 1.2) + 16))
        arr = arr[arr < window]
        reqs = []
        for _ in arr:
            gdir = rng.normal(size=3)
            reqs.append((int(rng.integers(len(pool))), float(rng.uniform(1 / 120, 1 / 30)),
                         tuple(gdir / np.linalg.norm(gdir)), float(np.exp(rng.uniform(np.log(10.0), np.log(1000.0))))))
        return arr, reqs

    def run(batched, rate, window, seed):
        prec = "mixed" if batched else "fp64"
        sv = serving.Server(ctx, budget_bytes=budget, batched=batched)
        for inst, m in zip(pool, meshes):
            sv.add_scene(serving.SceneSpec(build=lambda m=m: m,
                                           material=api.Material(inst["kind"], 1000.0, inst["E"], inst["nu"], 0.1),
                                           tol=1e-6, precision=prec))
        ctx.reset_counters()
        tw = time.perf_counter()
        warmed = sv.warm(range(len(pool)))
        warm_s = time.perf_counter() - tw
        arr, reqs = requests(rate, window, seed)

        def make(k):
            sid, dt, gdir, tr = reqs[k]
            return serving.StepRequest(scene=sid, arrival=0.0, dt=dt, gravity=gdir, traction=tr)
        done, wall, backlog = serving.wall_clock_loop(sv, arr, window, make)
        stats = sv.stats
        sv.close()
        lat = sorted(1000.0 * (r.done - r.arrival) for r in done)
        bad = [r for r in done if r.status != 0]
        its = sorted(r.pcg_iterations for r in done if r.status == 0)
        return {"offered_per_s": rate, "window_s": window, "offered": len(arr), "completed": len(done),
                "failed": len(bad), "backlog_at_end": backlog, "steps_per_s": len(done) / wall,
                "ok_steps_per_s": (len(done) - len(bad)) / wall,
                "p50_ms": lat[len(lat) // 2] if lat else None,
                "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))] if lat else None,
                "mean_batch": stats["steps"] / max(1, stats["ticks"]), "warmed_scenes": warmed, "warm_s": warm_s,
                "pcg_iterations": {"mean": float(np.mean(its)) if its else None,
                                   "p50": its[len(its) // 2] if its else None,
                                   "p99": its[min(len(its) - 1, int(0.99 * len(its)))] if its else None,
                                   "max": its[-1] if its else None},
                "fp64_fallbacks": ctx.counters().mix_fallbacks,
                "fp64_fallback_s": ctx.counters().mix_fallback_ms / 1000.0,
                "failed_detail": [{"scene": r.scene, "status": r.status, "iterations": r.pcg_iterations,
                                   "E": pool[r.scene]["E"], "kind": pool[r.scene]["kind"]} for r in bad][:4],
                **{k: stats[k] for k in ("ticks", "admissions", "restores", "evictions", "deferred", "s_admit",
                                         "s_loads", "s_step", "s_build", "s_device", "s_worker")}}

    window = args.serving_seconds
    sat_b = run(True, args.serving_rate, window, 9)
    sat_p = run(False, args.serving_rate, window, 9)
    # rate sweep below the batched capacity: the highest rate whose queue
    # stays flat (backlog at the end within 2% of the offered requests) is
    # the sustainable one, and its p50 / p99 are service latencies
    sweep = []
    for frac in (0.15, 0.3, 0.6):
        rate = max(5.0, frac * sat_b["ok_steps_per_s"])
        r = run(True, rate, max(5.0, 0.5 * window), 10)
        sweep.append({k: r[k] for k in ("offered_per_s", "ok_steps_per_s", "p50_ms", "p99_ms", "backlog_at_end",
                                        "offered", "mean_batch", "admissions", "evictions")})
    flat = [x for x in sweep if x["backlog_at_end"] <= 0.02 * max(1, x["offered"])]
    sustain = max(flat, key=lambda x: x["offered_per_s"]) if flat else min(sweep, key=lambda x: x["offered_per_s"])
    cpu = serving_cpu_baseline(len(pool)) if not args.no_cpu_baseline else None
    return {"workload": "serving_pool_poisson", "pool_scenes": len(pool), "pool_tets": n_tets,
            "scaled": (f"the configuration's full size: {len(pool)} scenes ({n_tets / 1e6:.0f}M tets, more than "
                       f"the {budget / 1e9:.0f} GB budget holds, so scenes are evicted and restored), {window:.0f} s "
                       f"windows" if len(pool) >= 4096 and window >= 60 else
                       f"pool {len(pool)} of the configuration's 4096 scenes and {window:.0f} s windows of its 60 s, "
                       f"so that the default bench run ends within minutes (--serving-pool 4096 --serving-seconds 60 "
                       f"runs the full size: about 12 minutes)"),
            "budget_bytes": budget, "tol": 1e-6, "mesh_s": mesh_s, "cpu_baseline": cpu,
            "saturation_steps_per_s": sat_b["ok_steps_per_s"], "plain_saturation_steps_per_s": sat_p["ok_steps_per_s"],
            "throughput_ratio_batched_vs_plain": sat_b["ok_steps_per_s"] / max(1e-9, sat_p["ok_steps_per_s"]),
            "sustainable": {**sustain, "queue_flat": bool(flat)},
            "rate_sweep": sweep,
            "note": "throughput counts successful steps (a diverged scene's requests fail and are not counted); "
                    "latency = completion - arrival on the server clock; at the saturating rate the queue grows "
                    "(p50/p99 there are queueing, not service); requests past the window are not waited for",
            "batched_mixed": sat_b, "plain_fp64": sat_p}


def tiers_summary(line):
    """The figures of every workload in a few hundred bytes."""
    def g(d, *path):
        for k in path:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return float(f"{d:.4g}") if isinstance(d, float) else d
    out = {"headline_steps_per_s": g(line, "value"), "e2e_steps_per_s": g(line, "e2e", "value"),
           "cpu_ref_steps_per_s": g(line, "cpu_baseline", "value"),
           "headline_rel_err_vs_oracle": g(line, "parity", "headline_rel_err"),
           "pcg_fp64_frac": g(line, "roofline", "fp64", "frac")}
    if "precision_tier" in line:
        t = line["precision_tier"]
        out["precision"] = {"speedup_mixed_vs_fp64": g(t, "speedup_mixed_vs_fp64"),
                            "speedup_full_layout": g(t, "speedup_mixed_full_vs_fp64"),
                            "mixed_steps_per_s": g(t, "mixed", "steps_per_s"),
                            "fp64_steps_per_s": g(t, "fp64", "steps_per_s"),
                            "inner_iters": g(t, "mixed", "pcg_iterations_per_step"),
                            "fp64_iters": g(t, "fp64", "pcg_iterations_per_step"),
                            "rel_err_vs_oracle": g(t, "oracle", "rel_err_mixed_vs_oracle"),
                            "spmv_frac": g(t, "spmv_roofline", "frac"),
                            "spmv_frac_with_sum": g(t, "spmv_roofline", "with_grid_sum", "frac"),
                            "cpu_steps_per_s": g(t, "oracle", "cpu_baseline", "value")}
    if "batched_tier" in line:
        t = line["batched_tier"]
        out["batched"] = {"speedup_vs_fp64_alone": g(t, "speedup_batched_mixed_vs_fp64_alone"),
                          "autotune_gain": g(t, "autotune", "gain"),
                          "batch_steps_per_s": g(t, "batched_mixed", "batch_steps_per_s"),
                          "rel_err_vs_fp64": g(t, "max_rel_err_vs_fp64"),
                          "cpu_batch_steps_per_s": g(t, "cpu_baseline", "value")}
    if "serving_tier" in line:
        t = line["serving_tier"]
        out["serving"] = {"ratio_vs_plain": g(t, "throughput_ratio_batched_vs_plain"),
                          "saturation_steps_per_s": g(t, "saturation_steps_per_s"),
                          "sustainable_rate": g(t, "sustainable", "offered_per_s"),
                          "queue_flat": g(t, "sustainable", "queue_flat"),
                          "p50_ms": g(t, "sustainable", "p50_ms"), "p99_ms": g(t, "sustainable", "p99_ms"),
                          "cpu_steps_per_s": g(t, "cpu_baseline", "value")}
    if "ic0_tier" in line:
        t = line["ic0_tier"]
        out["ic0"] = {"steps_per_s": g(t, "steps_per_s"), "levels": g(t, "apply", "levels"),
                      "iters": g(t, "pcg_iterations_per_step")}
    if "sweep_tier" in line:
        t = line["sweep_tier"]
        out["sweep"] = {k: g(t, k, "steps_per_s") for k in ("ic", "ldlt") if isinstance(t.get(k), dict)}
    if "modal_tier" in line:
        t = line["modal_tier"]
        out["modal"] = {"gpu_setup_s": g(t, "gpu_setup_s"), "cpu_setup_s": g(t, "cpu_setup_s"),
                        "speedup_setup": g(t, "speedup_setup"), "steps_per_s_e2e": g(t, "gpu_steps_per_s_e2e"),
                        "speedup_steps_e2e": g(t, "speedup_steps_e2e"),
                        "lambda_rel_err": g(t, "lambda_max_rel_err_vs_arpack"),
                        "u_rel_err": g(t, "u_rel_err_vs_oracle_after_50_steps")}
    return out


def run_gpu(args, wl):
    import torch
    from opendeformer_gb300 import api

    rank, world, local_rank = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local_rank)
    g = wl["mesh"]()
    cd = meshgen.constrained_dofs_for_nodes(g.face_nodes(0, 0))
    kind, rho, E, nu, thr = wl["material"]
    ctx = api.Context(local_rank)
    # the device's FP64 / FP32 multiply-add rates: the roofline of the FP64
    # solve and element kernels (measured here, outside the timed region)
    fma64, _ = ctx.measure_fma_rate(True)
    fma32, _ = ctx.measure_fma_rate(False)
    scene = api.Scene(ctx, g.X, g.tets, g.facets, cd, api.Material(kind, rho, E, nu, thr))
    solver = api.CGSolver(wl["tol"], 5000, api.Preconditioner(args.precond), precision=args.precision)
    integ = api.NewmarkIntegrator(0.25, 0.5, wl["alpha_m"], wl["beta_k"], wl["dt"], solver, wl["newton"])
    scene.setup_integrator(integ)
    groups = traction_groups(g, wl["traction"])
    scene.set_loads(body=wl["body"], tractions=groups)
    if wl["freq"]:
        scene.set_traction_schedule(wl["freq"])
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        st = scene.step(1)
        if st.status not in (0, 3):
            raise RuntimeError(f"step failed with status {st.status}")
    flush.zero_()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.5)   # let nvidia-smi start up before the timed steps (it competes for the host thread)
    ctx.reset_counters()
    ctx.set_profiling(True)
    dev_ms, iters, solves, worst = 0.0, 0, 0, 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = scene.step(1)
        dev_ms += st.device_ms
        iters += st.pcg_iterations
        solves += st.solves
        worst = max(worst, st.max_rel_residual)
        flush.zero_()          # L2 flush between timed steps (outside the step's events)
        torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ctx.set_profiling(False)
    counters = ctx.counters()
    # one more step, untimed, with the one-launch PCG's per-iteration phase
    # timers on (they add clock reads and a CTA barrier to every iteration)
    ctx.reset_counters()
    ctx.set_profiling(2)
    scene.step(1)
    ctx.set_profiling(False)
    phase_counters = ctx.counters()
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    total_ms = dev_ms
    if dist:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * args.steps / (total_ms / 1000.0)

    # end to end through the public API with host buffers: per step the
    # traction arrays go host->device (pinned), the displacement field comes back
    e2e = None
    if not args.no_e2e:
        fac = groups[0][1] if groups else np.zeros(0, np.int32)
        ids_h = torch.from_numpy(np.ascontiguousarray(fac, dtype=np.int32)).pin_memory()
        u_h = torch.empty((g.n_nodes, 3), dtype=torch.float64).pin_memory()
        scene.set_traction_schedule(0.0)
        h2d = ids_h.numel() * 4 + 3 * 8 + 4 + (24 if wl["body"] else 0)
        d2h = u_h.numel() * 8
        tt = scene_time = (args.warmup + args.steps) * wl["dt"]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(args.steps):
            tt += wl["dt"]
            scale = math.sin(2 * math.pi * wl["freq"] * tt) if wl["freq"] else 1.0
            ids = ids_h.numpy()
            tr = [([0.0, -wl["traction"] * scale, 0.0], ids)] if groups else []
            scene.set_loads(body=wl["body"], tractions=tr)
            scene.step(1)
            api._check(api.load_library().od_scene_get_displacements(
                scene.h, u_h.numpy().ctypes.data_as(api._dp)), "get_displacements")
        e2e_wall = time.perf_counter() - t1
        del scene_time
        e2e_v = args.steps / e2e_wall
        if dist:
            t = torch.tensor([e2e_wall], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_v = world * args.steps / float(t.item())
        e2e = {"value": e2e_v, "unit": "steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}

    info = scene.info
    peak, peak_kind = peaks()
    if counters.pcg_launches:
        # persistent PCG solve kernel: one launch per linear solve
        per_iter = pcg_iteration_bytes(info, args.precond)
        init = spmv_bytes(info) + 6 * 8 * info.dofs
        avg_iters = counters.pcg_iterations / counters.pcg_launches
        nbytes = init + avg_iters * per_iter
        avg_ms = counters.pcg_ms / counters.pcg_launches
        kname = "pcg_persistent_kernel<double> (whole FP64 PCG solve, one cooperative launch)"
        kms, kl = counters.pcg_ms, counters.pcg_launches
        tkey = "pcg_persistent_kernel"
    else:
        nbytes = spmv_bytes(info)
        avg_ms = counters.spmv_ms / max(1, counters.spmv_launches)
        kname = "pcg_spmv_kernel<double> (full-BSR FP64 SpMV + p.q)"
        kms, kl = counters.spmv_ms, counters.spmv_launches
        tkey = "pcg_spmv_kernel"
    achieved = nbytes / (avg_ms * 1e-3) / 1e9 if kl else None
    traffic = traffic_from_profiles(args.workload, tkey)
    fp64 = None
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    peak64 = 2.0 * fma64 / 1e9
    if counters.pcg_launches:
        fmas = 9 * info.num_full_blocks + avg_iters * pcg_iteration_fmas(info, args.precond)
        ach64 = 2.0 * fmas / (avg_ms * 1e-3) / 1e9
        fp64 = {"bound": "fp64", "achieved": ach64, "peak": peak64, "unit": "GFLOP/s", "frac": ach64 / peak64,
                "peak_source": "measured in this run: od_measure_fma_rate (independent FP64 multiply-add "
                               "chains on every SM at full occupancy, CUDA events)",
                "fma_per_launch": fmas,
                "peak_fma_per_sm_per_cycle": fma64 / (torch.cuda.get_device_properties(local_rank).multi_processor_count * sm_mhz * 1e6),
                "fp32_peak_gflops": 2.0 * fma32 / 1e9,
                "pipe_active_pct_ncu": traffic_from_profiles(args.workload, tkey, "fp64_pipe_pct"),
                "pipe_source": "ncu --set full capture of this kernel on this workload "
                               "(sm__pipe_fp64_cycles_active, of peak, active cycles)"}
    phases = None
    pc = phase_counters
    if pc.pcg_phase_iterations:
        names = ("spmv_pq", "pq_sum", "update_rz_rr", "rz_rr_sum", "direction", "barrier")
        phases = {k: round(1000.0 * pc.pcg_phase_ms[j] / pc.pcg_phase_iterations, 3) for j, k in enumerate(names)}
        for j, k in enumerate(("spmv_pq", "update_rz_rr", "direction")):
            phases[f"{k}_cta_max"] = round(1000.0 * pc.pcg_work_max_ms[j] / pc.pcg_phase_iterations, 3)
            phases[f"{k}_cta_mean"] = round(1000.0 * pc.pcg_work_mean_ms[j] / pc.pcg_phase_iterations, 3)
        phases["iterations"] = pc.pcg_phase_iterations
        phases["us_per_iteration_timed_steps"] = round(1000.0 * counters.pcg_ms / max(1, counters.pcg_iterations), 3)
        phases["note_pipelined"] = ("the pipelined form (one sync per iteration, the default for this tolerance "
                                    "and size) fills spmv_pq (the product and the recurrences), update_rz_rr (the "
                                    "dot partials and M^-1 w) and rz_rr_sum (its one grid-wide sum); the other "
                                    "phases and the per-CTA figures stay 0")
        phases["note"] = ("one extra step after the timed ones with the phase timers on: us per PCG iteration "
                          "on the clock of CTA 0 (%globaltimer); a *_sum or barrier phase includes the wait for "
                          "the slowest CTA; *_cta_max / *_cta_mean: every CTA's own work in the phase (its warps, "
                          "no waits), slowest CTA per solve and mean; the timers themselves add about 2 us")
    roofline = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "peak_source": peak_kind, "algorithmic_bytes_per_launch": nbytes,
                "avg_launch_ms": avg_ms, "launches": kl,
                "share_of_step_time": kms / total_ms if total_ms else None, "fp64": fp64,
                "pcg_phases_us_per_iteration": phases,
                "note": "the binding roofline is fp64 (FP64 pipe and grid barriers): the 98k-tet system "
                        "(18.6 MB) stays L2-resident, so DRAM traffic (traffic) is far below the algorithmic "
                        "bytes"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            n, secs = cpu_reference_sample(wl)
            cpu = {"value": n / secs, "unit": "steps/s", "cores": 1, "kind": "reference",
                   "sample": f"{n} Newmark steps of the same workload, reference CPU code (Jacobi PCG), "
                             f"single thread, {secs:.1f} s"}
        except Exception as exc:
            cpu = {"value": None, "unit": "steps/s", "cores": 1, "kind": "reference", "sample": f"failed: {exc}"}
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            parity = headline_parity(args, wl, api, ctx)
        except Exception as exc:
            parity = {"error": str(exc)}
    tiers = {}
    if world > 1 and not args.no_tiers:
        # a multi-rank job runs the sharded workload only (the others are
        # single-GPU configurations)
        del scene
        try:
            tiers["batched_tier"] = batched_tier(args, api, ctx)
        except Exception as exc:
            tiers["batched_tier"] = {"error": str(exc)}
    elif rank == 0 and not args.no_tiers:
        del scene
        only = [t for t in args.only_tiers.split(",") if t]
        for name, fn in (("precision_tier", precision_tier), ("batched_tier", batched_tier),
                         ("serving_tier", serving_tier), ("sweep_tier", sweep_tier),
                         ("ic0_tier", ic0_tier), ("relabel_tier", relabel_tier), ("modal_tier", modal_tier)):
            if only and name.split("_")[0] not in only:
                continue
            try:
                tiers[name] = fn(args, api, ctx)
            except Exception as exc:
                tiers[name] = {"error": str(exc)}
    if rank == 0:
        line = {"metric": "newmark_steps_per_s", "value": value, "unit": "steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32/f64",
                "data": "synthetic",
                "config": {"workload": args.workload, "n_tets": g.n_tets, "n_nodes": g.n_nodes,
                           "dofs": info.dofs, "precond": args.precond, "precision": args.precision,
                           "newton_iters": wl["newton"], "dt": wl["dt"], "tol": wl["tol"],
                           "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                           "l2": "flushed between timed steps (256 MiB write, outside the step events)",
                           "pcg_iterations_per_step": iters / args.steps,
                           "solves_per_step": solves / args.steps, "max_rel_residual": worst,
                           "wall_s_timed_region": wall},
                "e2e": e2e, "gpu_launches": counters.kernel_launches, "clocks": clocks, "roofline": roofline,
                "cpu_baseline": cpu, "parity": parity}
        line.update(tiers)
        line["tiers_summary"] = tiers_summary(line)   # last: the part of the line a log tail keeps
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="beam98k_nh_newmark")
    ap.add_argument("--precond", choices=["block_jacobi", "ic0", "jacobi", "none"], default="block_jacobi")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tiers", action="store_true", help="skip the mixed-precision and batched workloads")
    ap.add_argument("--tier-steps", type=int, default=5)
    ap.add_argument("--only-tiers", default="", help="comma list of precision,batched,serving,sweep,ic0,relabel,modal (default: all)")
    ap.add_argument("--precision-nz", type=int, default=64,
                    help="cube layers of the precision-tier block (64: 2,621,440 tets)")
    ap.add_argument("--precision-variants", default="fp64,mixed,mixed_full,mixed_ic0",
                    help="comma list of the precision tier's solvers (fp64, mixed, mixed_full, mixed_ic0)")
    ap.add_argument("--modal-modes", type=int, default=16)
    ap.add_argument("--serving-pool", type=int, default=512)
    ap.add_argument("--serving-rate", type=float, default=2000.0)
    ap.add_argument("--serving-seconds", type=float, default=15.0)
    ap.add_argument("--serving-budget-frac", type=float, default=0.5,
                    help="device budget as a fraction of the pool's estimated resident bytes")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_gpu(args, wl)


if __name__ == "__main__":
    sys.exit(main())
