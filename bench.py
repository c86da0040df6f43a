"""Benchmark: Stokes ms per time step to a 1e-6 residual on one GB300.

Workload (default, --workload cfg2): the 2 x 2 x 1 box of 128 x 128 x 64 Q1
elements, 6 multigrid levels (4 x 4 x 2 .. 128 x 128 x 64), eta =
exp(-ln(1e4) T) times 30 below z = 0.8, Ra 1e6, internal heating Q0 = 1,
free-slip walls, seeded initial T = 1 - z + U(-0.01, 0.01) (numpy PCG64 seed
0), multigrid knobs of the reference's example deck.  --workload cube is the
64^3 unit box (eta = exp(-ln(1e3) T), Ra 1e5), --workload sphere the
192 x 192 x 96 regional spherical segment.

Stopping: the residual rule.  Every Stokes solve runs until both FP64
residuals of its solution are at most 1e-6: |F - K U - G P| / |F| and
|B U| / (|U| sqrt(npno/neq)) (Uzawa iterations capped at 1000).  The
reference's own rule (dv/v and dp/p below 1e-6, at most 375 iterations) is
timed beside it on cold solves (`cold_solve.reference_rule`).

A step is one time step of the reference's loop (Citcom.c:111-161) on state
resident in HBM: PG_timestep, then general_stokes_solver (forces, viscosity
from T, projection to every level, operator assembly, the Uzawa/multigrid
solve from the previous step's U, P, and V).  Each mode starts from the
seeded state with one untimed cold solve, runs `--warmup` untimed steps and
then `--steps` timed ones.  `value` is the mean device time (CUDA events
inside the library, on its stream) of the Stokes part of a timed step in the
headline configuration: FP32 multigrid inside FP64 refinement with the
learned warm start.  `ms_per_step` adds PG_timestep.  The same loop runs
without the network (`mixed`) and on the FP64 plain path (`fp64_plain`); each
mode reports the errors of its U, P, Nu and Vrms against the FP64 plain path
after the same steps.  The network is trained online first on converged
solves of other seeds (training time reported, not timed into `value`).
`e2e` runs the headline loop through the C ABI with host buffers (pinned):
PG_timestep and general_stokes_solver per step, the copies inside the timed
region.  `drift` runs the 64^3 box (mixed vs FP64 plain) for --drift-steps
steps (200, that benchmark's run length) and reports the per-step Nu / Vrms
drift; with --drift-workload equal to --workload it also runs the trained
learned path against FP64 plain.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]
                  [--workload cfg2|cube|sphere] [--no-cpu] [--no-learned]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Stokes ms/step to 1e-6 residual: FP64 plain vs FP32 MG + learned warm start"
UNIT = "ms/step"
TOL = 1e-6
ITER_CAP = 1000


def workload(size: int):
    """The unit box of size^3 elements, eta = exp(-ln(1e3) T), Ra 1e5."""
    from citcomcu_gb300 import Config
    levels = {64: 5, 32: 4, 128: 6, 16: 3}[size]
    return Config(mgunit=(4, 4, 4), levels=levels, rayleigh=1e5, tdepv=True, visc0=(1.0,),
                  viscE=(math.log(1e3),), viscT=(0.0,), accuracy=TOL, piterations=ITER_CAP, stop_rule=1)


def cfg2_workload():
    """The 2 x 2 x 1 box of 128 x 128 x 64 elements, 6 multigrid levels,
    eta = exp(-ln(1e4) T) times 30 below z = 0.8, Ra 1e6, internal heating
    Q0 = 1."""
    from citcomcu_gb300 import Config
    return Config(mgunit=(4, 4, 2), levels=6, dimen=(2.0, 2.0, 1.0), rayleigh=1e6, Q0=1.0, tdepv=True,
                  visc0=(1.0, 30.0), viscE=(math.log(1e4), math.log(1e4)), viscT=(0.0, 0.0), z_layer=(0.8,),
                  accuracy=TOL, piterations=ITER_CAP, stop_rule=1)


def sphere_workload():
    """Regional spherical shell segment: colatitude 45-135 deg, longitude
    0-90 deg, radius 0.55-1.0, 192 x 192 x 96 elements, 6 multigrid levels,
    eta = exp(-ln(1e5) T) times 30 below r = 0.9, Ra 1e7."""
    from citcomcu_gb300 import Config
    return Config(mgunit=(6, 6, 3), levels=6, rayleigh=1e7, tdepv=True, visc0=(1.0, 30.0),
                  viscE=(math.log(1e5), math.log(1e5)), viscT=(0.0, 0.0), z_layer=(0.9,), accuracy=TOL,
                  piterations=ITER_CAP, stop_rule=1, sphere=(45.0, 135.0, 0.0, 90.0, 0.55, 1.0))


def seeded_T0_sphere(case, seed: int = 0):
    """Conductive shell profile T = (1/r - 1/ro) / (1/ri - 1/ro) plus seeded
    uniform noise of +-0.01 on the interior (numpy PCG64)."""
    ri, ro = case.sphere[4], case.sphere[5]
    rng = np.random.Generator(np.random.PCG64(seed))
    r = np.linspace(ri, ro, case.noz)
    T = np.empty((case.noy, case.nox, case.noz))
    T[:] = (1.0 / r - 1.0 / ro) / (1.0 / ri - 1.0 / ro)
    T += rng.uniform(-0.01, 0.01, size=T.shape)
    T[:, :, 0] = 1.0
    T[:, :, -1] = 0.0
    return T.reshape(-1)


def seeded_T0(case, seed: int = 0):
    rng = np.random.Generator(np.random.PCG64(seed))
    z = np.linspace(0.0, case.dimen[2], case.noz)
    T = np.empty((case.noy, case.nox, case.noz))
    T[:] = 1.0 - z / case.dimen[2]
    T += rng.uniform(-0.01, 0.01, size=T.shape)
    T[:, :, 0] = 1.0
    T[:, :, -1] = 0.0
    return T.reshape(-1)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(values, world: int, device: str = "cuda"):
    """The per-rank times reduced to their maximum over the replicas (a
    replica run is as slow as its slowest rank); identity for one rank."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def whole_job_value(ms_per_step_max: float, world: int) -> float:
    """Whole-job ms per step of N replicas that each ran the same steps in
    the same wall time: N steps complete per step time."""
    return ms_per_step_max / max(world, 1)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------- algorithmic bytes
def gs_sweep_bytes(nno: int, nel: int, word: int) -> int:
    """Algorithmic bytes of one Gauss-Seidel sweep (all 8 colours) of a
    level: read F, read and write d (9 words per node), read 1/diag K (3 words
    per node), the viscosity at the 8 Gauss points of every element (FP32)
    and one byte of boundary flags per node."""
    return nno * word * 12 + 32 * nel + nno


def bytes_per_sweep(nno: int, word: int) -> int:
    """Bytes one sweep of the stored-stencil smoother moves at the least: the
    243 coefficients and 3 inverse diagonals of every node, the right-hand
    side, one write of d, and the whole d vector read once per colour launch
    (its 27-neighbourhoods)."""
    return nno * word * (243 + 3 + 3 + 3 + 8 * 3)


# DRAM bytes (read + write) of one finest-level FP32 Gauss-Seidel colour launch
# of the stored-stencil kernel (k_tile<float, 0>) on the 1,081,665-node level
# of the 128x128x64 box: median of the 48 finest launches of one time step
# captured by ncu (dram__bytes_read.sum + dram__bytes_write.sum, cold caches);
# scaled by nodes for other levels.
TRAFFIC_PER_LAUNCH_NODES = 1081665
TRAFFIC_PER_LAUNCH = 150.02e6


# --------------------------------------------------------------- GPU arm
def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def rel_p(a, b):
    """Relative L2 difference of two pressure fields after removing their
    means (the free-slip box fixes the pressure only up to a constant)."""
    a, b = np.asarray(a), np.asarray(b)
    return rel(a - a.mean(), b - b.mean())


def nvtx_range(push: bool, pop: bool = False, name: str = "timed_step"):
    """Marks each timed step as an NVTX range (timed_learned, timed_mixed,
    timed_fp64, ...), so that a kernel profiler can capture exactly the
    launches of one mode's timed steps (ncu --nvtx --nvtx-include
    timed_learned/)."""
    if not (push or pop):
        return
    try:
        import torch
        if push:
            torch.cuda.nvtx.range_push(name)
        else:
            torch.cuda.nvtx.range_pop()
    except Exception:
        pass


def run_loop(cg, case, T0, precision, steps, warmup, solver=None, net=None, zero_start=False, tag="step"):
    """The reference's time loop on resident state: one cold solve of the
    seeded state (untimed), then per step PG_timestep and general_stokes_solver
    warm from the previous step's U, P (zero_start: from U = P = 0 instead).
    Device time per step (CUDA events inside the library), after `warmup`
    untimed steps."""
    s = solver or cg.Solver(cg.Config.like(case, precision=precision))
    if net is not None:
        net.attach(True)
    f = s.fine
    s.load_state(T=T0, Tdot=np.zeros(f["nno"]), U=np.zeros(f["neq"]), P=np.zeros(f["nel"]))
    s.stokes_resident()
    cold = s.stats()
    t = 0.0
    recs, nus, vrs = [], [], []
    l0 = None
    zu, zp = np.zeros(f["neq"]), np.zeros(f["nel"])
    for i in range(warmup + steps):
        if i == warmup:
            l0 = s.stats()["kernel_launches"]
        if zero_start:
            s.load_state(U=zu, P=zp)
        nvtx_range(i >= warmup, name=f"timed_{tag}")
        adv = s.step_resident(t)
        nvtx_range(False, i >= warmup)
        t = adv["elapsed_time"]
        st = s.stats()
        if i >= warmup:
            recs.append(st)
        nus.append(s.heat_flux()[0])
        vrs.append(s.vrms())
    launches = recs[-1]["kernel_launches"] - l0 if recs else 0
    state = s.store_state()
    if net is not None:
        net.attach(False)
    if solver is None:
        s.close()
    return {"recs": recs, "cold": cold, "launches": launches, "state": state, "nu": nus, "vrms": vrs,
            "elapsed_time": t}


def loop_summary(r, ref=None):
    recs = r["recs"]
    d = {"stokes_ms_per_step": float(np.mean([x["stokes_ms"] for x in recs])),
         "ms_per_step": float(np.mean([x["stokes_ms"] + x["energy_ms"] for x in recs])),
         "multigrid_ms_per_step": float(np.mean([x["pass_ms"] for x in recs])),
         "assembly_ms_per_step": float(np.mean([x["assembly_ms"] for x in recs])),
         "uzawa_iterations": [x["uzawa"] for x in recs], "mg_passes": [x["mg_passes"] for x in recs],
         "corrections": [x["corrections"] for x in recs],
         "residuals_final_max": [max(x["final_momentum"] for x in recs), max(x["final_continuity"] for x in recs)],
         "cold_solve_ms": r["cold"]["stokes_ms"], "cold_uzawa": r["cold"]["uzawa"],
         "nu_top": r["nu"][-1], "vrms": r["vrms"][-1]}
    if ref is not None:
        a, b = r["state"], ref["state"]
        d["errors_vs_fp64"] = {"U": rel(a["U"], b["U"]), "P": rel_p(a["P"], b["P"]), "T": rel(a["T"], b["T"]),
                               "Nu": abs(r["nu"][-1] - ref["nu"][-1]) / abs(ref["nu"][-1]),
                               "Vrms": abs(r["vrms"][-1] - ref["vrms"][-1]) / abs(ref["vrms"][-1])}
    return d


def cold_solves(cg, case, T0, precision, reps, solver=None, net=None, **over):
    """`reps` cold solves of the seeded state (U = P = 0) with the given
    stopping rule; device ms, iterations and passes of each."""
    s = solver or cg.Solver(cg.Config.like(case, precision=precision, **over))
    if net is not None:
        net.attach(True)
    f = s.fine
    out = []
    for _ in range(reps):
        s.load_state(T=T0, Tdot=np.zeros(f["nno"]), U=np.zeros(f["neq"]), P=np.zeros(f["nel"]))
        s.stokes_resident()
        st = s.stats()
        res = s.stokes_residuals()
        out.append({"ms": st["stokes_ms"], "uzawa": st["uzawa"], "mg_passes": st["mg_passes"],
                    "residuals": list(res), "warm_start": st["warm_start"]})
    if net is not None:
        net.attach(False)
    if solver is None:
        s.close()
    return {"ms": float(np.mean([o["ms"] for o in out])), "uzawa": [o["uzawa"] for o in out],
            "mg_passes": [o["mg_passes"] for o in out], "residuals": out[-1]["residuals"],
            "warm_start": [o["warm_start"] for o in out]}


def train_warm_start(cg, case, T0_of, seeds: int, steps_per_seed: int, train_steps: int, mode: int):
    """The learned warm start, trained online on the plain solver's own
    converged solves: for each training seed (never the benchmark's seed 0) a
    cold solve of its initial state and the time steps that follow, each
    recorded; then Adam steps on random minibatches of the snapshots.  In
    increment mode a snapshot is the change between consecutive steps."""
    s = cg.Solver(cg.Config.like(case, precision=cg.MIXED))
    f = s.fine
    n = cg.WarmStart(s, seed=7, capacity=seeds * (steps_per_seed + 1), mode=mode)
    zn, zu, zp = np.zeros(f["nno"]), np.zeros(f["neq"]), np.zeros(f["nel"])
    t0 = time.perf_counter()
    for seed in range(1, seeds + 1):
        s.load_state(T=T0_of(seed), Tdot=zn, U=zu, P=zp)
        s.stokes_resident()
        n.record()
        for _ in range(steps_per_seed):
            s.step_resident(0.0)
            n.record()
    t1 = time.perf_counter()
    losses = [n.train(1, 4, 1e-3)]
    for lr, k in ((1e-3, train_steps // 2), (3e-4, train_steps // 4), (1e-4, train_steps // 4)):
        losses.append(n.train(k, 4, lr))
    t2 = time.perf_counter()
    info = {"snapshots": n.recorded, "seeds": seeds, "steps_per_seed": steps_per_seed, "adam_steps": train_steps,
            "mode": "increment" if mode else "absolute",
            "batch": 4, "lr": "1e-3, 3e-4, 1e-4 (1/2, 1/4, 1/4 of the steps)", "loss_first": losses[0],
            "loss_final": losses[-1], "record_s": t1 - t0,
            "train_s": t2 - t1, "network_grid": list(n.grid), "params": n.n_params}
    return s, n, info


def e2e_loop(cg, s, T0, steps, warmup):
    """The headline loop through the C ABI with host buffers: per step
    PG_timestep (T, Tdot in/out, V in) and general_stokes_solver (T in, U, P
    in/out, V out), all in pinned host memory allocated once (as the
    reference's E->T, E->U, E->P, E->V); wall time of the Stokes call, its
    host<->device copies included."""
    import torch
    f = s.fine

    def pinned(n):
        return torch.zeros(n, dtype=torch.float64, pin_memory=True).numpy()

    T, Tdot, U, P = pinned(f["nno"]), pinned(f["nno"]), pinned(f["neq"]), pinned(f["nel"])
    V = pinned(3 * f["nno"])
    T[:] = T0
    # a new state sequence (the solver object has run other loops before)
    s.load_state(T=T, Tdot=Tdot, U=U, P=P)
    s.general_stokes_solver(T, U, P, V)  # the cold solve (untimed)
    t = 0.0
    ms, dev, passes, compared = [], [], [], []
    for i in range(warmup + steps):
        t = s.PG_timestep(T, Tdot, V, t)["elapsed_time"]
        t0 = time.perf_counter()
        s.general_stokes_solver(T, U, P, V)
        t1 = time.perf_counter()
        if i >= warmup:
            st = s.stats()
            ms.append(1e3 * (t1 - t0))
            dev.append(st["stokes_ms"])
            passes.append(st["mg_passes"])
            compared.append(st["warm_compared"])
    h2d = 8 * (f["nno"] + f["neq"] + f["nel"])
    d2h = 8 * (f["neq"] + f["nel"] + 3 * f["nno"])
    detail = {"device_stokes_ms": float(np.mean(dev)), "mg_passes": passes, "compared": compared}
    return float(np.mean(ms)), h2d, d2h, detail


def output_step(s, reps: int = 10):
    """One output step of the solved state (heat_flux and averages fields
    computed on the device: the six .ave layer profiles, heatflux,
    heatflux_adv, surface fluxes, Nu, Vrms; plus T, V, P) copied to pinned
    host buffers: wall time of output_async + output_wait."""
    bufs = s.output_buffers(pinned=True)
    for _ in range(3):
        s.output_async(bufs)
        s.output_wait()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        s.output_async(bufs)
        s.output_wait()
        ts.append(1e3 * (time.perf_counter() - t0))
    return {"ms": float(np.median(ts)), "d2h_bytes": 8 * sum(s.output_sizes().values()),
            "fields": "T, V, P, heatflux, heatflux_adv, Have (T, vrms, Vi, Rho, F, f), shflux, bhflux, Nut, Nub, Vrms"}


def drift_run(cg, which, steps, learned=None, control=False):
    """A workload from its seeded state (`which`: "cube" the 64^3 box, eta =
    exp(-ln(1e3) T), Ra 1e5; "cfg2" the 128x128x64 box): `steps` time steps of
    the mixed path and of the FP64 plain path, of the learned path when
    `learned` = (solver, trained network) of the same workload is given, and
    with `control` of the mixed path solving every step from U = P = 0 (the
    same stopping rule from another start); per path against FP64 plain the
    per-step relative differences of Nu and Vrms (every step, and their
    maxima), the Nu differences over the RMS of FP64 plain's Nu over the run,
    and the final U, P, T."""
    case = cfg2_workload() if which == "cfg2" else workload(64)
    T0 = seeded_T0(case)
    r = {"fp64_plain": run_loop(cg, case, T0, cg.FP64, steps, 0), "mixed": run_loop(cg, case, T0, cg.MIXED, steps, 0)}
    if learned is not None:
        r["learned"] = run_loop(cg, case, T0, cg.MIXED, steps, 0, solver=learned[0], net=learned[1])
    if control:
        r["zero_start"] = run_loop(cg, case, T0, cg.MIXED, steps, 0, zero_start=True)
    p = r["fp64_plain"]
    nu_scale = float(np.sqrt(np.mean(np.square(p["nu"]))))

    def against_fp64(m):
        dnu = [abs(a - b) / abs(b) for a, b in zip(m["nu"], p["nu"])]
        dvr = [abs(a - b) / abs(b) for a, b in zip(m["vrms"], p["vrms"])]
        dnus = [abs(a - b) / nu_scale for a, b in zip(m["nu"], p["nu"])]
        return {"nu_rel_drift_per_step": dnu, "vrms_rel_drift_per_step": dvr,
                "nu_rel_drift_max": max(dnu), "vrms_rel_drift_max": max(dvr),
                "nu_drift_over_rms_per_step": dnus, "nu_drift_over_rms_max": max(dnus),
                "final_errors": {"U": rel(m["state"]["U"], p["state"]["U"]),
                                 "P": rel_p(m["state"]["P"], p["state"]["P"]),
                                 "T": rel(m["state"]["T"], p["state"]["T"])}}

    out = {"workload": workload_name(case), "steps": steps, "fp64_nu_per_step": p["nu"],
           "fp64_vrms_per_step": p["vrms"], "fp64_nu_rms": nu_scale}
    out.update(against_fp64(r["mixed"]))
    out["stokes_ms_per_step"] = {k: loop_summary(v)["stokes_ms_per_step"] for k, v in r.items()}
    out["nu_top_final"] = {k: v["nu"][-1] for k, v in r.items()}
    out["uzawa_iterations_total"] = {k: int(sum(x["uzawa"] for x in v["recs"])) for k, v in r.items()}
    if learned is not None:
        lr = r["learned"]
        out["learned"] = against_fp64(lr)
        out["learned"]["warm_start_used"] = int(sum(x["warm_start"] for x in lr["recs"]))
    if control:
        out["zero_start"] = against_fp64(r["zero_start"])
    return out


# --------------------------------------------------------------- CPU side
def oracle_case(case, stop_rule=1):
    from oracle.decks import Case
    c = Case(**{k: getattr(case, k) for k in ("mgunit", "levels", "dimen", "rayleigh", "Q0", "tdepv", "visc0",
                                               "viscE", "viscT", "z_layer", "vmin", "vmax", "aug_lagr",
                                               "aug_number", "precond", "mg_cycle", "down_heavy", "up_heavy",
                                               "vlowstep", "vhighstep", "accuracy", "piterations")})
    c.stop_rule = stop_rule
    return c


def cpu_sample(case, T0, passes_per_step: float):
    """A bounded sample of the oracle port (FP64, lexicographic smoother = the
    reference's algorithm) on the same workload: the set-up of a Stokes solve
    (forces, viscosity on all levels, stiffness assembly) timed in full, then
    the head of the cold solve (one solve_del2_u) timed per multigrid pass;
    scaled to `passes_per_step` passes per time step."""
    from oracle import oracle as O
    O.build()
    c = oracle_case(case)
    o = O.Oracle(c, gs_colored=False)
    o.set_T(T0)
    t0 = time.perf_counter()
    o.setup_operators()
    t1 = time.perf_counter()
    info = o.solve_Ahat_p_fhat(c.accuracy, 0)
    t2 = time.perf_counter()
    per_pass = (t2 - t1) / max(info["mg_calls"], 1)
    value = 1e3 * ((t1 - t0) + per_pass * passes_per_step)
    return {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle (C, FP64, lexicographic Gauss-Seidel) on this workload: set-up {t1 - t0:.2f} s timed in "
                      f"full, then the velocity solve of the cold solve's head ({info['mg_calls']} multigrid passes, "
                      f"{t2 - t1:.1f} s): {1e3 * per_pass:.1f} ms per pass x {passes_per_step:.1f} passes per time "
                      f"step (the FP64 GPU path's mean over the timed steps, the same algorithm in 8 colours)"}


def reference_arm(args):
    """The oracle port (the reference's algorithm, lexicographic smoother, one
    host core) on the same workload and stopping rule.  A cold solve of the
    seeded state, then `--ref-full-steps` complete time steps (PG_timestep and
    the Stokes solve from the previous step), each timed in full: `value` is
    the mean wall time of those Stokes solves.  The --steps (after --warmup)
    bench steps are bounded samples of the same state: one multigrid pass
    each, timed, giving the per-pass time; set-up + passes x per-pass time of
    the complete steps is reported beside the measured value as the error of
    the sampled estimate."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    if args.workload == "sphere":
        print(json.dumps({"impl": "reference", "unavailable": "the spherical segment has no CPU port of the path "
                                                               "(the oracle is Cartesian)"}))
        return 0
    from oracle import oracle as O
    O.build()
    case = cfg2_workload() if args.workload == "cfg2" else workload(args.size)
    T0 = seeded_T0(case)
    c = oracle_case(case)
    o = O.Oracle(c, gs_colored=False)
    o.set_T(T0)
    o.thermal_buoyancy()
    t0 = time.perf_counter()
    cold = o.stokes()
    cold_s = time.perf_counter() - t0
    full, full_passes, full_uzawa, pg = [], [], [], []
    for _ in range(max(args.ref_full_steps, 1)):
        t0 = time.perf_counter()
        o.pg_timestep()
        t1 = time.perf_counter()
        info = o.stokes()
        t2 = time.perf_counter()
        full.append(1e3 * (t2 - t1))
        pg.append(1e3 * (t1 - t0))
        full_passes.append(info["mg_calls"])
        full_uzawa.append(info["uzawa"])
    v = float(np.mean(full))
    # set-up of the current state (forces, viscosity, stiffness), then the
    # bench steps: one multigrid pass each on the state's momentum residual
    t0 = time.perf_counter()
    o.setup_operators()
    setup_ms = 1e3 * (time.perf_counter() - t0)
    F = o.F()[: o.fine["neq"]].copy()
    samples = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        o.multi_grid(F)
        dt = 1e3 * (time.perf_counter() - t0)
        if i >= args.warmup:
            samples.append(dt)
    per_pass = float(np.mean(samples))
    est = setup_ms + per_pass * float(np.mean(full_passes))
    sample = (f"oracle port (C, FP64, lexicographic Gauss-Seidel: the reference's algorithm), one core: a cold solve "
              f"({cold_s:.1f} s, {cold['uzawa']} Uzawa iterations, untimed), then {len(full)} complete time steps "
              f"(PG_timestep + Stokes solve to the residual rule) timed in full: value = mean Stokes wall time; "
              f"the {args.steps} bench steps (after {args.warmup}) are one multigrid pass each")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(samples)), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_name(case), "step": STEP_DESC,
                       "bench_step": "one multigrid pass of the oracle on the state after the complete steps"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
            "complete_steps": {"stokes_ms": full, "pg_timestep_ms": pg, "uzawa_iterations": full_uzawa,
                               "mg_passes": full_passes, "cold_solve_s": cold_s, "cold_uzawa": cold["uzawa"],
                               "cold_mg_passes": cold["mg_calls"]},
            "sampled_estimate": {"setup_ms": setup_ms, "ms_per_pass": per_pass, "value": est,
                                 "rel_error_vs_complete": (est - v) / v},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


STEP_DESC = ("one time step of the reference's loop on resident state: PG_timestep, then general_stokes_solver "
             "(forces, viscosity, projection, operator assembly, Uzawa/multigrid solve from the previous step to the "
             "residual rule, V); value = the Stokes part")


def workload_name(case):
    rule = (f"residual rule |F-KU-GP|/|F| and |BU|/(|U| sqrt(npno/neq)) <= {case.accuracy:g}, "
            f"Uzawa cap {case.piterations}") if case.stop_rule == 1 else \
        f"reference rule dv/v, dp/p < {case.accuracy:g}, piterations {case.piterations}"
    if case.sphere is not None:
        return ("regional spherical shell segment, colatitude 45-135 deg, longitude 0-90 deg, r 0.55-1.0, "
                f"{case.nox - 1}x{case.noy - 1}x{case.noz - 1} Q1 elements, {case.levels} multigrid levels, "
                "eta=exp(-ln(1e5) T) x30 below r=0.9, Ra=1e7, conductive T0 + U(-0.01,0.01) seed 0, " + rule)
    if case.dimen[0] == 2.0:
        return (f"2x2x1 box, {case.nox - 1}x{case.noy - 1}x{case.noz - 1} Q1 elements, {case.levels} multigrid levels, "
                "eta=exp(-ln(1e4) T) x30 below z=0.8, Ra=1e6, Q0=1, free slip, T0=1-z+U(-0.01,0.01) seed 0, " + rule)
    return (f"{case.nox - 1}^3 Q1 elements, {case.levels} multigrid levels, eta=exp(-ln(1e3) T), Ra=1e5, free slip, "
            f"T0=1-z+U(-0.01,0.01) seed 0, " + rule)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=["cfg2", "cube", "sphere"],
                    help="cfg2: the 128x128x64 box with a 10^4 contrast (default); cube: the --size^3 unit box; "
                         "sphere: the 192x192x96 regional spherical segment")
    ap.add_argument("--size", type=int, default=64, choices=[16, 32, 64, 128])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--modes", default="all", choices=["all", "mixed"],
                    help="'mixed' skips the FP64 plain comparison (profiling runs)")
    ap.add_argument("--no-learned", action="store_true",
                    help="headline without the learned warm start (profiling runs)")
    ap.add_argument("--learn-seeds", type=int, default=10)
    ap.add_argument("--learn-steps", type=int, default=40, help="time steps recorded after each seed's cold solve")
    ap.add_argument("--learn-mode", default="increment", choices=["increment", "absolute"],
                    help="increment: the network predicts the change of U, P over a time step (default); "
                         "absolute: U, P themselves")
    ap.add_argument("--learn-adam", type=int, default=4000,
                    help="Adam steps of the online training (half at lr 1e-3, a quarter each at 3e-4 and 1e-4)")
    ap.add_argument("--learn-check", type=int, default=8,
                    help="compare the network's start with the previous step's on every k-th solve (and whenever "
                         "its initial residual grows past 4x the last winning one); 1: every solve")
    ap.add_argument("--cold-reps", type=int, default=2, help="cold solves per mode (0: skip)")
    ap.add_argument("--drift-steps", type=int, default=200, help="time steps of the drift run (0: skip)")
    ap.add_argument("--drift-control", action="store_true",
                    help="drift run: also the mixed path solving every step from U = P = 0")
    ap.add_argument("--drift-workload", default="cube", choices=["cube", "cfg2"],
                    help="drift run: the 64^3 box (200 steps by default) or the 128x128x64 box")
    ap.add_argument("--ref-full-steps", type=int, default=2,
                    help="reference arm: complete time steps timed in full after the cold solve")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import citcomcu_gb300 as cg
    cg.build()
    if args.workload == "sphere":
        case = sphere_workload()
        T0_of = lambda sd: seeded_T0_sphere(case, sd)  # noqa: E731
    else:
        case = cfg2_workload() if args.workload == "cfg2" else workload(args.size)
        T0_of = lambda sd: seeded_T0(case, sd)  # noqa: E731
    T0 = T0_of(0)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    learned = ls = ln = train_info = None
    if not args.no_learned:
        ls, ln, train_info = train_warm_start(cg, case, T0_of, args.learn_seeds, args.learn_steps, args.learn_adam,
                                              1 if args.learn_mode == "increment" else 0)
    barrier()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        if ls is not None:
            ln.set_check_interval(args.learn_check)
            learned = run_loop(cg, case, T0, cg.MIXED, args.steps, args.warmup, solver=ls, net=ln, tag="learned")
        mixed = run_loop(cg, case, T0, cg.MIXED, args.steps, args.warmup, tag="mixed")
        fp64 = run_loop(cg, case, T0, cg.FP64, args.steps, args.warmup, tag="fp64") if args.modes == "all" else None
        t1 = time.perf_counter()
    barrier()

    head = learned or mixed
    recs = head["recs"]
    stokes_ms = float(np.mean([r["stokes_ms"] for r in recs]))
    step_ms = float(np.mean([r["stokes_ms"] + r["energy_ms"] for r in recs]))
    stokes_ms, step_ms = max_over_ranks([stokes_ms, step_ms], world)
    value = whole_job_value(stokes_ms, world)

    # dominant kernel: the finest-level FP32 Gauss-Seidel colour launches, timed
    # live by CUDA events inside the multigrid pass (on the library's stream)
    sweeps = sum(r["smoother_sweeps"] for r in recs)
    sm_ms = sum(r["smoother_ms"] for r in recs)
    per_launch_s = sm_ms * 1e-3 / max(8 * sweeps, 1)
    nno, nel = case.nno, (case.nox - 1) * (case.noy - 1) * (case.noz - 1)
    alg_bytes = gs_sweep_bytes(nno, nel, 4) / 8.0
    stored_bytes = bytes_per_sweep(nno, 4) / 8.0
    peak, peak_kind = peaks()
    achieved = alg_bytes / per_launch_s / 1e9 if per_launch_s > 0 else None
    achieved_stored = stored_bytes / per_launch_s / 1e9 if per_launch_s > 0 else None

    if rank != 0:
        return 0

    ref = fp64 if fp64 is not None else None
    mode = ("FP32 multigrid + FP64 refinement + learned warm start" if learned
            else "FP32 multigrid + FP64 refinement")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": workload_name(case), "mode": mode + " (headline)", "step": STEP_DESC,
                   "parallelism": f"replicas{world}",
                   "l2": f"inputs larger than L2 (finest FP32 stencil {case.nno * 972 / 1e6:.0f} MB, FP64 "
                         f"{case.nno * 1944 / 1e6:.0f} MB)",
                   "timing": "CUDA events around each Stokes solve inside the library, mean over timed steps"},
        "mixed": loop_summary(mixed, ref),
        "roofline": {"bound": "hbm", "kernel": "k_tile<float, 0> (finest-level Gauss-Seidel colour)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": TRAFFIC_PER_LAUNCH * nno / TRAFFIC_PER_LAUNCH_NODES if nno >= 274625 else None,
                     "peak_kind": peak_kind, "bytes_per_launch": alg_bytes,
                     "bytes_kind": "algorithmic (per colour: F, d, 1/diag K, Gauss-point viscosity, flags)",
                     "launch_us": per_launch_s * 1e6,
                     "stored_stencil": {"bytes_per_launch": stored_bytes, "achieved": achieved_stored,
                                        "frac": (achieved_stored / peak) if achieved_stored else None}},
        "clocks": clk.summary(),
        "gpu_launches": int(head["launches"]),
        "wall_s_loops": t1 - t0,
    }
    if fp64 is not None:
        line["fp64_plain"] = loop_summary(fp64)
        line["speedup_vs_fp64"] = line["fp64_plain"]["stokes_ms_per_step"] / stokes_ms
    if learned:
        d = loop_summary(learned, ref)
        d.update({"check_interval": args.learn_check,
                  "compared": [r["warm_compared"] for r in learned["recs"]],
                  "warm_start_used": [r["warm_start"] for r in learned["recs"]],
                  "start_residual_previous_step": [r["base_residual"] for r in learned["recs"]],
                  "start_residual_network": [r["warm_residual"] for r in learned["recs"]],
                  "speedup_vs_mixed": line["mixed"]["stokes_ms_per_step"] / d["stokes_ms_per_step"],
                  "training": train_info})
        line["learned"] = d
    if ls is not None and args.learn_check != 1:
        # the same loop comparing the two starts on every solve (the fallback
        # decided afresh each step, at the price of a second head per step)
        ln.set_check_interval(1)
        strict = run_loop(cg, case, T0, cg.MIXED, args.steps, args.warmup, solver=ls, net=ln, tag="learned_every")
        ln.set_check_interval(args.learn_check)
        d = loop_summary(strict, ref)
        d["speedup_vs_mixed"] = line["mixed"]["stokes_ms_per_step"] / d["stokes_ms_per_step"]
        d["warm_start_used"] = [r["warm_start"] for r in strict["recs"]]
        line["learned_compare_every_step"] = d
    if args.cold_reps > 0:
        cs = {"mixed": cold_solves(cg, case, T0, cg.MIXED, args.cold_reps)}
        if ls is not None and args.learn_mode == "absolute":
            cs["learned"] = cold_solves(cg, case, T0, cg.MIXED, args.cold_reps, solver=ls, net=ln)
        if args.modes == "all":
            cs["fp64_plain"] = cold_solves(cg, case, T0, cg.FP64, args.cold_reps)
            cs["reference_rule"] = {
                "mixed": cold_solves(cg, case, T0, cg.MIXED, 1, stop_rule=0, piterations=375),
                "fp64_plain": cold_solves(cg, case, T0, cg.FP64, 1, stop_rule=0, piterations=375)}
        line["cold_solve"] = cs
    if not args.no_e2e:
        es = ls if ls is not None else cg.Solver(cg.Config.like(case, precision=cg.MIXED))
        if ln is not None:
            ln.attach(True)
        e2e_ms, h2d, d2h, detail = e2e_loop(cg, es, T0, args.steps, args.warmup)
        line["e2e"] = {"value": e2e_ms, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "mode": mode, "steps": args.steps, "warmup": args.warmup, **detail}
        line["output_step"] = output_step(es)
        if es is not ls:
            es.close()
    if args.drift_steps > 0 and args.workload != "sphere":
        same = ls is not None and args.drift_workload == args.workload
        line["drift"] = drift_run(cg, args.drift_workload, args.drift_steps, (ls, ln) if same else None,
                                  control=args.drift_control)
    if ln is not None:
        ln.close()
        ls.close()
    if not args.no_cpu and case.sphere is None:  # the oracle has no spherical geometry
        pps = float(np.mean([r["mg_passes"] for r in (fp64 or mixed)["recs"]]))
        line["cpu_baseline"] = cpu_sample(case, T0, pps)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
