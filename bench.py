#!/usr/bin/env python3
"""Benchmark of the sediment-column hot path on GB300.

Default line (the headline): the surrogate step with its plain fallback
against the plain solver on the 2048 x 2048 workload (30 % land, 30 layers,
11 OMEXDIA+P tracers, 3600 s coupling steps, per-column adaptive Euler, FP32
state), timed from simulated day 10 after the network is trained at its
configured size.  ``--solver plain --workload NAME`` times the plain solver
on another workload (e.g. plain_gpu_256x256).  One bench "step" is one
coupling step of every column; the unit is column-steps/s (one active column
advanced by one 3600 s coupling step, all its substeps included).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  ``value`` is device throughput with the state
resident in HBM (CUDA events around each step on the library's stream, L2
flushed between steps); ``e2e`` is the same metric through the drop-in call
(sed_ode_solver_surrogate, or sed_ode_solver for the plain solver) on
pinned FP64 host arrays, copies included; ``roofline`` is the plain column
kernel against the measured HBM copy bandwidth; ``cpu_baseline`` is the
FP64 oracle on the host cores on a column sample.  ``--impl reference``
times the reference algorithm on the host CPU (the FP64 restatement; the
Fortran reference cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "mossco-code_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = ("sediment column-steps/s on 1 GB300: surrogate vs plain, "
          "≤1e-3 rel err vs FP64")
UNIT = "column-steps/s"
WORKLOAD = "plain_gpu_256x256"
NTR, NCOEF, NFORCE, NDISS = 11, 4, 13, 5
L2_BYTES = 129 * 1024 * 1024
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the hot
# kernel, from an ncu --set full capture of the launch at day 10 of the run
# (surrogate_2048x2048: the capture of 183,315 active columns, 3,271 B per
# column-step, scaled to the grid's 2,936,778)
MEASURED_TRAFFIC = {"plain_gpu_256x256": 168.4e6,
                    "surrogate_2048x2048": 3271.0 * 2936778}
# ncu counters of the hot kernel in the headline's window (day 10), from
# an ncu --set full capture of one launch on the grid's first 262,144
# columns (python -m sedgpu.profcase plain --columns 262144 --day 10)
NCU_KERNEL = {"surrogate_2048x2048": {
    "issue_active": 0.809, "fp32_pipe": 0.560, "alu_pipe": 0.365, "lsu_pipe": 0.420,
    "warps_active": 0.372, "warp_instructions_per_attempt": 227,
    "traffic_per_column_step": 3271, "bound": "instruction issue",
    "capture": "ncu --set full, 183,315 active columns at day 10, budgets on"}}
# the same for one Run of the pelagic kernel (the first timed Run)
PEL_TRAFFIC = {"pelagic_1024x1024": 1384.8e6}
FALLBACK_HBM_GBS = 6800.0


def algorithmic_bytes(kact: np.ndarray, budgets: bool, rsize: int = 4) -> int:
    """Bytes one coupling step must move per the kernel's inputs/outputs:
    state read+write (2 r NTR K), coefficient rows (r NCOEF K), forcing
    (r NFORCE), kact (4), surface fluxes (r NDISS), attempts (4) and FP64
    budgets (4 x 8)."""
    K = kact[kact > 0].astype(np.int64)
    per = 2 * rsize * NTR * K + rsize * NCOEF * K + rsize * NFORCE + 4 \
        + rsize * NDISS + 4 + (32 if budgets else 0)
    return int(per.sum())


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for r in rows:
            for i, nm in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_run(cs, warmup: int, steps: int, threads: int):
    """FP64 oracle, per-column cuts, all given host threads: returns
    (column-steps/s of the timed steps, seconds, stats)."""
    import oracle
    om = oracle.OracleModel(cs)
    c = cs.conc.copy()
    fl = cs.fluxes.copy()
    if warmup:
        rc, _, fl = om.run(c, nsteps=warmup, percol=True, nthreads=threads,
                           fluxes=fl)
    t0 = time.perf_counter()
    rc, st, _ = om.run(c, nsteps=steps, percol=True, nthreads=threads, fluxes=fl)
    dt = time.perf_counter() - t0
    return cs.n_active * steps / dt, dt, st


def cpu_sample(ncol_full: int, n: int, seed: int, workload: str = WORKLOAD):
    from sedgpu import synth
    cols = np.linspace(0, ncol_full - 1, min(n, ncol_full)).astype(np.int64)
    return synth.make_workload(workload, seed=seed, cols=np.unique(cols))


def cpu_window(workload: str, seed: int, warmup: int, steps: int, threads: int,
               max_columns: int, target_s: float = 15.0):
    """The oracle over the same coupling steps as the GPU run, on an evenly
    spaced column sample sized (from a 2-columns-per-thread pilot over the
    same steps) to about target_s seconds of timed CPU work."""
    from sedgpu import synth
    full = synth.WORKLOADS[workload]
    ncol = full["inum"] * full["jnum"]
    n0 = min(max(2 * threads, 16), max_columns)
    cs = cpu_sample(ncol, n0, seed, workload)
    val, secs, st = cpu_run(cs, warmup, steps, threads)
    n = int(min(max_columns, max(n0, n0 * target_s / max(secs, 1e-3))))
    if n > 1.5 * n0:
        cs = cpu_sample(ncol, n, seed, workload)
        val, secs, st = cpu_run(cs, warmup, steps, threads)
    sample = (f"{cs.n_active} active of {ncol} columns (evenly spaced), coupling steps "
              f"{warmup + 1}..{warmup + steps}, {secs:.1f} s")
    return {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": sample, "seconds": secs}


def host_cpu() -> dict:
    """The host's CPU model (as /proc/cpuinfo names it) and core count."""
    import platform
    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu part") and ":" in line:
                    model = line.split(":", 1)[1].strip()
                    if key == "model name":
                        break
    except OSError:
        pass
    return {"machine": platform.machine(), "model": model, "nproc": os.cpu_count() or 1}


def cpu_context(workload: str, seed: int, warmup: int, steps: int, max_columns: int) -> dict:
    """The host beside the all-core baseline, and the same window on one
    core (about 5 s of work)."""
    one = cpu_window(workload, seed, warmup, steps, 1, max_columns, target_s=5.0)
    return {"host": host_cpu(),
            "one_core": {"value": one["value"], "unit": one["unit"], "sample": one["sample"]}}


def days(step0: int, step1: int, dt: float) -> str:
    return f"{step0 * dt / 86400.0:.3f}..{step1 * dt / 86400.0:.3f}"


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    from sedgpu import synth
    full = synth.make_workload(args.workload, cols=np.arange(1))
    steps = args.steps or full.nsteps
    threads = os.cpu_count() or 1
    cpu = cpu_window(args.workload, args.seed, args.warmup, steps, threads, args.cpu_columns)
    val = cpu["value"]
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup,
        "ms_per_step": cpu["seconds"] * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": args.workload, "tracers": NTR, "dt_s": full.dt,
                   "method": "adaptive_euler", "cut": "per_column",
                   "simulated_days_timed": days(args.warmup, args.warmup + steps, full.dt)},
        "cpu_baseline": dict({k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
                             **cpu_context(args.workload, args.seed, args.warmup, steps,
                                           args.cpu_columns)),
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("reference algorithm as the FP64 C restatement on the host "
                 "cores; the Fortran reference and its FABM reaction model "
                 "cannot be built on this machine"),
    }
    print(json.dumps(line), flush=True)


HEADLINE = "surrogate_2048x2048"
TRAIN_WORKLOAD = "surrogate_200k"
# tracers of the phosphorus and nitrogen inventories (mossco_sed.h order)
P_TRACERS, N_TRACERS = (4, 5, 10), (2, 3, 7, 8)


def grid_sample(inum: int, jnum: int, n: int = 64) -> np.ndarray:
    """Column ids of an n x n regular subsample of an inum x jnum grid
    (every inum/n-th column in each direction, offset to the cell centre)."""
    si, sj = inum // n, jnum // n
    i = si // 2 + si * np.arange(n)
    j = sj // 2 + sj * np.arange(n)
    return (i[None, :] + inum * j[:, None]).ravel().astype(np.int64)


def inventories(cs, conc) -> tuple:
    """P and N inventories per column, sum over active layers of phi dz C
    (mmol/m2), of the tracers that carry each element."""
    act = np.arange(cs.kmax)[:, None] < cs.kact[None, :]
    w = np.where(act, cs.phi * cs.dz, 0.0)
    P = sum((w * conc[n]).sum(axis=0) for n in P_TRACERS)
    N = sum((w * conc[n]).sum(axis=0) for n in N_TRACERS)
    return P, N


def rel_err_per_tracer(x, r, act) -> list:
    """max |x - r| / (|r| + 1e-4 max|r|) over the active cells, per tracer."""
    out = []
    for n in range(NTR):
        rn, xn = r[n][act], x[n][act]
        floor = 1e-4 * max(np.abs(rn).max(), 1e-300)
        out.append(float(np.max(np.abs(xn - rn) / (np.abs(rn) + floor))))
    return out


def cpu_window_from(cs, conc0, steps: int, threads: int, max_columns: int,
                    target_s: float = 12.0, seed: int = 0):
    """The FP64 oracle over ``steps`` coupling steps from the state conc0 of
    ``cs`` (e.g. a developed state), on a random column sample sized from a
    pilot to about target_s seconds of timed CPU work."""
    import oracle
    act = np.nonzero(cs.kact > 0)[0]
    rng = np.random.default_rng(seed)
    order = rng.permutation(act)

    def timed(n):
        cols = np.sort(order[:n])
        sub = cs.subset(cols)
        c = np.ascontiguousarray(conc0[:, :, cols], dtype=np.float64)
        om = oracle.OracleModel(sub)
        t0 = time.perf_counter()
        rc, st, _ = om.run(c, nsteps=steps, percol=True, nthreads=threads)
        return sub, time.perf_counter() - t0, st
    n0 = min(max(8 * threads, 64), len(act), max_columns)
    sub, secs, st = timed(n0)
    n = int(min(max_columns, len(act), max(n0, n0 * target_s / max(secs, 1e-3))))
    if n > 1.5 * n0:
        sub, secs, st = timed(n)
    return {"value": sub.n_active * steps / secs, "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": (f"{sub.n_active} of {len(act)} active columns (random), {steps} coupling "
                       f"steps from the timed window's start state, {secs:.1f} s"),
            "seconds": secs,
            "attempts_per_column_step": st["attempts"] / max(sub.n_active * steps, 1)}


def run_headline(args) -> None:
    """The headline: surrogate + fallback against the plain FP32 solver on
    the 2048 x 2048 workload (30 % land, 30 layers), timed from a developed
    state (args.start_day) over args.steps coupling steps.  The network is
    trained first, untimed, on rows the plain solver generates on the
    200 000-column training workload, by the library's own kernels."""
    import torch
    from sedgpu import capi, synth
    from sedgpu import surrogate as S

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    t_job = time.perf_counter()

    # 1. the network (untimed)
    ntrain = args.sur_train_columns
    train_cs = synth.make_workload(TRAIN_WORKLOAD, cols=np.arange(ntrain))
    test_cs = synth.make_workload(TRAIN_WORKLOAD,
                                  cols=np.arange(ntrain, ntrain + args.sur_test_columns))
    sur, training = S.train_surrogate(
        train_cs, test_cs, nsteps=train_cs.nsteps, every=args.sur_every, warm=24,
        train_steps=args.sur_train_steps, batch=8192,
        log_every=max(1, args.sur_train_steps // 10), test_nsteps=train_cs.nsteps)
    del train_cs, test_cs
    torch.cuda.empty_cache()

    # 2. the workload at its developed state (untimed): plain steps from the
    #    configured initial state, then the plain kernel's launch tuning
    cs = synth.make_workload(args.workload, seed=args.seed + 7919 * rank)
    p = capi.params_from(cs, capi.SED_FP32, budgets=False, device=local)
    s = capi.Solver(cs, params=p)
    s.set_forcing()
    s.set_state(cs.conc)
    spin = int(round(args.start_day * 86400.0 / cs.dt))
    t0 = time.perf_counter()
    for done in range(0, spin, 24):
        s.step(min(24, spin - done))
    spin_s = time.perf_counter() - t0
    tuning = None if args.no_autotune else s.autotune(flags=0)
    S0 = s.get_state()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    steps = args.steps or 24
    day0 = spin * cs.dt / 86400.0
    window_days = f"{day0:.3f}..{day0 + steps * cs.dt / 86400.0:.3f}"

    def window(tol):
        """W untimed steps from S0, then K timed steps from S0 again."""
        def one():
            return s.step(1) if tol is None else S.step_surrogate(s, sur, 1, tol=tol,
                                                                  res_atol=args.sur_res_atol)
        s.set_state(S0)
        for _ in range(args.warmup):
            one()
        s.set_state(S0)
        clocks = ClockSampler(local)
        clocks.start()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        tot = {"device_ms": 0.0, "gpu_launches": 0, "column_steps": 0, "attempts": 0,
               "surrogate_columns": 0}
        for _ in range(steps):
            flush.zero_()        # L2 flush between timed steps
            torch.cuda.synchronize()
            st = one()
            for k in tot:
                tot[k] += st[k]
        torch.cuda.synchronize()
        if dist:
            t = torch.tensor([tot["device_ms"]], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            tot["device_ms"] = float(t.item())
            dist.barrier()
        tot["clocks"] = clocks.stop()
        tot["value"] = world * cs.n_active * steps / (tot["device_ms"] / 1e3)
        tot["ms_per_step"] = tot["device_ms"] / steps
        tot["surrogate_fraction"] = tot["surrogate_columns"] / max(tot["column_steps"], 1)
        tot["attempts_per_column_step"] = tot["attempts"] / max(tot["column_steps"], 1)
        # substeps per column of the window's last step (power-of-two bins)
        tot["attempt_histogram"] = [int(v) for v in s.attempt_histogram()]
        return tot

    plain = window(None)
    head = window(args.sur_tol)

    # 3. accuracy against the FP64 path on the 64 x 64 subsample, one
    #    coupling step at a time from the surrogate run's own states
    #    (teacher forced: the reference algorithm amplifies any rounding
    #    difference ~100x per step, so free-running trajectories of FP32 and
    #    FP64 part within a day), for the headline tolerance and the sweep
    cols = grid_sample(cs.inum, cs.jnum, 64)
    cols = cols[cs.kact[cols] > 0]
    sub = cs.subset(cols)
    act = np.arange(sub.kmax)[:, None] < sub.kact[None, :]

    def accuracy(tol, nacc):
        h32 = capi.Solver(sub, params=capi.params_from(sub, capi.SED_FP32, device=local))
        h64 = capi.Solver(sub, params=capi.params_from(sub, capi.SED_FP64, device=local))
        for h in (h32, h64):
            h.set_forcing()
        cur = np.ascontiguousarray(S0[:, :, cols])
        errs = np.zeros(NTR)
        plain_errs = np.zeros(NTR)
        dP = dN = 0.0
        taken = total = 0
        live = sub.kact > 0
        for _ in range(nacc):
            h64.set_state(cur)
            h64.step(1)
            ref = h64.get_state()
            h32.set_state(cur)
            h32.step(1)
            plain_errs = np.maximum(plain_errs, rel_err_per_tracer(h32.get_state(), ref, act))
            h32.set_state(cur)
            st = h32.step(1) if tol is None else S.step_surrogate(h32, sur, 1, tol=tol,
                                                                  res_atol=args.sur_res_atol)
            out = h32.get_state()
            errs = np.maximum(errs, rel_err_per_tracer(out, ref, act))
            P1, N1 = inventories(sub, out)
            P0, N0 = inventories(sub, ref)
            dP = max(dP, float(np.max(np.abs(P1 - P0)[live] / np.abs(P0[live]))))
            dN = max(dN, float(np.max(np.abs(N1 - N0)[live] / np.abs(N0[live]))))
            taken += st["surrogate_columns"]
            total += st["column_steps"]
            cur = out
        h32.close()
        h64.close()
        return {"max_rel_err_per_tracer": [float(e) for e in errs],
                "max_rel_err": float(errs.max()),
                "plain_fp32_max_rel_err": float(plain_errs.max()),
                "budget_drift_vs_fp64": {"P": dP, "N": dN},
                "surrogate_fraction": taken / max(total, 1), "steps": nacc}

    acc = accuracy(args.sur_tol, min(steps, args.acc_steps))
    sweep = []
    for tol in args.sur_sweep:
        w = window(tol)
        a = accuracy(tol, min(steps, args.acc_steps))
        sweep.append({"tol": tol, "value": w["value"],
                      "speedup_vs_plain": w["value"] / plain["value"],
                      "surrogate_fraction": w["surrogate_fraction"],
                      "max_rel_err_vs_fp64": a["max_rel_err"],
                      "budget_drift_vs_fp64": a["budget_drift_vs_fp64"]})

    # 4. end to end through the drop-in call with host buffers: per step the
    #    FP64 state, bottom-water values and fluxes in, the gated surrogate
    #    step, the state and fluxes out (sed_ode_solver_surrogate, copies
    #    pipelined over the column segments)
    e2e = None
    if not args.no_e2e:
        # the caller's arrays in pinned host memory (sed_host_alloc)
        host = capi.host_empty(S0.shape)
        host[:] = S0
        bd = capi.host_empty(cs.bdys.shape)
        bd[:] = cs.bdys
        fl = capi.host_empty(cs.fluxes.shape)
        fl[:] = cs.fluxes
        n_e2e = args.e2e_steps or steps
        for _ in range(args.warmup):
            S.ode_solver_surrogate(s, sur, host, bd, fl, tol=args.sur_tol,
                                   res_atol=args.sur_res_atol)
        host[:] = S0
        fl[:] = cs.fluxes
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(n_e2e):
            S.ode_solver_surrogate(s, sur, host, bd, fl, tol=args.sur_tol,
                                   res_atol=args.sur_res_atol)
        e2e_s = time.perf_counter() - t1
        e2e = {"value": world * cs.n_active * n_e2e / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(host.nbytes + bd.nbytes + fl.nbytes),
               "d2h_bytes_per_step": int(host.nbytes + fl.nbytes),
               "steps": n_e2e,
               "call": "sed_ode_solver_surrogate (FP64 host state in and out, copies "
                       "pipelined over the column segments)",
               "host_arrays": "pinned (sed_host_alloc)"}
        del host, bd, fl
    t_now = s.tuning().as_dict()
    s.close()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # 5. the plain kernel against its roofline, in the same window
    bytes_step = algorithmic_bytes(cs.kact, budgets=False)
    peak, peak_kind = measured_peaks()
    achieved = bytes_step / (plain["ms_per_step"] / 1e3) / 1e9
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        cpu = cpu_window_from(cs, S0, steps, threads, args.cpu_columns)
        one = cpu_window_from(cs, S0, steps, 1, args.cpu_columns, target_s=5.0)
        cpu.pop("seconds")
        cpu["host"] = host_cpu()
        cpu["one_core"] = {"value": one["value"], "unit": one["unit"], "sample": one["sample"]}
    clk = head["clocks"] or plain["clocks"]
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "columns": cs.n_active,
                   "grid": f"{cs.inum}x{cs.jnum}", "layers": cs.kmax,
                   "land_fraction": float(np.mean(cs.kact == 0)), "tracers": NTR,
                   "dt_s": cs.dt, "method": "adaptive_euler", "cut": "per_column",
                   "state": "fp32", "solver": "surrogate+fallback",
                   "residual_tol": args.sur_tol, "residual_atol": args.sur_res_atol,
                   "simulated_days_timed": window_days,
                   "start": f"day {day0:g}, reached by {spin} untimed plain steps from the "
                            f"configured initial state",
                   "l2": "flushed between timed steps (state 5.5 GB, larger than L2)",
                   "network": f"{NTR * cs.kmax + S.NFORCE}->{S.HIDDEN}x{S.NHIDDEN}->"
                              f"{NTR * cs.kmax} (BF16 products, FP32 accumulation)",
                   "tuning": {k: t_now[k] for k in ("tile_columns", "threads")}},
        "plain": {"value": plain["value"], "ms_per_step": plain["ms_per_step"],
                  "attempts_per_column_step": plain["attempts_per_column_step"],
                  "attempt_histogram_last_step": plain["attempt_histogram"],
                  "gpu_launches": plain["gpu_launches"]},
        "speedup_vs_plain": head["value"] / plain["value"],
        "surrogate_fraction": head["surrogate_fraction"],
        "attempts_per_column_step": head["attempts_per_column_step"],
        "accuracy": dict(acc, columns=int(len(cols)),
                         reference="FP64 device path (bit-identical to the FP64 CPU "
                                   "restatement), one coupling step from the same state",
                         parity="stepper, transport, epilogue and boundary assembly pinned "
                                "to the reference's source and solver test; the OMEXDIA+P "
                                "rates are a restatement of the published model (FABM is not "
                                "in the reference tree): parity of the rates unpinned",
                         floor="1e-4 x tracer max", sample="64 x 64 regular subsample"),
        "sweep": sweep,
        "training": training,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": MEASURED_TRAFFIC.get(args.workload),
                     "peak_kind": peak_kind, "bytes_per_launch": bytes_step,
                     "kernel": "k_column_warp<float,1,...,ADAPT> (plain arm, same window)",
                     "ncu": NCU_KERNEL.get(args.workload)},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": head["gpu_launches"],
        "clocks": clk, "spin_s": round(spin_s, 1),
        "job_s": round(time.perf_counter() - t_job, 1),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_reference_headline(args) -> None:
    """The reference algorithm (the FP64 restatement, per-column cuts) on the
    host cores over the headline's window: a random column sample of the
    workload is integrated from the configured initial state to args.start_day
    (untimed), then args.steps coupling steps are timed."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    from sedgpu import synth
    spec = synth.WORKLOADS[args.workload]
    act = synth.active_columns(args.workload, seed=args.seed)
    steps = args.steps or 24
    dt = 3600.0
    spin = int(round(args.start_day * 86400.0 / dt))
    threads = os.cpu_count() or 1
    order = np.random.default_rng(0).permutation(act)
    n = min(args.ref_columns, len(act))
    cols = np.sort(order[:n])
    sub = synth.make_workload(args.workload, seed=args.seed, cols=cols)
    om = oracle.OracleModel(sub)
    c = sub.conc.copy()
    t0 = time.perf_counter()
    rc, _, _ = om.run(c, nsteps=spin, percol=True, nthreads=threads)
    spin_s = time.perf_counter() - t0
    for _ in range(args.warmup):
        w = c.copy()
        om.run(w, nsteps=1, percol=True, nthreads=threads)
    t0 = time.perf_counter()
    rc, st, _ = om.run(c, nsteps=steps, percol=True, nthreads=threads)
    secs = time.perf_counter() - t0
    val = sub.n_active * steps / secs
    day0 = spin * dt / 86400.0
    sample = (f"{sub.n_active} of {len(act)} active columns (random), coupling steps "
              f"{spin + 1}..{spin + steps} after {spin} untimed steps ({spin_s:.0f} s), "
              f"{secs:.1f} s")
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": args.workload, "columns": int(len(act)),
                   "grid": f"{spec['inum']}x{spec['jnum']}", "layers": spec["kmax"],
                   "tracers": NTR, "dt_s": dt, "method": "adaptive_euler", "cut": "per_column",
                   "solver": "plain (the reference algorithm)",
                   "simulated_days_timed": f"{day0:.3f}..{day0 + steps * dt / 86400.0:.3f}"},
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample, "host": host_cpu(),
                         "attempts_per_column_step":
                             st["attempts"] / max(sub.n_active * steps, 1)},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "status": rc,
        "note": ("reference algorithm as the FP64 C restatement on the host cores; the "
                 "Fortran reference and its FABM reaction model cannot be built on this "
                 "machine; the reference has no surrogate, so its arm is the plain method"),
    }
    print(json.dumps(line), flush=True)


MLP_METRIC = ("surrogate MLP inference on 1 GB300: rows/s of the 343->256x4->330 network "
              "(BF16 products, FP32 accumulation)")


def mlp_flops_per_row(K: int = 30) -> int:
    """Algorithmic multiply-adds x 2 of one row, unpadded widths."""
    dims = [NTR * K + NFORCE] + [256] * 4 + [NTR * K]
    return 2 * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))


def run_mlp(args) -> None:
    """Inference of the surrogate network on the rows of the 2048 x 2048
    workload's active columns (2 936 778, padded to 128), with random
    weights: the fused tcgen05 kernel and the mma.sync GEMMs, each timed with
    CUDA events on the stream it runs on, inputs larger than L2."""
    import ctypes
    import torch
    from sedgpu import capi
    from sedgpu import surrogate as S
    torch.cuda.set_device(0)
    lib = capi.load()
    K = 30
    m = S.pad128(args.mlp_rows)
    sur = S.Surrogate(K, batch=8192, seed=3)
    n = lib.sed_sur_num_params(sur.h)
    rng = np.random.default_rng(4)
    w = rng.normal(0, 1, n).astype(np.float32)
    dims = [sur.nin] + [S.HIDDEN] * S.NHIDDEN + [sur.nout]
    o = 0
    for i in range(len(dims) - 1):
        w[o:o + dims[i] * dims[i + 1]] /= np.sqrt(dims[i])
        o += dims[i] * dims[i + 1] + dims[i + 1]
    sur.set_weights(w)
    X = torch.zeros((m, sur.pin), dtype=torch.bfloat16, device="cuda")
    X[:, :sur.nin] = torch.randn((m, sur.nin), device="cuda").to(torch.bfloat16)
    Y = torch.empty((m, sur.pout), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    lib.sed_sur_set_stream(sur.h, ctypes.c_void_p(stream.cuda_stream))
    flops = mlp_flops_per_row(K) * m
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except Exception:
        peak = 1900.0
    out = {}
    clk = None
    for name, tc in (("tcgen05_fused", 1), ("mma_sync_gemms", 0)):
        got = lib.sed_sur_set_tensor_cores(sur.h, tc)
        if tc and got != 1:
            out[name] = {"unavailable": "network shape or tensor-map encoder"}
            continue

        def call():
            rc = lib.sed_sur_forward_device(sur.h, ctypes.c_void_p(X.data_ptr()),
                                            ctypes.c_void_p(Y.data_ptr()), m)
            if rc != 0:
                raise capi.SedError(rc, lib.sed_sur_last_error(sur.h).decode())
        for _ in range(args.warmup):
            call()
        clocks = ClockSampler(0) if tc else None
        if clocks:
            clocks.start()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps or 10)]
        for e0, e1 in ev:
            e0.record(stream)
            call()
            e1.record(stream)
        torch.cuda.synchronize()
        if clocks:
            clk = clocks.stop()
        ms = [e0.elapsed_time(e1) for e0, e1 in ev]
        med = statistics.median(ms)
        out[name] = {"ms": med, "rows_per_s": m / (med / 1e3),
                     "tflops": flops / (med / 1e3) / 1e12,
                     "frac_of_measured_bf16_peak": flops / (med / 1e3) / 1e12 / peak}
    lib.sed_sur_set_stream(sur.h, None)
    sur.close()
    fast = out["tcgen05_fused"]
    line = {"metric": MLP_METRIC, "value": fast.get("rows_per_s"), "unit": "rows/s",
            "n_gpus": 1, "steps": args.steps or 10, "warmup": args.warmup,
            "ms_per_step": fast.get("ms"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16", "data": "synthetic (random weights and rows)",
            "config": {"workload": "surrogate_mlp_2048x2048", "rows": m,
                       "network": "343->256x4->330 (padded 384/384)",
                       "flops_per_row": mlp_flops_per_row(K),
                       "l2": "inputs larger than L2 (rows 2.2 GB)"},
            "roofline": {"bound": "tensor", "achieved": fast.get("tflops"), "peak": peak,
                         "unit": "TFLOP/s",
                         "frac": fast.get("frac_of_measured_bf16_peak"),
                         "peak_kind": "measured (cuBLAS bf16 burst)"},
            "engines": out, "clocks": clk}
    print(json.dumps(line), flush=True)


def run_spinup(args) -> None:
    """Spin-up of the reference's 1-column model (sed1d, hourly steps for
    --spinup-years) through sed_spinup's column mode, against the oracle's
    1-column run on one host core (the reference runs sed1d on one PET)."""
    import torch
    import oracle
    from sedgpu import capi, synth
    torch.cuda.set_device(0)
    cs = synth.make_workload(args.workload, cols=np.arange(1))
    nsteps = int(round(args.spinup_years * 8760))
    b1 = np.array(cs.bdys[:, 0], dtype=np.float64)
    f1 = np.array(cs.fluxes[:, 0], dtype=np.float64)
    out = {}
    for prec, name in ((capi.SED_FP32, "fp32"), (capi.SED_FP64, "fp64")):
        s = capi.Solver(cs, precision=prec)
        s.set_forcing()
        s.set_state(cs.conc)
        s.spinup(24, capi.SED_SPINUP_COLUMN, bdys1=b1, fluxes1=f1)   # warm
        s.set_state(cs.conc)
        t0 = time.perf_counter()
        st = s.spinup(nsteps, capi.SED_SPINUP_COLUMN, bdys1=b1, fluxes1=f1)
        out[name] = {"seconds": time.perf_counter() - t0,
                     "attempts_per_step": st["attempts"] / max(nsteps, 1),
                     "gpu_launches": st["gpu_launches"]}
        s.close()
    # the oracle on one core over a bounded sample of the same run
    cpu_steps = min(nsteps, args.spinup_cpu_steps)
    c = cs.conc.copy()
    t0 = time.perf_counter()
    rc, sref, _ = oracle.OracleModel(cs).run(c, nsteps=cpu_steps, percol=True, nthreads=1)
    cpu_s = time.perf_counter() - t0
    line = {"metric": "spin-up of the 1-column model", "unit": "simulated years/s",
            "workload": f"{args.workload}, one column, {cs.kmax} layers, dt 3600 s, "
                        f"{args.spinup_years} years ({nsteps} steps)",
            "gpu_fp32": {**out["fp32"], "years_per_s": args.spinup_years / out["fp32"]["seconds"]},
            "gpu_fp64": {**out["fp64"], "years_per_s": args.spinup_years / out["fp64"]["seconds"]},
            "cpu_oracle_1core": {"seconds": cpu_s, "steps": cpu_steps,
                                 "years_per_s": cpu_steps / 8760 / cpu_s,
                                 "attempts_per_step": sref["attempts"] / max(cpu_steps, 1)}}
    print(json.dumps(line), flush=True)


def ensemble_sets(cs, seed: int) -> np.ndarray:
    """[SED_NBGC][ncol]: the workload's parameter set with the labile and
    semilabile decay rates, the oxic half saturation and the nitrification
    rate of each column scaled by exp(U[-0.7, 0.7]) (a factor of 2 either
    way), counter-based per column."""
    from sedgpu import synth
    from sedgpu.model import BGC_NAMES
    tab = cs.bgc_columns().copy()
    idx = np.arange(cs.ncol, dtype=np.int64)
    for f, name in enumerate(("rLabile", "rSemilabile", "ksO2oxic", "rnit")):
        u = synth.uniform(seed, 200 + f, idx)
        tab[BGC_NAMES.index(name)] *= np.exp(-0.7 + 1.4 * u)
    return tab


def run_ensemble_spinup(args) -> None:
    """An ensemble spin-up: --ensemble parameter sets as the columns of one
    grid (sed_set_column_bgc), all spun up together for --spinup-years of
    hourly steps by sed_spinup's all-columns mode, against the oracle with
    every host thread on a bounded sample of the same sets and steps."""
    import torch
    import oracle
    from sedgpu import capi, synth
    torch.cuda.set_device(0)
    n = args.ensemble
    cs = synth.make_workload(args.workload, cols=np.zeros(n, dtype=np.int64))
    tab = ensemble_sets(cs, args.seed)
    cs.bgc_col = tab
    nsteps = int(round(args.spinup_years * 8760))
    s = capi.Solver(cs)
    s.set_forcing()
    s.set_state(cs.conc)
    s.spinup(24, capi.SED_SPINUP_ALL)   # warm
    s.set_state(cs.conc)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = s.spinup(nsteps, capi.SED_SPINUP_ALL)
    gpu_s = time.perf_counter() - t0
    s.close()
    threads = os.cpu_count() or 1
    m = min(n, max(4 * threads, 64))
    sub = cs.subset(np.arange(m))
    cpu_steps = min(nsteps, args.spinup_cpu_steps)
    c = sub.conc.copy()
    t0 = time.perf_counter()
    rc, _, _ = oracle.OracleModel(sub).run(c, nsteps=cpu_steps, percol=True, nthreads=threads)
    cpu_s = time.perf_counter() - t0
    line = {"metric": "ensemble spin-up", "unit": "parameter-set years/s",
            "workload": f"{n} parameter sets on column 0 of {args.workload} "
                        f"({cs.kmax} layers), {args.spinup_years} years of 3600 s steps",
            "gpu_fp32": {"seconds": gpu_s, "value": n * args.spinup_years / gpu_s,
                         "attempts_per_column_step": st["attempts"] / max(st["column_steps"], 1),
                         "gpu_launches": st["gpu_launches"]},
            "cpu_oracle": {"value": m * cpu_steps / 8760 / cpu_s, "cores": threads,
                           "sample": f"{m} sets x {cpu_steps} steps, {cpu_s:.1f} s",
                           "status": rc}}
    print(json.dumps(line), flush=True)


def coupled_e2e(s, cs, warmup, nsteps, world):
    """Coupling steps with the state resident on the device: each step takes
    the pelagic fields at the soil surface in (sed_set_boundary), steps, and
    returns the surface fluxes (sed_get_fluxes), all on pinned host arrays.
    The particulate fields reproduce the workload's deposition fluxes
    (fluxes = -surface * velocity at a settling velocity of 1e-5 m/s)."""
    import ctypes
    from sedgpu import capi
    T = np.array(cs.bdys[0], dtype=np.float64, copy=True)
    surface = np.zeros((NTR, cs.ncol))
    velocity = np.zeros((NTR, cs.ncol))
    velocity[:6] = -1e-5
    surface[:6] = cs.fluxes[:6] / 1e-5
    surface[6:] = cs.bdys[7:]
    fl = np.zeros((NTR, cs.ncol))
    for a in (T, surface, velocity, fl):
        capi.host_register(a)
    s.set_state(cs.conc)
    dp = ctypes.POINTER(ctypes.c_double)
    args = [a.ctypes.data_as(dp) for a in (T, surface, velocity)]
    st = capi.SedStats()
    lib = s.lib
    parts = {"sed_set_boundary": [], "sed_step": [], "sed_get_fluxes": []}
    def one():
        t = time.perf_counter()
        s._check(lib.sed_set_boundary(s.h, *args, None), "sed_set_boundary")
        t1 = time.perf_counter()
        s._check(lib.sed_step(s.h, float(cs.dt), 2, 1, ctypes.byref(st)), "sed_step")
        t2 = time.perf_counter()
        s._check(lib.sed_get_fluxes(s.h, fl.ctypes.data_as(dp)), "sed_get_fluxes")
        t3 = time.perf_counter()
        for k, v in zip(parts, (t1 - t, t2 - t1, t3 - t2)):
            parts[k].append(v)
    for _ in range(warmup):
        one()
    for v in parts.values():
        v.clear()
    t0 = time.perf_counter()
    for _ in range(nsteps):
        one()
    sec = time.perf_counter() - t0
    for a in (T, surface, velocity, fl):
        capi.host_unregister(a)
    return {"value": world * cs.n_active * nsteps / sec, "unit": UNIT,
            "h2d_bytes_per_step": int(T.nbytes + surface.nbytes + velocity[:6].nbytes),
            "d2h_bytes_per_step": int(fl.nbytes), "steps": nsteps,
            "calls": "sed_set_boundary + sed_step + sed_get_fluxes (state on the device)",
            "ms_per_call": {k: round(1e3 * statistics.median(v), 3) for k, v in parts.items()}}


def run_gpu(args) -> None:
    import torch
    from sedgpu import capi, synth

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # weak scaling: every rank integrates its own block of columns
    cs = synth.make_workload(args.workload, seed=args.seed + 7919 * rank)
    p = capi.params_from(cs, capi.SED_FP32, budgets=True, device=local)
    s = capi.Solver(cs, params=p)
    s.set_forcing()
    s.set_state(cs.conc)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    steps = args.steps or cs.nsteps   # default: the configured run
    # launch tuning chosen by the library's autotuner on a developed state
    # (ten simulated days in, or the middle of a shorter window: the
    # reference algorithm's substep count grows ~10x over the first days and
    # the developed regime dominates the run), untimed; the timed run then
    # starts from the configured initial state
    tuning = None
    if args.tuning:
        tc0, tc1, th0, th1 = (int(v) for v in args.tuning.split(","))
        s.set_tuning(tile_columns=(tc0, tc1), threads=(th0, th1))
    elif not args.no_autotune:
        s.step(max(1, min(240, steps // 2)))
        tuning = s.autotune(flags=0 if args.no_e2e else capi.SED_TUNE_PIPELINE)
    s.set_state(cs.conc)
    for _ in range(args.warmup):
        s.step(1)

    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms = 0.0
    launches = 0
    col_steps = 0
    att = acc = 0
    max_att = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        flush.zero_()            # L2 flush between timed steps
        torch.cuda.synchronize()
        st = s.step(1)
        dev_ms += st["device_ms"]
        launches += st["gpu_launches"]
        col_steps += st["column_steps"]
        att += st["attempts"]
        acc += st["accepted"]
        max_att = max(max_att, st["max_col_attempts"])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        t = torch.tensor([dev_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
        # whole-job substep statistics (scalars only; no state crosses ranks)
        from sedgpu import shard
        red = shard.reduce_stats({"attempts": att, "accepted": acc, "column_steps": col_steps,
                                  "max_col_attempts": max_att})
        att, acc, col_steps, max_att = (red["attempts"], red["accepted"],
                                        red["column_steps"], red["max_col_attempts"])
        dist.barrier()
    clk = clocks.stop()
    ms_per_step = dev_ms / steps
    value = world * cs.n_active * steps / (dev_ms / 1e3)

    # accuracy: one FP32 coupling step against the FP64 device path (which
    # reproduces the FP64 CPU restatement bit for bit) from the same state,
    # on an evenly spaced column sample
    accuracy = None
    acc_cols = np.unique(np.linspace(0, cs.ncol - 1, min(args.acc_columns, cs.ncol)
                                     ).astype(np.int64)) if args.acc_columns > 0 else []
    S = s.get_state() if len(acc_cols) else None
    errs = []
    outs = []
    sub = cs.subset(acc_cols) if len(acc_cols) else None
    if sub is not None:
        sub.conc = np.ascontiguousarray(S[:, :, acc_cols])
    for prec in ((capi.SED_FP32, capi.SED_FP64) if sub is not None else ()):
        pp = capi.params_from(sub, prec, budgets=False, device=local)
        ss = capi.Solver(sub, params=pp)
        ss.set_forcing()
        ss.set_state(sub.conc)
        ss.step(1)
        outs.append(ss.get_state())
        ss.close()
    if sub is not None:
        act_mask = np.arange(sub.kmax)[:, None] < sub.kact[None, :]
        for n in range(NTR):
            r = outs[1][n][act_mask]
            x = outs[0][n][act_mask]
            floor = 1e-4 * max(np.abs(r).max(), 1e-300)
            errs.append(float(np.max(np.abs(x - r) / (np.abs(r) + floor))))
        accuracy = {"max_rel_err_per_tracer": errs, "max_rel_err": max(errs),
                    "columns": int(len(acc_cols)),
                    "reference": "FP64 device path (bit-identical to the FP64 CPU "
                                 "restatement), one coupling step from the same state",
                    "parity": "OMEXDIA+P rates unpinned (a restatement of the published "
                              "model; FABM is not in the reference tree)",
                    "floor": "1e-4 x tracer max"}

    # budgets of the last timed step
    bud = s.budgets()
    act = cs.kact > 0
    drift_P = float(np.max(np.abs(bud[1][act]) / bud[0][act]))
    drift_N = float(np.max(np.abs(bud[3][act]) / bud[2][act]))

    # end-to-end through the drop-in call on pinned FP64 host arrays, over
    # the same coupling steps as the device run (from the initial state)
    e2e = None
    coupled = None
    if not args.no_e2e:
        n_e2e = args.e2e_steps or steps
        # the caller's arrays in pinned host memory (sed_host_alloc)
        conc = capi.host_empty(cs.conc.shape)
        conc[:] = cs.conc
        fluxes = capi.host_empty(cs.fluxes.shape)
        fluxes[:] = cs.fluxes
        bdys = capi.host_empty(cs.bdys.shape)
        bdys[:] = cs.bdys
        for _ in range(args.warmup):
            s.ode_solver(conc, bdys, fluxes, cs.dt)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(n_e2e):
            s.ode_solver(conc, bdys, fluxes, cs.dt)
        e2e_s = time.perf_counter() - t1
        h2d = conc.nbytes + bdys.nbytes + fluxes.nbytes
        d2h = conc.nbytes + fluxes.nbytes
        e2e = {"value": world * cs.n_active * n_e2e / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "steps": n_e2e, "call": "sed_ode_solver", "host_arrays": "pinned (sed_host_alloc)",
               "simulated_days_timed": days(args.warmup, args.warmup + n_e2e, cs.dt)}
        coupled = coupled_e2e(s, cs, args.warmup, n_e2e, world)

    t_now = s.tuning().as_dict()
    s_tuning = {k: t_now[k] for k in ("tile_columns", "threads", "pipeline_chunks",
                                       "segments")}
    s_tuning["chosen_by"] = ("--tuning" if args.tuning else
                             "sed_autotune" if tuning else "defaults")
    if tuning:
        s_tuning["autotune_trials"] = tuning["trials"]
    s.close()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    bytes_step = algorithmic_bytes(cs.kact, budgets=True)
    peak, peak_kind = measured_peaks()
    achieved = bytes_step / (ms_per_step / 1e3) / 1e9
    # FP32 work estimate of the column kernel (per cell: ~130 flops per
    # right-hand side + 11 per accepted update, 22 per attempt's test)
    K = float(np.mean(cs.kact[act]))
    flops = (acc * (130 + 11) + att * 22) * K
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_ach = flops / (dev_ms / 1e3) / 1e12

    cpu = None
    if not args.no_cpu:
        cpu = cpu_window(args.workload, args.seed, args.warmup, steps, os.cpu_count() or 1,
                         args.cpu_columns)
        cpu.pop("seconds")
        cpu.update(cpu_context(args.workload, args.seed, args.warmup, steps, args.cpu_columns))

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "columns": cs.n_active,
                   "layers": cs.kmax if cs.kact.min() == cs.kmax else
                   f"{int(cs.kact[cs.kact > 0].min())}..{int(cs.kact.max())}",
                   "land_fraction": float(np.mean(cs.kact == 0)),
                   "tracers": NTR, "dt_s": cs.dt,
                   "method": "adaptive_euler", "cut": "per_column",
                   "state": "fp32", "budgets": "fp64",
                   "l2": "flushed between timed steps",
                   "simulated_days_timed": days(args.warmup, args.warmup + steps, cs.dt),
                   "window": ("the configured run" if steps == cs.nsteps else
                              f"the first {steps} coupling steps"),
                   "solver": "plain",
                   "tuning": s_tuning},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": MEASURED_TRAFFIC.get(args.workload),
                     "peak_kind": peak_kind,
                     "bytes_per_launch": bytes_step,
                     "kernel": ("k_column_warp<float,1,...,ADAPT>" if s_tuning["tile_columns"][0] == 0
                                else "k_column<float,1,...,ADAPT>")},
        "compute": {"fp32_tflops_est": fp32_ach, "fp32_peak_tflops": fp32_peak,
                    "frac": fp32_ach / fp32_peak,
                    "note": "nominal 152 SM x 128 FMA/clk at the sampled clock"},
        "substeps": {"attempts_per_column_step": att / max(col_steps, 1),
                     "accepted_per_column_step": acc / max(col_steps, 1),
                     "max_attempts": max_att},
        "budget_drift": {"P": drift_P, "N": drift_N},
        "accuracy": accuracy,
        "e2e": e2e, "e2e_coupled": coupled, "cpu_baseline": cpu, "gpu_launches": launches,
        "clocks": clk, "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


PEL_METRIC = "pelagic water-column Runs/s on 1 GB300 (fabm_pelagic driver, gotm_npzd)"
PEL_WORKLOAD = "pelagic_1024x1024"


def pel_bytes(pcs, rsize: int = 4) -> int:
    """Bytes one Run must move: state read + write (2 r 4) and the PAR the
    handle keeps for later driver calls (r) per water cell, layer height (r)
    and mask (1) per cell of a water column, I_0 and albedo (2 r) and the
    bottom and surface flux rows (2 r 4) per water column."""
    water = int(pcs.water().sum())
    wcols = pcs.water_columns()
    return int(2 * rsize * 4 * water + rsize * water + (rsize + 1) * pcs.knum * wcols
               + 2 * rsize * wcols + 2 * rsize * 4 * wcols)


def pel_cpu(pcs, nruns: int, threads: int, max_columns: int, target_s: float = 15.0):
    """The pelagic oracle (all host threads) on an evenly spaced column
    sample sized, from a pilot, to about target_s seconds: the whole grid
    and more Runs when one Run of it is shorter than that."""
    import pel_oracle

    def timed(n, runs):
        cols = np.unique(np.linspace(0, pcs.ncol - 1, n).astype(np.int64))
        sub = pcs.subset(cols)
        c = sub.conc.copy()
        t0 = time.perf_counter()
        rc, _, _ = pel_oracle.PelOracle(sub).run(c, nthreads=threads, nruns=runs)
        return sub, time.perf_counter() - t0, rc
    n0 = min(max(64 * threads, 256), max_columns, pcs.ncol)
    sub, secs, rc = timed(n0, 1)
    per_col = secs / n0
    n = int(min(max_columns, pcs.ncol, max(n0, target_s / max(per_col, 1e-9))))
    nruns = max(nruns, int(target_s / max(per_col * n, 1e-9)))
    if n > 1.5 * n0 or nruns > 1:
        sub, secs, rc = timed(n, nruns)
    val = sub.water_columns() * nruns / secs
    return {"value": val, "unit": "column-runs/s", "cores": threads, "kind": "port",
            "sample": (f"{sub.water_columns()} water columns of {pcs.ncol} (evenly spaced), "
                       f"{nruns} Runs, {secs:.1f} s"), "seconds": secs, "status": rc,
            "runs": nruns}


def run_pelagic(args) -> None:
    """The pelagic driver path: Runs of the component (light, 10 internal
    RUNGE_KUTTA_4 steps of 360 s with their epilogues) on every water column
    of a 1024 x 1024 grid, FP32 state resident in HBM."""
    import torch
    from sedgpu import capi, pelagic

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pcs = pelagic.make_pelagic_workload(args.workload if args.workload != WORKLOAD
                                        else PEL_WORKLOAD, seed=args.seed + 7919 * rank)
    p = pcs.params(capi.SED_FP32)
    p.device = local
    s = pelagic.PelagicSolver(pcs, params=p)
    s.set_state(pcs.conc)
    runs = args.steps or pcs.nruns
    for _ in range(args.warmup):
        s.step(1)
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    dev_ms = 0.0
    launches = 0
    t0 = time.perf_counter()
    for _ in range(runs):
        st = s.step(1)
        dev_ms += st["device_ms"]
        launches += st["gpu_launches"]
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        t = torch.tensor([dev_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
        dist.barrier()
    clk = clocks.stop()
    wcols = pcs.water_columns()
    value = world * wcols * runs / (dev_ms / 1e3)

    # accuracy: one FP32 Run against the FP64 device path (bit-identical to
    # the FP64 CPU restatement) from the same state on a column sample
    S = s.get_state()
    cols = np.unique(np.linspace(0, pcs.ncol - 1, min(4096, pcs.ncol)).astype(np.int64))
    sub = pcs.subset(cols)
    sub.conc = np.ascontiguousarray(S[:, :, cols])
    outs = []
    for prec in (capi.SED_FP32, capi.SED_FP64):
        ss = pelagic.PelagicSolver(sub, precision=prec)
        ss.set_state(sub.conc)
        ss.step(1)
        outs.append(ss.get_state())
        ss.close()
    w = sub.water()
    errs = [float(np.max(np.abs(outs[0][n][w] - outs[1][n][w]) /
                         max(np.abs(outs[1][n][w]).max(), 1e-300))) for n in range(4)]

    e2e = None
    if not args.no_e2e:
        # the caller's array in pinned host memory (sed_host_alloc)
        conc = capi.host_empty(pcs.conc.shape)
        conc[:] = pcs.conc
        for _ in range(args.warmup):
            s.run(conc)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(runs):
            s.run(conc)
        e2e_s = time.perf_counter() - t1
        e2e = {"value": world * wcols * runs / e2e_s, "unit": "column-runs/s",
               "h2d_bytes_per_step": int(conc.nbytes), "d2h_bytes_per_step": int(conc.nbytes),
               "steps": runs, "call": "pel_run", "host_arrays": "pinned (sed_host_alloc)"}
    s.close()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    ms = dev_ms / runs
    bytes_run = pel_bytes(pcs)
    peak, peak_kind = measured_peaks()
    achieved = bytes_run / (ms / 1e3) / 1e9
    cells = int(pcs.water().sum())
    nsub = int(np.ceil(pcs.t_couple / pcs.dt))
    # FP32 work per cell and internal step of RUNGE_KUTTA_4: 4 rate
    # evaluations of ~35 flops (plus one exp and one division each) and
    # ~52 flops of stage updates
    flops = cells * nsub * (4 * 35 + 52)
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    cpu = None
    if not args.no_cpu:
        cpu = pel_cpu(pcs, 1, os.cpu_count() or 1, args.pel_cpu_columns or pcs.ncol)
        for k in ("seconds", "status", "runs"):
            cpu.pop(k)
    line = {
        "metric": PEL_METRIC, "value": value, "unit": "column-runs/s", "n_gpus": world,
        "steps": runs, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic (seeded)",
        "config": {"workload": PEL_WORKLOAD, "columns": pcs.ncol, "water_columns": wcols,
                   "layers": pcs.knum, "tracers": 4, "model": "gotm_npzd",
                   "t_couple_s": pcs.t_couple, "dt_s": pcs.dt, "method": "runge_kutta_4",
                   "state": "fp32",
                   "l2": "inputs larger than L2 (state 0.5 GB)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": PEL_TRAFFIC.get(PEL_WORKLOAD),
                     "peak_kind": peak_kind, "bytes_per_launch": bytes_run,
                     "kernel": "k_pel_run<float,float,RK4,light,epilogue>"},
        "compute": {"fp32_tflops_est": flops / (ms / 1e3) / 1e12,
                    "fp32_peak_tflops": fp32_peak,
                    "frac": flops / (ms / 1e3) / 1e12 / fp32_peak,
                    "note": "nominal 152 SM x 128 FMA/clk at the sampled clock"},
        "accuracy": {"max_rel_err_per_tracer": errs, "max_rel_err": max(errs),
                     "columns": int(len(cols)),
                     "reference": "FP64 device path (bit-identical to the FP64 CPU "
                                  "restatement), one Run from the same state",
                     "scale": "tracer max"},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches,
        "clocks": clk, "wall_s": wall,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_reference_pelagic(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import pel_oracle
    pel_oracle.build()
    from sedgpu import pelagic
    pcs = pelagic.make_pelagic_workload(PEL_WORKLOAD, seed=args.seed)
    runs = args.steps or 1
    cpu = pel_cpu(pcs, runs, os.cpu_count() or 1, args.pel_cpu_columns or pcs.ncol)
    line = {
        "metric": PEL_METRIC, "value": cpu["value"], "unit": "column-runs/s",
        "n_gpus": args.gpus, "steps": cpu["runs"], "warmup": args.warmup,
        "ms_per_step": cpu["seconds"] * 1e3 / cpu["runs"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": PEL_WORKLOAD, "layers": pcs.knum, "tracers": 4,
                   "model": "gotm_npzd", "t_couple_s": pcs.t_couple, "dt_s": pcs.dt,
                   "method": "runge_kutta_4"},
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cpu["value"], "unit": "column-runs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("reference algorithm as the FP64 C restatement on the host cores; the "
                 "Fortran reference and FABM cannot be built on this machine"),
    }
    print(json.dumps(line), flush=True)


CPL_METRIC = ("pelagic->soil coupling: horizontal columns mapped into the soil boundary per "
              "second on 1 GB300 (pelagic_soil_connector Run + get_boundary_conditions)")
CPL_PEL, CPL_SED = "pelagic_1024x1024", "soil_1024x1024"


def cpl_bytes(ncol: int, as_named: bool, depth: bool, rsize: int = 4) -> int:
    """Bytes one k_pelagic_soil launch must move for gotm_npzd's fields: the
    bottom-layer detritus and nutrient values (2 r), the water depth (8 when
    given), the eleven surface rows and the velocity rows the Run writes (8
    each: phosphorus only as the Run is written, the five detritus rows as
    named) per column."""
    return int(ncol * (2 * rsize + (8 if depth else 0) + 8 * (11 + (5 if as_named else 1))))


def cpl_cpu(conc, depth, target_s: float = 10.0):
    """The connector oracle on the whole grid (its column loops split over
    the host threads by OpenMP), repeated for about target_s seconds."""
    import pel_oracle
    fields = {"detN": 3, "din": 0}
    t0 = time.perf_counter()
    pel_oracle.cpl_run(conc, fields, None, False, depth)
    one = max(time.perf_counter() - t0, 1e-6)
    reps = max(1, int(target_s / one))
    t0 = time.perf_counter()
    for _ in range(reps):
        rc, *_ = pel_oracle.cpl_run(conc, fields, None, False, depth)
    secs = time.perf_counter() - t0
    ncol = conc.shape[2]
    return {"value": ncol * reps / secs, "unit": "columns/s", "cores": os.cpu_count() or 1,
            "kind": "port",
            "sample": f"the whole grid ({ncol} columns), {reps} calls, {secs:.1f} s",
            "seconds": secs, "calls": reps, "status": rc}


def cpl_bottom(pcs):
    """The pelagic state the oracle needs: the bottom layer only (k = 0)."""
    return np.ascontiguousarray(pcs.conc[:, :1, :])


def run_coupling(args) -> None:
    """The pelagic -> soil coupling on a 1024 x 1024 grid: the connector's
    mapping from the FP32 pelagic state of pelagic_1024x1024 into the
    boundary of the soil_1024x1024 sediment handle (gotm_npzd fields, the
    Run as written, water depth from the pelagic layer heights), state
    resident in HBM; bottom-water temperature and water depth come from
    host arrays each call, as the API takes them."""
    import torch
    from sedgpu import capi, coupling, pelagic, synth

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pcs = pelagic.make_pelagic_workload(CPL_PEL, seed=args.seed + 7919 * rank)
    cs = synth.make_workload(CPL_SED, seed=args.seed + 7919 * rank)
    assert pcs.ncol == cs.ncol
    pp = pcs.params(capi.SED_FP32)
    pp.device = local
    pel = pelagic.PelagicSolver(pcs, params=pp)
    pel.set_state(pcs.conc)
    sed = capi.Solver(cs, params=capi.params_from(cs, capi.SED_FP32, device=local))
    sed.set_state(cs.conc)
    T = np.array(cs.bdys[0], dtype=np.float64, copy=True)
    depth = np.ascontiguousarray(pcs.layer_height.sum(axis=0))
    for a in (T, depth):
        capi.host_register(a)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    calls = args.steps or 200
    st = coupling.CplStats()
    for _ in range(args.warmup):
        coupling.pelagic_soil(pel, sed, T, depth, stats=st, read_back=False)
    clocks = ClockSampler(local)
    clocks.start()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    kern_ms = dev_ms = 0.0
    launches = 0
    t0 = time.perf_counter()
    for _ in range(calls):
        flush.zero_()            # L2 flush between timed calls
        torch.cuda.synchronize()
        coupling.pelagic_soil(pel, sed, T, depth, stats=st, read_back=False)
        kern_ms += st.kernel_ms
        dev_ms += st.device_ms
        launches += st.gpu_launches
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    # the reverse direction (soil_pelagic_connector) on the fluxes of one
    # soil step, timed the same way
    sed.step(1)
    for _ in range(args.warmup):
        coupling.soil_pelagic(sed, pel, stats=st, read_back=False)
    rev_kern = rev_dev = 0.0
    for _ in range(calls):
        flush.zero_()
        torch.cuda.synchronize()
        coupling.soil_pelagic(sed, pel, stats=st, read_back=False)
        rev_kern += st.kernel_ms
        rev_dev += st.device_ms
        launches += st.gpu_launches
    torch.cuda.synchronize()
    if dist:
        t = torch.tensor([dev_ms, kern_ms, rev_dev, rev_kern], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms, kern_ms, rev_dev, rev_kern = (float(v) for v in t.tolist())
        dist.barrier()
    clk = clocks.stop()
    e2e = None
    if not args.no_e2e:
        t1 = time.perf_counter()
        for _ in range(calls):
            _, _, present = coupling.pelagic_soil(pel, sed, T, depth, read_back=False)
        e2e_s = time.perf_counter() - t1
        e2e = {"value": world * cs.ncol * calls / e2e_s, "unit": "columns/s",
               "h2d_bytes_per_step": int(T.nbytes + depth.nbytes),
               "d2h_bytes_per_step": int(present.nbytes), "steps": calls,
               "call": "cpl_pelagic_soil (host temperature and water depth in, the "
                       "present flags out; the boundary stays on the device)"}
    for a in (T, depth):
        capi.host_unregister(a)
    pel.close()
    sed.close()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    nbytes = cpl_bytes(cs.ncol, False, True)
    # reverse, gotm_npzd: four soil flux rows read (8 B each), two pelagic
    # bottom-flux rows written (4 B each) per column
    rev_bytes = cs.ncol * (4 * 8 + 2 * 4)
    peak, peak_kind = measured_peaks()
    achieved = nbytes / (kern_ms / calls / 1e3) / 1e9
    cpu = None
    if not args.no_cpu:
        cpu = cpl_cpu(cpl_bottom(pcs), depth, args.cpl_cpu_seconds)
        for k in ("seconds", "status", "calls"):
            cpu.pop(k)
    line = {
        "metric": CPL_METRIC, "value": world * cs.ncol * calls / (dev_ms / 1e3),
        "unit": "columns/s", "n_gpus": world, "steps": calls, "warmup": args.warmup,
        "ms_per_step": dev_ms / calls, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": f"{CPL_PEL} -> {CPL_SED}", "columns": cs.ncol,
                   "fields": "gotm_npzd (detN = detritus, DIN = nutrients)",
                   "mode": "CPL_AS_RUN", "water_depth": "given", "tke": "absent",
                   "pelagic_state": "f32", "l2": "L2 flushed between timed calls"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                     "bytes_per_launch": nbytes, "kernel": "k_pelagic_soil<float>",
                     "kernel_ms": kern_ms / calls},
        "reverse": {"kernel": "k_soil_pelagic<float>", "calls": calls,
                    "kernel_ms": rev_kern / calls, "device_ms": rev_dev / calls,
                    "bytes_per_launch": rev_bytes,
                    "achieved_gbs": rev_bytes / (rev_kern / calls / 1e3) / 1e9,
                    "frac": rev_bytes / (rev_kern / calls / 1e3) / 1e9 / peak,
                    "note": ("cpl_soil_pelagic: the soil's flux scatter and the mapping of "
                             "its nitrate, ammonium and detritus N fluxes into the pelagic "
                             "nutrient and detritus bottom fluxes")},
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches,
        "clocks": clk, "wall_s": wall,
        "note": ("ms_per_step and value: the call's device span (temperature and depth "
                 "copies, the mapping, the boundary assembly and the forcing rows); "
                 "gpu_launches counts both directions"),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_reference_coupling(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import pel_oracle
    pel_oracle.build()
    from sedgpu import pelagic
    pcs = pelagic.make_pelagic_workload(CPL_PEL, seed=args.seed)
    depth = np.ascontiguousarray(pcs.layer_height.sum(axis=0))
    cpu = cpl_cpu(cpl_bottom(pcs), depth, args.cpl_cpu_seconds)
    line = {
        "metric": CPL_METRIC, "value": cpu["value"], "unit": "columns/s",
        "n_gpus": args.gpus, "steps": cpu["calls"], "warmup": args.warmup,
        "ms_per_step": cpu["seconds"] * 1e3 / cpu["calls"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)", "impl": "reference",
        "config": {"workload": f"{CPL_PEL} -> {CPL_SED}", "columns": pcs.ncol,
                   "fields": "gotm_npzd (detN = detritus, DIN = nutrients)",
                   "mode": "CPL_AS_RUN", "water_depth": "given", "tke": "absent"},
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cpu["value"], "unit": "columns/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the connector's Run as the C restatement on the host cores (the "
                 "mapping only); the Fortran reference and ESMF cannot be built here"),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0,
                    help="coupling steps timed (default: the workload's configured run)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="",
                    help=f"default: {HEADLINE} (surrogate), {WORKLOAD} (plain)")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--cpu-columns", type=int, default=8192)
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end legs (default: --steps)")
    ap.add_argument("--acc-columns", type=int, default=4096)
    ap.add_argument("--solver", default="surrogate", choices=["plain", "surrogate"],
                    help="surrogate: the headline (surrogate + fallback vs plain on the "
                         "2048 x 2048 workload); plain: the plain solver alone")
    ap.add_argument("--start-day", type=float, default=10.0,
                    help="surrogate: simulated day the timed window starts at")
    ap.add_argument("--sur-tol", type=float, default=1e-3)
    ap.add_argument("--sur-res-atol", type=float, default=1e-2)
    ap.add_argument("--sur-sweep", type=float, nargs="*", default=[1e-2, 1e-1, 1.0, 1e30],
                    help="residual tolerances of the sweep (1e30: every proposal taken)")
    ap.add_argument("--sur-train-columns", type=int, default=200000)
    ap.add_argument("--sur-test-columns", type=int, default=20000)
    ap.add_argument("--sur-every", type=int, default=15,
                    help="training rows from every n-th coupling step")
    ap.add_argument("--sur-train-steps", type=int, default=50000)
    ap.add_argument("--acc-steps", type=int, default=8,
                    help="surrogate: teacher-forced accuracy steps on the subsample")
    ap.add_argument("--ref-columns", type=int, default=2048,
                    help="surrogate reference arm: columns of the CPU sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default="",
                    help="tile columns and threads per depth class, 'tc0,tc1,th0,th1' "
                         "(replaces the autotuner)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--spinup-years", type=float, default=0.0,
                    help="time sed_spinup's 1-column model for this many years instead")
    ap.add_argument("--spinup-cpu-steps", type=int, default=2000)
    ap.add_argument("--ensemble", type=int, default=0,
                    help="with --spinup-years: spin up this many parameter sets at once")
    ap.add_argument("--mlp-rows", type=int, default=2936778,
                    help="--path mlp: rows of the inference batch")
    ap.add_argument("--path", default="sediment",
                    choices=["sediment", "pelagic", "coupling", "mlp"],
                    help="pelagic: the fabm_pelagic driver path instead; coupling: the "
                         "pelagic -> soil connector; mlp: the surrogate network's "
                         "inference on the tensor cores")
    ap.add_argument("--cpl-cpu-seconds", type=float, default=8.0,
                    help="coupling CPU baseline: about this many seconds of oracle calls")
    ap.add_argument("--pel-cpu-columns", type=int, default=0,
                    help="pelagic CPU baseline: at most this many columns (0: the grid)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    headline = (args.path == "sediment" and args.solver == "surrogate"
                and args.spinup_years <= 0)
    if not args.workload:
        args.workload = HEADLINE if headline else WORKLOAD
    if args.path == "mlp":
        run_mlp(args)
        return
    if args.path == "pelagic":
        if args.impl == "reference":
            run_reference_pelagic(args)
        else:
            run_pelagic(args)
    elif args.path == "coupling":
        if args.impl == "reference":
            run_reference_coupling(args)
        else:
            run_coupling(args)
    elif args.impl == "reference":
        if headline:
            run_reference_headline(args)
        else:
            run_reference(args)
    elif args.spinup_years > 0 and args.ensemble > 0:
        run_ensemble_spinup(args)
    elif args.spinup_years > 0:
        run_spinup(args)
    elif headline:
        run_headline(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
