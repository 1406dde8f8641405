"""Profiling cases: the launches of one coupling step in a stated regime,
bracketed by cudaProfilerStart / cudaProfilerStop so that
``ncu --profile-from-start off`` captures them and nothing of the set-up.

    python -m sedgpu.profcase plain --columns 262144 --day 10
        one plain FP32 step (budgets on) of the first COLUMNS columns of the
        2048 x 2048 workload, from the state DAY simulated days in
    python -m sedgpu.profcase surrogate --day 10 [--sur-columns N]
        the whole 2048 x 2048 workload (or its first N columns) at day DAY:
        one plain step, then one gated surrogate step (tolerance 1e-3) with
        a briefly trained network; budgets off as in the bench's headline
        (--budgets: on)
    python -m sedgpu.profcase train --engine tcgen05
        one training step of the surrogate network at batch 8192 on rows
        of the 200 000-column workload (ENGINE: tcgen05 or mma_sync), after
        TIMED steps measured with CUDA events on the library's stream

The tuning is the workload's autotuned one at DAY.  Run from the repository
root with ``mossco-code_gb300`` on the path (``python -m`` from that folder,
or PYTHONPATH)."""
import argparse
import json
import time

import numpy as np

from . import capi, synth


def _develop(cs, day: float, budgets: bool = True):
    s = capi.Solver(cs, budgets=budgets)
    s.set_forcing()
    s.set_state(cs.conc)
    n = int(round(day * 86400.0 / cs.dt))
    done = 0
    while done < n:
        k = min(24, n - done)
        s.step(k)
        done += k
    s.autotune()
    return s


def plain(columns: int, day: float) -> dict:
    import torch
    cs = synth.make_workload("surrogate_2048x2048", cols=np.arange(columns))
    s = _develop(cs, day)
    s.step(1)   # the graph and tuning in place
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    st = s.step(1)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    t = s.tuning().as_dict()
    s.close()
    return {"case": "plain", "columns": int(cs.n_active), "day": day,
            "tuning": {k: t[k] for k in ("tile_columns", "threads")},
            "attempts": st["attempts"], "accepted": st["accepted"],
            "column_steps": st["column_steps"], "device_ms": st["device_ms"]}


def surrogate(day: float, train_steps: int = 300, columns: int = 0,
              budgets: bool = False) -> dict:
    import torch
    from . import surrogate as S
    train = synth.make_workload("surrogate_200k", cols=np.arange(8192))
    sur, _ = S.train_surrogate(train, None, nsteps=48, every=3, warm=12,
                               train_steps=train_steps, batch=2048, log_every=100)
    cs = synth.make_workload("surrogate_2048x2048",
                             cols=np.arange(columns) if columns > 0 else None)
    s = _develop(cs, day, budgets=budgets)
    s0 = s.get_state()
    # one untimed pass of each, then the profiled pair from the same state
    s.step(1)
    s.set_state(s0)
    S.step_surrogate(s, sur, 1, tol=1e-3)
    s.set_state(s0)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    p = s.step(1)
    s.set_state(s0)
    q = S.step_surrogate(s, sur, 1, tol=1e-3)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    s.close()
    sur.close()
    return {"case": "surrogate", "columns": int(cs.n_active), "day": day, "budgets": budgets,
            "plain_ms": p["device_ms"], "surrogate_ms": q["device_ms"],
            "surrogate_columns": q["surrogate_columns"],
            "launches": {"plain": p["gpu_launches"], "surrogate": q["gpu_launches"]}}


def train(engine: str, timed: int = 200) -> dict:
    import ctypes

    import torch
    from . import surrogate as S
    cs = synth.make_workload("surrogate_200k", cols=np.arange(16384))
    rows = S.collect_rows(cs, 48, 3, warm=12)
    nz = S.fit_normalizer(rows)
    X, Y = S.standardised(rows, nz)
    m = 8192
    sur = S.Surrogate(cs.kmax, batch=m)
    sur.set_norm(nz)
    lib = sur.lib
    lib.sed_sur_set_tensor_cores(sur.h, 1 if engine == "tcgen05" else 0)
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    sur._check(lib.sed_sur_set_stream(sur.h, ctypes.c_void_p(st.cuda_stream)), "stream")
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1)
    with torch.cuda.stream(st):
        idx = torch.randint(0, X.shape[0], (m,), device="cuda", generator=gen)
        xb = X.index_select(0, idx)
        yb = Y.index_select(0, idx)

        def step():
            sur._check(lib.sed_sur_train_step(sur.h, ctypes.c_void_p(xb.data_ptr()),
                                              ctypes.c_void_p(yb.data_ptr()), m, 1e-4, None),
                       "train step")

        for _ in range(5):
            step()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(timed):
            step()
        e1.record(st)
        st.synchronize()
        ms = e0.elapsed_time(e1) / timed
        torch.cuda.profiler.start()
        step()
        st.synchronize()
        torch.cuda.profiler.stop()
    sur._check(lib.sed_sur_set_stream(sur.h, None), "stream")
    # products per step: forward, input gradients (not of the first layer)
    # and weight gradients, 2 m n k FLOPs each at the padded widths
    dims = [(384, 256), (256, 256), (256, 256), (256, 256), (256, 384)]
    flops = sum(2 * m * a * b * (3 if l > 0 else 2) for l, (a, b) in enumerate(dims))
    sur.close()
    return {"case": "train", "engine": engine, "batch": m, "ms_per_step": round(ms, 4),
            "gemm_tflops_per_step": flops / 1e12,
            "tflop_s": round(flops / (ms * 1e-3) / 1e12, 1)}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("case", choices=("plain", "surrogate", "train"))
    ap.add_argument("--columns", type=int, default=262144)
    ap.add_argument("--day", type=float, default=10.0)
    ap.add_argument("--sur-columns", type=int, default=0,
                    help="surrogate case: the first SUR_COLUMNS columns (0: the whole grid)")
    ap.add_argument("--budgets", action="store_true",
                    help="surrogate case: budgets on (the plain case always has them)")
    ap.add_argument("--engine", default="tcgen05", choices=("tcgen05", "mma_sync"))
    ap.add_argument("--timed", type=int, default=200)
    a = ap.parse_args(argv)
    t = time.perf_counter()
    if a.case == "plain":
        out = plain(a.columns, a.day)
    elif a.case == "surrogate":
        out = surrogate(a.day, columns=a.sur_columns, budgets=a.budgets)
    else:
        out = train(a.engine, a.timed)
    out["wall_s"] = round(time.perf_counter() - t, 1)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
