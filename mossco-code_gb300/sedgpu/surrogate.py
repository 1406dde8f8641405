"""Column-increment surrogate: training rows, normalisation, training, use.

The network (nin = 11 K + 13 -> 256 x 4, GELU -> nout = 11 K) maps a
column's state and its 13 forcing rows to the change of log(C + c0) over one
coupling step.  It serves the columns whose plain step is expensive: those
whose first adaptive attempt -- the whole coupling step at once -- is
rejected, so that the plain solver takes hundreds of substeps.  In
sed_step_surrogate that attempt is the gate (accepted columns are finished
exactly as the plain step), the network proposes a state for the others, a
residual test with the plain right-hand side takes or rejects each proposal,
and rejected columns are stepped by the plain solver.

Training rows come from the plain FP32 GPU solver (sed_sur_collect: one
plain step, then a row for every column whose step took more than one
attempt), written straight into device arrays.  The network's products, loss,
backward pass and Adam run in the library's own kernels (sed_sur_*); torch
only holds the rows on the device, standardises them and draws batches.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import time
from typing import Optional, Tuple

import numpy as np

from . import capi
from .model import NTR, ColumnSet

NFORCE = 13
HIDDEN, NHIDDEN = 256, 4


def pad128(n: int) -> int:
    return (n + 127) // 128 * 128


def forcing_rows(cs: ColumnSet) -> np.ndarray:
    """The 13 per-column forcing rows the solver forms for a coupling step
    (bioturbation x f_T, molecular multiplier, 11 surface values), rounded to
    FP32 as the device holds them."""
    d = cs.driver
    T = cs.bdys[0]
    fT = np.exp(-4500.0 * (1.0 / (T + 273.0) - 1.0 / 288.0))
    rows = np.zeros((NFORCE, cs.ncol))
    rows[0] = d.bioturbation * fT
    rows[1] = 1.0 if d.mol_diff_mode == 1 else d.diffusivity + 0.035 * T
    for n in range(NTR):
        part = n < 6
        rows[2 + n] = cs.fluxes[n] if (part or d.bcup_dissolved == 1) else cs.bdys[n + 1]
    return rows.astype(np.float32).astype(np.float64)


@dataclasses.dataclass
class Normalizer:
    c0: np.ndarray     # [11] offsets of the log transform
    mu_x: np.ndarray   # [nin]
    sd_x: np.ndarray
    mu_d: np.ndarray   # [nout]
    sd_d: np.ndarray

    def pack(self) -> np.ndarray:
        return np.concatenate([self.c0, self.mu_x, self.sd_x, self.mu_d,
                               self.sd_d]).astype(np.float32)

    @staticmethod
    def unpack(v: np.ndarray, K: int) -> "Normalizer":
        nin, nout = NTR * K + NFORCE, NTR * K
        o = [0, NTR, NTR + nin, NTR + 2 * nin, NTR + 2 * nin + nout,
             NTR + 2 * nin + 2 * nout]
        return Normalizer(*(np.asarray(v[o[i]:o[i + 1]], dtype=np.float64)
                            for i in range(5)))


# Flat checkpoint for hosts without numpy (a Fortran component reads it with
# stream access): nine little-endian int64 -- RAW_MAGIC, K, nin, nout,
# hidden, nhidden, the state's length (sed_sur_state_size), the
# normalisation's length (11 + 2 nin + 2 nout) and Adam's step count --
# then the FP32 state (sed_sur_get_state's layout) and the FP32
# normalisation (sed_sur_set_norm's layout).
RAW_MAGIC = 0x5345445355524731  # "SEDSURG1"
RAW_HEADER = 9


def write_raw(path: str, ck: dict) -> None:
    """Write a checkpoint (Surrogate.checkpoint()) in the flat format."""
    K = int(ck["K"])
    nin, nout = NTR * K + NFORCE, NTR * K
    state = np.ascontiguousarray(ck["state"], dtype="<f4")
    norm = np.ascontiguousarray(ck["norm"], dtype="<f4")
    if norm.size != NTR + 2 * nin + 2 * nout:
        raise ValueError(f"normalisation of {norm.size} floats for K = {K}")
    hdr = np.array([RAW_MAGIC, K, nin, nout, HIDDEN, NHIDDEN, state.size, norm.size,
                    int(ck["step"])], dtype="<i8")
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(state.tobytes())
        f.write(norm.tobytes())


def read_raw(path: str) -> dict:
    """Read a flat checkpoint back into Surrogate.restore()'s form."""
    with open(path, "rb") as f:
        hdr = np.frombuffer(f.read(8 * RAW_HEADER), dtype="<i8")
        if hdr.size != RAW_HEADER or hdr[0] != RAW_MAGIC:
            raise ValueError(f"{path}: not a flat surrogate checkpoint")
        K, nin, nout, hidden, nhidden, nstate, nnorm, step = (int(v) for v in hdr[1:])
        if (nin, nout) != (NTR * K + NFORCE, NTR * K) or (hidden, nhidden) != (HIDDEN, NHIDDEN) \
                or nnorm != NTR + 2 * nin + 2 * nout:
            raise ValueError(f"{path}: header {hdr.tolist()} does not describe this network")
        state = np.frombuffer(f.read(4 * nstate), dtype="<f4")
        norm = np.frombuffer(f.read(4 * nnorm), dtype="<f4")
        if state.size != nstate or norm.size != nnorm or f.read(1):
            raise ValueError(f"{path}: length does not match its header")
    return {"state": state.astype(np.float32), "step": step,
            "norm": norm.astype(np.float32), "K": K}


def log_state(conc: np.ndarray, c0: np.ndarray) -> np.ndarray:
    """[ntr][K][cols] -> [cols][ntr*K] of log(max(C, 0) + c0)."""
    ntr, K, n = conc.shape
    u = np.log(np.maximum(conc, 0.0) + c0[:, None, None])
    return u.reshape(ntr * K, n).T


def c0_of(cs: ColumnSet) -> np.ndarray:
    """Offsets of the log transform: 1e-3 of each tracer's median magnitude
    over the active cells of the initial state, at least 1e-6."""
    act = np.arange(cs.kmax)[:, None] < cs.kact[None, :]
    med = np.array([np.median(np.abs(cs.conc[n][act])) for n in range(NTR)])
    return np.maximum(1e-3 * med, 1e-6)


@dataclasses.dataclass
class Rows:
    """Training rows on the device (torch FP32 tensors): x [m][11K+13] of
    log-state and forcing, y [m][11K] of log-state change."""
    x: "object"
    y: "object"
    c0: np.ndarray
    K: int
    columns: int
    steps: int
    collect_steps: int
    full: bool          # the arrays filled up: later rows were dropped


def collect_rows(cs: ColumnSet, nsteps: int, every: int, warm: int = 0,
                 c0: Optional[np.ndarray] = None, capacity: Optional[int] = None,
                 heavy_share: float = 1.0) -> Rows:
    """Run the plain FP32 solver over ``cs`` for ``nsteps`` coupling steps
    from its initial state and collect the rows of every ``every``-th step
    from ``warm`` on (sed_sur_collect).  The default capacity holds a row
    for every column at every collected step."""
    import torch
    K = cs.kmax
    nin, nout = NTR * K + NFORCE, NTR * K
    c0 = c0_of(cs) if c0 is None else np.asarray(c0, dtype=np.float64)
    picks = list(range(warm, nsteps, every))
    if capacity is None:
        capacity = max(1, int(heavy_share * len(picks) * cs.n_active))
    x = torch.empty((capacity, nin), dtype=torch.float32, device="cuda")
    y = torch.empty((capacity, nout), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    c0f = np.ascontiguousarray(c0, dtype=np.float32)
    count = ctypes.c_longlong(0)
    s = capi.Solver(cs, precision=capi.SED_FP32)
    try:
        s.set_forcing()
        s.set_state(cs.conc)
        t = 0
        for p in picks:
            if p > t:
                s.step(p - t)
            st = capi.SedStats()
            rc = s.lib.sed_sur_collect(
                s.h, c0f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), float(cs.dt),
                ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), nin, nout,
                capacity, ctypes.byref(count), ctypes.byref(st))
            s._check(rc, "sed_sur_collect")
            t = p + 1
    finally:
        s.close()
    m = count.value
    return Rows(x=x[:m], y=y[:m], c0=c0, K=K, columns=cs.n_active, steps=nsteps,
                collect_steps=len(picks), full=m >= capacity)


def fit_normalizer(rows: Rows, chunk: int = 1 << 18) -> Normalizer:
    """Means and standard deviations of the features and targets (FP64
    accumulation over row chunks)."""
    import torch

    def moments(a):
        s1 = torch.zeros(a.shape[1], dtype=torch.float64, device=a.device)
        s2 = torch.zeros_like(s1)
        for i in range(0, a.shape[0], chunk):
            b = a[i:i + chunk].double()
            s1 += b.sum(0)
            s2 += (b * b).sum(0)
        n = max(a.shape[0], 1)
        mu = s1 / n
        var = torch.clamp(s2 / n - mu * mu, min=0.0)
        return mu.cpu().numpy(), torch.sqrt(var).cpu().numpy()

    mu_x, sd_x = moments(rows.x)
    mu_d, sd_d = moments(rows.y)
    sd_x[sd_x < 1e-8 * (np.abs(mu_x) + 1.0)] = 1.0
    sd_d[sd_d < 1e-12] = 1e-12
    return Normalizer(rows.c0, mu_x, sd_x, mu_d, sd_d)


def standardised(rows: Rows, nz: Normalizer, chunk: int = 1 << 18):
    """BF16 device arrays of the standardised rows, padded to multiples of
    128 columns (the layout sed_sur_train_step reads)."""
    import torch
    nin, nout = rows.x.shape[1], rows.y.shape[1]
    m = rows.x.shape[0]
    X = torch.zeros((m, pad128(nin)), dtype=torch.bfloat16, device="cuda")
    Y = torch.zeros((m, pad128(nout)), dtype=torch.bfloat16, device="cuda")
    mx = torch.tensor(nz.mu_x, dtype=torch.float32, device="cuda")
    sx = torch.tensor(nz.sd_x, dtype=torch.float32, device="cuda")
    md = torch.tensor(nz.mu_d, dtype=torch.float32, device="cuda")
    sdd = torch.tensor(nz.sd_d, dtype=torch.float32, device="cuda")
    for i in range(0, m, chunk):
        X[i:i + chunk, :nin] = ((rows.x[i:i + chunk] - mx) / sx).to(torch.bfloat16)
        Y[i:i + chunk, :nout] = ((rows.y[i:i + chunk] - md) / sdd).to(torch.bfloat16)
    return X, Y


class Surrogate:
    """A library surrogate handle (sed_sur_*) with its normalisation."""

    def __init__(self, K: int, batch: int = 8192, seed: int = 7, device: int = 0):
        self.lib = capi.load()
        self.K = K
        self.nin, self.nout = NTR * K + NFORCE, NTR * K
        self.pin, self.pout = pad128(self.nin), pad128(self.nout)
        h = capi._H()
        rc = self.lib.sed_sur_create(self.nin, self.nout, HIDDEN, NHIDDEN, batch, seed,
                                     device, ctypes.byref(h))
        if rc != 0:
            raise capi.SedError(rc, "sed_sur_create")
        self.h = h
        self.batch = batch
        self.norm: Optional[Normalizer] = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.sed_sur_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise capi.SedError(rc, f"{what}: {self.lib.sed_sur_last_error(self.h).decode()}")

    def set_norm(self, nz: Normalizer):
        self.norm = nz
        v = nz.pack()
        self._check(self.lib.sed_sur_set_norm(
            self.h, v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(v)),
            "sed_sur_set_norm")

    def weights(self) -> np.ndarray:
        n = self.lib.sed_sur_num_params(self.h)
        w = np.zeros(n, dtype=np.float32)
        self._check(self.lib.sed_sur_get_weights(
            self.h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "get weights")
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self.lib.sed_sur_set_weights(
            self.h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "set weights")

    def checkpoint(self) -> dict:
        """The training state: parameters, Adam moments and step count
        (sed_sur_get_state), with the normalisation."""
        n = self.lib.sed_sur_state_size(self.h)
        st = np.zeros(n, dtype=np.float32)
        step = ctypes.c_longlong(0)
        self._check(self.lib.sed_sur_get_state(
            self.h, st.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(step)),
            "get state")
        return {"state": st, "step": int(step.value),
                "norm": None if self.norm is None else self.norm.pack(), "K": self.K}

    def restore(self, ck: dict):
        st = np.ascontiguousarray(ck["state"], dtype=np.float32)
        self._check(self.lib.sed_sur_set_state(
            self.h, st.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), int(ck["step"])),
            "set state")
        if ck.get("norm") is not None:
            self.set_norm(Normalizer.unpack(ck["norm"], int(ck["K"])))

    def save(self, path: str):
        """Parameters, Adam state and normalisation to an .npz file."""
        ck = self.checkpoint()
        np.savez_compressed(path, state=ck["state"], step=ck["step"], norm=ck["norm"],
                            K=self.K)

    @staticmethod
    def load(path: str, batch: int = 8192) -> "Surrogate":
        d = np.load(path)
        s = Surrogate(int(d["K"]), batch=batch)
        s.restore({"state": d["state"], "step": int(d["step"]), "norm": d["norm"],
                   "K": int(d["K"])})
        return s

    def save_raw(self, path: str):
        """The checkpoint in the flat format of write_raw (for a Fortran
        host: sed_sur_create, sed_sur_set_state, sed_sur_set_norm)."""
        write_raw(path, self.checkpoint())

    @staticmethod
    def load_raw(path: str, batch: int = 8192) -> "Surrogate":
        ck = read_raw(path)
        s = Surrogate(ck["K"], batch=batch)
        s.restore(ck)
        return s

    def train(self, X, Y, steps: int, lr: float = 1e-3, lr_final: float = 2e-5,
              log_every: int = 1000, seed: int = 0):
        """Adam on random batches of standardised rows (cosine decay of the
        learning rate).  X, Y: BF16 device tensors padded to pin / pout
        columns (``standardised``).  Returns [(step, loss, seconds)]."""
        import torch
        n = X.shape[0]
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        loss = np.zeros(1, dtype=np.float32)
        lp = loss.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        log = []
        m = self.batch
        # The batches are gathered and the library's steps run on one torch
        # stream of their own, so each step's copy of its batch is ordered
        # after the gather that writes it and before the caching allocator
        # hands the batch's memory to a later gather.  (With the steps on
        # another stream, a step could copy a batch that a later gather was
        # already overwriting.)  The stream is a created one: the library
        # reads a null stream as "its own stream".
        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        self._check(self.lib.sed_sur_set_stream(self.h, ctypes.c_void_p(stream.cuda_stream)),
                    "sed_sur_set_stream")
        t0 = time.perf_counter()
        try:
            with torch.cuda.stream(stream):
                for it in range(steps):
                    idx = torch.randint(0, n, (m,), device="cuda", generator=gen)
                    xb = X.index_select(0, idx)
                    yb = Y.index_select(0, idx)
                    frac = it / max(steps - 1, 1)
                    lr_t = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * frac))
                    want = (it % log_every == 0) or it == steps - 1
                    self._check(self.lib.sed_sur_train_step(
                        self.h, ctypes.c_void_p(xb.data_ptr()), ctypes.c_void_p(yb.data_ptr()),
                        m, float(lr_t), lp if want else None), "train step")
                    if want:
                        log.append((it, float(loss[0]), time.perf_counter() - t0))
        finally:
            self._check(self.lib.sed_sur_set_stream(self.h, None), "sed_sur_set_stream")
            torch.cuda.current_stream().wait_stream(stream)
        return log

    def predict_device(self, X):
        """Standardised predictions [m][nout] (torch FP32) of BF16 device rows
        X [m][pin] (sed_sur_forward_device)."""
        import torch
        m = X.shape[0]
        mp = pad128(m)
        if mp != m:
            Xp = torch.zeros((mp, self.pin), dtype=torch.bfloat16, device="cuda")
            Xp[:m] = X
        else:
            Xp = X.contiguous()
        Yp = torch.empty((mp, self.pout), dtype=torch.float32, device="cuda")
        torch.cuda.current_stream().synchronize()
        self._check(self.lib.sed_sur_forward_device(
            self.h, ctypes.c_void_p(Xp.data_ptr()), ctypes.c_void_p(Yp.data_ptr()), mp),
            "forward")
        return Yp[:m, :self.nout]

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.nout), dtype=np.float32)
        self._check(self.lib.sed_sur_forward(
            self.h, X.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            Y.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), X.shape[0]), "forward")
        return Y

    def next_state(self, conc: np.ndarray, force: np.ndarray) -> np.ndarray:
        """Proposed state after one coupling step, [ntr][K][cols] (host rows
        through sed_sur_forward)."""
        nz = self.norm
        u0 = log_state(conc, nz.c0)
        X = (np.concatenate([u0, force.T], axis=1) - nz.mu_x) / nz.sd_x
        d = self.predict(X).astype(np.float64) * nz.sd_d + nz.mu_d
        u1 = u0 + d
        ntr, K, n = conc.shape
        out = np.exp(u1.T.reshape(ntr, K, n)) - nz.c0[:, None, None]
        return np.maximum(out, 0.0)


def evaluate(sur: Surrogate, rows: Rows, chunk: int = 1 << 17) -> dict:
    """Held-out error of the network on collected rows: standardised MSE,
    and per row the largest relative error of the proposed state against the
    plain solver's (floor 1e-4 x the tracer's largest value in the set)."""
    import torch
    nz = sur.norm
    K = rows.K
    mx = torch.tensor(nz.mu_x, dtype=torch.float32, device="cuda")
    sx = torch.tensor(nz.sd_x, dtype=torch.float32, device="cuda")
    md = torch.tensor(nz.mu_d, dtype=torch.float32, device="cuda")
    sdd = torch.tensor(nz.sd_d, dtype=torch.float32, device="cuda")
    c0 = torch.tensor(np.repeat(nz.c0, K), dtype=torch.float32, device="cuda")
    m = rows.x.shape[0]
    # tracer maxima of the true next states
    tmax = torch.zeros(NTR, dtype=torch.float32, device="cuda")
    for i in range(0, m, chunk):
        u1 = rows.x[i:i + chunk, :NTR * K] + rows.y[i:i + chunk]
        c1 = torch.clamp(torch.exp(u1) - c0, min=0.0).view(-1, NTR, K)
        tmax = torch.maximum(tmax, c1.amax(dim=(0, 2)))
    floor = (1e-4 * tmax).repeat_interleave(K)
    mse, errs, per_tr = 0.0, [], []
    for i in range(0, m, chunk):
        xb, yb = rows.x[i:i + chunk], rows.y[i:i + chunk]
        Xn = torch.zeros((xb.shape[0], sur.pin), dtype=torch.bfloat16, device="cuda")
        Xn[:, :sur.nin] = ((xb - mx) / sx).to(torch.bfloat16)
        pred = sur.predict_device(Xn)
        ytrue = (yb - md) / sdd
        mse += float(((pred - ytrue) ** 2).sum())
        u0 = xb[:, :NTR * K]
        c_true = torch.clamp(torch.exp(u0 + yb) - c0, min=0.0)
        c_pred = torch.clamp(torch.exp(u0 + pred * sdd + md) - c0, min=0.0)
        e = (c_pred - c_true).abs() / torch.maximum(c_true.abs(), floor)
        errs.append(e.amax(dim=1).cpu())
        per_tr.append(e.view(-1, NTR, K).amax(dim=2).cpu())
    err = torch.cat(errs).numpy()
    per = torch.cat(per_tr).numpy()
    return {"rows": int(m), "mse_standardised": mse / max(m * sur.nout, 1),
            "row_max_rel_err_quantiles": {q: float(np.percentile(err, q)) for q in (10, 50, 90)},
            "rows_within": {t: float(np.mean(err <= t)) for t in (1e-3, 1e-2, 1e-1)},
            "per_tracer_median_row_max": [float(v) for v in np.median(per, axis=0)]}


def train_surrogate(train_cs: ColumnSet, test_cs: Optional[ColumnSet], nsteps: int,
                    every: int, train_steps: int, batch: int = 8192, warm: int = 24,
                    lr: float = 1e-3, seed: int = 7, log_every: int = 1000,
                    test_nsteps: Optional[int] = None) -> Tuple[Surrogate, dict]:
    """Collect rows on ``train_cs``, fit the normalisation, train a network
    and, with ``test_cs``, measure it on held-out columns.  Returns the
    surrogate and a report."""
    import torch
    t0 = time.perf_counter()
    rows = collect_rows(train_cs, nsteps, every, warm=warm)
    t_rows = time.perf_counter() - t0
    nz = fit_normalizer(rows)
    X, Y = standardised(rows, nz)
    nrows = rows.x.shape[0]
    full = rows.full
    del rows
    torch.cuda.empty_cache()
    sur = Surrogate(train_cs.kmax, batch=batch, seed=seed)
    sur.set_norm(nz)
    t1 = time.perf_counter()
    log = sur.train(X, Y, steps=train_steps, lr=lr, log_every=log_every)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    del X, Y
    torch.cuda.empty_cache()
    report = {"train_columns": train_cs.n_active, "simulated_steps": nsteps,
              "collected_every": every, "rows": int(nrows), "rows_full": bool(full),
              "train_steps": train_steps, "batch": batch,
              "loss_log": [(int(i), round(l, 5)) for i, l, _ in log],
              "seconds_rows": round(t_rows, 2), "seconds_train": round(t_train, 2)}
    if test_cs is not None:
        test = collect_rows(test_cs, test_nsteps or nsteps, every, warm=warm, c0=nz.c0)
        report["held_out"] = evaluate(sur, test)
        report["held_out"]["columns"] = test_cs.n_active
        del test
        torch.cuda.empty_cache()
    return sur, report


def step_surrogate(solver: capi.Solver, sur: Surrogate, nsteps: int = 1,
                   tol: float = 1e-3, res_atol: float = 1e-2,
                   dt: Optional[float] = None) -> dict:
    """nsteps coupling steps of solver's device state with the surrogate and
    per-column fallback (sed_step_surrogate)."""
    st = capi.SedStats()
    dt = solver.cs.dt if dt is None else dt
    rc = solver.lib.sed_step_surrogate(solver.h, sur.h, float(dt), int(nsteps), float(tol),
                                       float(res_atol), ctypes.byref(st))
    solver._check(rc, "sed_step_surrogate")
    return st.as_dict()


def ode_solver_surrogate(solver: capi.Solver, sur: Surrogate, conc: np.ndarray,
                         bdys: np.ndarray, fluxes: np.ndarray, tol: float = 1e-3,
                         res_atol: float = 1e-2, dt: Optional[float] = None) -> dict:
    """The drop-in call with the surrogate (sed_ode_solver_surrogate): conc
    [ntr][kmax][ncol] FP64 in place, bdys in, fluxes in and out; copies
    pipelined over the column segments."""
    for a in (conc, fluxes):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    bdys = np.ascontiguousarray(bdys, dtype=np.float64)
    st = capi.SedStats()
    dt = solver.cs.dt if dt is None else dt
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = solver.lib.sed_ode_solver_surrogate(solver.h, sur.h, p(conc), p(bdys), p(fluxes),
                                             float(dt), float(tol), float(res_atol),
                                             ctypes.byref(st))
    solver._check(rc, "sed_ode_solver_surrogate")
    return st.as_dict()
