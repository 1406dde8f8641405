"""Column-increment surrogate: data, normalisation, training and use.

The network (nin = 11 K + 13 -> 256 x 4, GELU -> nout = 11 K) maps a
column's state and its 13 forcing rows to the change of log(C + c0) over one
coupling step.  It is trained on (state, next state) pairs that the plain
GPU solver generates, by the library's own BF16 tensor-core forward /
backward / Adam kernels (sed_sur_*).  In use (sed_step_surrogate) every
column's proposal is checked with the plain right-hand side and rejected
columns are advanced by the plain solver.

torch is used only as device storage for the training set and for random
batching; all arithmetic of the network runs in the library.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import time
from typing import Dict, Optional, Tuple

import numpy as np

from . import capi, synth
from .model import NTR, ColumnSet

NFORCE = 13
HIDDEN, NHIDDEN = 256, 4


def pad128(n: int) -> int:
    return (n + 127) // 128 * 128


def forcing_rows(cs: ColumnSet) -> np.ndarray:
    """The 13 per-column forcing rows the solver forms for a coupling step
    (bioturbation x f_T, molecular multiplier, 11 surface values)."""
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


def log_state(conc: np.ndarray, c0: np.ndarray) -> np.ndarray:
    """[ntr][K][cols] -> [cols][ntr*K] of log(C + c0)."""
    ntr, K, n = conc.shape
    u = np.log(np.maximum(conc, 0.0) + c0[:, None, None])
    return u.reshape(ntr * K, n).T


def generate_pairs(cs: ColumnSet, nsteps: int, samples: int, warm: int = 24,
                   seed: int = 0) -> Dict[str, np.ndarray]:
    """Run the plain FP32 GPU solver on ``cs`` for ``nsteps`` coupling steps
    and keep (state, next state) at ``samples`` step indices in
    [warm, nsteps)."""
    rng = np.random.default_rng(seed)
    pick = np.sort(rng.choice(np.arange(warm, nsteps), size=min(samples, nsteps - warm),
                              replace=False))
    s = capi.Solver(cs, precision=capi.SED_FP32)
    s.set_forcing()
    s.set_state(cs.conc)
    xs, ys = [], []
    t = 0
    for target in pick:
        if target > t:
            s.step(int(target - t))
            t = int(target)
        s0 = s.get_state().astype(np.float32)
        s.step(1)
        t += 1
        s1 = s.get_state().astype(np.float32)
        xs.append(s0)
        ys.append(s1)
    s.close()
    return {"x": np.stack(xs), "y": np.stack(ys), "force": forcing_rows(cs),
            "steps": pick}


def fit_normalizer(pairs: Dict[str, np.ndarray], K: int) -> Normalizer:
    x, y = pairs["x"].astype(np.float64), pairs["y"].astype(np.float64)
    # log offset: a small fraction of each tracer's typical magnitude
    med = np.array([np.median(np.abs(x[:, n])) for n in range(NTR)])
    c0 = np.maximum(1e-3 * med, 1e-6)
    u0 = np.concatenate([log_state(xi, c0) for xi in x])
    u1 = np.concatenate([log_state(yi, c0) for yi in y])
    f = np.tile(pairs["force"].T, (x.shape[0], 1))
    feat = np.concatenate([u0, f], axis=1)
    mu_x = feat.mean(axis=0)
    sd_x = feat.std(axis=0)
    sd_x[sd_x < 1e-8 * (np.abs(mu_x) + 1.0)] = 1.0
    d = u1 - u0
    mu_d = d.mean(axis=0)
    sd_d = d.std(axis=0)
    sd_d[sd_d < 1e-12] = 1e-12
    return Normalizer(c0, mu_x, sd_x, mu_d, sd_d)


def training_arrays(pairs: Dict[str, np.ndarray], nz: Normalizer
                    ) -> Tuple[np.ndarray, np.ndarray]:
    x, y = pairs["x"].astype(np.float64), pairs["y"].astype(np.float64)
    u0 = np.concatenate([log_state(xi, nz.c0) for xi in x])
    u1 = np.concatenate([log_state(yi, nz.c0) for yi in y])
    f = np.tile(pairs["force"].T, (x.shape[0], 1))
    X = (np.concatenate([u0, f], axis=1) - nz.mu_x) / nz.sd_x
    Y = ((u1 - u0) - nz.mu_d) / nz.sd_d
    return X.astype(np.float32), Y.astype(np.float32)


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

    def save(self, path: str):
        np.savez_compressed(path, weights=self.weights(), norm=self.norm.pack(), K=self.K)

    @staticmethod
    def load(path: str, batch: int = 8192) -> "Surrogate":
        d = np.load(path)
        s = Surrogate(int(d["K"]), batch=batch)
        s.set_weights(d["weights"])
        s.set_norm(Normalizer.unpack(d["norm"], int(d["K"])))
        return s

    def train(self, X: np.ndarray, Y: np.ndarray, steps: int, lr: float = 1e-3,
              lr_final: float = 2e-5, log_every: int = 1000, seed: int = 0):
        """Adam on random batches of (X, Y) held on the device (cosine decay
        of the learning rate).  Returns the logged losses."""
        import torch
        n = X.shape[0]
        Xp = np.zeros((n, self.pin), dtype=np.float32)
        Yp = np.zeros((n, self.pout), dtype=np.float32)
        Xp[:, :self.nin] = X
        Yp[:, :self.nout] = Y
        xd = torch.from_numpy(Xp).to("cuda").to(torch.bfloat16)
        yd = torch.from_numpy(Yp).to("cuda").to(torch.bfloat16)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        loss = np.zeros(1, dtype=np.float32)
        lp = loss.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        log = []
        m = self.batch
        t0 = time.perf_counter()
        for it in range(steps):
            idx = torch.randint(0, n, (m,), device="cuda", generator=gen)
            xb = xd.index_select(0, idx)
            yb = yd.index_select(0, idx)
            torch.cuda.current_stream().synchronize()
            frac = it / max(steps - 1, 1)
            lr_t = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * frac))
            want = (it % log_every == 0) or it == steps - 1
            self._check(self.lib.sed_sur_train_step(
                self.h, ctypes.c_void_p(xb.data_ptr()), ctypes.c_void_p(yb.data_ptr()), m,
                float(lr_t), lp if want else None), "train step")
            if want:
                log.append((it, float(loss[0]), time.perf_counter() - t0))
        return log

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.nout), dtype=np.float32)
        self._check(self.lib.sed_sur_forward(
            self.h, X.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
            Y.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), X.shape[0]), "forward")
        return Y

    def next_state(self, conc: np.ndarray, force: np.ndarray) -> np.ndarray:
        """Proposed state after one coupling step, [ntr][K][cols]."""
        nz = self.norm
        u0 = log_state(conc, nz.c0)
        X = (np.concatenate([u0, force.T], axis=1) - nz.mu_x) / nz.sd_x
        d = self.predict(X).astype(np.float64) * nz.sd_d + nz.mu_d
        u1 = u0 + d
        ntr, K, n = conc.shape
        out = np.exp(u1.T.reshape(ntr, K, n)) - nz.c0[:, None, None]
        return np.maximum(out, 0.0)


def step_surrogate(solver: capi.Solver, sur: Surrogate, nsteps: int = 1,
                   tol: float = 1e-3, res_atol: float = 1e-6,
                   dt: Optional[float] = None) -> dict:
    """nsteps coupling steps of solver's device state with the surrogate and
    per-column fallback (sed_step_surrogate)."""
    st = capi.SedStats()
    dt = solver.cs.dt if dt is None else dt
    rc = solver.lib.sed_step_surrogate(solver.h, sur.h, float(dt), int(nsteps), float(tol),
                                       float(res_atol), ctypes.byref(st))
    solver._check(rc, "sed_step_surrogate")
    return st.as_dict()
