"""Checkpoint and resume.

The reference's component restarts from `<var>_in_soil` fields of a restart
file (src/components/fabm_sediment_component.F90:1328-1489): the state is all
a sediment run carries from one coupling step to the next.  A run split at
step n -- the state read out with sed_get_state, written into a new handle
with sed_set_state -- must equal the uninterrupted run bit for bit, in FP32
and FP64.  The surrogate's training state (parameters, Adam moments and
step count, sed_sur_get_state / sed_sur_set_state) must resume the same
way: training continued from a checkpoint, in a new handle, on the same
batches, gives the same parameters bit for bit."""
import ctypes

import numpy as np
import pytest

from sedgpu import capi, synth
from sedgpu import surrogate as S

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [capi.SED_FP32, capi.SED_FP64])
def test_split_run_equals_uninterrupted(precision):
    cs = synth.make_workload("uneven_1024x1024", cols=np.arange(0, 1024 * 1024, 2048))
    n1, n2 = 30, 18

    def solver():
        s = capi.Solver(cs, precision=precision)
        s.set_forcing()
        return s

    a = solver()
    a.set_state(cs.conc)
    a.step(n1 + n2)
    whole = a.get_state()
    fl_whole = a.fluxes()
    a.close()
    b = solver()
    b.set_state(cs.conc)
    b.step(n1)
    checkpoint = b.get_state()
    b.close()
    c = solver()
    c.set_state(checkpoint)
    c.step(n2)
    resumed = c.get_state()
    fl_resumed = c.fluxes()
    c.close()
    np.testing.assert_array_equal(resumed, whole)
    np.testing.assert_array_equal(fl_resumed, fl_whole)


def test_training_resumes_bit_for_bit():
    import torch
    K, m = 30, 1024
    nin, nout = 11 * K + 13, 11 * K
    rng = np.random.default_rng(5)
    A = rng.normal(0, 1 / np.sqrt(nin), (nin, nout))
    x = rng.normal(0, 1, (8 * m, nin))
    y = np.tanh(x @ A)
    xp = np.zeros((8 * m, 384), dtype=np.float32)
    yp = np.zeros((8 * m, 384), dtype=np.float32)
    xp[:, :nin] = x
    yp[:, :nout] = y
    X = torch.tensor(xp, device="cuda").to(torch.bfloat16)
    Y = torch.tensor(yp, device="cuda").to(torch.bfloat16)
    batches = [torch.tensor(rng.choice(8 * m, m, replace=False), device="cuda")
               for _ in range(60)]

    def train(sur, bs):
        for idx in bs:
            xb = X.index_select(0, idx).contiguous()
            yb = Y.index_select(0, idx).contiguous()
            torch.cuda.synchronize()
            rc = sur.lib.sed_sur_train_step(sur.h, ctypes.c_void_p(xb.data_ptr()),
                                            ctypes.c_void_p(yb.data_ptr()), m, 1e-3, None)
            assert rc == 0, sur.lib.sed_sur_last_error(sur.h)
            # the step runs on the library's stream: keep the batch until it is read
            torch.cuda.synchronize()

    a = S.Surrogate(K, batch=m, seed=3)
    train(a, batches)
    whole = a.weights()
    a.close()
    b = S.Surrogate(K, batch=m, seed=3)
    train(b, batches[:25])
    ck = b.checkpoint()
    b.close()
    assert ck["step"] == 25
    c = S.Surrogate(K, batch=m, seed=99)   # other initial weights: all restored
    c.restore(ck)
    train(c, batches[25:])
    resumed = c.weights()
    ck2 = c.checkpoint()
    c.close()
    assert ck2["step"] == 60
    np.testing.assert_array_equal(resumed, whole)
