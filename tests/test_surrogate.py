"""Surrogate MLP kernels: the FP64 reference is checked by finite
differences on the CPU; the GPU forward pass and gradients (BF16 tensor-core
products, FP32 accumulation) are checked against it; training reduces the
loss."""
import ctypes

import numpy as np
import pytest

import mlp_oracle as M

SHAPE = dict(nin=343, nout=330, hidden=256, nhidden=4)


def test_reference_mlp_finite_differences():
    rng = np.random.default_rng(0)
    shapes = M.layer_shapes(7, 5, 6, 2)
    n = sum(r * c + r for r, c in shapes)
    p = rng.normal(0, 0.5, n)
    x = rng.normal(0, 1, (9, 7))
    y = rng.normal(0, 1, (9, 5))
    loss, g = M.loss_and_grads(p, shapes, x, y)
    h = 1e-6
    for i in rng.choice(n, 25, replace=False):
        q = p.copy()
        q[i] += h
        lp, _ = M.loss_and_grads(q, shapes, x, y)
        q[i] -= 2 * h
        lm, _ = M.loss_and_grads(q, shapes, x, y)
        assert abs((lp - lm) / (2 * h) - g[i]) < 1e-6 * max(1.0, abs(g[i]))


def test_bf16_rounding_matches_definition():
    v = np.array([1.0, 1.00390625, 1.01171875, 1.001953125, 3.14159],
                 dtype=np.float32)
    r = M.bf16_round(v)
    # 1 + 2^-8 and 1 + 3 2^-8 are ties: to the even significand
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625 and r[3] == 1.0
    assert r[4] == 3.140625


def test_flat_checkpoint_round_trip(tmp_path):
    """The flat checkpoint a Fortran host reads with stream access: nine
    little-endian int64 (magic, K, nin, nout, hidden, nhidden, state and
    normalisation lengths, Adam step), the FP32 state, the FP32
    normalisation; read back unchanged, and refused when cut short or
    described for another network."""
    from sedgpu import surrogate as S
    K = 30
    nin, nout = 11 * K + 13, 11 * K
    rng = np.random.default_rng(4)
    ck = {"state": rng.normal(0, 1, 1000).astype(np.float32), "step": 50000,
          "norm": rng.normal(0, 1, 11 + 2 * nin + 2 * nout).astype(np.float32), "K": K}
    path = str(tmp_path / "sur.raw")
    S.write_raw(path, ck)
    raw = open(path, "rb").read()
    hdr = np.frombuffer(raw[:72], dtype="<i8")
    assert hdr.tolist() == [S.RAW_MAGIC, K, nin, nout, 256, 4, 1000, ck["norm"].size, 50000]
    assert len(raw) == 72 + 4 * (1000 + ck["norm"].size)
    assert np.array_equal(np.frombuffer(raw[72:72 + 4000], dtype="<f4"), ck["state"])
    back = S.read_raw(path)
    assert back["K"] == K and back["step"] == 50000
    assert np.array_equal(back["state"], ck["state"])
    assert np.array_equal(back["norm"], ck["norm"])
    open(path, "wb").write(raw[:-4])
    with pytest.raises(ValueError):
        S.read_raw(path)
    bad = bytearray(raw)
    bad[8:16] = np.array([K + 1], dtype="<i8").tobytes()
    open(path, "wb").write(bytes(bad))
    with pytest.raises(ValueError):
        S.read_raw(path)
    with pytest.raises(ValueError):
        S.write_raw(path, dict(ck, K=K + 1))


def _sur(nin, nout, hidden, nhidden, batch, seed=3):
    from sedgpu import capi
    lib = capi.load()
    h = capi._H()
    rc = lib.sed_sur_create(nin, nout, hidden, nhidden, batch, seed, 0, ctypes.byref(h))
    assert rc == 0, rc
    return lib, h


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


@pytest.mark.gpu
@pytest.mark.parametrize("tc", [True, False], ids=["tcgen05", "mma_sync"])
def test_gpu_forward_and_gradients_match_fp64_reference(tc):
    """Forward pass and gradients of both engines: the tcgen05 GEMMs (TMA
    operands, TMEM accumulators, the weight gradient split over K) and the
    mma.sync GEMMs.  Against the FP64 MLP on the BF16-rounded operands the
    bar is the BF16 storage of activations and gradients (5e-2); against the
    FP64 MLP that also rounds those stores to BF16 it is the FP32
    accumulation (1e-3 forward, 3e-3 per gradient block)."""
    lib, h = _sur(**SHAPE, batch=256)
    try:
        lib.sed_sur_set_tensor_cores(h, 1 if tc else 0)
        shapes = M.layer_shapes(**SHAPE)
        n = lib.sed_sur_num_params(h)
        assert n == sum(r * c + r for r, c in shapes)
        rng = np.random.default_rng(1)
        params = rng.normal(0, 1, n).astype(np.float32)
        o = 0
        for r, c in shapes:   # scale so activations stay O(1)
            params[o:o + r * c] *= 1.0 / np.sqrt(c)
            o += r * c + r
        assert lib.sed_sur_set_weights(h, _fp(params)) == 0
        m = 200  # not a multiple of 128: padded rows must not count
        x = rng.normal(0, 1, (m, SHAPE["nin"])).astype(np.float32)
        y = (0.3 * rng.normal(0, 1, (m, SHAPE["nout"]))).astype(np.float32)
        # reference with the BF16 rounding of the GPU operands
        pb = params.astype(np.float64).copy()
        o = 0
        for r, c in shapes:
            pb[o:o + r * c] = M.bf16_round(params[o:o + r * c])
            o += r * c + r
        xb = M.bf16_round(x)
        yb = M.bf16_round(y)
        yref, _, _ = M.forward(pb, shapes, xb)
        yemu, _, _ = M.forward(pb, shapes, xb, bf16=True)
        yg = np.zeros((m, SHAPE["nout"]), dtype=np.float32)
        assert lib.sed_sur_forward(h, _fp(x), _fp(yg), m) == 0
        rel = np.linalg.norm(yg - yref) / np.linalg.norm(yref)
        assert rel < 1e-2, rel
        # with the activations rounded to BF16 where the GPU stores them the
        # reference leaves only the FP32 accumulation: far closer
        rel_e = np.linalg.norm(yg - yemu) / np.linalg.norm(yemu)
        assert rel_e < 1e-3, rel_e   # measured 1.8e-4 on GB300
        lref, gref = M.loss_and_grads(pb, shapes, xb, yb)
        _, gemu = M.loss_and_grads(pb, shapes, xb, yb, bf16=True)
        g = np.zeros(n, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        assert lib.sed_sur_grads(h, _fp(x), _fp(y), m, _fp(g), _fp(loss)) == 0
        assert abs(loss[0] - lref) < 2e-2 * lref
        o = 0
        worst = 0.0
        for r, c in shapes:
            for blk in (slice(o, o + r * c), slice(o + r * c, o + r * c + r)):
                a, b = g[blk].astype(np.float64), gref[blk]
                relg = np.linalg.norm(a - b) / np.linalg.norm(b)
                cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
                assert relg < 5e-2 and cos > 0.998, (relg, cos)
                # against the BF16-storage emulation
                e = gemu[blk]
                rel_g = np.linalg.norm(a - e) / np.linalg.norm(e)
                worst = max(worst, rel_g)
                # measured: at most 8.9e-4 over the blocks, both engines
                assert rel_g < 3e-3 and a @ e / (np.linalg.norm(a) * np.linalg.norm(e)) > 0.99999, \
                    rel_g
            o += r * c + r
        print(f"forward vs emulation {rel_e:.2e}, worst gradient block {worst:.2e}")
    finally:
        lib.sed_sur_destroy(h)


@pytest.mark.gpu
@pytest.mark.parametrize("tc", [True, False], ids=["tcgen05", "mma_sync"])
def test_gpu_training_reduces_loss(tc):
    import torch
    lib, h = _sur(**SHAPE, batch=1024)
    try:
        lib.sed_sur_set_tensor_cores(h, 1 if tc else 0)
        rng = np.random.default_rng(2)
        m = 1024
        A = rng.normal(0, 1 / np.sqrt(SHAPE["nin"]), (SHAPE["nin"], SHAPE["nout"]))
        x = rng.normal(0, 1, (m, SHAPE["nin"]))
        y = np.tanh(x @ A)
        xp = np.zeros((m, 384), dtype=np.float32)
        yp = np.zeros((m, 384), dtype=np.float32)
        xp[:, :SHAPE["nin"]] = x
        yp[:, :SHAPE["nout"]] = y
        xd = torch.tensor(xp, device="cuda").to(torch.bfloat16).contiguous()
        yd = torch.tensor(yp, device="cuda").to(torch.bfloat16).contiguous()
        torch.cuda.synchronize()
        loss = np.zeros(1, dtype=np.float32)
        losses = []
        for it in range(300):
            rc = lib.sed_sur_train_step(h, ctypes.c_void_p(xd.data_ptr()),
                                        ctypes.c_void_p(yd.data_ptr()), m, 1e-3,
                                        _fp(loss) if it % 50 == 0 or it == 299 else None)
            assert rc == 0, lib.sed_sur_last_error(h)
            if it % 50 == 0 or it == 299:
                losses.append(float(loss[0]))
        assert losses[-1] < 0.33 * losses[0], losses
    finally:
        lib.sed_sur_destroy(h)


def _device_forward(lib, h, x, tc):
    """sed_sur_forward_device on BF16 rows of x with the fused tcgen05
    kernel (tc) or the mma.sync GEMMs; returns the FP32 outputs."""
    import torch
    m = x.shape[0]
    xp = np.zeros((m, 384), dtype=np.float32)
    xp[:, :x.shape[1]] = x
    xd = torch.tensor(xp, device="cuda").to(torch.bfloat16).contiguous()
    yd = torch.zeros((m, 384), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert lib.sed_sur_set_tensor_cores(h, 1 if tc else 0) == (1 if tc else 0)
    rc = lib.sed_sur_forward_device(h, ctypes.c_void_p(xd.data_ptr()),
                                    ctypes.c_void_p(yd.data_ptr()), m)
    assert rc == 0, lib.sed_sur_last_error(h)
    return yd[:, :SHAPE["nout"]].cpu().numpy().astype(np.float64)


@pytest.mark.gpu
def test_tensor_core_inference_matches_fp64_reference():
    """The fused tcgen05 inference kernel (TMEM accumulators, TMA-staged
    operands) against the FP64 MLP on the same BF16-rounded operands, at the
    bar of the GEMM path above; and against the GEMM path on a batch of 400
    tiles of 128 rows, so that every CTA of the persistent grid walks
    several tiles through its barrier phases."""
    lib, h = _sur(**SHAPE, batch=256, seed=5)
    try:
        shapes = M.layer_shapes(**SHAPE)
        n = lib.sed_sur_num_params(h)
        rng = np.random.default_rng(3)
        params = rng.normal(0, 1, n).astype(np.float32)
        o = 0
        for r, c in shapes:
            params[o:o + r * c] *= 1.0 / np.sqrt(c)
            params[o + r * c:o + r * c + r] *= 0.1
            o += r * c + r
        assert lib.sed_sur_set_weights(h, _fp(params)) == 0
        pb = params.astype(np.float64).copy()
        o = 0
        for r, c in shapes:
            pb[o:o + r * c] = M.bf16_round(params[o:o + r * c])
            o += r * c + r
        x = rng.normal(0, 1, (256, SHAPE["nin"])).astype(np.float32)
        yref, _, _ = M.forward(pb, shapes, M.bf16_round(x))
        for tc in (True, False):
            yg = _device_forward(lib, h, x, tc)
            rel = np.linalg.norm(yg - yref) / np.linalg.norm(yref)
            assert rel < 1e-2, (tc, rel)
        xl = rng.normal(0, 1, (128 * 400, SHAPE["nin"])).astype(np.float32)
        a = _device_forward(lib, h, xl, True)
        b = _device_forward(lib, h, xl, False)
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel < 1e-2, rel
        # row by row: no tile is missing or misplaced
        rrow = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
        assert rrow.max() < 5e-2, rrow.max()
    finally:
        lib.sed_sur_destroy(h)


@pytest.mark.gpu
def test_tensor_core_inference_output_alignment():
    """The fused kernel writes 32-byte row pieces when the output rows start
    on 32-byte boundaries and 16-byte pieces when they start on 16-byte ones:
    the same values either way.  An output or input that is not 16-byte
    aligned is refused before any launch."""
    import torch
    lib, h = _sur(**SHAPE, batch=256, seed=5)
    try:
        m = 256
        rng = np.random.default_rng(11)
        n = lib.sed_sur_num_params(h)
        params = (rng.normal(0, 1, n) * 0.05).astype(np.float32)
        assert lib.sed_sur_set_weights(h, _fp(params)) == 0
        assert lib.sed_sur_set_tensor_cores(h, 1) == 1
        xp = np.zeros((m, 384), dtype=np.float32)
        xp[:, :SHAPE["nin"]] = rng.normal(0, 1, (m, SHAPE["nin"]))
        xd = torch.tensor(xp, device="cuda").to(torch.bfloat16).contiguous()
        # one buffer, the rows placed at byte offsets 0 (32-byte pieces),
        # 16 (16-byte pieces) and 4 (refused)
        buf = torch.zeros(m * 384 + 8, dtype=torch.float32, device="cuda")
        base = buf.data_ptr()
        assert base % 32 == 0
        out = {}
        for off in (0, 4):
            buf.zero_()
            torch.cuda.synchronize()
            rc = lib.sed_sur_forward_device(h, ctypes.c_void_p(xd.data_ptr()),
                                            ctypes.c_void_p(base + 4 * off), m)
            assert rc == 0, lib.sed_sur_last_error(h)
            torch.cuda.synchronize()
            out[off] = buf[off:off + m * 384].reshape(m, 384).cpu().numpy().copy()
        assert np.array_equal(out[0], out[4])
        assert np.abs(out[0][:, :SHAPE["nout"]]).max() > 0
        assert lib.sed_sur_forward_device(h, ctypes.c_void_p(xd.data_ptr()),
                                          ctypes.c_void_p(base + 4), m) == -1
        assert lib.sed_sur_forward_device(h, ctypes.c_void_p(xd.data_ptr() + 2),
                                          ctypes.c_void_p(base), m) == -1
    finally:
        lib.sed_sur_destroy(h)


@pytest.mark.gpu
def test_tcgen05_training_products_match_mma_sync_at_full_batch():
    """At the training batch (8192 rows) the weight gradients' K is split
    over the SMs and added in a fixed order: the gradients of the two
    engines agree, and the tcgen05 ones repeat bit for bit."""
    lib, h = _sur(**SHAPE, batch=8192, seed=7)
    try:
        shapes = M.layer_shapes(**SHAPE)
        n = lib.sed_sur_num_params(h)
        rng = np.random.default_rng(4)
        m = 8192
        x = rng.normal(0, 1, (m, SHAPE["nin"])).astype(np.float32)
        y = (0.3 * rng.normal(0, 1, (m, SHAPE["nout"]))).astype(np.float32)
        out = {}
        for tc in (True, False, True):
            lib.sed_sur_set_tensor_cores(h, 1 if tc else 0)
            g = np.zeros(n, dtype=np.float32)
            loss = np.zeros(1, dtype=np.float32)
            assert lib.sed_sur_grads(h, _fp(x), _fp(y), m, _fp(g), _fp(loss)) == 0, \
                lib.sed_sur_last_error(h)
            if tc and tc in out:
                np.testing.assert_array_equal(g, out[tc])
            out[tc] = g
        o = 0
        for r, c in shapes:
            for blk in (slice(o, o + r * c), slice(o + r * c, o + r * c + r)):
                a, b = out[True][blk].astype(np.float64), out[False][blk].astype(np.float64)
                relg = np.linalg.norm(a - b) / np.linalg.norm(b)
                cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
                assert relg < 2e-2 and cos > 0.9995, (relg, cos)
            o += r * c + r
    finally:
        lib.sed_sur_destroy(h)


@pytest.mark.gpu
def test_adam_step_matches_the_update_formula():
    """One sed_sur_train_step from known weights equals Adam's first update
    (m = (1-b1) g, v = (1-b2) g^2, bias-corrected: w - lr g / (|g| + eps))
    applied in numpy to the gradients sed_sur_grads gives on the same batch,
    for the FP32 master weights and biases."""
    import torch
    shapes = M.layer_shapes(**SHAPE)
    m, lr, eps = 256, 1e-3, 1e-8
    rng = np.random.default_rng(6)
    x = rng.normal(0, 1, (m, SHAPE["nin"])).astype(np.float32)
    y = (0.3 * rng.normal(0, 1, (m, SHAPE["nout"]))).astype(np.float32)
    lib, h = _sur(**SHAPE, batch=m, seed=9)
    try:
        n = lib.sed_sur_num_params(h)
        w0 = np.zeros(n, dtype=np.float32)
        assert lib.sed_sur_get_weights(h, _fp(w0)) == 0
        g = np.zeros(n, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        assert lib.sed_sur_grads(h, _fp(x), _fp(y), m, _fp(g), _fp(loss)) == 0
        xp = np.zeros((m, 384), dtype=np.float32)
        yp = np.zeros((m, 384), dtype=np.float32)
        xp[:, :SHAPE["nin"]] = x
        yp[:, :SHAPE["nout"]] = y
        xd = torch.tensor(xp, device="cuda").to(torch.bfloat16).contiguous()
        yd = torch.tensor(yp, device="cuda").to(torch.bfloat16).contiguous()
        torch.cuda.synchronize()
        rc = lib.sed_sur_train_step(h, ctypes.c_void_p(xd.data_ptr()),
                                    ctypes.c_void_p(yd.data_ptr()), m, lr, _fp(loss))
        assert rc == 0, lib.sed_sur_last_error(h)
        w1 = np.zeros(n, dtype=np.float32)
        assert lib.sed_sur_get_weights(h, _fp(w1)) == 0
    finally:
        lib.sed_sur_destroy(h)
    g64 = g.astype(np.float64)
    mhat = (1 - 0.9) * g64 / (1 - 0.9)
    vhat = (1 - 0.999) * g64 * g64 / (1 - 0.999)
    expect = w0.astype(np.float64) - lr * mhat / (np.sqrt(vhat) + eps)
    step = w1.astype(np.float64) - w0
    # the same gradients (deterministic products) give the same step; the
    # FP32 arithmetic of the update rounds to within a few ulp of w
    assert np.abs(w1 - expect).max() <= 4 * np.spacing(np.abs(w0).max() + lr), \
        np.abs(w1 - expect).max()
    # Adam's first step moves every parameter with a nonzero gradient by lr
    nz = np.abs(g64) > 1e-6
    assert np.allclose(np.abs(step[nz]), lr, rtol=1e-2), np.abs(step[nz]).min()
