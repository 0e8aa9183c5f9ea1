"""The tensor-core MLP kernels (sph_mlp_*) through the C ABI against the
NumPy oracle (oracle/mlp.py), which rounds to BF16 at the same places.

Tolerances: outputs within 1e-2 of the output scale; each gradient block
(W1, b1, W2, b2, W3, b3) within GRAD_RTOL relative in the 2-norm; the loss
within 1e-3 relative.  The residual differences come from tanh (the hardware
approximation, accurate to about 2^-11, vs double) occasionally flipping a
BF16 rounding, and from FP32 accumulation order.
"""
import ctypes

import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu

# Measured: each gradient block within 7.1e-4 of the oracle at 64 samples,
# 4e-5 at 50,000 (both passes); the two passes within 7.2e-7 of each other.
GRAD_RTOL = 2e-3          # each gradient block against the oracle (2-norm, relative)
GRAD_TC_MMA_RTOL = 1e-5   # tcgen05 pass against the mma.sync pass


def _lib():
    from pibiti_gb300 import _lib
    return _lib, _lib.lib()


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _pack(torch, params):
    _l, L = _lib()
    prm = torch.from_numpy(np.asarray(params, np.float32)).cuda()
    img = torch.zeros(L.sph_mlp_packed_bytes(), dtype=torch.uint8, device="cuda")
    _l.check(L.sph_mlp_pack(_p(prm), _p(img), None))
    return prm, img


def _x(torch, x):
    return torch.from_numpy(omlp.bf16_bits(x).view(np.int16).copy()).cuda()


def test_sizes(cuda):
    _l, L = _lib()
    assert L.sph_mlp_param_count() == omlp.COUNT == 5443


@pytest.mark.parametrize("n", [1, 37, 4096, 100_003])
def test_forward(cuda, n):
    torch = cuda
    _l, L = _lib()
    rng = np.random.default_rng(n)
    params = omlp.init(3)
    params[1024:1088] = rng.normal(0, 0.1, 64)  # nonzero biases
    x = rng.normal(0, 1, size=(n, 16)).astype(np.float32)
    _, img = _pack(torch, params)
    y = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    _l.check(L.sph_mlp_forward(_p(img), _p(_x(torch, x)), n, _p(y), None))
    torch.cuda.synchronize()
    ref, _ = omlp.forward(params, x)
    scale = max(np.abs(ref).max(), 1e-3)
    np.testing.assert_allclose(y.cpu().numpy(), ref, rtol=0, atol=1e-2 * scale)


@pytest.mark.parametrize("n", [1, 37, 128, 4096, 100_003])
def test_forward_tc(cuda, n):
    """The tcgen05 forward pass: against the oracle with the same bound as
    the mma.sync pass, and bit-identical to the mma.sync pass (both seed the
    accumulators with the bias, add the K = 16 products in the same order and
    round to BF16 at the same places)."""
    torch = cuda
    _l, L = _lib()
    rng = np.random.default_rng(100 + n)
    params = omlp.init(4)
    params[1024:1088] = rng.normal(0, 0.1, 64)
    params[1088 + 4096:1088 + 4096 + 64] = rng.normal(0, 0.1, 64)
    params[5440:5443] = rng.normal(0, 0.1, 3)
    x = rng.normal(0, 1, size=(n, 16)).astype(np.float32)
    _, img = _pack(torch, params)
    xd = _x(torch, x)
    y_tc = torch.full((n, 3), float("nan"), dtype=torch.float32, device="cuda")
    y_mma = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    _l.check(L.sph_mlp_forward_tc(_p(img), _p(xd), n, _p(y_tc), None))
    _l.check(L.sph_mlp_forward(_p(img), _p(xd), n, _p(y_mma), None))
    status = ctypes.c_uint32(7)
    _l.check(L.sph_mlp_status(ctypes.byref(status)))
    assert status.value == 0
    ref, _ = omlp.forward(params, x)
    scale = max(np.abs(ref).max(), 1e-3)
    a, b = y_tc.cpu().numpy(), y_mma.cpu().numpy()
    np.testing.assert_allclose(a, ref, rtol=0, atol=1e-2 * scale)
    np.testing.assert_array_equal(a, b)


def test_forward_tc_timeout_path(cuda):
    """A pass whose tensor-core work is withheld (test hook): every thread
    block's wait runs out; its rows become NaN, the status word reports it
    once, and the next pass runs normally (the tensor memory was freed)."""
    torch = cuda
    _l, L = _lib()
    n = 100_003
    rng = np.random.default_rng(3)
    _, img = _pack(torch, omlp.init(2))
    xd = _x(torch, rng.normal(0, 1, size=(n, 16)).astype(np.float32))
    y = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    _l.check(L.sph_mlp_forward_tc_withheld(_p(img), _p(xd), n, _p(y), None))
    status = ctypes.c_uint32(0)
    _l.check(L.sph_mlp_status(ctypes.byref(status)))
    assert status.value == 1
    assert bool(torch.isnan(y).all())
    _l.check(L.sph_mlp_status(ctypes.byref(status)))
    assert status.value == 0
    y_tc = torch.zeros_like(y)
    y_mma = torch.zeros_like(y)
    _l.check(L.sph_mlp_forward_tc(_p(img), _p(xd), n, _p(y_tc), None))
    _l.check(L.sph_mlp_forward(_p(img), _p(xd), n, _p(y_mma), None))
    _l.check(L.sph_mlp_status(ctypes.byref(status)))
    assert status.value == 0
    assert torch.equal(y_tc, y_mma)


def test_forward_tc_arguments(cuda):
    torch = cuda
    _l, L = _lib()
    _, img = _pack(torch, omlp.init(1))
    x = torch.zeros(64 * 16 + 8, dtype=torch.int16, device="cuda")
    y = torch.zeros((64, 3), dtype=torch.float32, device="cuda")
    misaligned = ctypes.c_void_p(x.data_ptr() + 2)
    assert L.sph_mlp_forward_tc(_p(img), misaligned, 64, _p(y), None) != 0
    assert L.sph_mlp_forward_tc(_p(img), _p(x), 0, _p(y), None) == 0


def _grad_case(torch, n):
    rng = np.random.default_rng(7 + n)
    params = omlp.init(5)
    params[1024:1088] = rng.normal(0, 0.1, 64)
    params[5440:5443] = rng.normal(0, 0.1, 3)
    x = rng.normal(0, 1, size=(n, 16)).astype(np.float32)
    t = rng.normal(0, 0.5, size=(n, 3)).astype(np.float32)
    return params, x, t


def _train(torch, entry, img, x, t):
    n = len(x)
    grad = torch.zeros(omlp.COUNT, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    _l, L = _lib()
    xd, td = _x(torch, x), torch.from_numpy(t).cuda()  # held until the pass has run
    _l.check(getattr(L, entry)(_p(img), _p(xd), _p(td), n, _p(grad), _p(loss), None))
    torch.cuda.synchronize()
    return grad.cpu().numpy().astype(np.float64), loss.item()


def _block_errors(g, ref_g):
    out, o = {}, 0
    for name, shape in omlp.SIZES:
        k = int(np.prod(shape))
        a, b = g[o:o + k], ref_g[o:o + k]
        out[name] = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        o += k
    return out


@pytest.mark.parametrize("entry", ["sph_mlp_train_pass", "sph_mlp_train_pass_tc"])
@pytest.mark.parametrize("n", [64, 1000, 50_000])
def test_gradients(cuda, n, entry):
    """Both training passes (mma.sync and tcgen05) against the oracle."""
    torch = cuda
    params, x, t = _grad_case(torch, n)
    _, img = _pack(torch, params)
    g, loss = _train(torch, entry, img, x, t)
    ref_loss, ref_g = omlp.loss_and_grad(params, x, t)
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss
    errs = _block_errors(g, ref_g)
    print(entry, n, {k: f"{v:.2e}" for k, v in errs.items()})
    for name, rel in errs.items():
        assert rel <= GRAD_RTOL, (name, rel)


@pytest.mark.parametrize("n", [64, 1000, 50_000, 262_144])
def test_gradients_tc_vs_mma(cuda, n):
    """The two training passes round to BF16 at the same places and differ
    only in the FP32 summation order of the products and sums."""
    torch = cuda
    params, x, t = _grad_case(torch, n)
    _, img = _pack(torch, params)
    g_tc, l_tc = _train(torch, "sph_mlp_train_pass_tc", img, x, t)
    g_mma, l_mma = _train(torch, "sph_mlp_train_pass", img, x, t)
    assert abs(l_tc - l_mma) <= 1e-5 * l_mma
    errs = _block_errors(g_tc, g_mma)
    print("tc vs mma.sync", n, {k: f"{v:.2e}" for k, v in errs.items()})
    for name, rel in errs.items():
        assert rel <= GRAD_TC_MMA_RTOL, (name, rel)
    status = ctypes.c_uint32(7)
    _l, L = _lib()
    _l.check(L.sph_mlp_status(ctypes.byref(status)))
    assert status.value == 0


def test_train_tc_timeout_path(cuda):
    """A training pass whose tensor-core work is withheld (test hook): the
    loss becomes NaN, no gradient is added, status bit 1 is set once, and the
    next pass runs normally (the tensor memory was freed)."""
    torch = cuda
    _l, L = _lib()
    params, x, t = _grad_case(torch, 5000)
    _, img = _pack(torch, params)
    g, loss = _train(torch, "sph_mlp_train_pass_tc_withheld", img, x, t)
    assert np.isnan(loss)
    assert not g.any()
    status = ctypes.c_uint32(0)
    _l.check(L.sph_mlp_status(ctypes.byref(status)))
    assert status.value == 2
    g_tc, l_tc = _train(torch, "sph_mlp_train_pass_tc", img, x, t)
    g_mma, l_mma = _train(torch, "sph_mlp_train_pass", img, x, t)
    _l.check(L.sph_mlp_status(ctypes.byref(status)))
    assert status.value == 0
    assert abs(l_tc - l_mma) <= 1e-5 * l_mma
    assert max(_block_errors(g_tc, g_mma).values()) <= GRAD_TC_MMA_RTOL


def test_train_tc_arguments(cuda):
    torch = cuda
    _l, L = _lib()
    _, img = _pack(torch, omlp.init(1))
    x = torch.zeros(64 * 16 + 8, dtype=torch.int16, device="cuda")
    t = torch.zeros((64, 3), dtype=torch.float32, device="cuda")
    grad = torch.zeros(omlp.COUNT, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    misaligned = ctypes.c_void_p(x.data_ptr() + 2)
    assert L.sph_mlp_train_pass_tc(_p(img), misaligned, _p(t), 64, _p(grad), _p(loss), None) != 0
    assert L.sph_mlp_train_pass_tc(_p(img), _p(x), _p(t), 0, _p(grad), _p(loss), None) == 0


@pytest.mark.parametrize("entry", ["sph_mlp_train_pass", "sph_mlp_train_pass_tc"])
def test_adam_fits(cuda, entry):
    """The kernels train: a smooth target is fitted, the loss falls 10x."""
    torch = cuda
    _l, L = _lib()
    rng = np.random.default_rng(0)
    n = 32768
    x = rng.normal(0, 1, size=(n, 16)).astype(np.float32)
    t = np.stack([np.sin(x[:, 0]), 0.5 * x[:, 1] * x[:, 2], np.tanh(x[:, 3] - x[:, 4])], 1)
    t = t.astype(np.float32)
    prm, img = _pack(torch, omlp.init(11))
    m = torch.zeros_like(prm)
    v = torch.zeros_like(prm)
    grad = torch.zeros_like(prm)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    xd, td = _x(torch, x), torch.from_numpy(t).cuda()
    losses = []
    for step in range(1, 401):
        grad.zero_()
        loss.zero_()
        _l.check(getattr(L, entry)(_p(img), _p(xd), _p(td), n, _p(grad), _p(loss), None))
        _l.check(L.sph_mlp_adam(_p(prm), _p(m), _p(v), _p(grad), 3e-3, 0.9, 0.999, 1e-8, step, None))
        _l.check(L.sph_mlp_pack(_p(prm), _p(img), None))
        if step in (1, 400):
            torch.cuda.synchronize()
            losses.append(loss.item())
    assert losses[1] < 0.1 * losses[0], losses
