"""The learned stencil classifier on the tensor cores: forward pass and gradients against the
CPU check in float64 (oracle/mlp_ref.py, same BF16 roundings), and training on a learnable task."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mref():
    import mlp_ref

    return mlp_ref


def bf16_bits(x, mref):
    """float rows [n, 6] -> (BF16 values float64 [n, 6], bits uint16 [n, 8])."""
    v = mref.bf16(x)
    bits = (v.astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
    out = np.zeros((x.shape[0], 8), dtype=np.uint16)
    out[:, :6] = bits
    return v, out


def to_dev(cuda, a):
    t = cuda.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a)
    return t.cuda()


def random_params(rng, mref, scale=0.5):
    return (rng.standard_normal(mref.N_PARAMS) * scale).astype(np.float32)


def test_mlp_params_roundtrip(hteno_lib, cuda):
    with hteno_lib.Mlp(seed=3) as m:
        p = m.params()
        assert p.shape == (1379,) and np.isfinite(p).all() and np.abs(p[:192]).max() > 0
        q = np.arange(1379, dtype=np.float32) * 1e-3
        m.set_params(q)
        np.testing.assert_array_equal(m.params(), q)


def test_mlp_predict_matches_cpu(hteno_lib, cuda, mref):
    rng = np.random.default_rng(1)
    n = 777
    xv, xb = bf16_bits(rng.standard_normal((n, 6)) * 0.5, mref)
    p = random_params(rng, mref)
    with hteno_lib.Mlp() as m:
        m.set_params(p)
        out = cuda.empty((n, 3), dtype=cuda.float32, device="cuda")
        m.predict(to_dev(cuda, xb), out)
        cuda.cuda.synchronize()
        got = out.cpu().numpy()
    want = mref.predict(p.astype(np.float64), xv)
    assert np.abs(got - want).max() <= 2e-3


def test_mlp_pack_rounds_like_cpu(hteno_lib, cuda, mref):
    rng = np.random.default_rng(2)
    x = (rng.standard_normal((300, 6)) * 3).astype(np.float32)
    _, want = bf16_bits(x, mref)
    with hteno_lib.Mlp() as m:
        out = cuda.empty((300, 8), dtype=cuda.int16, device="cuda")
        m.pack(cuda.from_numpy(x).cuda(), out)
        got = out.cpu().numpy().view(np.uint16)
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("n", [128, 1000, 40000])
def test_mlp_gradient_matches_cpu(hteno_lib, cuda, mref, n):
    """Gradients of the mean BCE on the tensor cores (forward, back-propagation, weight-gradient
    products accumulated in tensor memory across tiles and CTAs) against float64 on the CPU."""
    rng = np.random.default_rng(n)
    xv, xb = bf16_bits(rng.standard_normal((n, 6)) * 0.5, mref)
    y = rng.integers(0, 8, size=n).astype(np.uint8)
    p = random_params(rng, mref)
    with hteno_lib.Mlp() as m:
        m.set_params(p)
        g, loss = m.grad(to_dev(cuda, xb), to_dev(cuda, y))
    loss_ref, g_ref = mref.loss_and_grad(p.astype(np.float64), xv, y.astype(np.int64))
    assert loss == pytest.approx(loss_ref, rel=1e-4)
    blocks = {"W1": (0, 192), "b1": (192, 224), "W2": (224, 1248), "b2": (1248, 1280),
              "W3": (1280, 1376), "b3": (1376, 1379)}
    for name, (a, b) in blocks.items():
        err = np.linalg.norm(g[a:b] - g_ref[a:b]) / (np.linalg.norm(g_ref[a:b]) + 1e-30)
        assert err <= 2e-3, (name, err)


def test_mlp_learns_a_separable_rule(hteno_lib, cuda, mref):
    rng = np.random.default_rng(5)
    n = 60000
    x = rng.standard_normal((n, 6)) * 0.5
    y = ((x[:, 0] > x[:, 3]).astype(np.uint8) | ((x[:, 1] > x[:, 4]).astype(np.uint8) << 1)
         | ((x[:, 2] + x[:, 5] > 0).astype(np.uint8) << 2))
    xv, xb = bf16_bits(x, mref)
    ntr = 50000
    with hteno_lib.Mlp(seed=11) as m:
        xd, yd = to_dev(cuda, xb), to_dev(cuda, y)
        loss0 = m.grad(xd[:ntr], yd[:ntr])[1]
        loss = m.train(xd[:ntr], yd[:ntr], epochs=25, batch=2048, lr=5e-3)
        out = cuda.empty((n - ntr, 3), dtype=cuda.float32, device="cuda")
        m.predict(xd[ntr:].contiguous(), out)
        pr = out.cpu().numpy()
    bits = np.stack([(y[ntr:] >> k) & 1 for k in range(3)], axis=1)
    acc = ((pr > 0.5) == bits).mean()
    assert loss < 0.5 * loss0 and acc >= 0.95, (loss0, loss, acc)


def test_mlp_training_is_deterministic(hteno_lib, cuda, mref):
    """Per-CTA partial gradients summed in CTA order: two trainings from the same seed on the same
    rows give the same parameters bit for bit (and so the same router)."""
    rng = np.random.default_rng(9)
    n = 70000
    x = rng.standard_normal((n, 6)) * 0.5
    y = rng.integers(0, 8, size=n).astype(np.uint8)
    _, xb = bf16_bits(x, mref)
    xd, yd = to_dev(cuda, xb), to_dev(cuda, y)
    params, losses = [], []
    for _ in range(2):
        with hteno_lib.Mlp(seed=4) as m:
            losses.append(m.train(xd, yd, epochs=3, batch=8192, lr=3e-3))
            params.append(m.params())
    np.testing.assert_array_equal(params[0], params[1])
    assert losses[0] == losses[1]


def test_mlp_wait_timeout_reported_and_handle_recovers(hteno_lib, cuda, mref):
    """The bounded tensor-core waits: with a limit of 0 polls every main-loop wait gives up at once;
    the kernels then wait (with the default bound) for their own products in flight, free their
    tensor memory and return, and the call reports HTENO_ERR_TIMEOUT.  The same handle then
    predicts and computes gradients normally."""
    rng = np.random.default_rng(3)
    n = 1000
    xv, xb = bf16_bits(rng.standard_normal((n, 6)) * 0.5, mref)
    y = rng.integers(0, 8, size=n).astype(np.uint8)
    p = random_params(rng, mref)
    with hteno_lib.Mlp() as m:
        m.set_params(p)
        xd, yd = to_dev(cuda, xb), to_dev(cuda, y)
        out = cuda.empty((n, 3), dtype=cuda.float32, device="cuda")
        m.set_wait_limit(0)
        for call in (lambda: m.predict(xd, out), lambda: m.grad(xd, yd)):
            with pytest.raises(hteno_lib.HtenoError) as e:
                call()
            assert e.value.code == 6  # HTENO_ERR_TIMEOUT
        m.set_wait_limit(1 << 22)
        m.predict(xd, out)
        got = out.cpu().numpy()
        g, loss = m.grad(xd, yd)
    assert np.abs(got - mref.predict(p.astype(np.float64), xv)).max() <= 2e-3
    loss_ref, g_ref = mref.loss_and_grad(p.astype(np.float64), xv, y.astype(np.int64))
    assert loss == pytest.approx(loss_ref, rel=1e-4)
