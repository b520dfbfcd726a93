"""Learned screen MLP: the NumPy reference's analytic gradient against finite differences (CPU), and the CUDA
kernels (tensor-core inference, FP32 training gradient) against the NumPy reference (GPU)."""
import numpy as np
import pytest

from oracle import mlp_ref as R


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = R.init_params(1)
    X = rng.standard_normal((40, R.NIN))
    X[:, 14:] = 0
    y = rng.standard_normal(40) * 0.1
    g, _ = R.grad(X, y, p, rounded=False)
    eps = 1e-6
    for q in rng.choice(R.NPARAM, 60, replace=False):
        pp = p.copy()
        pp[q] += eps
        lp = 0.5 * ((R.forward(X, pp, False)[0] - y) ** 2).sum()
        pp[q] -= 2 * eps
        lm = 0.5 * ((R.forward(X, pp, False)[0] - y) ** 2).sum()
        assert abs((lp - lm) / (2 * eps) - g[q]) < 1e-6 * max(1.0, abs(g[q]))


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159], dtype=np.float64)
    r = R.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even
    assert r[2] == 1.0 + 2 ** -7
    assert r[3] == -2.5


def _data(n, seed):
    rng = np.random.default_rng(seed)
    X = np.zeros((n, R.NIN))
    X[:, :14] = rng.standard_normal((n, 14))
    y = 0.05 * np.tanh(X[:, 0]) + 0.02 * X[:, 5] ** 2
    return X, y


@pytest.mark.gpu
def test_tensor_core_inference_matches_reference():
    import torch
    from curvedspacesim_gb300 import api
    ctx = api.Context(0)
    p = R.init_params(3)
    X, _ = _data(1000, 4)
    Xt = torch.tensor(R.bf16(X), dtype=torch.bfloat16, device="cuda")
    pt = torch.tensor(p, dtype=torch.float32, device="cuda")
    y = api.mlp_infer(ctx, Xt, pt).cpu().numpy()
    yr, _ = R.forward(X, p.astype(np.float32).astype(np.float64))
    err = np.abs(y - yr)
    scale = np.abs(yr).mean() + 1e-3
    # rare BF16 re-rounding flips of a hidden activation are tolerated; a layout error is not
    assert np.quantile(err, 0.995) < 2e-3 * scale + 1e-5, np.quantile(err, 0.995)
    assert err.max() < 5e-2 * scale + 1e-4, err.max()


@pytest.mark.gpu
def test_inference_rejects_misaligned_rows_and_covers_many_tiles():
    """Rows are read as 16-byte words: a feature array that does not start on a 16-byte boundary is an argument
    error (no launch); a batch of many tiles on the persistent grid (more tiles than resident CTAs, a ragged last
    tile) still matches the reference."""
    import torch
    from curvedspacesim_gb300 import _lib, api
    ctx = api.Context(0)
    p = R.init_params(7)
    pt = torch.tensor(p, dtype=torch.float32, device="cuda")
    X, _ = _data(200_003, 8)
    Xt = torch.tensor(R.bf16(X), dtype=torch.bfloat16, device="cuda")
    flat = torch.zeros(Xt.numel() + 8, dtype=torch.bfloat16, device="cuda")
    shifted = flat[4:4 + Xt.numel()].view(-1, 16)  # 8 bytes past an aligned base
    shifted.copy_(Xt)
    with pytest.raises(_lib.CssgError, match="16-byte aligned"):
        api.mlp_infer(ctx, shifted, pt)
    y = api.mlp_infer(ctx, Xt, pt).cpu().numpy()
    yr, _ = R.forward(X, p.astype(np.float32).astype(np.float64))
    err = np.abs(y - yr)
    scale = np.abs(yr).mean() + 1e-3
    assert np.quantile(err, 0.995) < 2e-3 * scale + 1e-5, np.quantile(err, 0.995)
    assert err.max() < 5e-2 * scale + 1e-4, err.max()


@pytest.mark.gpu
def test_training_gradient_matches_reference():
    import torch
    from curvedspacesim_gb300 import api
    ctx = api.Context(0)
    p = R.init_params(5).astype(np.float32).astype(np.float64)
    X, y = _data(777, 6)
    Xt = torch.tensor(R.bf16(X), dtype=torch.bfloat16, device="cuda")
    yt = torch.tensor(y, dtype=torch.float32, device="cuda")
    pt = torch.tensor(p, dtype=torch.float32, device="cuda")
    g, loss = api.mlp_grad(ctx, Xt, yt, pt)
    g = g.cpu().numpy().astype(np.float64)
    gr, lr = R.grad(X, y.astype(np.float32).astype(np.float64), p)
    assert abs(float(loss.item()) - lr) < 2e-3 * lr
    for a, b in [(R.OFF_W1, R.OFF_B1), (R.OFF_B1, R.OFF_W2), (R.OFF_W2, R.OFF_B2), (R.OFF_B2, R.OFF_W3),
                 (R.OFF_W3, R.OFF_B3), (R.OFF_B3, R.OFF_W4), (R.OFF_W4, R.OFF_B4), (R.OFF_B4, R.NPARAM)]:
        rel = np.linalg.norm(g[a:b] - gr[a:b]) / (np.linalg.norm(gr[a:b]) + 1e-12)
        assert rel < 5e-3, (a, rel)


@pytest.mark.gpu
def test_training_reduces_loss():
    import torch
    from curvedspacesim_gb300 import api
    ctx = api.Context(0)
    X, y = _data(8192, 8)
    Xt = torch.tensor(R.bf16(X), dtype=torch.bfloat16, device="cuda")
    yt = torch.tensor(y, dtype=torch.float32, device="cuda")
    pt = torch.tensor(R.init_params(9) * 0.5, dtype=torch.float32, device="cuda")
    m = torch.zeros_like(pt)
    v = torch.zeros_like(pt)
    losses = []
    for step in range(1, 301):
        g, loss = api.mlp_grad(ctx, Xt, yt, pt)
        api.mlp_adam(ctx, pt, g, m, v, Xt.shape[0], 2e-3, step)
        losses.append(float(loss.item()) / Xt.shape[0])
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
