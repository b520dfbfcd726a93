"""Learned distance screen: training data from the exact GPU solver, training with the library's own kernels,
margin calibration on held-out surfaces, and the audit against the exact path.

The screen predicts, for a candidate pair (chord < range), y = (d - |chord|) / sigma, the normalised excess of the
geodesic over the chord.  A pair is skipped when |chord| / sigma + y_hat > 1 + margin.  The margin is the largest
over-prediction seen on held-out in-range pairs plus a safety term, so no held-out in-range pair is skipped; the
periodic audit (`audit`) reruns the exact path and reports any in-range pair the screen dropped.
"""
from __future__ import annotations

import math

import numpy as np

from . import api
from . import meshes as ms


def _torch():
    import torch
    return torch


def pairs_from_exact_solver(ctx, V, F, n, sigma, seed, data_cutoff=1.5, mesh=None):
    """Exact candidate-pair distances of one random configuration (reference patches, cell list with range sigma,
    geodesics followed to data_cutoff * sigma).  Returns device tensors X (bf16 features), y, chord/sigma, d/sigma.
    mesh: the api.Mesh of (V, F) when the caller already holds one."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    M = mesh if mesh is not None else api.Mesh(V, F, device=ctx.device)
    p = api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=data_cutoff * sigma, dt=1e-3)
    S = api.System(ctx, M, n, p)
    S.set_state(f, b, np.zeros((n, 3)), np.zeros((n, 3)))
    S.enable_pairs()
    S.compute_forces()
    bits, cnt = S.check()
    if bits:
        raise RuntimeError(f"exact solver reported errors {bits:#x} {cnt}")
    i, j, d, _ = S.pairs()
    dev = f"cuda:{ctx.device}"
    pos = torch.tensor(ms.bary_to_r3(V, F, f, b), dtype=torch.float64, device=dev)
    face = torch.tensor(f, dtype=torch.int32, device=dev)
    ti = torch.tensor(i, dtype=torch.int32, device=dev)
    tj = torch.tensor(j, dtype=torch.int32, device=dev)
    X, chord = api.screen_features(ctx, M, sigma, ti, tj, face, pos)
    dd = np.where(np.isfinite(d), d, data_cutoff * sigma) / sigma
    ds = torch.tensor(dd, dtype=torch.float32, device=dev)
    y = ds - chord
    return X, y, chord, ds


def generate(ctx, mesh_fn, seeds, n, sigma, pairs_per_seed=None, configs_per_seed=1):
    """Concatenated training pairs from several surfaces (mesh_fn(seed) -> (V, F)) and configurations."""
    torch = _torch()
    Xs, ys, cs, ds = [], [], [], []
    for s in seeds:
        V, F = mesh_fn(s)
        M = api.Mesh(V, F, device=ctx.device)
        for c in range(configs_per_seed):
            X, y, ch, d = pairs_from_exact_solver(ctx, V, F, n, sigma, 1000 * s + c, mesh=M)
            Xs.append(X)
            ys.append(y)
            cs.append(ch)
            ds.append(d)
    return torch.cat(Xs), torch.cat(ys), torch.cat(cs), torch.cat(ds)


def init_params(seed=0):
    """He-style initialisation of the 14 -> 64 -> 64 -> 64 -> 1 network (FP32)."""
    P = api.mlp_param_count()
    nin, nh = 16, 64
    rng = np.random.default_rng(seed)
    p = np.zeros(P, dtype=np.float64)
    o = 0
    p[o:o + nh * nin] = rng.standard_normal(nh * nin) * math.sqrt(2.0 / 14)
    o += nh * nin + nh
    p[o:o + nh * nh] = rng.standard_normal(nh * nh) * math.sqrt(2.0 / nh)
    o += nh * nh + nh
    p[o:o + nh * nh] = rng.standard_normal(nh * nh) * math.sqrt(2.0 / nh)
    o += nh * nh + nh
    p[o:o + nh] = rng.standard_normal(nh) * math.sqrt(1.0 / nh)
    return p.astype(np.float32)


def train(ctx, X, y, steps=2000, batch=8192, lr=2e-3, seed=0, log_every=0):
    """Adam on the mean squared error with the library's FP32 forward/backward kernels; returns FP32 params."""
    torch = _torch()
    dev = X.device
    params = torch.tensor(init_params(seed), device=dev)
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = X.shape[0]
    history = []
    for step in range(1, steps + 1):
        idx = torch.randint(0, n, (min(batch, n),), generator=g).to(dev)
        Xb = X[idx].contiguous()
        yb = y[idx].contiguous()
        grad, loss = api.mlp_grad(ctx, Xb, yb, params)
        lr_t = lr * (0.5 * (1 + math.cos(math.pi * step / steps)))  # cosine decay
        api.mlp_adam(ctx, params, grad, m, v, Xb.shape[0], lr_t, step)
        if log_every and step % log_every == 0:
            history.append(float(loss.item()) / Xb.shape[0])
    return params.cpu().numpy(), history


def predict(ctx, X, params):
    torch = _torch()
    pt = torch.tensor(np.asarray(params, dtype=np.float32), device=X.device)
    return api.mlp_infer(ctx, X, pt)


def calibrate(ctx, params, X, y, chord, safety=0.01):
    """Margin = max over in-range pairs (d <= sigma) of the over-prediction y_hat - y, plus `safety`."""
    yh = predict(ctx, X, params)
    inr = (chord + y) <= 1.0
    over = (yh - y)[inr]
    worst = float(over.max().item()) if over.numel() else 0.0
    return max(worst, 0.0) + safety, {"in_range_pairs": int(inr.sum().item()),
                                      "worst_over_prediction": worst,
                                      "rmse": float(((yh - y) ** 2).mean().sqrt().item())}


def skipped_fraction(ctx, params, margin, X, y, chord):
    """Fraction of candidate pairs the screen would skip, and in-range pairs it would wrongly skip."""
    yh = predict(ctx, X, params)
    skip = (chord + yh) > 1.0 + margin
    inr = (chord + y) <= 1.0
    return float(skip.float().mean().item()), int((skip & inr).sum().item())


def audit(plain_pairs, screened_pairs, sigma):
    """Compare in-range pair sets and distances of the exact and the screened path.
    Each argument: (i, j, d) arrays from System.pairs().  Returns (missing, extra, max relative distance error)."""
    def inr(p):
        i, j, d = p[:3]
        return {(int(a), int(b)): float(x) for a, b, x in zip(i, j, d) if x <= sigma}
    A = inr(plain_pairs)
    B = inr(screened_pairs)
    missing = set(A) - set(B)
    extra = set(B) - set(A)
    err = max([abs(A[k] - B[k]) / max(A[k], 1e-300) for k in set(A) & set(B)] or [0.0])
    return missing, extra, err
