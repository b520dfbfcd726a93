"""Learned screen on a bumpy sphere: trained on the exact GPU solver's pairs from other seeds, calibrated on held-out
surfaces; the screened force pass must keep the exact path's in-range pair set and distances."""
import os

import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


def test_screened_path_keeps_pairs_and_distances():
    from curvedspacesim_gb300 import api, screen
    ctx = api.Context(0)
    sub, n, sigma = 5, 3000, 0.06

    def mesh(seed):
        return ms.bumpy_sphere(sub, amplitude=0.05, seed=seed)

    X, y, c, _ = screen.generate(ctx, mesh, [11, 12, 13], n, sigma)
    params, _ = screen.train(ctx, X, y, steps=600, batch=4096, lr=3e-3)
    Xh, yh, ch, _ = screen.generate(ctx, mesh, [21, 22], n, sigma)
    margin, info = screen.calibrate(ctx, params, Xh, yh, ch)
    frac, wrong = screen.skipped_fraction(ctx, params, margin, Xh, yh, ch)
    assert wrong == 0
    # evaluation surface (seed 0): exact vs screened force pass
    V, F = mesh(0)
    rng = np.random.default_rng(5)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    M = api.Mesh(V, F)
    p = api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=1e-3)
    plain = api.System(ctx, M, n, p)
    plain.set_state(f, b, np.zeros((n, 3)), np.zeros((n, 3)))
    plain.enable_pairs()
    plain.compute_forces()
    assert plain.check()[0] == 0
    scr = api.System(ctx, M, n, p)
    scr.set_state(f, b, np.zeros((n, 3)), np.zeros((n, 3)))
    scr.enable_pairs()
    scr.set_screen(params, margin)
    scr.compute_forces()
    bits, cnt = scr.check()
    assert bits == 0, cnt
    sc = scr.screen_counters()
    assert sc["tc_errors"] == 0 and sc["pairs"] > 0
    missing, extra, err = screen.audit(plain.pairs(), scr.pairs(), sigma)
    assert not missing and not extra
    assert err <= 1e-12
    fp = plain.get_state()[3]
    fs = scr.get_state()[3]
    np.testing.assert_allclose(fs, fp, atol=1e-12)


def test_screen_gain_on_thin_torus():
    """What the trained network gains over the method without it: on a thin-tubed torus (tube radius 0.3,
    sigma 0.5) candidate pairs across the tube have chords below sigma and geodesics above it.  Such a pair holds the
    exact path's early exit open until the propagation reaches the cutoff; the screen skips it, and the source stops
    once its in-range targets are settled.  At 40 particles a source has few candidates, so this is most of the
    propagation's reach: the measured bound (every out-of-range pair skipped, from the exact distances) and the
    trained screen's saving are both real, and the in-range pair set stays identical."""
    import sys
    from curvedspacesim_gb300 import api, screen
    ctx = api.Context(0)
    sigma = 0.5

    def mesh(seed):
        return ms.noisy_torus(60, 30, 1.0, 0.3, std=0.01, smoothing_rings=2, seed=seed)

    X, y, c, _ = screen.generate(ctx, mesh, [1, 2, 3], 400, sigma, configs_per_seed=2)
    params, _ = screen.train(ctx, X, y, steps=800, batch=4096, lr=3e-3)
    Xh, yh, ch, _ = screen.generate(ctx, mesh, [4, 5], 400, sigma, configs_per_seed=2)
    margin, info = screen.calibrate(ctx, params, Xh, yh, ch)
    frac, wrong = screen.skipped_fraction(ctx, params, margin, Xh, yh, ch)
    assert wrong == 0
    V, F = mesh(0)
    n = 40
    rng = np.random.default_rng(9)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    M = api.Mesh(V, F)
    p = api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=1e-3)
    runs = {}
    for name in ("plain", "screened"):
        S = api.System(ctx, M, n, p)
        S.set_state(f, b, np.zeros((n, 3)), np.zeros((n, 3)))
        S.enable_pairs()
        if name == "screened":
            S.set_screen(params, margin)
        S.compute_forces()
        bits, cnt = S.check()
        assert bits == 0, cnt
        runs[name] = (S, cnt)
    sc = runs["screened"][0].screen_counters()
    missing, extra, err = screen.audit(runs["plain"][0].pairs(), runs["screened"][0].pairs(), sigma)
    assert not missing and not extra and err <= 1e-12
    w_plain, w_scr = runs["plain"][1]["windows"], runs["screened"][1]["windows"]
    sys.path.insert(0, ROOT)
    import bench
    bound = bench.screen_bound(ctx, M, sigma, runs["plain"][0].get_state(), runs["plain"][0].pairs())
    print(f"thin torus, N={n}: holdout skip fraction {frac:.3f}, evaluation skipped {sc['screened']} of "
          f"{sc['pairs']} candidate pairs ({bound['out_of_range_candidate_pairs']} out of range), windows "
          f"{w_plain} -> {w_scr}; every out-of-range pair skipped: {bound['windows_in_range_only']} "
          f"(saving {bound['max_window_saving']:.3f})")
    assert sc["screened"] > 0
    assert bound["max_window_saving"] > 0.1  # the configuration has something to gain
    # window counts vary by a few tenths of a percent between runs (the order in which the threads of a source group
    # take windows); the screen's saving is several percent
    assert w_scr < 0.97 * w_plain, (w_plain, w_scr)


def test_screen_audit_switches_off_a_screen_that_drops_pairs():
    """Periodic exact audit with automatic fallback (cssg_system_set_screen_audit): a screen with a negative margin
    skips every candidate pair, in range or not.  The steps before the first audit run with it; the audit step runs
    the exact pass too, drives the step with it, finds the dropped in-range pairs and switches the screen off on the
    device, after which the screened system's force passes equal the plain exact path's."""
    from curvedspacesim_gb300 import api, screen
    ctx = api.Context(0)
    sub, n, sigma = 5, 3000, 0.06
    V, F = ms.bumpy_sphere(sub, amplitude=0.05, seed=0)
    rng = np.random.default_rng(3)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, 0.1, rng)
    M = api.Mesh(V, F)
    p = api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=1e-3)

    def exact_at(state):
        P = api.System(ctx, M, n, p)
        P.set_state(*state)
        P.enable_pairs()
        P.compute_forces()
        assert P.check()[0] == 0
        return P

    # a screen that skips nothing passes its audits and stays on
    good = api.System(ctx, M, n, p)
    good.set_state(f, b, vel, np.zeros((n, 3)))
    good.set_screen(screen.init_params(0), 1e6)
    good.set_screen_audit(2)
    good.step(4, graph=True)
    st = good.screen_audit_status()
    assert st == {"audits": 2, "sources_with_dropped_pairs": 0, "screen_off": False}, st

    bad = api.System(ctx, M, n, p)
    bad.set_state(f, b, vel, np.zeros((n, 3)))
    bad.set_screen(screen.init_params(0), -10.0)
    bad.set_screen_audit(3)
    bad.step(2, graph=True)
    st = bad.screen_audit_status()
    assert st["audits"] == 0 and not st["screen_off"]
    assert np.all(bad.get_state()[3] == 0)  # every pair skipped: zero forces
    bad.step(1, graph=True)  # the audit step
    st = bad.screen_audit_status()
    assert st["audits"] == 1 and st["screen_off"] and st["sources_with_dropped_pairs"] > 0, st
    assert bad.check()[0] == 0
    # the audited step's forces are the exact ones at its positions
    state = bad.get_state()
    np.testing.assert_allclose(state[3], exact_at(state).get_state()[3], atol=1e-12)
    # after the fallback the screened system computes the exact pairs and forces
    bad.step(2, graph=True)
    state = bad.get_state()
    ref = exact_at(state)
    bad.set_state(*state)
    bad.enable_pairs()
    bad.compute_forces()
    missing, extra, err = screen.audit(ref.pairs(), bad.pairs(), sigma)
    assert not missing and not extra and err <= 1e-12
    np.testing.assert_allclose(bad.get_state()[3], ref.get_state()[3], atol=1e-12)
    # enabling the screen again clears the fallback
    bad.set_screen(screen.init_params(0), 1e6)
    assert not bad.screen_audit_status()["screen_off"]
