"""The CUDA path against the FP64 oracle at the sizes of the benchmark workloads (GPU).

* bumpy sphere, subdivision 7 (163,842 vertices), N=20,000, sigma 0.02: one exact force pass and one learned-screen
  force pass, each against the oracle's neighbour distances and forces on the same positions;
* the 64 uneven systems of the batched workload (53,606 particles): three velocity-Verlet steps of the one batched
  system object, each system against the oracle;
* noisy torus 1000x500 (500,000 vertices), N=100,000: one exact force pass, 2,000 sampled sources against the oracle.

Reference path matched: simpleModel::findNeighbors (src/models/simpleModel.cpp:68-112) with
triangulatedMeshSpace::distanceWithSubmeshing (src/models/triangulatedMeshSpace.cpp:155-205) and force::computeForces
(src/forces/baseForce.cpp:12-28).  Tolerances: distances 1e-6 relative is the bar; the tests require 1e-10."""
import os
import sys

import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REL_DIST = 1e-10
THREADS = os.cpu_count() or 1


def _bench():
    sys.path.insert(0, ROOT)
    import bench
    return bench


def _compare_pairs(i, j, d, src, idx, do, sigma, sources=None):
    """In-range pair sets (d <= sigma) identical, distances within REL_DIST; returns the largest relative error."""
    gpu = {(int(a), int(c)): float(x) for a, c, x in zip(i, j, d) if c >= 0 and x <= sigma}
    ora = {(int(a), int(c)): float(x) for a, c, x in zip(src, idx, do) if x <= sigma}
    if sources is not None:
        keep = set(int(s) for s in sources)
        gpu = {k: v for k, v in gpu.items() if k[0] in keep}
    assert set(gpu) == set(ora), (len(set(gpu) - set(ora)), len(set(ora) - set(gpu)))
    rel = max([abs(gpu[k] - ora[k]) / ora[k] for k in ora if ora[k] > 0] or [0.0])
    assert rel <= REL_DIST, rel
    return rel


@pytest.mark.parametrize("lanes,build", [(0, 0), (32, 0), (0, 3)])
def test_bumpy_sphere7_exact_and_screened_match_oracle(gpu, oracle_mod, lanes, build):
    """Config 4 (bumpy sphere 7, N=20,000): one exact and one screened force pass against the oracle, with the
    source-group pass (default build, and the 255-register build with out-of-line probes) and the lane pass."""
    api, ctx = gpu
    from curvedspacesim_gb300 import screen
    bench = _bench()
    cfg = bench.workload_config("bumpy_screen")
    V, F, f, b, vel = bench.build_inputs(cfg)
    n, sigma = cfg["n"], cfg["sigma"]
    M = api.Mesh(V, F)
    p = api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=cfg["dt"])
    OM = oracle_mod.OracleMesh(V, F)
    off, idx, mc = OM.candidates(f, b, sigma)
    do, _, _ = OM.neighbor_distances(f, b, off, idx, mc, 1, sigma, sigma, threads=THREADS)
    src = np.repeat(np.arange(n), np.diff(off))
    prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma)
    fo, _, _ = OM.forces(f, b, prm, threads=THREADS)

    # a small screen trained on two other surfaces, calibrated on a third
    mesh_fn = lambda seed: ms.bumpy_sphere(7, amplitude=0.05, seed=seed)
    X, y, _, _ = screen.generate(ctx, mesh_fn, [1, 2], n, sigma, configs_per_seed=2)
    params, _ = screen.train(ctx, X, y, steps=400, batch=8192, lr=3e-3)
    Xh, yh, ch, _ = screen.generate(ctx, mesh_fn, [9], n, sigma, configs_per_seed=1)
    margin, _ = screen.calibrate(ctx, params, Xh, yh, ch)
    del X, y, Xh, yh, ch

    for screened in (False, True):
        S = api.System(ctx, M, n, p)
        S.set_lanes(lanes)
        if build:
            S.set_tuning(2.0, 8, 0, 0, True, 1, build)
        S.set_state(f, b, vel, np.zeros((n, 3)))
        if screened:
            S.set_screen(params, margin)
        S.enable_pairs()
        S.compute_forces()
        bits, cnt = S.check()
        assert bits == 0, cnt
        i, j, d, _ = S.pairs()
        rel = _compare_pairs(i, j, d, src, idx, do, sigma)
        np.testing.assert_allclose(S.get_state()[3], fo, atol=1e-9)
        print(f"bumpy sphere 7, lanes {lanes}, build {build}, {'screened' if screened else 'exact'}: {cnt['in_range_pairs']} pairs, "
              f"max relative distance error {rel:.2e}")


@pytest.mark.parametrize("lanes", [0, 32])
def test_batch64_three_steps_match_oracle(gpu, oracle_mod, lanes):
    api, ctx = gpu
    bench = _bench()
    cfg = bench.workload_config("batch64")
    systems = bench.build_batch(cfg)
    meshes = [api.Mesh(sy["V"], sy["F"]) for sy in systems]
    params = [api.make_params("nve", "harmonic", k=1.0 / sy["sigma"] ** 2, sigma=sy["sigma"], range_=sy["sigma"],
                              submesh=True, max_dist=sy["sigma"], cutoff=sy["sigma"], dt=cfg["dt"]) for sy in systems]
    counts = [sy["n"] for sy in systems]
    assert len(systems) == 64 and sum(counts) == 53606
    S = api.System(ctx, meshes, counts, params)
    S.set_lanes(lanes)
    S.set_state(np.concatenate([sy["f"] for sy in systems]), np.concatenate([sy["b"] for sy in systems]),
                np.concatenate([sy["vel"] for sy in systems]), np.zeros((sum(counts), 3)))
    S.step(3, graph=True)
    bits, cnt = S.check()
    assert bits == 0, cnt
    fg, bg, vg, frc = S.get_state()
    off = np.cumsum([0] + counts)
    worst = 0.0
    for k, sy in enumerate(systems):
        OM = oracle_mod.OracleMesh(sy["V"], sy["F"])
        sg = sy["sigma"]
        prm = OM.params(0, k=1.0 / sg ** 2, sigma=sg, rng=sg, submesh=1, max_dist=sg, cutoff=sg, dt=cfg["dt"])
        fo, bo, vo, fco, _, err, _ = OM.simulate(0, 3, sy["f"], sy["b"], sy["vel"], np.zeros((sy["n"], 3)), prm,
                                                 threads=THREADS)
        assert err == 0
        a, e = off[k], off[k + 1]
        pe = np.linalg.norm(OM.r3(fg[a:e], bg[a:e]) - OM.r3(fo, bo), axis=1).max()
        assert pe < 1e-9, (k, sy["kind"], pe)
        np.testing.assert_allclose(vg[a:e], vo, atol=1e-9)
        np.testing.assert_allclose(frc[a:e], fco, atol=1e-7 * max(1.0, np.abs(fco).max()))
        worst = max(worst, pe)
    print(f"64 systems, 3 NVE steps: largest position difference {worst:.2e}")


@pytest.mark.parametrize("lanes", [0, 32])
def test_noisy_torus_sampled_sources_match_oracle(gpu, oracle_mod, lanes):
    api, ctx = gpu
    bench = _bench()
    cfg = bench.workload_config("noisy_torus_nvt")
    sy = bench.systems_of(cfg)[0]
    V, F, f, b, n, sigma = sy["V"], sy["F"], sy["f"], sy["b"], sy["n"], sy["sigma"]
    M = api.Mesh(V, F)
    p = api.make_params("nvt", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=cfg["dt"], temperature=cfg["T"])
    S = api.System(ctx, M, n, p)
    S.set_lanes(lanes)
    S.set_state(f, b, sy["vel"], np.zeros((n, 3)))
    S.enable_pairs()
    S.compute_forces()
    bits, cnt = S.check()
    assert bits == 0, cnt
    i, j, d, _ = S.pairs()
    OM = oracle_mod.OracleMesh(V, F)
    off, idx, mc = OM.candidates(f, b, sigma)
    sample = np.sort(np.random.default_rng(11).choice(n, 2000, replace=False))
    counts = np.zeros(n, dtype=np.int64)
    counts[sample] = np.diff(off)[sample]
    off2 = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    idx2 = np.concatenate([idx[off[s]:off[s + 1]] for s in sample]).astype(np.int32)
    do, _, _ = OM.neighbor_distances(f, b, off2, idx2, mc, 1, sigma, sigma, threads=THREADS)
    src = np.repeat(np.arange(n), counts)
    rel = _compare_pairs(i, j, d, src, idx2, do, sigma, sources=sample)
    # forces of the sampled sources: the oracle's force sum over the same pairs
    fg = S.get_state()[3]
    fs = np.zeros((n, 3))
    ts = OM.neighbor_distances(f, b, off2, idx2, mc, 1, sigma, sigma, threads=THREADS)[1]
    mag = np.where(do <= sigma, -(1.0 / sigma ** 2) * (sigma - do), 0.0)
    np.add.at(fs, src, mag[:, None] * np.where(np.isfinite(do)[:, None], ts, 0.0))
    np.testing.assert_allclose(fg[sample], fs[sample], atol=1e-9)
    print(f"noisy torus 1000x500, N=100000: 2000 sources, max relative distance error {rel:.2e}")
