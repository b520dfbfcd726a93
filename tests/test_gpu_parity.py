"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle on the same seeded inputs."""
import math

import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms

pytestmark = pytest.mark.gpu


def _tangent(V, F, f, rng, scale):
    N = ms.face_normals(V, F)[f]
    raw = rng.standard_normal((len(f), 3))
    d = raw - (raw * N).sum(1, keepdims=True) * N
    return d * scale


@pytest.mark.parametrize("mesh,scale", [("ico4", 0.02), ("ico4", 0.3), ("torus", 0.1), ("torus", 1.5)])
def test_walk_matches_oracle(gpu, oracle_mod, mesh, scale):
    api, ctx = gpu
    rng = np.random.default_rng(100)
    V, F = ms.icosphere(4) if mesh == "ico4" else ms.torus(200, 100)
    OM = oracle_mod.OracleMesh(V, F)
    M = api.Mesh(V, F)
    n = 4000
    f, b = ms.area_weighted_positions(V, F, n, rng)
    disp = _tangent(V, F, f, rng, scale)
    vel = _tangent(V, F, f, rng, 1.0)
    fo, bo, do, to, so, co = OM.transport(f, b, disp, vel[:, None, :])
    fg, bg, dg, tg, sg, cg = api.transport_batch(ctx, M, f, b, disp, vel[:, None, :])
    assert np.all(so == 0) and np.all(sg == 0), (np.unique(so), np.unique(sg))
    vertex = co >> 16
    edge = co & 0xFFFF
    assert cg == int(edge.sum() + vertex.sum()) and cg > 0
    mism = np.nonzero(fg != fo)[0]
    assert len(mism) == 0, ("face mismatch", mism[:10], vertex[mism[:10]], edge[mism[:10]])
    # walks with edge crossings only use the same IEEE operations on both sides (no FMA contraction): bitwise
    # equal; vertex crossings evaluate acos/sin/cos (libm vs CUDA) and are compared with a tolerance
    e = vertex == 0
    np.testing.assert_array_equal(bg[e], bo[e])
    np.testing.assert_array_equal(tg[e, 0], to[e, 0])
    np.testing.assert_array_equal(dg[e], do[e])
    if (~e).any():
        np.testing.assert_allclose(bg[~e], bo[~e], atol=1e-9)
        np.testing.assert_allclose(tg[~e, 0], to[~e, 0], atol=1e-9)


def test_distances_full_mesh_match_oracle(gpu, oracle_mod):
    """All-to-all geodesics on the icosphere-4 (N=100): whole mesh, no cutoff (triangulatedMeshSpace::distance)."""
    api, ctx = gpu
    rng = np.random.default_rng(1)
    V, F = ms.icosphere(4)
    OM = oracle_mod.OracleMesh(V, F)
    M = api.Mesh(V, F)
    n = 100
    f, b = ms.area_weighted_positions(V, F, n, rng)
    src = np.arange(0, 100, 10)
    off = [0]
    cf, cb = [], []
    for s in src:
        o = np.array([i for i in range(n) if i != s])
        cf.append(f[o])
        cb.append(b[o])
        off.append(off[-1] + len(o))
    cf = np.concatenate(cf)
    cb = np.concatenate(cb)
    d, ts, te, st = api.distance_batch(ctx, M, f[src], b[src], np.array(off), cf, cb, submesh=False)
    assert np.all(st == 0)
    for q, s in enumerate(src):
        a, e = off[q], off[q + 1]
        do, tso, teo, _ = OM.distance(f[s], b[s], cf[a:e], cb[a:e])
        np.testing.assert_allclose(d[a:e], do, rtol=1e-12, atol=1e-13)
        np.testing.assert_allclose(ts[a:e], tso, atol=1e-9)
        np.testing.assert_allclose(te[a:e], teo, atol=1e-9)


@pytest.mark.parametrize("cutoff", [math.inf, 0.3])
def test_distances_patch_mode_match_oracle(gpu, oracle_mod, cutoff):
    """Torus 200x100, N=2000, range 0.3: reference patches (distanceWithSubmeshing)."""
    api, ctx = gpu
    rng = np.random.default_rng(2)
    V, F = ms.torus(200, 100)
    OM = oracle_mod.OracleMesh(V, F)
    M = api.Mesh(V, F)
    n = 2000
    f, b = ms.area_weighted_positions(V, F, n, rng)
    off, idx, mc = OM.candidates(f, b, 0.3)
    d, ts, te, st = api.distance_batch(ctx, M, f, b, off, f[idx], b[idx], submesh=True, max_dist=0.3,
                                       threshold=mc, cutoff=cutoff)
    stats = api.distance_batch.last_stats
    assert np.all(st == 0), (np.nonzero(st)[0][:10], stats[st != 0][:5])
    do, tso, _ = OM.neighbor_distances(f, b, off, idx, mc, 1, 0.3, cutoff)
    if not math.isfinite(cutoff):
        do = np.where(np.isfinite(do), do, 0.6)
    fin = np.isfinite(do)
    assert np.array_equal(fin, np.isfinite(d))
    np.testing.assert_allclose(d[fin], do[fin], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(ts[fin], tso[fin], atol=1e-9)


def _system(api, ctx, V, F, n, seed, integrator, sigma, submesh, range_, dt, T):
    rng = np.random.default_rng(seed)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, T if T > 0 else 0.1, rng)
    M = api.Mesh(V, F)
    p = api.make_params(integrator, "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=range_, submesh=submesh,
                        max_dist=sigma, cutoff=sigma, dt=dt, temperature=T)
    S = api.System(ctx, M, n, p)
    S.set_state(f, b, vel, np.zeros((n, 3)))
    return S, f, b, vel


@pytest.mark.parametrize("group", [1, 4, 8])
def test_nve_all_to_all_matches_oracle(gpu, oracle_mod, group):
    """Icosphere-4, N=100, sigma=0.2, all-to-all, velocity Verlet dt=0.005, 100 steps: positions within 1e-5
    (one warp per source, and four warps per source)."""
    api, ctx = gpu
    V, F = ms.icosphere(4)
    n, sigma, dt = 100, 0.2, 0.005
    S, f, b, vel = _system(api, ctx, V, F, n, 1, "nve", sigma, False, 0.0, dt, 0.1)
    S.set_tuning(1.0, 8, 0, 0, False, group)
    S.step(100, graph=True)
    bits, cnt = S.check()
    assert bits == 0, cnt
    fg, bg, vg, _ = S.get_state()
    OM = oracle_mod.OracleMesh(V, F)
    prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=0.0, submesh=0, max_dist=sigma, cutoff=sigma, dt=dt)
    fo, bo, vo, _, _, err, _ = OM.simulate(0, 100, f, b, vel, np.zeros((n, 3)), prm)
    assert err == 0
    err = np.linalg.norm(OM.r3(fg, bg) - OM.r3(fo, bo), axis=1)
    assert err.max() < 1e-5, err.max()
    np.testing.assert_allclose(vg, vo, atol=1e-5)


@pytest.mark.parametrize("lanes", [0, 32])
def test_nvt_patch_matches_oracle(gpu, oracle_mod, lanes):
    """Torus 200x100, N=2000, sigma=cutoff=0.3, patches, Nose-Hoover T=0.05 dt=0.002: 20 steps."""
    api, ctx = gpu
    V, F = ms.torus(200, 100)
    n, sigma, dt, T = 2000, 0.3, 0.002, 0.05
    S, f, b, vel = _system(api, ctx, V, F, n, 2, "nvt", sigma, True, sigma, dt, T)
    S.set_lanes(lanes)
    S.step(20, graph=True)
    bits, cnt = S.check()
    assert bits == 0, cnt
    fg, bg, vg, _ = S.get_state()
    OM = oracle_mod.OracleMesh(V, F)
    prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma, dt=dt,
                    T=T)
    fo, bo, vo, _, ch, err, _ = OM.simulate(1, 20, f, b, vel, np.zeros((n, 3)), prm)
    assert err == 0
    pe = np.linalg.norm(OM.r3(fg, bg) - OM.r3(fo, bo), axis=1)
    assert pe.max() < 1e-7, pe.max()
    np.testing.assert_allclose(vg, vo, atol=1e-7)
    np.testing.assert_allclose(S.chain(), ch, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("lanes,split", [(0, 0), (16, 0), (32, 0), (32, 500)])
def test_pair_sets_identical(gpu, oracle_mod, lanes, split):
    """Torus 200x100, N=2000: in-range pair sets, distances and forces of one force pass against the oracle, with the
    source-group pass (lanes = 0), the one-source-per-lane pass (16 or 32 sources per warp) and the split of the two
    (the 500 costliest sources of a first evaluation to the group pass)."""
    api, ctx = gpu
    V, F = ms.torus(200, 100)
    n, sigma = 2000, 0.3
    S, f, b, vel = _system(api, ctx, V, F, n, 3, "nvt", sigma, True, sigma, 0.002, 0.05)
    S.set_lanes(lanes)
    S.set_lane_split(split)
    if split:
        S.set_tuning(1.0, 8, 0, 0, True, 1)
        S.compute_forces()  # costs for the split
    S.enable_pairs()
    S.compute_forces()
    i, j, d, t = S.pairs()
    cost = S.source_costs()  # windows + launches (+ rounds in the group pass) of each source: every source did work
    assert cost.shape == (n,) and (cost >= 1).all() and cost.max() > 10
    OM = oracle_mod.OracleMesh(V, F)
    off, idx, mc = OM.candidates(f, b, sigma)
    do, tso, _ = OM.neighbor_distances(f, b, off, idx, mc, 1, sigma, sigma)
    gpu_pairs = {(a, c) for a, c, x in zip(i, j, d) if x <= sigma}
    src = np.repeat(np.arange(n), np.diff(off))
    ora_pairs = {(a, c) for a, c, x in zip(src, idx, do) if x <= sigma}
    assert gpu_pairs == ora_pairs
    gd = {(a, c): x for a, c, x in zip(i, j, d)}
    for a, c, x in zip(src, idx, do):
        if np.isfinite(x):
            assert abs(gd[(a, c)] - x) <= 1e-12 * max(1, x)
    # forces against the oracle's force evaluation
    _, _, _, fg = S.get_state()
    prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma)
    fo, _, _ = OM.forces(f, b, prm)
    np.testing.assert_allclose(fg, fo, atol=1e-11)


@pytest.mark.parametrize("group,lanes", [(1, 0), (4, 0), (1, 32)])
def test_batched_systems_match_oracle(gpu, oracle_mod, group, lanes):
    """Three independent systems (different meshes, counts and ranges) in one system object: each must evolve
    exactly as it does alone (velocity Verlet, cell lists, patches, 20 steps; one and four warps per source)."""
    api, ctx = gpu
    rng = np.random.default_rng(7)
    specs = [ms.icosphere(3), ms.torus(50, 25, 3.0, 1.0), ms.ellipsoid(3, (1.5, 1.0, 0.7))]
    counts = [60, 150, 40]
    meshes, params, states = [], [], []
    for (V, F), n in zip(specs, counts):
        sigma = ms.sigma_for_area_fraction(ms.total_area(V, F), n, 0.4)
        f, b = ms.area_weighted_positions(V, F, n, rng)
        vel = ms.tangent_velocities(V, F, f, 0.05, rng)
        meshes.append(api.Mesh(V, F))
        params.append(api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                                      max_dist=sigma, cutoff=sigma, dt=0.002))
        states.append((V, F, f, b, vel, sigma))
    S = api.System(ctx, meshes, counts, params)
    S.set_state(np.concatenate([s[2] for s in states]), np.concatenate([s[3] for s in states]),
                np.concatenate([s[4] for s in states]), np.zeros((sum(counts), 3)))
    S.set_tuning(2.0, 8, 0, 0, True, group)
    S.set_lanes(lanes)
    S.step(20, graph=True)
    bits, cnt = S.check()
    assert bits == 0, cnt
    fg, bg, vg, _ = S.get_state()
    off = np.cumsum([0] + counts)
    for k, (V, F, f, b, vel, sigma) in enumerate(states):
        OM = oracle_mod.OracleMesh(V, F)
        prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma,
                        dt=0.002)
        fo, bo, vo, _, _, err, _ = OM.simulate(0, 20, f, b, vel, np.zeros((len(f), 3)), prm)
        assert err == 0
        a, e = off[k], off[k + 1]
        pe = np.linalg.norm(OM.r3(fg[a:e], bg[a:e]) - OM.r3(fo, bo), axis=1)
        assert pe.max() < 1e-8, (k, pe.max())
        np.testing.assert_allclose(vg[a:e], vo, atol=1e-8)


def test_autotune_keeps_results(gpu, oracle_mod):
    """The autotuner only changes the work order: forces before and after tuning agree, and a forced extreme
    tuning (narrow bands, small CTAs) still matches the oracle."""
    api, ctx = gpu
    V, F = ms.torus(60, 30, 3.0, 1.0)
    n, sigma = 300, 0.45
    S, f, b, _ = _system(api, ctx, V, F, n, 3, "nve", sigma, True, sigma, 1e-3, 0.0)
    S.compute_forces()
    f0 = S.get_state()[3]
    tune = S.autotune(reps=1)
    assert tune["delta_scale"] in (0.5, 1.0, 2.0, 4.0) and tune["warps_per_block"] in (4, 8)
    f1 = S.get_state()[3]
    np.testing.assert_allclose(f1, f0, rtol=0, atol=1e-12)
    for args in ((0.5, 4, 0, 0, False, 1), (2.0, 8, 0, 2, True, 1), (1.0, 8, 0, 4, True, 1), (1.0, 8, 0, 0, True, 2),
                 (4.0, 8, 0, 0, False, 4), (0.5, 4, 0, 8, True, 4), (2.0, 8, 0, 0, True, 8),
                 (4.0, 8, 0, 0, True, 2, True), (1.0, 8, 0, 0, True, 1, True), (2.0, 8, 0, 0, True, 1, 3),
                 (1.0, 8, 0, 0, True, 2, 2), (0.5, 4, 0, 0, False, 4, 3)):
        S.set_tuning(*args)
        S.compute_forces()
        S.compute_forces()  # the second evaluation uses the longest-first order built from the first
        assert S.check()[0] == 0
        np.testing.assert_allclose(S.get_state()[3], f0, rtol=0, atol=1e-12)


def test_device_reciprocal_accuracy(gpu):
    """The Newton-Raphson reciprocal used for window geometry stays within a few ulps of 1/x (and falls back to the
    division outside the float range)."""
    import ctypes
    import torch
    from curvedspacesim_gb300 import _lib
    api, ctx = gpu
    rng = np.random.default_rng(0)
    x = np.concatenate([10.0 ** rng.uniform(-12, 12, 200000) * rng.choice([-1.0, 1.0], 200000),
                        [1.0, -1.0, 3.0, 1e-40, 1e40, 2.0 ** -1022]])
    xd = torch.tensor(x, device="cuda:0")
    od = torch.empty_like(xd)
    with ctx.use():
        assert _lib.load().cssg_diag_reciprocal(ctx.h, len(x), ctypes.c_void_p(xd.data_ptr()),
                                                ctypes.c_void_p(od.data_ptr())) == 0
    ctx.synchronize()
    out = od.cpu().numpy()
    rel = np.abs(out * x - 1.0)
    assert rel.max() < 2.0 ** -50, rel.max()
