"""FIRE minimisation (fireMinimization::minimizeByFire) and the monodisperse stress (simulation::
computeMonodisperseStress): the oracle's restatement on the CPU, the device path against it on the GPU."""
import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms


def _setup(n=60, sigma=0.4, seed=4, T=0.0):
    V, F = ms.icosphere(3)
    rng = np.random.default_rng(seed)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, T, rng) if T > 0 else np.zeros((n, 3))
    return V, F, f, b, vel


def test_oracle_fire_converges_and_stress_is_symmetric(oracle_mod):
    V, F, f, b, vel = _setup()
    OM = oracle_mod.OracleMesh(V, F)
    prm = OM.params(0, k=1 / 0.16, sigma=0.4, rng=0.4, submesh=1, max_dist=0.4, cutoff=0.4, dt=0.01)
    f0 = OM.forces(f, b, prm)[0]
    fa, ba, va, fo, st, it, fmax, err = OM.fire(f, b, vel, np.zeros_like(vel), prm, maximum_iterations=400,
                                               force_cutoff=1e-10)
    assert err == 0
    assert fmax <= 1e-10 and it < 400
    assert np.max(np.linalg.norm(fo, axis=1)) == pytest.approx(fmax, rel=1e-12)
    assert fmax < 1e-6 * np.max(np.linalg.norm(f0, axis=1))
    # stress of an overlapping, moving configuration: symmetric (f_ij is parallel to t_ij), negative virial trace
    V2, F2, f2, b2, v2 = _setup(n=80, seed=7, T=0.1)
    OM2 = oracle_mod.OracleMesh(V2, F2)
    s = OM2.stress(f2, b2, v2, prm)
    np.testing.assert_allclose(s, s.T, atol=1e-15)
    s0 = OM2.stress(f2, b2, np.zeros_like(v2), prm)
    assert np.trace(s0) < 0


@pytest.mark.gpu
@pytest.mark.parametrize("group", [1, 2])
def test_fire_matches_oracle(gpu, oracle_mod, group):
    """20 iterations step for step (sums differ only in order: tolerance 1e-9), then a full minimisation converges
    (one and two warps per source)."""
    api, ctx = gpu
    V, F, f, b, vel = _setup()
    n, sigma = len(f), 0.4
    OM = oracle_mod.OracleMesh(V, F)
    prm = OM.params(0, k=1 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma, dt=0.01)
    M = api.Mesh(V, F)
    p = api.make_params("nve", "harmonic", k=1 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True, max_dist=sigma,
                        cutoff=sigma, dt=0.01)
    S = api.System(ctx, M, n, p)
    S.set_state(f, b, vel, np.zeros((n, 3)))
    S.set_tuning(1.0, 8, 0, 0, False, group)
    res = S.fire(maximum_iterations=20, force_cutoff=1e-300, reset=True)
    fo, bo, vo, fco, st, it, fmax, err = OM.fire(f, b, vel, np.zeros((n, 3)), prm, maximum_iterations=20,
                                                 force_cutoff=1e-300)
    assert err == 0 and it == 20 and res["iterations"] == 20
    bits, _ = S.check()
    assert bits == 0
    fg, bg, vg, fcg = S.get_state()
    assert np.array_equal(fg, fo)
    np.testing.assert_allclose(OM.r3(fg, bg), OM.r3(fo, bo), atol=1e-9)
    np.testing.assert_allclose(vg, vo, atol=1e-9)
    np.testing.assert_allclose(fcg, fco, atol=1e-9)
    assert res["dt"] == pytest.approx(st[0], rel=1e-12) and res["alpha"] == pytest.approx(st[1], rel=1e-12)
    assert res["n_since_negative_power"] == int(st[2])
    assert res["force_max"] == pytest.approx(fmax, rel=1e-9)
    # continue (state persists) until converged
    res2 = S.fire(maximum_iterations=1000, force_cutoff=1e-10)
    assert res2["force_max"] <= 1e-10 and res2["iterations"] < 1000
    fcg2 = S.get_state()[3]
    assert np.max(np.linalg.norm(fcg2, axis=1)) <= 1e-10


@pytest.mark.gpu
def test_stress_matches_oracle(gpu, oracle_mod):
    api, ctx = gpu
    V, F, f, b, vel = _setup(n=80, seed=7, T=0.1)
    n, sigma = len(f), 0.4
    OM = oracle_mod.OracleMesh(V, F)
    for kind, k in ((0, 1 / sigma ** 2), (1, 0.5)):
        prm = OM.params(kind, k=k, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma, dt=0.01)
        M = api.Mesh(V, F)
        p = api.make_params("nve", "harmonic" if kind == 0 else "gaussian", k=k, sigma=sigma, range_=sigma,
                            submesh=True, max_dist=sigma, cutoff=sigma, dt=0.01)
        S = api.System(ctx, M, n, p)
        S.set_state(f, b, vel, np.zeros((n, 3)))
        sg = S.stress()
        so = OM.stress(f, b, vel, prm)
        np.testing.assert_allclose(sg, so, rtol=1e-9, atol=1e-14)


def test_oracle_gradient_descent_lowers_energy(oracle_mod):
    """gradientDescent::performUpdate in the oracle: with a small step the energy of an overlapping configuration
    falls every step."""
    V, F, f, b, vel = _setup()
    OM = oracle_mod.OracleMesh(V, F)
    prm = OM.params(0, k=1 / 0.16, sigma=0.4, rng=0.4, submesh=1, max_dist=0.4, cutoff=0.4, dt=0.01)
    energies = []
    face, bary = f, b
    for _ in range(5):
        energies.append(OM.forces(face, bary, prm)[1])
        face, bary, _, _, err = OM.gradient_descent(face, bary, prm, 1, 0.01)
        assert err == 0
    assert all(e1 < e0 for e0, e1 in zip(energies, energies[1:])), energies


@pytest.mark.gpu
@pytest.mark.parametrize("transport_velocity", [False, True])
def test_gradient_descent_matches_oracle(gpu, oracle_mod, transport_velocity):
    """20 gradient-descent updates (forces, then a move by dt * force through the walk) against the oracle."""
    api, ctx = gpu
    V, F, f, b, vel = _setup(T=0.1)
    n, sigma, dt = len(f), 0.4, 0.01
    OM = oracle_mod.OracleMesh(V, F)
    prm = OM.params(0, k=1 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma, dt=dt)
    M = api.Mesh(V, F)
    p = api.make_params("nve", "harmonic", k=1 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True, max_dist=sigma,
                        cutoff=sigma, dt=dt)
    S = api.System(ctx, M, n, p)
    S.set_state(f, b, vel, np.zeros((n, 3)))
    S.gradient_descent(20, dt, transport_velocity)
    bits, _ = S.check()
    assert bits == 0
    fg, bg, vg, fcg = S.get_state()
    fo, bo, vo, fco, err = OM.gradient_descent(f, b, prm, 20, dt, vel if transport_velocity else None)
    assert err == 0
    np.testing.assert_allclose(OM.r3(fg, bg), OM.r3(fo, bo), atol=1e-9)
    np.testing.assert_allclose(fcg, fco, atol=1e-9)
    np.testing.assert_allclose(vg, vo if transport_velocity else vel, atol=1e-9)


@pytest.mark.gpu
def test_batched_fire_matches_oracle_and_single_systems(gpu, oracle_mod):
    """FIRE on a batched object of three systems (different meshes, counts and sigmas): 20 iterations of each system
    against the oracle's minimizeByFire on that system alone, then minimisation to convergence against the same calls
    on each system as its own object (each system stops on its own rule; a converged one no longer moves)."""
    api, ctx = gpu
    rng = np.random.default_rng(11)
    specs = [(ms.icosphere(3), 60), (ms.torus(50, 25, 3.0, 1.0), 150), (ms.ellipsoid(3, (1.5, 1.0, 0.7)), 40)]
    dt = 0.01
    systems = []
    for (V, F), n in specs:
        sigma = ms.sigma_for_area_fraction(ms.total_area(V, F), n, 0.6)
        f, b = ms.area_weighted_positions(V, F, n, rng)
        systems.append((V, F, n, sigma, f, b))

    def make(group):
        meshes = [api.Mesh(V, F) for V, F, *_ in group]
        params = [api.make_params("nve", "harmonic", k=1 / sg ** 2, sigma=sg, range_=sg, submesh=True, max_dist=sg,
                                  cutoff=sg, dt=dt) for _, _, _, sg, _, _ in group]
        S = api.System(ctx, meshes if len(meshes) > 1 else meshes[0], [g[2] for g in group] if len(group) > 1
                       else group[0][2], params if len(params) > 1 else params[0])
        n = sum(g[2] for g in group)
        S.set_state(np.concatenate([g[4] for g in group]), np.concatenate([g[5] for g in group]), np.zeros((n, 3)),
                    np.zeros((n, 3)))
        return S

    B = make(systems)
    res = B.fire(maximum_iterations=20, force_cutoff=1e-300, reset=True)
    assert isinstance(res, list) and len(res) == 3
    assert B.check()[0] == 0
    fg, bg, vg, fcg = B.get_state()
    off = np.cumsum([0] + [g[2] for g in systems])
    for k, (V, F, n, sg, f, b) in enumerate(systems):
        OM = oracle_mod.OracleMesh(V, F)
        prm = OM.params(0, k=1 / sg ** 2, sigma=sg, rng=sg, submesh=1, max_dist=sg, cutoff=sg, dt=dt)
        fo, bo, vo, fco, st, it, fmax, err = OM.fire(f, b, np.zeros((n, 3)), np.zeros((n, 3)), prm,
                                                     maximum_iterations=20, force_cutoff=1e-300)
        a, e = off[k], off[k + 1]
        assert err == 0 and it == 20 and res[k]["iterations"] == 20
        assert np.array_equal(fg[a:e], fo)
        np.testing.assert_allclose(OM.r3(fg[a:e], bg[a:e]), OM.r3(fo, bo), atol=1e-9)
        np.testing.assert_allclose(vg[a:e], vo, atol=1e-9)
        np.testing.assert_allclose(fcg[a:e], fco, atol=1e-9)
        assert res[k]["dt"] == pytest.approx(st[0], rel=1e-12)
        assert res[k]["force_max"] == pytest.approx(fmax, rel=1e-9)
    res2 = B.fire(maximum_iterations=3000, force_cutoff=1e-10)
    fg2, bg2, _, fcg2 = B.get_state()
    iters = [r["iterations"] for r in res2]
    for k, g in enumerate(systems):
        S = make([g])
        S.fire(maximum_iterations=20, force_cutoff=1e-300, reset=True)
        r = S.fire(maximum_iterations=3000, force_cutoff=1e-10)
        a, e = off[k], off[k + 1]
        assert res2[k]["force_max"] <= 1e-10 and abs(res2[k]["iterations"] - r["iterations"]) <= 1, (k, res2[k], r)
        fs, bs, _, _ = S.get_state()
        OM = oracle_mod.OracleMesh(g[0], g[1])
        np.testing.assert_allclose(OM.r3(fg2[a:e], bg2[a:e]), OM.r3(fs, bs), atol=1e-7)
        assert np.max(np.linalg.norm(fcg2[a:e], axis=1)) <= 1e-10
    assert len(set(iters)) > 1, iters  # the systems converged at different iterations
