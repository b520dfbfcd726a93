"""Open meshes: the tangential and absorbing boundary conditions of the walk (openMeshSpace.cpp,
tangentialOpenMeshSpace.cpp, absorbingOpenMeshSpace.cpp) - known answers on a planar square in the oracle, and the
device walk against the oracle on a silo (hemispherical bowl + cylinder, open rim)."""
import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms


def _locate(V, F, x, y):
    for f in range(len(F)):
        a, b, c = V[F[f]]
        T = np.array([[a[0], b[0], c[0]], [a[1], b[1], c[1]], [1, 1, 1]])
        w = np.linalg.solve(T, [x, y, 1])
        if (w >= -1e-12).all():
            return f, w
    raise ValueError("outside")


@pytest.fixture()
def boundary(oracle_mod):
    yield oracle_mod.set_boundary
    oracle_mod.set_boundary(0)


def test_oracle_planar_square_known_answers(oracle_mod, boundary):
    V, F = ms.planar_grid(10, 1.0)
    OM = oracle_mod.OracleMesh(V, F)
    f0, b0 = _locate(V, F, 0.51, 0.93)
    disp = np.array([[0.3, 0.3, 0.0]])
    vel = np.array([[[0.5, 0.5, 0.0]]])
    # closed-mesh semantics: reaching the border is an error
    boundary(0)
    assert OM.transport([f0], [b0], disp, vel)[4][0] == 1
    # tangential: reach y = 1 at x = 0.58, then slide along +x by the tangential part of the whole displacement
    # (0.3 / sqrt(2) * |(0.3, 0.3)| = 0.3); the velocity loses its outward component
    boundary(1)
    fo, bo, _, to, st, _ = OM.transport([f0], [b0], disp, vel)
    assert st[0] == 0
    np.testing.assert_allclose(OM.r3(fo, bo)[0], [0.88, 1.0, 0.0], atol=1e-12)
    np.testing.assert_allclose(to[0, 0], [0.5, 0.0, 0.0], atol=1e-15)
    # absorbing: stop where the border was reached
    boundary(2)
    fo, bo, _, to, st, _ = OM.transport([f0], [b0], disp, vel)
    assert st[0] == 0
    np.testing.assert_allclose(OM.r3(fo, bo)[0], [0.58, 1.0, 0.0], atol=1e-12)
    np.testing.assert_allclose(to[0, 0], [0.5, 0.0, 0.0], atol=1e-15)
    # sliding into the corner: the slide continues through border vertices along the border edges
    boundary(1)
    f1, b1 = _locate(V, F, 0.75, 0.95)
    fo, bo, _, _, st, _ = OM.transport([f1], [b1], np.array([[0.1, 0.1, 0.0]]))
    assert st[0] == 0
    p = OM.r3(fo, bo)[0]
    assert p[1] == pytest.approx(1.0, abs=1e-12) and 0.75 < p[0] <= 1.0


def test_oracle_silo_walks_stay_on_the_surface(oracle_mod, boundary):
    V, F = ms.silo()
    OM = oracle_mod.OracleMesh(V, F)
    rng = np.random.default_rng(3)
    n = 300
    f, b = ms.area_weighted_positions(V, F, n, rng)
    disp = ms.tangent_velocities(V, F, f, 1.0, rng) * 2.0
    for bc in (1, 2):
        boundary(bc)
        fo, bo, _, to, st, _ = OM.transport(f, b, disp, disp[:, None, :])
        assert np.all(st == 0)
        assert np.all(bo >= -1e-11)
        p = OM.r3(fo, bo)
        assert np.all(p[:, 2] <= 4.0 + 1e-12)
        # transported vectors stay in the tangent plane of the final face
        nrm = ms.face_normals(V, F)[fo]
        assert np.max(np.abs(np.einsum("ij,ij->i", to[:, 0], nrm))) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("bc", ["tangential", "absorbing"])
def test_open_walk_matches_oracle(gpu, oracle_mod, boundary, bc):
    api, ctx = gpu
    V, F = ms.silo()
    OM = oracle_mod.OracleMesh(V, F)
    boundary({"tangential": 1, "absorbing": 2}[bc])
    rng = np.random.default_rng(11)
    n = 2000
    f, b = ms.area_weighted_positions(V, F, n, rng)
    disp = ms.tangent_velocities(V, F, f, 1.0, rng) * rng.uniform(0.1, 3.0, size=(n, 1))
    M = api.Mesh(V, F, boundary=bc)
    fg, bg, dg, tg, sg, _ = api.transport_batch(ctx, M, f, b, disp, disp[:, None, :])
    fo, bo, do, to, so, cr = OM.transport(f, b, disp, disp[:, None, :])
    assert np.all(so == 0) and np.all(sg == 0)
    assert np.array_equal(fg, fo)
    exact = (cr >> 16) == 0  # no interior vertex crossing (those use acos/sin/cos): bitwise
    assert exact.mean() > 0.9
    assert np.array_equal(bg[exact], bo[exact])
    assert np.array_equal(tg[exact], to[exact])
    np.testing.assert_allclose(bg, bo, atol=1e-9)
    np.testing.assert_allclose(tg, to, atol=1e-9)
    # some walks must actually have met the rim
    p = OM.r3(fo, bo)
    assert np.sum(np.abs(p[:, 2] - 4.0) < 1e-9) > 10


@pytest.mark.gpu
def test_open_system_nve_matches_oracle(gpu, oracle_mod, boundary):
    """Velocity-Verlet on the silo with tangential walls: 30 steps against the oracle."""
    api, ctx = gpu
    V, F = ms.silo(nsides=32, ncap=8, nz=12)
    boundary(1)
    OM = oracle_mod.OracleMesh(V, F)
    n, sigma, dt = 200, 0.5, 0.01
    rng = np.random.default_rng(2)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, 1.0, rng)
    M = api.Mesh(V, F, boundary="tangential")
    p = api.make_params("nve", "harmonic", k=1 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True, max_dist=sigma,
                        cutoff=sigma, dt=dt)
    S = api.System(ctx, M, n, p)
    S.set_state(f, b, vel, np.zeros((n, 3)))
    S.step(30, graph=True)
    bits, _ = S.check()
    assert bits == 0
    fg, bg, vg, _ = S.get_state()
    prm = OM.params(0, k=1 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma, dt=dt)
    fo, bo, vo, _, _, err, _ = OM.simulate(0, 30, f, b, vel, np.zeros((n, 3)), prm)
    assert err == 0
    np.testing.assert_allclose(OM.r3(fg, bg), OM.r3(fo, bo), atol=1e-8)
    np.testing.assert_allclose(vg, vo, atol=1e-8)


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", ["nve", "nvt"])
def test_closed_rule_on_open_mesh_reports_border(gpu, integrator):
    """A system on the open silo with the closed-mesh rule: walks that reach the rim fail with CSSG_ST_BORDER, and
    the failure reaches System.check() (the walk kernel reduces the failure bits itself)."""
    api, ctx = gpu
    V, F = ms.silo(nsides=32, ncap=8, nz=12)
    rng = np.random.default_rng(8)
    n, sigma = 200, 0.3
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, 50.0, rng)
    M = api.Mesh(V, F)  # closed rule
    p = api.make_params(integrator, "harmonic", k=1 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=0.05, temperature=1.0)
    S = api.System(ctx, M, n, p)
    S.set_state(f, b, vel, np.zeros((n, 3)))
    S.step(5, graph=True)
    bits, _ = S.check()
    assert bits & (1 << 1), bits
    # the same system with the tangential rule: no failure
    M2 = api.Mesh(V, F, boundary="tangential")
    S2 = api.System(ctx, M2, n, p)
    S2.set_state(f, b, vel, np.zeros((n, 3)))
    S2.step(5, graph=True)
    bits2, _ = S2.check()
    assert bits2 == 0, bits2
