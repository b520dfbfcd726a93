"""CPU tests of the oracle (the checker of the CUDA path) against closed-form geometry and an independent
brute-force unfolding solver.  The reference ships no tests or golden vectors and its geodesic code (CGAL) cannot
be built here, so these known answers are what pins the oracle."""
import math

import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms


@pytest.fixture(scope="module")
def O(oracle_mod):
    return oracle_mod


def test_planar_distance_is_chord(O):
    rng = np.random.default_rng(1)
    V, F = ms.planar_grid(10, 1.0, jitter=0.35, seed=3)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 30, rng)
    P = M.r3(f, b)
    for s in range(5):
        others = [i for i in range(30) if i != s]
        d, ts, te, _ = M.distance(f[s], b[s], f[others], b[others])
        ch = np.linalg.norm(P[others] - P[s], axis=1)
        np.testing.assert_allclose(d, ch, rtol=0, atol=1e-14)
        u = (P[others] - P[s]) / ch[:, None]
        np.testing.assert_allclose(ts, u, atol=1e-13)
        np.testing.assert_allclose(te, u, atol=1e-13)


def _unroll_prism(P, nsides, radius):
    ang = np.arctan2(P[:, 1], P[:, 0]) % (2 * np.pi)
    step = 2 * np.pi / nsides
    side = 2 * radius * math.sin(step / 2)
    k = np.floor(ang / step).astype(int) % nsides
    a0 = k * step
    c0 = np.stack([radius * np.cos(a0), radius * np.sin(a0)], 1)
    along = np.linalg.norm(P[:, :2] - c0, axis=1)
    return k * side + along, P[:, 2], nsides * side


def test_prism_distance_equals_unrolled(O):
    rng = np.random.default_rng(2)
    nsides = 12
    V, F = ms.prism(nsides, 8, radius=1.0, height=2.0)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 25, rng)
    P = M.r3(f, b)
    s, z, perim = _unroll_prism(P, nsides, 1.0)
    for src in range(4):
        others = np.array([i for i in range(25) if i != src])
        d, _, _, _ = M.distance(f[src], b[src], f[others], b[others])
        ds = np.abs(s[others] - s[src])
        ds = np.minimum(ds, perim - ds)
        exp = np.hypot(ds, z[others] - z[src])
        np.testing.assert_allclose(d, exp, rtol=1e-12, atol=1e-13)


def test_cone_distance_equals_unrolled(O):
    rng = np.random.default_rng(3)
    nsides, rings = 10, 6
    V, F = ms.pyramid_cone(nsides, rings, radius=1.0, height=1.5)
    M = O.OracleMesh(V, F)
    apex = V[0]
    # unrolled apex angle per side (isosceles face apex angle)
    e0 = V[1] - apex
    e1 = V[2] - apex
    theta = math.acos(np.dot(e0, e1) / (np.linalg.norm(e0) * np.linalg.norm(e1)))
    total = nsides * theta
    assert total < 2 * np.pi
    f, b = ms.area_weighted_positions(V, F, 20, rng)
    P = M.r3(f, b)
    r = np.linalg.norm(P - apex, axis=1)
    # unrolled angle: side index + angle inside the side sector
    ang3 = np.arctan2(P[:, 1], P[:, 0]) % (2 * np.pi)
    step = 2 * np.pi / nsides
    k = np.floor(ang3 / step).astype(int) % nsides
    ring_dir = V[1 + k] - apex
    phi = np.array([math.acos(np.clip(np.dot(P[i] - apex, ring_dir[i]) / (r[i] * np.linalg.norm(ring_dir[i])), -1, 1))
                    for i in range(20)])
    unrolled = k * theta + phi
    for src in range(4):
        others = np.array([i for i in range(20) if i != src])
        d, _, _, _ = M.distance(f[src], b[src], f[others], b[others])
        dphi = np.abs(unrolled[others] - unrolled[src])
        dphi = np.minimum(dphi, total - dphi)
        exp = np.sqrt(r[others] ** 2 + r[src] ** 2 - 2 * r[others] * r[src] * np.cos(dphi))
        np.testing.assert_allclose(d, exp, rtol=1e-11, atol=1e-12)


def test_icosphere_matches_bruteforce(O):
    rng = np.random.default_rng(4)
    V, F = ms.icosphere(2)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 10, rng)
    d, _, _, _ = M.distance(f[0], b[0], f[1:], b[1:])
    P = M.r3(f, b)
    for i in range(1, 10):
        if np.linalg.norm(P[i] - P[0]) > 1.0:
            continue  # keep the brute force shallow
        bf = M.distance_bruteforce(f[0], b[0], f[i], b[i], max_depth=10)
        assert abs(d[i - 1] - bf) < 1e-12 * max(1.0, bf), (i, d[i - 1], bf)


def test_torus_saddles_match_bruteforce(O):
    rng = np.random.default_rng(5)
    V, F = ms.torus(18, 9, 3.0, 1.0)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 40, rng)
    P = M.r3(f, b)
    checked = 0
    for s in range(3):
        others = np.array([i for i in range(40) if i != s and np.linalg.norm(P[i] - P[s]) < 1.6])
        if len(others) == 0:
            continue
        d, _, _, _ = M.distance(f[s], b[s], f[others], b[others])
        for q, i in enumerate(others[:4]):
            bf = M.distance_bruteforce(f[s], b[s], f[i], b[i], max_depth=9)
            assert abs(d[q] - bf) < 1e-11 * max(1.0, bf), (s, i, d[q], bf)
            checked += 1
    assert checked >= 6


def test_patch_distances_match_bruteforce_on_patch(O):
    rng = np.random.default_rng(6)
    V, F = ms.torus(40, 20, 3.0, 1.0)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 300, rng)
    off, idx, mc = M.candidates(f, b, 0.8)
    done = 0
    for s in range(300):
        c = idx[off[s]:off[s + 1]]
        if len(c) < 2:
            continue
        r = min(0.8, mc[s])
        patch = M.patch(f[s], b[s], f[c], r)
        d, _, _, st = M.distance(f[s], b[s], f[c], b[c], submesh=True, max_dist=0.8, threshold=mc[s])
        for q in range(min(2, len(c))):
            bf = M.distance_bruteforce(f[s], b[s], f[c[q]], b[c[q]], face_set=patch, max_depth=9)
            if not np.isfinite(bf):
                assert d[q] == pytest.approx(1.6)  # disconnected patch target: 2 * max_dist
            else:
                assert abs(d[q] - bf) < 1e-11, (s, q, d[q], bf)
            done += 1
        if done >= 8:
            break
    assert done >= 8


def test_distance_symmetry_and_bounds(O):
    rng = np.random.default_rng(7)
    V, F = ms.torus(30, 15, 3.0, 1.0)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 12, rng)
    P = M.r3(f, b)
    D = np.zeros((12, 12))
    for s in range(12):
        others = [i for i in range(12) if i != s]
        d, ts, te, _ = M.distance(f[s], b[s], f[others], b[others])
        D[s, others] = d
        np.testing.assert_allclose(np.linalg.norm(ts, axis=1), 1.0, atol=1e-12)
        np.testing.assert_allclose(np.linalg.norm(te, axis=1), 1.0, atol=1e-12)
    np.testing.assert_allclose(D, D.T, rtol=1e-11, atol=1e-12)
    chord = np.linalg.norm(P[:, None] - P[None], axis=2)
    assert np.all(D >= chord - 1e-12)
    for i in range(12):
        for j in range(12):
            assert np.all(D[i, j] <= D[i] + D[:, j] + 1e-11)


def test_walk_planar_straight_line_and_isometry(O):
    rng = np.random.default_rng(8)
    V, F = ms.icosphere(3)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 200, rng)
    N = ms.face_normals(V, F)[f]
    raw = rng.standard_normal((200, 3))
    disp = raw - (raw * N).sum(1, keepdims=True) * N
    disp *= (rng.random((200, 1)) * 0.3)
    vel = rng.standard_normal((200, 3))
    vel -= (vel * N).sum(1, keepdims=True) * N
    f2, b2, d2, tv, st, cr = M.transport(f, b, disp, vel[:, None, :])
    assert np.all(st == 0)
    assert cr.sum() > 50
    # unfolding rotations preserve the lengths of the displacement and of transported vectors
    np.testing.assert_allclose(np.linalg.norm(tv[:, 0], axis=1), np.linalg.norm(vel, axis=1), rtol=1e-12)
    np.testing.assert_allclose(np.linalg.norm(d2, axis=1)[cr == 0], np.linalg.norm(disp, axis=1)[cr == 0],
                               rtol=1e-10)
    assert np.all(b2 >= 0) and np.allclose(b2.sum(1), 1.0)
    # planar: straight line, identity transport
    V, F = ms.planar_grid(12, 1.0, jitter=0.3, seed=2)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 400, rng)
    P = M.r3(f, b)
    disp = np.zeros((400, 3))
    disp[:, :2] = rng.standard_normal((400, 2)) * 0.05
    target = P + disp
    ok = (target[:, 0] > 0.01) & (target[:, 0] < 0.99) & (target[:, 1] > 0.01) & (target[:, 1] < 0.99)
    f2, b2, d2, tv, st, cr = M.transport(f[ok], b[ok], disp[ok], disp[ok][:, None, :])
    assert np.all(st == 0)
    np.testing.assert_allclose(M.r3(f2, b2), target[ok], atol=1e-12)
    np.testing.assert_allclose(tv[:, 0], disp[ok], atol=1e-15)


def test_walk_reversibility_on_sphere(O):
    rng = np.random.default_rng(9)
    V, F = ms.icosphere(4)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 300, rng)
    N = ms.face_normals(V, F)[f]
    raw = rng.standard_normal((300, 3))
    disp = raw - (raw * N).sum(1, keepdims=True) * N
    disp *= 0.08 / np.linalg.norm(disp, axis=1, keepdims=True)
    f2, b2, d2, tv, st, cr = M.transport(f, b, disp, disp[:, None, :])
    assert np.all(st == 0) and cr.sum() > 100
    back = -tv[:, 0]
    f3, b3, _, _, st3, _ = M.transport(f2, b2, back)
    assert np.all(st3 == 0)
    err = np.linalg.norm(M.r3(f3, b3) - M.r3(f, b), axis=1)
    assert err.max() < 1e-10


def test_nve_energy_and_nvt_temperature(O):
    rng = np.random.default_rng(10)
    V, F = ms.icosphere(3)
    M = O.OracleMesh(V, F)
    n = 60
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, 0.05, rng)
    sigma = 0.35
    prm = O.OracleMesh.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sigma, submesh=0, max_dist=sigma, cutoff=sigma,
                              dt=0.002)
    force, e0, _ = M.forces(f, b, prm)
    ke0 = 0.5 * (vel ** 2).sum()
    out = M.simulate(0, 200, f, b, vel, force, prm)
    f2, b2, v2, fo2, _, err, _ = out
    assert err == 0
    _, e1, _ = M.forces(f2, b2, prm)
    # computeEnergy counts each pair from both sides
    E0 = ke0 + 0.5 * e0
    E1 = 0.5 * (v2 ** 2).sum() + 0.5 * e1
    assert abs(E1 - E0) < 2e-3 * max(abs(E0), 1e-3)


def test_candidates_are_exact_chord_ball(O):
    rng = np.random.default_rng(11)
    V, F = ms.torus(50, 25, 3.0, 1.0)
    M = O.OracleMesh(V, F)
    f, b = ms.area_weighted_positions(V, F, 500, rng)
    P = M.r3(f, b)
    off, idx, mc = M.candidates(f, b, 0.4)
    D = np.linalg.norm(P[:, None] - P[None], axis=2)
    for i in range(500):
        got = set(idx[off[i]:off[i + 1]].tolist())
        exp = set(np.nonzero((D[i] ** 2 < 0.16) & (np.arange(500) != i))[0].tolist())
        assert got == exp
