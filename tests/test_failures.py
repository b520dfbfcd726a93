"""Failure detection without a GPU fault: every failure below is made on the host (an input, a cap), every loop it
triggers is bounded, and the failure comes back as a per-item status that the host reads.

The reference's loops are unbounded and its failures throw (ERRORERROR, inc/debuggingHelp.h:19-31): the walk loop of
triangulatedMeshSpace::transportParticleAndVectors (src/models/triangulatedMeshSpace.cpp:474) and checkBaryNan
(src/utility/meshUtilities.cpp:184-195).  Here the walk stops after 100,000 passes with CSSG_ST_ITER, a NaN weight
reports CSSG_ST_NAN, and a source that exceeds the propagation caps of all three passes reports CSSG_ST_CAPACITY."""
import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms

ST_NAN, ST_ITER, ST_CAPACITY = 2, 4, 6


def _long_walks(n=4, length=2e5):
    V, F = ms.icosphere(1)
    rng = np.random.default_rng(0)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    N = ms.face_normals(V, F)[f]
    raw = rng.standard_normal((n, 3))
    d = raw - (raw * N).sum(1, keepdims=True) * N
    d *= length / np.linalg.norm(d, axis=1, keepdims=True)
    return V, F, f, b, d


def test_oracle_walk_iteration_cap_and_nan(oracle_mod):
    V, F, f, b, d = _long_walks()
    M = oracle_mod.OracleMesh(V, F)
    st = M.transport(f, b, d)[4]
    assert np.all(st == ST_ITER)  # ~190,000 edge crossings needed, the cap is 100,000 passes
    b2 = b.copy()
    b2[0, 0] = np.nan
    st = M.transport(f, b2, d * 1e-6)[4]
    assert st[0] == ST_NAN and np.all(st[1:] == 0)


@pytest.mark.gpu
def test_gpu_walk_iteration_cap_and_nan(gpu, oracle_mod):
    api, ctx = gpu
    V, F, f, b, d = _long_walks()
    mesh = api.Mesh(V, F)
    st = api.transport_batch(ctx, mesh, f, b, d)[4]
    assert np.all(st == ST_ITER)
    b2 = b.copy()
    b2[0, 0] = np.nan
    st = api.transport_batch(ctx, mesh, f, b2, d * 1e-6)[4]
    assert st[0] == ST_NAN and np.all(st[1:] == 0)


@pytest.mark.gpu
def test_nan_position_reaches_system_check(gpu):
    """A particle with a NaN barycentric weight: its walk reports NaN, its source in the force pass reports NaN (no
    geodesics from a position that is not finite), the other particles step normally, and System.check() sees it."""
    api, ctx = gpu
    V, F = ms.icosphere(3)
    n, sigma = 200, 0.3
    rng = np.random.default_rng(4)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, 0.1, rng)
    M = api.Mesh(V, F)
    for integrator in ("nve", "nvt"):
        p = api.make_params(integrator, "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                            max_dist=sigma, cutoff=sigma, dt=1e-3, temperature=0.1)
        S = api.System(ctx, M, n, p)
        b2 = b.copy()
        b2[7] = [np.nan, 0.5, 0.5]
        S.set_state(f, b2, vel, np.zeros((n, 3)))
        S.step(3, graph=True)
        bits, cnt = S.check()
        assert bits & (1 << ST_NAN), bits
        assert not bits & ~((1 << ST_NAN) | 1), bits
        fg, bg, _, frc = S.get_state()
        ok = np.arange(n) != 7
        assert np.all(np.isfinite(bg[ok])) and np.all(np.isfinite(frc))


@pytest.mark.gpu
@pytest.mark.parametrize("lanes,pass_warps", [(0, 0), (32, 0), (0, 8), (32, 2)])
def test_propagation_caps_escalate_then_report_capacity(gpu, oracle_mod, lanes, pass_warps):
    """Host-forced tiny work caps: sources that exceed the regular pass's cap are redone by the medium (then large)
    pass with the same results; when every pass's cap is exceeded they report CSSG_ST_CAPACITY."""
    api, ctx = gpu
    V, F = ms.torus(60, 30, 3.0, 1.0)
    n, sigma = 300, 0.45
    rng = np.random.default_rng(3)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    M = api.Mesh(V, F)
    p = api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=1e-3)
    S = api.System(ctx, M, n, p)
    S.set_lanes(lanes)
    S.set_pass_groups(pass_warps, pass_warps)  # group size of the medium and large passes (0: the regular one's)
    S.set_state(f, b, np.zeros((n, 3)), np.zeros((n, 3)))
    S.compute_forces()
    assert S.check()[0] == 0
    ref = S.get_state()[3]
    for caps in ((5, 0, 0), (5, 5, 0)):  # regular (then medium) cap exceeded: the next pass redoes the source
        S.set_work_caps(*caps)
        S.compute_forces()
        bits, cnt = S.check()
        assert bits == 0 and cnt["capacity_hits"] == 0, (caps, bits, cnt)
        np.testing.assert_allclose(S.get_state()[3], ref, atol=1e-12)
    S.set_work_caps(5, 5, 5)  # every pass's cap exceeded
    S.compute_forces()
    bits, cnt = S.check()
    assert bits & (1 << ST_CAPACITY) and cnt["capacity_hits"] > 0, (bits, cnt)
    OM = oracle_mod.OracleMesh(V, F)
    off, idx, mc = OM.candidates(f, b, sigma)
    assert cnt["capacity_hits"] <= n and (np.diff(off) > 0).sum() >= cnt["capacity_hits"]
