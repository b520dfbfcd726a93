"""Randomised properties of the oracle's geodesics and walk on irregular closed surfaces (bumpy icospheres with
random radial noise: obtuse triangles and saddle vertices), beyond the fixed-seed cases of test_oracle.py:
symmetry d(a, b) = d(b, a), chord <= d, the triangle inequality, unit tangents, and walk reversibility."""
import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402


def _surface(seed, amplitude):
    V, F = ms.icosphere(3)
    rng = np.random.default_rng(seed)
    V = V * (1.0 + amplitude * rng.uniform(-1.0, 1.0, size=(len(V), 1)))
    return V, F


@settings(max_examples=30, deadline=None)
@given(seed=st.integers(0, 10_000), amplitude=st.floats(0.0, 0.15), npts=st.integers(3, 7))
def test_distances_symmetric_bounded_triangle(oracle_mod, seed, amplitude, npts):
    V, F = _surface(seed, amplitude)
    OM = oracle_mod.OracleMesh(V, F)
    rng = np.random.default_rng(seed + 1)
    f, b = ms.area_weighted_positions(V, F, npts, rng)
    P = OM.r3(f, b)
    D = np.zeros((npts, npts))
    for s in range(npts):
        o = [i for i in range(npts) if i != s]
        d, ts, te, _ = OM.distance(f[s], b[s], f[o], b[o])
        D[s, o] = d
        np.testing.assert_allclose(np.linalg.norm(ts, axis=1), 1.0, atol=1e-12)
        np.testing.assert_allclose(np.linalg.norm(te, axis=1), 1.0, atol=1e-12)
    np.testing.assert_allclose(D, D.T, rtol=1e-10, atol=1e-12)
    chord = np.linalg.norm(P[:, None] - P[None], axis=2)
    assert np.all(D >= chord - 1e-12)
    for i in range(npts):
        for j in range(npts):
            assert np.all(D[i, j] <= D[i] + D[:, j] + 1e-10)


@settings(max_examples=30, deadline=None)
@given(seed=st.integers(0, 10_000), amplitude=st.floats(0.0, 0.15), length=st.floats(0.01, 0.4))
def test_walk_there_and_back(oracle_mod, seed, amplitude, length):
    """Walk a tangent displacement, then the transported displacement reversed: back at the start when the walk
    crossed edges only (vertex crossings follow the reference's heuristic and need not be reversible)."""
    V, F = _surface(seed, amplitude)
    OM = oracle_mod.OracleMesh(V, F)
    rng = np.random.default_rng(seed + 2)
    n = 40
    f, b = ms.area_weighted_positions(V, F, n, rng)
    N = ms.face_normals(V, F)[f]
    raw = rng.standard_normal((n, 3))
    disp = raw - (raw * N).sum(1, keepdims=True) * N
    disp *= length / np.linalg.norm(disp, axis=1, keepdims=True)
    f2, b2, _, tv, s2, c2 = OM.transport(f, b, disp, disp[:, None, :])
    assert np.all(s2 == 0)
    np.testing.assert_allclose(np.linalg.norm(tv[:, 0], axis=1), length, rtol=1e-12)
    f3, b3, _, _, s3, c3 = OM.transport(f2, b2, -tv[:, 0])
    assert np.all(s3 == 0)
    edge_only = ((c2 >> 16) == 0) & ((c3 >> 16) == 0)
    err = np.linalg.norm(OM.r3(f3, b3) - OM.r3(f, b), axis=1)
    assert np.all(err[edge_only] < 1e-9), err[edge_only].max()
