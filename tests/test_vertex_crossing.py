"""Walks that cross an interior vertex and continue (triangulatedMeshSpace.cpp:448-564 with
updateForVertexIntersection, :566-611).

The reference passes its loop's vertexPositions to updateForVertexIntersection BY VALUE (.h:106-110), so after a
vertex crossing the caller keeps the previous face's triangle: the next pass computes the target's barycentric
weights against that old triangle (:478) and reads them in the new face (clampAndUpdatePosition,
meshUtilities.cpp:170-182).  Only an edge crossing (updateForEdgeIntersection, by reference) refreshes it.  The
oracle and the CUDA walk reproduce this.  On a flat grid the straightest continuation through a vertex is the
straight line, so the reference loop can be restated here in a few lines of numpy (no unfolding rotations, the
through-vertex face is the one that contains the continued ray); the oracle is pinned against that restatement."""
import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms


def _bary(tri, x):
    v0, v1, v2 = tri[1] - tri[0], tri[2] - tri[0], x - tri[0]
    d00, d01, d11 = v0 @ v0, v0 @ v1, v1 @ v1
    d20, d21 = v2 @ v0, v2 @ v1
    den = d00 * d11 - d01 * d01
    v = (d11 * d20 - d01 * d21) / den
    w = (d00 * d21 - d01 * d20) / den
    return np.array([1.0 - v - w, v, w])


def _construct(tri, b):
    return (b[0] * tri[0] + b[1] * tri[1] + b[2] * tri[2]) / (b[0] + b[1] + b[2])


def _clamp_below(b, tol=1e-11):
    b = np.maximum(b, tol)
    return b / b.sum()


def _clamp_near(b, tol=1e-13):
    b = b.copy()
    b[(b > -tol) & (b < tol)] = tol
    return b / b.sum()


def _hits(s, e):
    """meshUtilities.cpp:229-281: crossings of the segment s->e (barycentric) with edges v1v2, v2v3, v3v1."""
    out = []
    den = s[0] + s[1] - e[0] - e[1]
    if den != 0:
        t1 = (-e[1] + e[1] * s[0] + s[1] - e[0] * s[1]) / den
        t2 = (-1 + s[0] + s[1]) / den
        out.append((0, 1, 0 <= t1 <= 1 and 0 <= t2 <= 1, s + t2 * (e - s)))
    else:
        out.append((0, 1, False, None))
    den = -e[0] + s[0]
    if den != 0:
        t1 = -(e[0] - s[0] + e[1] * s[0] - e[0] * s[1]) / den
        t2 = s[0] / den
        out.append((1, 2, 0 <= t1 <= 1 and 0 <= t2 <= 1, s + t2 * (e - s)))
    else:
        out.append((1, 2, False, None))
    den = s[1] - e[1]
    if den != 0:
        t1 = (e[0] * s[1] - e[1] * s[0]) / den
        t2 = s[1] / den
        out.append((2, 0, 0 <= t1 <= 1 and 0 <= t2 <= 1, s + t2 * (e - s)))
    else:
        out.append((2, 0, False, None))
    return out


def reference_walk_flat(V, F, f, b, disp):
    """The reference loop on a flat mesh (no rotations), with its by-value vertexPositions."""
    tri = lambda g: V[F[g]]
    sb = np.array(b, dtype=np.float64)
    sp = _construct(tri(f), sb)
    target = sp + disp
    frame = tri(f)  # vertexPositions of the reference loop
    last = None
    for _ in range(1000):
        tb = _clamp_near(_bary(frame, target))
        target = _construct(tri(f), tb)
        sb = _clamp_below(sb)
        sp = _construct(tri(f), sb)
        disp = target - sp
        if np.all(tb >= 0):
            return f, tb
        vl = F[f]
        hit = [(vl[a], vl[c], ip) for a, c, ok, ip in _hits(sb, tb)
               if ok and not (last is not None and {vl[a], vl[c]} == last)]
        assert hit, "no crossing"
        ip = _clamp_below(hit[-1][2])
        ep = _construct(tri(f), ip)
        to_i = ep - sp
        sb, sp = ip, ep
        if len(hit) == 2:
            v = hit[0][0]  # involvedVertex[0]: first vertex of the first edge hit
            heading = to_i / np.linalg.norm(to_i)  # flat: the straightest continuation is the straight line
            disp = heading * np.linalg.norm(disp)  # remaining length measured before moving to the vertex
            target = sp + disp
            probe = V[v] + 1e-7 * heading
            g = [h for h in np.nonzero((F == v).any(axis=1))[0] if np.all(_bary(tri(h), probe) >= 0)]
            assert len(g) == 1
            f = int(g[0])
            sb = _bary(tri(f), sp)
            last = None  # vertexPositions (frame) is NOT refreshed
        else:
            a, c = hit[0][0], hit[0][1]
            g = [h for h in np.nonzero((F == a).any(axis=1) & (F == c).any(axis=1))[0] if h != f]
            f = int(g[0])
            frame = tri(f)
            sb = _bary(tri(f), sp)
            last = {a, c}
    raise AssertionError("walk did not end")


def vertex_crossing_cases(n_try=3000, seed=0):
    """Walks on a flat 6x6 grid of unit squares aimed through the interior vertex (3, 3)."""
    V, F = ms.planar_grid(6, 6.0)
    rng = np.random.default_rng(seed)
    fs, bs, ds = [], [], []
    for _ in range(n_try):
        f = int(rng.integers(len(F)))
        b = rng.random(3)
        b /= b.sum()
        P = _construct(V[F[f]], b)
        d = np.array([3.0, 3.0, 0.0]) - P
        L = np.linalg.norm(d)
        if not 0.3 < L < 2.5:
            continue
        t = P + 1.6 * d
        if not (0.2 < t[0] < 5.8 and 0.2 < t[1] < 5.8):
            continue
        fs.append(f)
        bs.append(b)
        ds.append(1.6 * d)
    return V, F, np.array(fs, dtype=np.int32), np.array(bs), np.array(ds)


def test_oracle_vertex_crossing_keeps_the_previous_frame(oracle_mod):
    V, F, f, b, d = vertex_crossing_cases()
    M = oracle_mod.OracleMesh(V, F)
    fo, bo, _, _, st, cr = M.transport(f, b, d, d[:, None, :])
    # a ray that grazes a vertex can find no crossing after the clamps (the reference throws there, :534-541); the
    # comparison uses the walks that end normally
    ok = st == 0
    assert ok.mean() > 0.99
    f, b, d, fo, bo, cr = f[ok], b[ok], d[ok], fo[ok], bo[ok], cr[ok]
    crossed = (cr >> 16) > 0
    assert crossed.sum() >= 20  # interior vertex crossings (counted in the high half)
    moved_off_line = 0
    for k in np.nonzero(crossed)[0]:
        g, tb = reference_walk_flat(V, F, int(f[k]), b[k], d[k])
        assert g == fo[k]
        np.testing.assert_allclose(bo[k], tb, atol=1e-9)
        straight = _construct(V[F[f[k]]], b[k]) + d[k]
        moved_off_line += np.linalg.norm(_construct(V[F[g]], tb) - straight) > 1e-6
    # the old frame moves most of these walks away from the straight-line end point (the reference's behaviour)
    assert moved_off_line >= crossed.sum() // 2
    # walks without a vertex crossing end on the straight line
    P = np.array([_construct(V[F[g]], x) for g, x in zip(fo[~crossed], bo[~crossed])])
    S = np.array([_construct(V[F[g]], x) for g, x in zip(f[~crossed], b[~crossed])]) + d[~crossed]
    np.testing.assert_allclose(P, S, atol=1e-12)


@pytest.mark.gpu
def test_gpu_vertex_crossing_matches_oracle(oracle_mod, gpu):
    api, ctx = gpu
    V, F, f, b, d = vertex_crossing_cases()
    M = oracle_mod.OracleMesh(V, F)
    fo, bo, do, tvo, st, cr = M.transport(f, b, d, d[:, None, :])
    mesh = api.Mesh(V, F)
    fg, bg, dg, tvg, sg, crg = api.transport_batch(ctx, mesh, f, b, d, d[:, None, :])
    np.testing.assert_array_equal(sg, st)
    ok = st == 0
    assert ((cr[ok] >> 16) > 0).sum() >= 20
    np.testing.assert_array_equal(fg[ok], fo[ok])
    np.testing.assert_allclose(bg[ok], bo[ok], atol=1e-12)
    np.testing.assert_allclose(tvg[ok, 0], tvo[ok, 0], atol=1e-12)
