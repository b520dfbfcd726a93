"""cssg_distance_batch_noalloc (fixed file-scope scratch, no allocation) against cssg_distance_batch, both called
through the C ABI on the same inputs, two calls in a row (the second reuses the scratch the first left behind), and
against the FP64 oracle on a sample of the sources."""
import ctypes

import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # both entry points run the same kernels; only the number of scratch slots may differ


def _P(t):
    return ctypes.c_void_p(t.data_ptr())


def _call(L, name, ctx, mesh, args, ns, m, dev, torch):
    d = torch.full((max(m, 1),), -1.0, dtype=torch.float64, device=dev)
    ts = torch.zeros((max(m, 1), 3), dtype=torch.float64, device=dev)
    te = torch.zeros((max(m, 1), 3), dtype=torch.float64, device=dev)
    st = torch.full((ns,), -1, dtype=torch.int32, device=dev)
    stats = torch.zeros((ns, 4), dtype=torch.int64, device=dev)
    sf, sb, co, cf, cb, submesh, max_dist, cutoff = args
    rc = getattr(L, name)(ctx.h, mesh.h, ns, _P(sf), _P(sb), _P(co), _P(cf), _P(cb), submesh, max_dist, None, cutoff,
                          _P(d), _P(ts), _P(te), _P(st), _P(stats))
    assert rc == 0, (name, rc, L.cssg_last_error().decode())
    ctx.synchronize()
    return d.cpu().numpy()[:m], ts.cpu().numpy()[:m], te.cpu().numpy()[:m], st.cpu().numpy()


@pytest.mark.parametrize("submesh,r", [(0, None), (1, 0.5), (1, 1.5)])
def test_noalloc_matches_distance_batch(submesh, r, oracle_mod):
    """Two calls in a row against cssg_distance_batch and against the FP64 oracle.  With r = 1.5 one propagation slot
    needs a few MiB, so the fixed scratch holds fewer slots than the 16 per SM the allocating call uses: the path
    that runs with fewer slots is exercised."""
    import torch
    from curvedspacesim_gb300 import _lib, api
    L = _lib.load()
    ctx = api.Context(0)
    dev = "cuda:0"
    V, F = ms.torus(100, 50, 3.0, 1.0)
    mesh = api.Mesh(V, F)
    rng = np.random.default_rng(7)
    n = 600
    f, b = ms.area_weighted_positions(V, F, n, rng)
    pos = ms.bary_to_r3(V, F, f, b)
    # candidates: chord < r (every other particle for the whole-mesh case on a few sources)
    if submesh:
        ns = n if r < 1 else 200
        lists = [np.nonzero((np.sum((pos - pos[i]) ** 2, axis=1) < r * r) & (np.arange(n) != i))[0]
                 for i in range(ns)]
        max_dist, cutoff = r, r
    else:
        ns = 8
        lists = [np.array([j for j in range(n) if j != i]) for i in range(ns)]
        max_dist, cutoff = 1.0, float("inf")
    off = np.zeros(ns + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(x) for x in lists])
    idx = np.concatenate(lists).astype(np.int64)
    m = int(off[-1])
    args = (torch.tensor(f[:ns], dtype=torch.int32, device=dev),
            torch.tensor(b[:ns], dtype=torch.float64, device=dev),
            torch.tensor(off, device=dev),
            torch.tensor(f[idx], dtype=torch.int32, device=dev),
            torch.tensor(b[idx], dtype=torch.float64, device=dev),
            submesh, max_dist, cutoff)
    if submesh:
        # the scratch must hold fewer slots than the allocating call's min(16 x SMs, sources) in the large case
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        if r > 1:
            caps_slot = _slot_bytes_estimate(mesh, max(len(x) for x in lists), max_dist)
            assert (64 << 20) // caps_slot < min(16 * sms, ns), caps_slot
    with ctx.use():
        ref = _call(L, "cssg_distance_batch", ctx, mesh, args, ns, m, dev, torch)
        for _ in range(2):
            got = _call(L, "cssg_distance_batch_noalloc", ctx, mesh, args, ns, m, dev, torch)
            assert np.all(got[3] == 0) and np.all(ref[3] == 0)
            fin = np.isfinite(ref[0])
            assert np.array_equal(fin, np.isfinite(got[0]))
            np.testing.assert_allclose(got[0][fin], ref[0][fin], rtol=RTOL, atol=0)
            np.testing.assert_allclose(got[1][fin], ref[1][fin], rtol=0, atol=1e-12)
            np.testing.assert_allclose(got[2][fin], ref[2][fin], rtol=0, atol=1e-12)
    # against the FP64 oracle (the CPU restatement of triangulatedMeshSpace::distance / distanceWithSubmeshing)
    OM = oracle_mod.OracleMesh(V, F)
    for q in range(0, ns, max(1, ns // 40)):
        a, e = off[q], off[q + 1]
        do, tso, teo, _ = OM.distance(f[q], b[q], f[idx[a:e]], b[idx[a:e]], submesh=bool(submesh),
                                      max_dist=max_dist, cutoff=cutoff)
        fin = np.isfinite(do)
        assert np.array_equal(fin, np.isfinite(got[0][a:e]))
        np.testing.assert_allclose(got[0][a:e][fin], do[fin], rtol=1e-12, atol=1e-13)
        np.testing.assert_allclose(got[1][a:e][fin], tso[fin], atol=1e-9)


def _slot_bytes_estimate(mesh, max_targets, reach):
    """Bytes of one propagation slot by the distance calls' sizing rule (the table capacities and record sizes of
    geodesic.cu), for the assertion that the fixed scratch caps the slot count."""
    import math
    est = min(mesh.nF, int(1.3 * math.pi * (reach + mesh_mean_edge(mesh)) ** 2 / (mesh.area / mesh.nF)) + 32)
    CW = min(1 << 22, 16 * est + 1024)
    CLOG = min(1 << 22, 32 * max(32, max_targets) + 16 * est + 1024)
    return 64 * (2 * CW + CLOG)  # the window frontiers and the log alone


def mesh_mean_edge(mesh):
    E = np.concatenate([mesh.V[mesh.F[:, k]] - mesh.V[mesh.F[:, (k + 1) % 3]] for k in range(3)])
    return float(np.linalg.norm(E, axis=1).mean())


def test_noalloc_rejects_oversize_slot():
    """A whole-mesh call on a large mesh needs one slot larger than the fixed scratch: rejected, nothing launched."""
    import torch
    from curvedspacesim_gb300 import _lib, api
    L = _lib.load()
    ctx = api.Context(0)
    dev = "cuda:0"
    V, F = ms.torus(400, 200, 3.0, 1.0)  # 160,000 faces: the whole-mesh tables exceed 64 MiB per slot
    mesh = api.Mesh(V, F)
    rng = np.random.default_rng(1)
    f, b = ms.area_weighted_positions(V, F, 4, rng)
    args = (torch.tensor(f[:1], dtype=torch.int32, device=dev), torch.tensor(b[:1], dtype=torch.float64, device=dev),
            torch.tensor(np.array([0, 3], dtype=np.int32), device=dev),
            torch.tensor(f[1:], dtype=torch.int32, device=dev), torch.tensor(b[1:], dtype=torch.float64, device=dev))
    d = torch.zeros(3, dtype=torch.float64, device=dev)
    ts = torch.zeros((3, 3), dtype=torch.float64, device=dev)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    with ctx.use():
        rc = L.cssg_distance_batch_noalloc(ctx.h, mesh.h, 1, *[_P(a) for a in args], 0, 1.0, None, float("inf"),
                                           _P(d), _P(ts), None, _P(st), None)
    assert rc == 4  # CSSG_ERR_CAPACITY
    assert "fixed scratch" in L.cssg_last_error().decode()
