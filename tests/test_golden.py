"""Regression fixtures on the reference's example meshes (tests/golden/*.npz, made by tests/golden/make_golden.py
from exampleMeshes/*.off with the oracle): the oracle must reproduce them (CPU), and the CUDA path must match them
(GPU) on remeshed surfaces with irregular and obtuse triangles, saddle vertices (the elephant, the torus) and an open
rim (the silo)."""
import glob
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
NAMES = [os.path.basename(p)[:-4] for p in FIXTURES]
CLOSED = [n for n in NAMES if not n.startswith("silo")]


def load(name):
    return dict(np.load(os.path.join(HERE, "golden", name + ".npz")))


def test_fixtures_present():
    assert {"torus_isotropic_remesh", "sphere_rb10_remesh", "triangulatedElephant",
            "silo_omega0.012_R2.0"} <= set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_fixture(oracle_mod, name):
    z = load(name)
    OM = oracle_mod.OracleMesh(z["V"], z["F"])
    if "full_d" in z:
        off = z["full_off"]
        f, b = z["pos_face"], z["pos_bary"]
        for q, s in enumerate(z["full_src"]):
            a, e = off[q], off[q + 1]
            d, ts, te, _ = OM.distance(f[s], b[s], z["full_tf"][a:e], z["full_tb"][a:e])
            np.testing.assert_allclose(d, z["full_d"][a:e], rtol=1e-14, atol=0)
            np.testing.assert_allclose(ts, z["full_ts"][a:e], atol=1e-13)
            np.testing.assert_allclose(te, z["full_te"][a:e], atol=1e-13)
        r = float(z["patch_range"])
        d, ts, _ = OM.neighbor_distances(f, b, z["patch_off"], z["patch_idx"], z["patch_maxchord"], 1, r, math.inf)
        np.testing.assert_allclose(d, z["patch_d"], rtol=1e-14, atol=0)
        np.testing.assert_allclose(ts, z["patch_ts"], atol=1e-13)
    for bc in (0, 1, 2):
        if f"walk{bc}_face" not in z:
            continue
        oracle_mod.set_boundary(bc)
        try:
            fo, bo, _, to, st, cr = OM.transport(z["walk_face"], z["walk_bary"], z["walk_disp"],
                                                 z["walk_vel"][:, None, :])
        finally:
            oracle_mod.set_boundary(0)
        np.testing.assert_array_equal(st, z[f"walk{bc}_status"])
        np.testing.assert_array_equal(fo, z[f"walk{bc}_face"])
        np.testing.assert_array_equal(cr, z[f"walk{bc}_cross"])
        np.testing.assert_array_equal(bo, z[f"walk{bc}_bary"])
        np.testing.assert_array_equal(to[:, 0], z[f"walk{bc}_tv"])


def test_through_vertex_case_of_the_reference(oracle_mod):
    """meshTesting.cpp:205-240: face 1 of torus_isotropic_remesh.off, weights (0.4, 0.3, 0.3), moved by twice the
    vector to weights (0.7, 0.3, 0)."""
    z = load("torus_isotropic_remesh")
    OM = oracle_mod.OracleMesh(z["V"], z["F"])
    w1, w2 = np.array([[0.4, 0.3, 0.3]]), np.array([[0.7, 0.3, 0.0]])
    dv = 2 * OM.r3([1], w2) - 2 * OM.r3([1], w1)
    np.testing.assert_array_equal(dv, z["tv_disp"])
    fo, bo, _, _, st, cr = OM.transport([1], w1, dv)
    assert st[0] == 0
    assert fo[0] == z["tv_face"][0] and cr[0] == z["tv_cross"][0]
    np.testing.assert_array_equal(bo, z["tv_bary"])
    assert np.all(bo >= -1e-12) and abs(bo.sum() - 1) < 1e-12


# ---- the CUDA path against the fixtures ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("name", CLOSED)
def test_gpu_whole_mesh_distances_match_fixture(gpu, name):
    api, ctx = gpu
    z = load(name)
    M = api.Mesh(z["V"], z["F"])
    f, b, src, off = z["pos_face"], z["pos_bary"], z["full_src"], z["full_off"]
    d, ts, te, st = api.distance_batch(ctx, M, f[src], b[src], off, z["full_tf"], z["full_tb"], submesh=False)
    assert np.all(st == 0)
    np.testing.assert_allclose(d, z["full_d"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(ts, z["full_ts"], atol=1e-9)
    np.testing.assert_allclose(te, z["full_te"], atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CLOSED)
def test_gpu_patch_distances_match_fixture(gpu, name):
    api, ctx = gpu
    z = load(name)
    M = api.Mesh(z["V"], z["F"])
    f, b, idx, r = z["pos_face"], z["pos_bary"], z["patch_idx"], float(z["patch_range"])
    d, ts, te, st = api.distance_batch(ctx, M, f, b, z["patch_off"], f[idx], b[idx], submesh=True, max_dist=r,
                                       threshold=z["patch_maxchord"], cutoff=math.inf)
    assert np.all(st == 0)
    do = np.where(np.isfinite(z["patch_d"]), z["patch_d"], 2 * r)
    np.testing.assert_allclose(d, do, rtol=1e-12, atol=1e-13)
    fin = np.isfinite(z["patch_d"])
    np.testing.assert_allclose(ts[fin], z["patch_ts"][fin], atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("name,bc", [(n, 0) for n in NAMES] + [("silo_omega0.012_R2.0", 1),
                                                                 ("silo_omega0.012_R2.0", 2)])
def test_gpu_walks_match_fixture(gpu, name, bc):
    """Edge-only walks bitwise, walks through interior vertices (acos/sin/cos) within 1e-9; on the open silo with the
    closed-mesh rule (bc 0) the walks that reach the rim must report it (status 1) as the oracle does."""
    api, ctx = gpu
    z = load(name)
    M = api.Mesh(z["V"], z["F"], boundary={0: "closed", 1: "tangential", 2: "absorbing"}[bc])
    fg, bg, _, tg, sg, _ = api.transport_batch(ctx, M, z["walk_face"], z["walk_bary"], z["walk_disp"],
                                               z["walk_vel"][:, None, :])
    np.testing.assert_array_equal(sg, z[f"walk{bc}_status"])
    ok = sg == 0
    np.testing.assert_array_equal(fg[ok], z[f"walk{bc}_face"][ok])
    exact = ok & ((z[f"walk{bc}_cross"] >> 16) == 0)
    np.testing.assert_array_equal(bg[exact], z[f"walk{bc}_bary"][exact])
    np.testing.assert_array_equal(tg[exact, 0], z[f"walk{bc}_tv"][exact])
    np.testing.assert_allclose(bg[ok], z[f"walk{bc}_bary"][ok], atol=1e-9)
    np.testing.assert_allclose(tg[ok, 0], z[f"walk{bc}_tv"][ok], atol=1e-9)


@pytest.mark.gpu
def test_gpu_through_vertex_case_of_the_reference(gpu):
    api, ctx = gpu
    z = load("torus_isotropic_remesh")
    M = api.Mesh(z["V"], z["F"])
    fg, bg, _, _, sg, _ = api.transport_batch(ctx, M, [1], np.array([[0.4, 0.3, 0.3]]), z["tv_disp"])
    assert sg[0] == 0 and fg[0] == z["tv_face"][0]
    np.testing.assert_array_equal(bg, z["tv_bary"])


@pytest.mark.gpu
def test_gpu_nve_on_remeshed_sphere_matches_fixture(gpu):
    """20 velocity-Verlet steps with harmonic repulsion on reference patches (sigma from area fraction 0.4)."""
    api, ctx = gpu
    z = load("sphere_rb10_remesh")
    n, sigma, dt = len(z["nve_face"]), float(z["nve_sigma"]), float(z["nve_dt"])
    M = api.Mesh(z["V"], z["F"])
    p = api.make_params("nve", "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=sigma, submesh=True,
                        max_dist=sigma, cutoff=sigma, dt=dt)
    S = api.System(ctx, M, n, p)
    S.set_state(z["nve_face"], z["nve_bary"], z["nve_vel"], np.zeros((n, 3)))
    S.step(int(z["nve_steps"]), graph=True)
    bits, cnt = S.check()
    assert bits == 0, cnt
    fg, bg, vg, fcg = S.get_state()
    from curvedspacesim_gb300 import meshes as ms
    np.testing.assert_allclose(ms.bary_to_r3(z["V"], z["F"], fg, bg),
                               ms.bary_to_r3(z["V"], z["F"], z["nve_face_out"], z["nve_bary_out"]), atol=1e-9)
    np.testing.assert_allclose(vg, z["nve_vel_out"], atol=1e-9)
    np.testing.assert_allclose(fcg, z["nve_force_out"], atol=1e-8)
