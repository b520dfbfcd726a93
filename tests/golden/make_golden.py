"""Regression fixtures on the reference's example meshes (exampleMeshes/*.off), produced by the oracle.

The reference has no test suite and records no expected values, so these fixtures hold the oracle's outputs on the
reference's own remeshed surfaces (irregular and obtuse triangles, saddle vertices, an open rim).  They pin the
oracle against drift (tests/test_golden.py, CPU) and compare the CUDA path with it on those surfaces (GPU).  The
walk that the reference's meshTesting.cpp:205-240 runs as its throughVertex check (torus_isotropic_remesh.off,
face 1, weights (0.4, 0.3, 0.3) moved by twice the vector to weights (0.7, 0.3, 0)) is one of the cases; the oracle
finds that it crosses two edges and no vertex.

Run where the reference tree is present (it is read here only; the tests use the .npz files):

    python tests/golden/make_golden.py REFERENCE_ROOT

Each tests/golden/<mesh>.npz holds the mesh as read from the .off file (vertex and face order kept, so face indices
are the reference's) and, per case, the inputs and the oracle's outputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from curvedspacesim_gb300 import meshes as ms  # noqa: E402

MESHES = {
    "torus_isotropic_remesh": dict(closed=True, through_vertex=True),
    "sphere_rb10_remesh": dict(closed=True, nve=True),
    "triangulatedElephant": dict(closed=True),
    "silo_omega0.012_R2.0": dict(closed=False),
}


def mean_edge(V, F):
    e = np.concatenate([V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 1]], V[F[:, 0]] - V[F[:, 2]]])
    return float(np.mean(np.linalg.norm(e, axis=1)))


def make(name, path, opts, seed):
    V, F = ms.read_off(path)
    OM = oracle.OracleMesh(V, F)
    rng = np.random.default_rng(seed)
    h = mean_edge(V, F)
    out = dict(V=V, F=F, mean_edge=h)
    n = 64
    f, b = ms.area_weighted_positions(V, F, n, rng)
    out.update(pos_face=f, pos_bary=b)
    if opts["closed"]:
        # whole-mesh distances (triangulatedMeshSpace::distance): 8 sources to every other point
        src = np.arange(8)
        off, tf, tb, d_all, ts_all, te_all = [0], [], [], [], [], []
        for s in src:
            o = np.array([i for i in range(n) if i != s])
            d, ts, te, _ = OM.distance(f[s], b[s], f[o], b[o])
            tf.append(f[o])
            tb.append(b[o])
            d_all.append(d)
            ts_all.append(ts)
            te_all.append(te)
            off.append(off[-1] + len(o))
        out.update(full_src=src, full_off=np.array(off, dtype=np.int32), full_tf=np.concatenate(tf),
                   full_tb=np.concatenate(tb), full_d=np.concatenate(d_all), full_ts=np.concatenate(ts_all),
                   full_te=np.concatenate(te_all))
        # reference patches (distanceWithSubmeshing) within a range of 4 mean edges
        r = 4.0 * h
        off, idx, mc = OM.candidates(f, b, r)
        d, ts, _ = OM.neighbor_distances(f, b, off, idx, mc, 1, r, np.inf)
        out.update(patch_range=r, patch_off=off, patch_idx=idx, patch_maxchord=mc, patch_d=d, patch_ts=ts)
    # walks with the velocity transported: displacements of 0.2 to 6 mean edges in the tangent plane
    nw = 128
    wf, wb = ms.area_weighted_positions(V, F, nw, rng)
    dirs = ms.tangent_velocities(V, F, wf, 1.0, rng)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    disp = dirs * (h * rng.uniform(0.2, 6.0, size=(nw, 1)))
    vel = ms.tangent_velocities(V, F, wf, 1.0, rng)
    out.update(walk_face=wf, walk_bary=wb, walk_disp=disp, walk_vel=vel)
    for bc in ((0,) if opts["closed"] else (0, 1, 2)):
        oracle.set_boundary(bc)
        fo, bo, do, to, st, cr = OM.transport(wf, wb, disp, vel[:, None, :])
        out.update({f"walk{bc}_face": fo, f"walk{bc}_bary": bo, f"walk{bc}_tv": to[:, 0], f"walk{bc}_status": st,
                    f"walk{bc}_cross": cr})
    oracle.set_boundary(0)
    if opts.get("through_vertex"):
        w1, w2 = np.array([[0.4, 0.3, 0.3]]), np.array([[0.7, 0.3, 0.0]])
        e1, e2 = OM.r3([1], w1)[0], OM.r3([1], w2)[0]
        dv = (2 * e2 - 2 * e1)[None, :]
        fo, bo, _, _, st, cr = OM.transport([1], w1, dv)
        out.update(tv_disp=dv, tv_face=fo, tv_bary=bo, tv_status=st, tv_cross=cr)
    if opts.get("nve"):
        # 20 velocity-Verlet steps, harmonic repulsion on reference patches, sigma from area fraction 0.4
        N = 60
        nf, nb = ms.area_weighted_positions(V, F, N, rng)
        nv = ms.tangent_velocities(V, F, nf, 0.1, rng)
        sigma = ms.sigma_for_area_fraction(ms.total_area(V, F), N, 0.4)
        prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma,
                        dt=0.005)
        fo, bo, vo, fco, _, err, _ = OM.simulate(0, 20, nf, nb, nv, np.zeros((N, 3)), prm)
        assert err == 0
        out.update(nve_face=nf, nve_bary=nb, nve_vel=nv, nve_sigma=sigma, nve_dt=0.005, nve_steps=20,
                   nve_face_out=fo, nve_bary_out=bo, nve_vel_out=vo, nve_force_out=fco)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return out


def main():
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py REFERENCE_ROOT  (the curvedSpaceSim source tree)")
    ref = sys.argv[1]
    oracle.build()
    for k, (name, opts) in enumerate(MESHES.items()):
        out = make(name, os.path.join(ref, "exampleMeshes", name + ".off"), opts, seed=100 + k)
        print(name, len(out["V"]), "vertices", len(out["F"]), "faces")


if __name__ == "__main__":
    main()
