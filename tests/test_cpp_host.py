"""The C++ host classes (include/curvedSpaceSimGPU.hpp) used like reference driver code, against the oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

from curvedspacesim_gb300 import meshes as ms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path):
    from curvedspacesim_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "host_classes_test")
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "host_classes_test.cpp"), "-I",
           os.path.join(ROOT, "include"), "-I", f"{cuda}/include", "-o", exe, lib, f"-L{cuda}/lib64", "-lcudart",
           f"-Wl,-rpath,{os.path.dirname(lib)}", f"-Wl,-rpath,{cuda}/lib64"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_host_classes_compile(tmp_path):
    if subprocess.run(["which", "g++"], capture_output=True).returncode != 0:
        pytest.skip("no g++")
    _compile(tmp_path)


@pytest.mark.gpu
def test_host_classes_match_oracle(tmp_path, oracle_mod):
    exe = _compile(tmp_path)
    V, F = ms.icosphere(3)
    rng = np.random.default_rng(5)
    n = 40
    f, b = ms.area_weighted_positions(V, F, n, rng)
    vel = ms.tangent_velocities(V, F, f, 0.1, rng)
    mp = tmp_path / "mesh.txt"
    pp = tmp_path / "parts.txt"
    with open(mp, "w") as fh:
        fh.write(f"{len(V)} {len(F)}\n")
        fh.write("\n".join(" ".join(repr(float(x)) for x in row) for row in V) + "\n")
        fh.write("\n".join(" ".join(str(int(x)) for x in row) for row in F) + "\n")
    with open(pp, "w") as fh:
        fh.write(f"{n}\n")
        for i in range(n):
            vals = " ".join(repr(float(x)) for x in (*b[i], *vel[i]))  # plain decimal text, round-trip exact
            fh.write(f"{int(f[i])} {vals}\n")
    run = subprocess.run([exe, str(mp), str(pp)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr[-2000:]
    out = run.stdout
    res = json.loads(out)
    OM = oracle_mod.OracleMesh(V, F)
    assert res["area"] == pytest.approx(OM.area, rel=1e-12)
    d, ts, _, _ = OM.distance(f[0], b[0], f[1:], b[1:])
    np.testing.assert_allclose(res["d"], d, rtol=1e-12)
    np.testing.assert_allclose(np.array(res["ts"]).reshape(-1, 3), ts, atol=1e-9)
    fo, bo, _, to, st, _ = OM.transport(f[1:2], b[1:2], vel[1:2], vel[1:2, None, :])
    assert res["walk"][0] == fo[0]
    np.testing.assert_allclose(res["walk"][1:4], bo[0], atol=1e-14)
    np.testing.assert_allclose(res["walk"][4:], to[0, 0], atol=1e-14)
    prm = OM.params(0, k=1.0 / 0.09, sigma=0.3, rng=0.0, submesh=0, max_dist=0.3, cutoff=0.3, dt=0.005)
    fs, bs, _, _, _, err, _ = OM.simulate(0, 10, f, b, vel, np.zeros((n, 3)), prm)
    assert err == 0
    pg = OM.r3(np.array(res["face"]), np.array(res["bary"]).reshape(-1, 3))
    np.testing.assert_allclose(pg, OM.r3(fs, bs), atol=1e-9)
    # gpuSimulation::performTimestepFromHost (cssg_system_step_host): the same device steps, state in and out of the
    # public vectors in one call
    assert res["face2"] == res["face"]
    np.testing.assert_allclose(res["bary2"], res["bary"], atol=1e-13)
    # gpuSimulation::findNeighbors (all-to-all): particle 0's candidates are all others in index order, with the
    # oracle's distances inside the 0.3 cutoff and +inf (printed -1) beyond it
    assert res["nb0"] == list(range(1, n))
    nd0 = np.array(res["nd0"])
    inside = d < 0.3
    np.testing.assert_allclose(nd0[inside], d[inside], rtol=1e-12)
    assert np.all(nd0[~inside] == -1)


def test_random_position_and_tangent_without_gpu(tmp_path):
    """cssg::randomPosition / randomVectorAtPosition (triangulatedMeshSpace.cpp:108-138), host-side: weights in the
    simplex, faces in range, vectors in the face's tangent plane with unit-variance Gaussian components."""
    if subprocess.run(["which", "g++"], capture_output=True).returncode != 0:
        pytest.skip("no g++")
    V, F = ms.icosphere(2)
    src = tmp_path / "rnd.cpp"
    vals = ", ".join(repr(float(x)) for x in V.reshape(-1))
    fids = ", ".join(str(int(x)) for x in F.reshape(-1))
    src.write_text(r'''
#include <cstdio>
#include "curvedSpaceSimGPU.hpp"
int main() {
    std::vector<double> V{''' + vals + r'''};
    std::vector<int> F{''' + fids + r'''};
    std::mt19937 rng(5);
    const int nF = (int)(F.size() / 3);
    double worstDot = 0, sum2 = 0, minW = 1, worstSum = 0;
    int badFace = 0;
    const int n = 20000;
    for (int i = 0; i < n; ++i) {
        cssg::meshPosition p;
        cssg::randomPosition(nF, p, rng);
        if (p.faceIndex < 0 || p.faceIndex >= nF) ++badFace;
        for (int c = 0; c < 3; ++c) minW = std::min(minW, p.x[c]);
        worstSum = std::max(worstSum, std::fabs(p.x[0] + p.x[1] + p.x[2] - 1.0));
        cssg::vector3 v;
        cssg::randomVectorAtPosition(V, F, p, v, rng);
        const double* a = &V[3 * F[3 * p.faceIndex]];
        const double* b = &V[3 * F[3 * p.faceIndex + 1]];
        const double* c = &V[3 * F[3 * p.faceIndex + 2]];
        double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        double nn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        double nl = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        worstDot = std::max(worstDot, std::fabs(v[0] * nn[0] + v[1] * nn[1] + v[2] * nn[2]) / nl);
        sum2 += v.squared_length();
    }
    std::printf("%d %.17g %.17g %.17g %.17g\n", badFace, minW, worstSum, worstDot, sum2 / n);
    return 0;
}
''')
    exe = str(tmp_path / "rnd")
    cuda = "/usr/local/cuda"
    subprocess.run(["g++", "-O2", "-std=c++17", str(src), "-I", os.path.join(ROOT, "include"), "-I", f"{cuda}/include",
                    "-o", exe], check=True, capture_output=True, text=True)
    bad, min_w, worst_sum, worst_dot, mean_sq = subprocess.run([exe], capture_output=True, text=True,
                                                                check=True).stdout.split()
    assert int(bad) == 0 and float(min_w) >= 0.0 and float(worst_sum) < 1e-15
    assert float(worst_dot) < 1e-12
    assert abs(float(mean_sq) - 2.0) < 0.1  # two unit-variance components


def test_pairs_to_neighbor_lists_without_gpu(tmp_path):
    """cssg::pairsToNeighborLists: pair records grouped into simpleModel's neighbour lists (screened pairs decoded,
    their distance +inf)."""
    if subprocess.run(["which", "g++"], capture_output=True).returncode != 0:
        pytest.skip("no g++")
    src = tmp_path / "nl.cpp"
    src.write_text(r'''
#include <cstdio>
#include "curvedSpaceSimGPU.hpp"
int main() {
    int i[] = {0, 0, 2, 2, 2};
    int j[] = {1, 2, 0, -2, 3};
    double d[] = {0.1, 0.2, 0.2, 0.9, INFINITY};
    double t[15];
    for (int k = 0; k < 15; ++k) t[k] = k;
    std::vector<std::vector<int>> nb;
    std::vector<std::vector<cssg::vector3>> nv;
    std::vector<std::vector<double>> nd;
    cssg::pairsToNeighborLists(4, 5, i, j, d, t, nb, nv, nd);
    std::printf("%zu %zu %zu %zu %d %d %d %g %g %g %g\n", nb.size(), nb[0].size(), nb[1].size(), nb[2].size(), nb[2][0],
                nb[2][1], nb[2][2], nd[0][1], nd[2][1], nv[2][1][0], nv[0][1][2]);
    return 0;
}
''')
    exe = str(tmp_path / "nl")
    cuda = "/usr/local/cuda"
    subprocess.run(["g++", "-O2", "-std=c++17", str(src), "-I", os.path.join(ROOT, "include"), "-I", f"{cuda}/include",
                    "-o", exe], check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert out[:7] == ["4", "2", "0", "3", "0", "1", "3"]
    assert float(out[7]) == 0.2 and out[8] == "inf" and float(out[9]) == 9.0 and float(out[10]) == 5.0
