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
