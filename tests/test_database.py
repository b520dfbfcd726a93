"""State persistence (simpleModelDatabase datasets, flat binary layout shared by the C++ header and Python)."""
import os
import subprocess

import numpy as np
import pytest

from curvedspacesim_gb300 import database as dbm
from curvedspacesim_gb300 import meshes as ms

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _state(n, seed):
    V, F = ms.icosphere(2)
    rng = np.random.default_rng(seed)
    f, b = ms.area_weighted_positions(V, F, n, rng)
    return V, F, f, b, rng.standard_normal((n, 3)), rng.standard_normal((n, 3))


def test_python_round_trip(tmp_path):
    n = 37
    fn = str(tmp_path / "traj.cssgdb")
    db = dbm.SimpleModelDatabase(n, fn, dbm.REPLACE, save_velocities=True, save_forces=True)
    states = [_state(n, s) for s in range(3)]
    for k, (V, F, f, b, v, fo) in enumerate(states):
        db.write_state(0.5 * k, ms.bary_to_r3(V, F, f, b), b, f, v, fo)
    db2 = dbm.SimpleModelDatabase(n, fn, dbm.READONLY)
    assert db2.velocity and db2.force and not db2.type
    assert db2.current_number_of_records() == 3
    for k, (V, F, f, b, v, fo) in enumerate(states):
        r = db2.read_state(k)
        assert r["time"] == 0.5 * k
        assert np.array_equal(r["faceIndex"], f) and np.array_equal(r["barycentricPosition"], b)
        assert np.array_equal(r["velocity"], v) and np.array_equal(r["force"], fo)
    with pytest.raises(ValueError):
        dbm.SimpleModelDatabase(n + 1, fn, dbm.READONLY)
    with pytest.raises(IndexError):
        db2.read_state(3)


def test_cpp_header_reads_python_records(tmp_path):
    """The C++ reader (curvedSpaceSimDatabase.hpp) sees the same records the Python writer stored."""
    if subprocess.run(["which", "g++"], capture_output=True).returncode != 0:
        pytest.skip("no g++")
    n = 11
    fn = str(tmp_path / "traj.cssgdb")
    db = dbm.SimpleModelDatabase(n, fn, dbm.REPLACE, save_velocities=True)
    V, F, f, b, v, _ = _state(n, 5)
    db.write_state(2.25, ms.bary_to_r3(V, F, f, b), b, f, v)
    src = tmp_path / "rd.cpp"
    src.write_text(r'''
#include <cstdio>
#include "curvedSpaceSimDatabase.hpp"
int main(int argc, char** argv) {
    cssg::simpleModelDatabase db(11, argv[1], cssg::fileMode::readonly);
    std::vector<double> b, v, f; std::vector<int> face, t;
    double time = db.readState(0, b, face, v, f, t);
    std::printf("%lu %.17g %d %.17g %.17g\n", db.currentNumberOfRecords(), time, face[3], b[7], v[10]);
    cssg::simpleModelDatabase w(11, argv[1], cssg::fileMode::readwrite);
    std::vector<double> r3(33, 1.0);
    w.writeState(r3, b, face, v, f, t, 3.5);
    return 0;
}
''')
    exe = str(tmp_path / "rd")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    out = subprocess.run([exe, fn], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == 1 and float(out[1]) == 2.25 and int(out[2]) == f[3]
    assert float(out[3]) == b.reshape(-1)[7] and float(out[4]) == v.reshape(-1)[10]
    db2 = dbm.SimpleModelDatabase(n, fn, dbm.READONLY)
    assert db2.current_number_of_records() == 2 and db2.read_state(1)["time"] == 3.5


def test_value_vector_database_python_and_cpp(tmp_path):
    """valueVectorDatabase: records written in Python read back in Python and by the C++ header, and records
    appended by the C++ header read back in Python."""
    fn = str(tmp_path / "energies.cssgvv")
    db = dbm.ValueVectorDatabase(fn, 5, dbm.REPLACE)
    rng = np.random.default_rng(3)
    rows = [(0.25 * k, rng.standard_normal(5)) for k in range(3)]
    for v, vec in rows:
        db.write_state(v, vec)
    db2 = dbm.ValueVectorDatabase(fn, 5, dbm.READONLY)
    assert db2.current_number_of_records() == 3
    for k, (v, vec) in enumerate(rows):
        rv, rvec = db2.read_state(k)
        assert rv == v and np.array_equal(rvec, vec)
    with pytest.raises(ValueError):
        dbm.ValueVectorDatabase(fn, 6, dbm.READONLY)
    if subprocess.run(["which", "g++"], capture_output=True).returncode != 0:
        pytest.skip("no g++")
    src = tmp_path / "vv.cpp"
    src.write_text(r'''
#include <cstdio>
#include "curvedSpaceSimDatabase.hpp"
int main(int argc, char** argv) {
    cssg::valueVectorDatabase db(argv[1], 5, cssg::fileMode::readwrite);
    db.readState(2);
    std::printf("%lu %.17g %.17g\n", db.currentNumberOfRecords(), db.valueVector[0], db.dataVector[4]);
    std::vector<double> v{1, 2, 3, 4, 5};
    db.writeState(9.5, v);
    return 0;
}
''')
    exe = str(tmp_path / "vv")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    out = subprocess.run([exe, fn], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == 3 and float(out[1]) == rows[2][0] and float(out[2]) == rows[2][1][4]
    rv, rvec = dbm.ValueVectorDatabase(fn, 5, dbm.READONLY).read_state(3)
    assert rv == 9.5 and np.array_equal(rvec, [1, 2, 3, 4, 5])
