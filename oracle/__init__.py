"""ctypes front end of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs as the
checker or the timed CPU baseline.  The product path never imports it.  Parity against the reference itself is
unpinned (CGAL is absent here; the reference ships no golden vectors); see the header of oracle.cpp for what pins it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

ST_NAMES = {0: "ok", 1: "border", 2: "nan", 3: "vertex", 4: "iteration cap", 5: "no intersection", 6: "capacity"}


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "oracle.cpp")):
        subprocess.run(["bash", os.path.join(_HERE, "build.sh")], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        I = ctypes.c_int
        D = ctypes.c_double
        LL = ctypes.c_longlong
        L.oracle_mesh_create.restype = P
        L.oracle_mesh_create.argtypes = [P, I, P, I]
        L.oracle_mesh_destroy.argtypes = [P]
        L.oracle_mesh_area.restype = D
        L.oracle_mesh_area.argtypes = [P]
        L.oracle_mesh_bbox.argtypes = [P, P]
        L.oracle_angle_sums.argtypes = [P, P]
        L.oracle_positions_r3.argtypes = [P, I, P, P, P]
        L.oracle_transport.argtypes = [P, I, P, P, P, P, I, I, P, P]
        L.oracle_patch.restype = I
        L.oracle_patch.argtypes = [P, I, P, I, P, D, P, I]
        L.oracle_distance.argtypes = [P, I, P, I, P, P, I, D, D, D, P, P, P, P]
        L.oracle_distance_bruteforce.restype = D
        L.oracle_distance_bruteforce.argtypes = [P, I, P, I, P, P, I, I]
        L.oracle_candidates.restype = LL
        L.oracle_candidates.argtypes = [P, I, P, P, D, P, P, LL, P]
        L.oracle_neighbor_distances.argtypes = [P, I, P, P, P, P, P, I, D, D, P, P, P, I]
        L.oracle_forces.argtypes = [P, I, P, P, P, P, P, I, P]
        L.oracle_simulate.restype = I
        L.oracle_simulate.argtypes = [P, I, I, I, P, P, P, P, P, P, I, P]
        L.oracle_nvt_init.argtypes = [I, D, D, I, P]
        L.oracle_set_order.argtypes = [I, D, I]
        L.oracle_fire.restype = I
        L.oracle_fire.argtypes = [P, I, P, P, P, P, P, P, P, I, P]
        L.oracle_stress.argtypes = [P, I, P, P, P, P, P]
        L.oracle_set_boundary.argtypes = [I]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def set_order(order: int = 0, delta: float = 0.0, bfs: bool = False):
    """Processing order of the oracle's propagation: 0 priority queue (default), 1 distance-banded rounds of width
    delta (the CUDA kernel's order; bfs=True drops the banding).  Results are identical; only the work differs."""
    lib().oracle_set_order(int(order), float(delta), int(bool(bfs)))


def set_boundary(bc: int = 0):
    """Boundary condition of the oracle's walks: 0 closed mesh, 1 tangential, 2 absorbing (open meshes)."""
    lib().oracle_set_boundary(int(bc))


class OracleMesh:
    """A mesh held by the oracle (its own connectivity, independent of the CUDA library's)."""

    def __init__(self, V, F):
        self.V = np.ascontiguousarray(V, dtype=np.float64)
        self.F = np.ascontiguousarray(F, dtype=np.int32)
        self.h = lib().oracle_mesh_create(_p(self.V), self.V.shape[0], _p(self.F), self.F.shape[0])

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.oracle_mesh_destroy(self.h)
            self.h = None

    @property
    def area(self):
        return lib().oracle_mesh_area(self.h)

    def bbox(self):
        out = np.zeros(6)
        lib().oracle_mesh_bbox(self.h, _p(out))
        return out[:3], out[3:]

    def angle_sums(self):
        out = np.zeros(self.V.shape[0])
        lib().oracle_angle_sums(self.h, _p(out))
        return out

    def r3(self, face, bary):
        face = np.ascontiguousarray(face, dtype=np.int32)
        bary = np.ascontiguousarray(bary, dtype=np.float64)
        out = np.zeros((len(face), 3))
        lib().oracle_positions_r3(self.h, len(face), _p(face), _p(bary), _p(out))
        return out

    # ----- walk ------------------------------------------------------------------------------------------------
    def transport(self, face, bary, disp, transport=None, max_iter=100000):
        """Batched transportParticleAndVectors.  Returns (face, bary, disp, transport, status, crossings)."""
        face = np.array(face, dtype=np.int32, copy=True)
        bary = np.array(bary, dtype=np.float64, copy=True)
        disp = np.array(disp, dtype=np.float64, copy=True)
        n = len(face)
        ntv = 0
        tv = None
        if transport is not None:
            tv = np.array(transport, dtype=np.float64, copy=True).reshape(n, -1, 3)
            ntv = tv.shape[1]
        status = np.zeros(n, dtype=np.int32)
        cross = np.zeros(n, dtype=np.int32)
        lib().oracle_transport(self.h, n, _p(face), _p(bary), _p(disp), _p(tv) if tv is not None else None, ntv,
                               max_iter, _p(status), _p(cross))
        return face, bary, disp, tv, status, cross

    # ----- patch / distances -------------------------------------------------------------------------------------
    def patch(self, f0, b0, target_faces, r):
        tf = np.ascontiguousarray(target_faces, dtype=np.int32)
        b0 = np.ascontiguousarray(b0, dtype=np.float64)
        cap = self.F.shape[0]
        out = np.zeros(cap, dtype=np.int32)
        n = lib().oracle_patch(self.h, int(f0), _p(b0), len(tf), _p(tf), float(r), _p(out), cap)
        return out[:n]

    def distance(self, f0, b0, target_faces, target_bary, submesh=False, max_dist=1.0, threshold=1e20,
                 cutoff=np.inf):
        tf = np.ascontiguousarray(target_faces, dtype=np.int32)
        tb = np.ascontiguousarray(target_bary, dtype=np.float64).reshape(-1, 3)
        b0 = np.ascontiguousarray(b0, dtype=np.float64)
        n = len(tf)
        d = np.zeros(n)
        ts = np.zeros((n, 3))
        te = np.zeros((n, 3))
        stats = np.zeros(4, dtype=np.int64)
        lib().oracle_distance(self.h, int(f0), _p(b0), n, _p(tf), _p(tb), int(bool(submesh)), float(max_dist),
                              float(threshold), float(cutoff), _p(d), _p(ts), _p(te), _p(stats))
        return d, ts, te, stats

    def distance_bruteforce(self, fa, ba, fb, bb, face_set=None, max_depth=12):
        ba = np.ascontiguousarray(ba, dtype=np.float64)
        bb = np.ascontiguousarray(bb, dtype=np.float64)
        if face_set is None:
            return lib().oracle_distance_bruteforce(self.h, int(fa), _p(ba), int(fb), _p(bb), None, 0, max_depth)
        fs = np.ascontiguousarray(face_set, dtype=np.int32)
        return lib().oracle_distance_bruteforce(self.h, int(fa), _p(ba), int(fb), _p(bb), _p(fs), len(fs), max_depth)

    def candidates(self, face, bary, rng):
        """Candidate CSR (offsets, indices, max chord) as the reference's neighbour structures produce it."""
        face = np.ascontiguousarray(face, dtype=np.int32)
        bary = np.ascontiguousarray(bary, dtype=np.float64)
        n = len(face)
        off = np.zeros(n + 1, dtype=np.int32)
        mc = np.zeros(n)
        cap = max(1024, n * 32)
        while True:
            idx = np.zeros(cap, dtype=np.int32)
            tot = lib().oracle_candidates(self.h, n, _p(face), _p(bary), float(rng), _p(off), _p(idx), cap, _p(mc))
            if tot >= 0:
                return off, idx[:tot], mc
            cap = -tot

    def neighbor_distances(self, face, bary, off, idx, max_chord, submesh, max_dist, cutoff, threads=0):
        face = np.ascontiguousarray(face, dtype=np.int32)
        bary = np.ascontiguousarray(bary, dtype=np.float64)
        off = np.ascontiguousarray(off, dtype=np.int32)
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        mc = np.ascontiguousarray(max_chord, dtype=np.float64)
        m = len(idx)
        d = np.full(m, np.inf)
        ts = np.zeros((m, 3))
        stats = np.zeros(5, dtype=np.int64)
        lib().oracle_neighbor_distances(self.h, len(face), _p(face), _p(bary), _p(off), _p(idx), _p(mc),
                                        int(submesh), float(max_dist), float(cutoff), _p(d), _p(ts), _p(stats),
                                        int(threads))
        return d, ts, stats

    # ----- forces / integrators ----------------------------------------------------------------------------------
    @staticmethod
    def params(force_kind=0, k=1.0, sigma=1.0, rng=1.0, submesh=0, max_dist=1.0, cutoff=None, dt=0.001, T=0.0,
               tau=1.0, chain=2):
        if cutoff is None:
            cutoff = sigma
        return np.array([force_kind, k, sigma, rng, submesh, max_dist, cutoff, dt, T, tau, chain], dtype=np.float64)

    def forces(self, face, bary, params, threads=0):
        face = np.ascontiguousarray(face, dtype=np.int32)
        bary = np.ascontiguousarray(bary, dtype=np.float64)
        f = np.zeros((len(face), 3))
        e = np.zeros(1)
        stats = np.zeros(4, dtype=np.int64)
        lib().oracle_forces(self.h, len(face), _p(face), _p(bary), _p(params), _p(f), _p(e), int(threads),
                            _p(stats))
        return f, float(e[0]), stats

    def simulate(self, kind, steps, face, bary, vel, force, params, chain=None, threads=0):
        """Advance in place (arrays are copied and returned): kind 0 NVE, 1 NVT."""
        face = np.array(face, dtype=np.int32, copy=True)
        bary = np.array(bary, dtype=np.float64, copy=True)
        vel = np.array(vel, dtype=np.float64, copy=True)
        force = np.array(force, dtype=np.float64, copy=True)
        if chain is None:
            chain = self.nvt_chain(len(face), params)
        chain = np.array(chain, dtype=np.float64, copy=True)
        stats = np.zeros(4, dtype=np.int64)
        err = lib().oracle_simulate(self.h, int(kind), int(steps), len(face), _p(face), _p(bary), _p(vel), _p(force),
                                    _p(params), _p(chain), int(threads), _p(stats))
        return face, bary, vel, force, chain, err, stats

    def fire(self, face, bary, vel, force, params, maximum_iterations=1000, alpha_start=0.99, dt_max=0.1, dt_min=1e-5,
             dt_inc=1.1, dt_dec=0.95, alpha_dec=0.9, n_min=4, force_cutoff=1e-12, alpha_min=0.0, state=None,
             threads=0):
        """fireMinimization::minimizeByFire; state = [deltaT, alpha, nSinceNegativePower] (default: params' dt,
        alpha_start, 0).  Returns (face, bary, vel, force, state, iterations, forceMax, err)."""
        face = np.array(face, dtype=np.int32, copy=True)
        bary = np.array(bary, dtype=np.float64, copy=True)
        vel = np.array(vel, dtype=np.float64, copy=True)
        force = np.array(force, dtype=np.float64, copy=True)
        fire = np.array([maximum_iterations, alpha_start, dt_max, dt_min, dt_inc, dt_dec, alpha_dec, n_min,
                         force_cutoff, alpha_min], dtype=np.float64)
        st = np.array(state if state is not None else [params[7], alpha_start, 0], dtype=np.float64)
        out = np.zeros(2)
        err = lib().oracle_fire(self.h, len(face), _p(face), _p(bary), _p(vel), _p(force), _p(params), _p(fire),
                                _p(st), int(threads), _p(out))
        return face, bary, vel, force, st, int(out[0]), float(out[1]), err

    def gradient_descent(self, face, bary, params, steps, delta_t, vel=None, threads=0):
        """gradientDescent::performUpdate (src/updaters/gradientDescent.cpp:6-18), `steps` times: the forces at the
        current positions, then every particle moved by delta_t * force through the walk (simpleModel::moveParticles,
        simpleModel.cpp:44-66), the velocity carried along when `vel` is given.  Returns (face, bary, vel, force, err)
        with the last forces computed (before the last move); err = 1 when a walk failed."""
        face = np.array(face, dtype=np.int32, copy=True)
        bary = np.array(bary, dtype=np.float64, copy=True)
        vel = None if vel is None else np.array(vel, dtype=np.float64, copy=True)
        f = np.zeros((len(face), 3))
        for _ in range(int(steps)):
            f, _, _ = self.forces(face, bary, params, threads)
            fo, bo, _, tv, st, _ = self.transport(face, bary, delta_t * f, None if vel is None else vel[:, None, :])
            if np.any(st != 0):
                return face, bary, vel, f, 1
            face, bary = fo, bo
            if vel is not None:
                vel = tv[:, 0]
        return face, bary, vel, f, 0

    def stress(self, face, bary, vel, params):
        face = np.ascontiguousarray(face, dtype=np.int32)
        bary = np.ascontiguousarray(bary, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        out = np.zeros(9)
        lib().oracle_stress(self.h, len(face), _p(face), _p(bary), _p(vel), _p(params), _p(out))
        return out.reshape(3, 3)

    @staticmethod
    def nvt_chain(n, params):
        Mc = int(params[10])
        chain = np.zeros(4 * (Mc + 1) + 2)
        lib().oracle_nvt_init(int(n), float(params[8]), float(params[9]), Mc, _p(chain))
        return chain
