"""Python front end of libcssg.so: device meshes, batched walks and distance queries, device-resident systems.

Every call goes through the C ABI (include/cssg.h).  Device buffers for the batched calls are torch tensors (torch
is used only for allocation and streams); the library launches on the stream of the context, which by default is
torch's current stream so ordering with torch copies is implicit.
"""
from __future__ import annotations

import atexit
import ctypes
import math
import weakref

import numpy as np

from . import _lib
from ._lib import check, cssg_params

_P = ctypes.c_void_p

# Library objects still alive at interpreter exit are released in dependency order (systems, then meshes, then
# contexts) by an exit hook registered after torch's own, so none is released after the CUDA context it uses.
_live = {"system": weakref.WeakSet(), "mesh": weakref.WeakSet(), "context": weakref.WeakSet()}
_exit_hook = []


def _register(kind, obj):
    _live[kind].add(obj)
    if not _exit_hook:
        atexit.register(_release_all)
        _exit_hook.append(True)


def _release_all():
    for kind in ("system", "mesh", "context"):
        for obj in list(_live[kind]):
            obj.close()


def _np_ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise _lib.CssgError("CUDA device required: libcssg has no CPU path")
    return torch


class Context:
    """cssg_ctx: the CUDA stream the library launches on.

    By default a dedicated torch stream is created and shared with the library (torch's default stream cannot be
    used: it is the legacy NULL stream, which does not support graph capture), so torch copies and events issued
    under ``with ctx.use():`` are ordered with the library's kernels."""

    def __init__(self, device: int = 0, stream=None):
        L = _lib.load()
        torch = _torch()
        self.device = device
        if stream is None:
            self.tstream = torch.cuda.Stream(device=device)
        elif isinstance(stream, int):
            self.tstream = torch.cuda.ExternalStream(stream, device=device)
        else:
            self.tstream = stream
        h = ctypes.c_void_p()
        check(L.cssg_ctx_create(device, ctypes.c_void_p(self.tstream.cuda_stream), ctypes.byref(h)),
              "cssg_ctx_create")
        self.h = h
        _register("context", self)

    def use(self):
        """Context manager: make the library's stream torch's current stream."""
        return _torch().cuda.stream(self.tstream)

    @property
    def stream(self):
        return _lib.load().cssg_ctx_stream(self.h)

    def synchronize(self):
        check(_lib.load().cssg_ctx_synchronize(self.h), "cssg_ctx_synchronize")

    def close(self):
        if getattr(self, "h", None) is not None and _lib._lib is not None:
            _lib._lib.cssg_ctx_destroy(self.h)
        self.h = None

    def __del__(self):
        self.close()


class Mesh:
    """cssg_mesh: the triangulated surface on the device (triangulatedMeshSpace::loadMeshFromFile)."""

    BOUNDARY = {"closed": 0, "tangential": 1, "absorbing": 2}

    def __init__(self, V, F, device: int = 0, boundary="closed"):
        """boundary: walk condition at border edges/vertices - "closed" (an error, triangulatedMeshSpace),
        "tangential" (tangentialOpenMeshSpace) or "absorbing" (absorbingOpenMeshSpace)."""
        L = _lib.load()
        self.V = np.ascontiguousarray(V, dtype=np.float64)
        self.F = np.ascontiguousarray(F, dtype=np.int32)
        h = ctypes.c_void_p()
        check(L.cssg_mesh_create(_np_ptr(self.V), self.V.shape[0], _np_ptr(self.F), self.F.shape[0], device,
                                 ctypes.byref(h)), "cssg_mesh_create")
        self.h = h
        nv, nf = ctypes.c_int(), ctypes.c_int()
        area = ctypes.c_double()
        bbox = np.zeros(6)
        check(L.cssg_mesh_info(h, ctypes.byref(nv), ctypes.byref(nf), ctypes.byref(area), _np_ptr(bbox)),
              "cssg_mesh_info")
        self.nV, self.nF, self.area = nv.value, nf.value, area.value
        self.bbox = (bbox[:3].copy(), bbox[3:].copy())
        self.boundary = "closed"
        _register("mesh", self)
        if boundary != "closed":
            self.set_boundary(boundary)

    def set_boundary(self, boundary):
        bc = self.BOUNDARY[boundary] if isinstance(boundary, str) else int(boundary)
        check(_lib.load().cssg_mesh_set_boundary(self.h, bc), "cssg_mesh_set_boundary")
        self.boundary = boundary

    def close(self):
        if getattr(self, "h", None) is not None and _lib._lib is not None:
            _lib._lib.cssg_mesh_destroy(self.h)
        self.h = None

    def __del__(self):
        self.close()


def transport_batch(ctx: Context, mesh: Mesh, face, bary, disp, transport=None):
    """Batched transportParticleAndVectors on host arrays; returns (face, bary, disp, transport, status)."""
    with ctx.use():
        return _transport_batch(ctx, mesh, face, bary, disp, transport)


def _transport_batch(ctx, mesh, face, bary, disp, transport):
    torch = _torch()
    dev = f"cuda:{ctx.device}"
    n = len(face)
    f = torch.tensor(np.asarray(face, dtype=np.int32), device=dev)
    b = torch.tensor(np.asarray(bary, dtype=np.float64).reshape(n, 3), device=dev)
    d = torch.tensor(np.asarray(disp, dtype=np.float64).reshape(n, 3), device=dev)
    ntv = 0
    tv = None
    if transport is not None:
        tvh = np.asarray(transport, dtype=np.float64).reshape(n, -1, 3)
        ntv = tvh.shape[1]
        tv = torch.tensor(tvh, device=dev)
    st = torch.zeros(n, dtype=torch.int32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    L = _lib.load()
    check(L.cssg_transport_batch(ctx.h, mesh.h, n, _P(f.data_ptr()), _P(b.data_ptr()), _P(d.data_ptr()),
                                 _P(tv.data_ptr()) if tv is not None else None, ntv, _P(st.data_ptr()),
                                 _P(cnt.data_ptr())), "cssg_transport_batch")
    ctx.synchronize()
    return (f.cpu().numpy(), b.cpu().numpy(), d.cpu().numpy(), tv.cpu().numpy() if tv is not None else None,
            st.cpu().numpy(), int(cnt.cpu().item()))


def distance_batch(ctx: Context, mesh: Mesh, src_face, src_bary, cand_off, cand_face, cand_bary, submesh=False,
                   max_dist=1.0, threshold=None, cutoff=math.inf):
    """Batched triangulatedMeshSpace::distance over sources with CSR candidate lists (host arrays in and out)."""
    with ctx.use():
        return _distance_batch(ctx, mesh, src_face, src_bary, cand_off, cand_face, cand_bary, submesh, max_dist,
                               threshold, cutoff)


def _distance_batch(ctx, mesh, src_face, src_bary, cand_off, cand_face, cand_bary, submesh, max_dist, threshold,
                    cutoff):
    torch = _torch()
    dev = f"cuda:{ctx.device}"
    ns = len(src_face)
    sf = torch.tensor(np.asarray(src_face, dtype=np.int32), device=dev)
    sb = torch.tensor(np.asarray(src_bary, dtype=np.float64).reshape(ns, 3), device=dev)
    co = torch.tensor(np.asarray(cand_off, dtype=np.int32), device=dev)
    m = int(cand_off[-1])
    cf = torch.tensor(np.asarray(cand_face, dtype=np.int32).reshape(m), device=dev)
    cb = torch.tensor(np.asarray(cand_bary, dtype=np.float64).reshape(m, 3), device=dev)
    th = torch.tensor(np.asarray(threshold, dtype=np.float64), device=dev) if threshold is not None else None
    d = torch.zeros(max(m, 1), dtype=torch.float64, device=dev)
    ts = torch.zeros((max(m, 1), 3), dtype=torch.float64, device=dev)
    te = torch.zeros((max(m, 1), 3), dtype=torch.float64, device=dev)
    st = torch.zeros(max(ns, 1), dtype=torch.int32, device=dev)
    stats = torch.zeros((max(ns, 1), 4), dtype=torch.int64, device=dev)
    L = _lib.load()
    check(L.cssg_distance_batch(ctx.h, mesh.h, ns, _P(sf.data_ptr()), _P(sb.data_ptr()), _P(co.data_ptr()),
                                _P(cf.data_ptr()), _P(cb.data_ptr()), int(bool(submesh)), float(max_dist),
                                _P(th.data_ptr()) if th is not None else None, float(cutoff), _P(d.data_ptr()),
                                _P(ts.data_ptr()), _P(te.data_ptr()), _P(st.data_ptr()), _P(stats.data_ptr())),
          "cssg_distance_batch")
    ctx.synchronize()
    distance_batch.last_stats = stats.cpu().numpy()[:ns]
    return d.cpu().numpy()[:m], ts.cpu().numpy()[:m], te.cpu().numpy()[:m], st.cpu().numpy()[:ns]


def flops_per_window() -> int:
    """FP64 flops of one processed window of the propagation (the library's own count, window.cuh)."""
    return int(_lib.load().cssg_diag_flops_per_window())


def fp64_peak_gflops(ctx: Context) -> float:
    out = ctypes.c_double()
    check(_lib.load().cssg_diag_fp64_peak(ctx.h, ctypes.byref(out)), "cssg_diag_fp64_peak")
    return out.value


def pairs_to_neighbor_lists(n, i, j, d, t):
    """Group pair records (source i, target j, distance d, start tangent t; grouped by source as cssg_system_pairs
    returns them) into simpleModel's per-particle lists: (neighbors, neighborVectors, neighborDistances).  Pairs the
    learned screen skipped (j < 0, index -j - 1) keep their index with distance +inf."""
    neighbors = [[] for _ in range(n)]
    vectors = [[] for _ in range(n)]
    distances = [[] for _ in range(n)]
    for a, b, dist, tan in zip(np.asarray(i), np.asarray(j), np.asarray(d), np.asarray(t).reshape(-1, 3)):
        if not 0 <= a < n:
            continue
        screened = b < 0
        neighbors[a].append(int(-b - 1 if screened else b))
        vectors[a].append(np.array(tan, dtype=np.float64))
        distances[a].append(math.inf if screened else float(dist))
    return neighbors, vectors, distances


def make_params(integrator="nve", force="harmonic", k=1.0, sigma=1.0, range_=None, submesh=False, max_dist=None,
                cutoff=None, dt=0.001, temperature=0.0, tau=1.0, chain_length=2):
    p = cssg_params()
    p.integrator = {"nve": 0, "nvt": 1}[integrator] if isinstance(integrator, str) else int(integrator)
    p.force_kind = {"harmonic": 0, "gaussian": 1}[force] if isinstance(force, str) else int(force)
    p.k = float(k)
    p.sigma = float(sigma)
    p.range = float(sigma if range_ is None else range_)
    p.submesh = int(bool(submesh))
    p.max_dist = float(sigma if max_dist is None else max_dist)
    p.cutoff = float(sigma if cutoff is None else cutoff)
    p.dt = float(dt)
    p.temperature = float(temperature)
    p.tau = float(tau)
    p.chain_length = int(chain_length)
    return p


class System:
    """cssg_system: particles, forces and the updater resident on the device.

    ``mesh``/``n``/``params`` may be lists (one entry per independent system) to batch several systems; state
    arrays are then the concatenation of the systems' particles."""

    def __init__(self, ctx: Context, mesh, n, params):
        L = _lib.load()
        meshes = list(mesh) if isinstance(mesh, (list, tuple)) else [mesh]
        counts = list(n) if isinstance(n, (list, tuple)) else [n]
        plist = list(params) if isinstance(params, (list, tuple)) else [params]
        if not (len(meshes) == len(counts) == len(plist)):
            raise ValueError("one mesh, count and parameter set per system")
        self.ctx, self.meshes, self.counts, self.params = ctx, meshes, counts, plist[0]
        self.mesh = meshes[0]
        self.K = len(meshes)
        self.n = int(sum(counts))
        h = ctypes.c_void_p()
        if self.K == 1:
            check(L.cssg_system_create(ctx.h, meshes[0].h, counts[0], ctypes.byref(plist[0]), ctypes.byref(h)),
                  "cssg_system_create")
        else:
            mh = (ctypes.c_void_p * self.K)(*[m.h.value for m in meshes])
            cn = (ctypes.c_int * self.K)(*counts)
            pa = (cssg_params * self.K)(*plist)
            check(L.cssg_system_create_batched(ctx.h, self.K, mh, cn, pa, ctypes.byref(h)),
                  "cssg_system_create_batched")
        self.h = h
        _register("system", self)

    def close(self):
        if getattr(self, "h", None) is not None and _lib._lib is not None:
            _lib._lib.cssg_system_destroy(self.h)
        self.h = None

    def __del__(self):
        self.close()

    def set_state(self, face=None, bary=None, vel=None, force=None):
        def prep(a, dt, shape):
            if a is None:
                return None, None
            arr = np.ascontiguousarray(np.asarray(a, dtype=dt).reshape(shape))
            return arr, _np_ptr(arr)
        fa, fp = prep(face, np.int32, (self.n,))
        ba, bp = prep(bary, np.float64, (self.n, 3))
        va, vp = prep(vel, np.float64, (self.n, 3))
        qa, qp = prep(force, np.float64, (self.n, 3))
        check(_lib.load().cssg_system_set_state(self.h, fp, bp, vp, qp), "cssg_system_set_state")

    def reset_thermostat(self):
        check(_lib.load().cssg_system_reset_thermostat(self.h), "cssg_system_reset_thermostat")

    def kernels_per_audit_step(self):
        c = ctypes.c_int()
        check(_lib.load().cssg_system_kernels_per_audit_step(self.h, ctypes.byref(c)),
              "cssg_system_kernels_per_audit_step")
        return c.value

    def kernels_per_step(self):
        c = ctypes.c_int()
        check(_lib.load().cssg_system_kernels_per_step(self.h, ctypes.byref(c)), "cssg_system_kernels_per_step")
        return c.value

    def get_state(self):
        face = np.zeros(self.n, dtype=np.int32)
        bary = np.zeros((self.n, 3))
        vel = np.zeros((self.n, 3))
        force = np.zeros((self.n, 3))
        check(_lib.load().cssg_system_get_state(self.h, _np_ptr(face), _np_ptr(bary), _np_ptr(vel), _np_ptr(force)),
              "cssg_system_get_state")
        return face, bary, vel, force

    def device_state(self):
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        check(_lib.load().cssg_system_device_state(self.h, *[ctypes.byref(p) for p in ptrs]),
              "cssg_system_device_state")
        return [p.value for p in ptrs]

    def step(self, steps: int = 1, graph: bool = True):
        check(_lib.load().cssg_system_step(self.h, int(steps), int(bool(graph))), "cssg_system_step")

    def step_host(self, steps, face, bary, vel, force, out=None):
        """cssg_system_step_host: host state in, `steps` graph-replayed steps, host state out (into `out`, a tuple of
        four arrays, or into the input arrays when out is None), one synchronisation."""
        arrs = [np.asarray(a) for a in (face, bary, vel, force)]
        for a, dt in zip(arrs, (np.int32, np.float64, np.float64, np.float64)):
            if a.dtype != dt or not a.flags.c_contiguous:
                raise ValueError("step_host wants C-contiguous int32 face and float64 bary, vel, force arrays")
        outs = arrs if out is None else [np.asarray(a) for a in out]
        check(_lib.load().cssg_system_step_host(self.h, int(steps), *[_np_ptr(a) for a in arrs],
                                                *[_np_ptr(a) for a in outs]), "cssg_system_step_host")
        return outs

    def gradient_descent(self, steps: int, delta_t: float, transport_velocity: bool = False):
        """gradientDescent::performUpdate x steps: forces, then every particle moved by delta_t * force."""
        rc = _lib.load().cssg_system_gradient_descent(self.h, int(steps), float(delta_t), int(bool(transport_velocity)))
        check(rc, "cssg_system_gradient_descent")

    def compute_forces(self):
        check(_lib.load().cssg_system_compute_forces(self.h), "cssg_system_compute_forces")

    def check(self):
        bits = ctypes.c_int()
        cnt = np.zeros(5, dtype=np.uint64)
        check(_lib.load().cssg_system_check(self.h, ctypes.byref(bits), _np_ptr(cnt)), "cssg_system_check")
        return bits.value, {"crossings": int(cnt[0]), "windows": int(cnt[1]), "launches": int(cnt[2]),
                            "in_range_pairs": int(cnt[3]), "capacity_hits": int(cnt[4])}

    def enable_pairs(self):
        cnt = ctypes.c_int()
        check(_lib.load().cssg_system_pairs(self.h, 0, None, None, None, None, ctypes.byref(cnt)), "pairs")

    def pairs(self):
        L = _lib.load()
        cnt = ctypes.c_int()
        check(L.cssg_system_pairs(self.h, 0, None, None, None, None, ctypes.byref(cnt)), "pairs")
        m = cnt.value
        i = np.zeros(m, dtype=np.int32)
        j = np.zeros(m, dtype=np.int32)
        d = np.zeros(m)
        t = np.zeros((m, 3))
        check(L.cssg_system_pairs(self.h, m, _np_ptr(i), _np_ptr(j), _np_ptr(d), _np_ptr(t), ctypes.byref(cnt)),
              "pairs")
        return i, j, d, t

    def neighbors(self):
        """simpleModel::findNeighbors (simpleModel.cpp:68-112) for analysis: forces at the current state, then the
        neighbour lists (indices, start tangents, distances; +inf beyond the force cutoff) from the pair records."""
        if not getattr(self, "_pairs_on", False):
            self.enable_pairs()
            self._pairs_on = True
        self.compute_forces()
        i, j, d, t = self.pairs()
        return pairs_to_neighbor_lists(self.n, i, j, d, t)

    def chain(self):
        cap = (4 * (max(1, self.params.chain_length) + 1) + 2) * self.K
        out = np.zeros(cap)
        check(_lib.load().cssg_system_chain(self.h, _np_ptr(out), cap), "cssg_system_chain")
        return out

    def set_screen(self, params=None, margin: float = 0.0, enable: bool = True):
        """Learned screen: params = FP32 MLP parameters (host array); enable=False returns to the exact path."""
        ptr = None
        arr = None
        if params is not None:
            arr = np.ascontiguousarray(np.asarray(params, dtype=np.float32))
            ptr = _np_ptr(arr)
        check(_lib.load().cssg_system_set_screen(self.h, ptr, float(margin), int(bool(enable))),
              "cssg_system_set_screen")

    def set_lanes(self, lanes_per_warp: int):
        """Regular propagation pass with one source per lane (16 or 32 per warp) or source groups (0)."""
        check(_lib.load().cssg_system_set_lanes(self.h, int(lanes_per_warp)), "cssg_system_set_lanes")

    def lanes(self):
        out = ctypes.c_int()
        check(_lib.load().cssg_system_lanes(self.h, ctypes.byref(out)), "cssg_system_lanes")
        return out.value

    def set_lane_split(self, group_sources: int):
        """With the lane pass: the `group_sources` costliest sources of the last evaluation go to the source-group
        pass, the rest to the lane pass (cssg_system_set_lane_split)."""
        check(_lib.load().cssg_system_set_lane_split(self.h, int(group_sources)), "cssg_system_set_lane_split")

    def lane_split(self):
        out = ctypes.c_int()
        check(_lib.load().cssg_system_lane_split(self.h, ctypes.byref(out)), "cssg_system_lane_split")
        return out.value

    def set_pass_groups(self, medium_warps: int = 0, large_warps: int = 0):
        """Warps per source of the medium and large passes (0: the regular pass's; cssg_system_set_pass_groups)."""
        check(_lib.load().cssg_system_set_pass_groups(self.h, int(medium_warps), int(large_warps)),
              "cssg_system_set_pass_groups")

    def pass_groups(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        check(_lib.load().cssg_system_pass_groups(self.h, ctypes.byref(a), ctypes.byref(b)), "cssg_system_pass_groups")
        return a.value, b.value

    def source_costs(self):
        """Work of each source in the last force evaluation (cssg_system_source_costs)."""
        out = np.zeros(self.n, dtype=np.int32)
        check(_lib.load().cssg_system_source_costs(self.h, int(self.n), _np_ptr(out)), "cssg_system_source_costs")
        return out

    def set_work_caps(self, regular: int = 0, medium: int = 0, large: int = 0):
        """Per-source window caps of the regular, medium and large propagation passes (<= 0 keeps a cap)."""
        check(_lib.load().cssg_system_set_work_caps(self.h, int(regular), int(medium), int(large)),
              "cssg_system_set_work_caps")

    def set_screen_audit(self, every: int):
        """Periodic exact audit of the screen every `every` steps (0: off); a dropped in-range pair switches the
        screen off on the device (cssg_system_set_screen_audit)."""
        check(_lib.load().cssg_system_set_screen_audit(self.h, int(every)), "cssg_system_set_screen_audit")

    def screen_audit_status(self):
        out = np.zeros(3, dtype=np.int64)
        check(_lib.load().cssg_system_screen_audit_status(self.h, _np_ptr(out)), "cssg_system_screen_audit_status")
        return {"audits": int(out[0]), "sources_with_dropped_pairs": int(out[1]), "screen_off": bool(out[2])}

    def screen_counters(self):
        out = np.zeros(3, dtype=np.uint64)
        check(_lib.load().cssg_system_screen_counters(self.h, _np_ptr(out)), "cssg_system_screen_counters")
        return {"pairs": int(out[0]), "screened": int(out[1]), "tc_errors": int(out[2])}

    def set_tuning(self, delta_scale: float = 1.0, warps_per_block: int = 8, mid_slots: int = 0,
                   warps_per_sm: int = 0, lpt_order: bool = False, warps_per_source: int = 1,
                   wide_registers: int = 0):
        """Band width scale, block size (warps), medium-pass slots, per-SM warp cap, longest-first source order,
        warps per source and the kernel build (bit 0: 255 registers, bit 1: out-of-line hash-table probes)."""
        check(_lib.load().cssg_system_set_tuning(self.h, float(delta_scale), int(warps_per_block), int(mid_slots),
                                                 int(warps_per_sm), int(bool(lpt_order)), int(warps_per_source),
                                                 int(wide_registers)), "cssg_system_set_tuning")

    def autotune(self, reps: int = 3):
        """Pick the fastest tuning on the current state (cssg_system_autotune); returns it with its time."""
        out = np.zeros(8)
        with self.ctx.use():
            check(_lib.load().cssg_system_autotune(self.h, int(reps), _np_ptr(out)), "cssg_system_autotune")
        return {"delta_scale": float(out[0]), "warps_per_block": int(out[1]), "mid_slots": int(out[2]),
                "warps_per_sm": int(out[3]), "lpt_order": bool(out[4]), "ms_per_force_pass": float(out[5]),
                "warps_per_source": int(out[6]), "wide_registers": bool(int(out[7]) & 1),
                "outlined_probes": bool(int(out[7]) & 2), "lanes_per_warp": self.lanes(),
                "lane_split": self.lane_split(), "pass_groups": list(self.pass_groups())}

    def fire(self, maximum_iterations=1000, alpha_start=0.99, dt_max=0.1, dt_min=1e-5, dt_inc=1.1, dt_dec=0.95,
             alpha_dec=0.9, n_min=4, force_cutoff=1e-12, alpha_min=0.0, reset=False):
        """FIRE energy minimisation on the device (fireMinimization::minimizeByFire); defaults are the reference's
        member defaults.  Returns iterations, forceMax and the persistent deltaT / alpha / nSinceNegativePower."""
        p = _lib.cssg_fire_params(int(maximum_iterations), float(alpha_start), float(dt_max), float(dt_min),
                                  float(dt_inc), float(dt_dec), float(alpha_dec), int(n_min), float(force_cutoff),
                                  float(alpha_min))
        out = np.zeros(5 * self.K)
        with self.ctx.use():
            check(_lib.load().cssg_system_fire(self.h, ctypes.byref(p), int(bool(reset)), _np_ptr(out)),
                  "cssg_system_fire")
        res = [{"iterations": int(o[0]), "force_max": float(o[1]), "dt": float(o[2]), "alpha": float(o[3]),
                "n_since_negative_power": int(o[4])} for o in out.reshape(self.K, 5)]
        return res[0] if self.K == 1 else res

    def stress(self):
        """simulation::computeMonodisperseStress on the current state: 3x3 array."""
        out = np.zeros(9)
        with self.ctx.use():
            check(_lib.load().cssg_system_stress(self.h, _np_ptr(out)), "cssg_system_stress")
        return out.reshape(3, 3)

    def timing(self, enable: bool):
        check(_lib.load().cssg_system_timing(self.h, int(bool(enable))), "cssg_system_timing")

    def last_times(self):
        out = np.zeros(2)
        check(_lib.load().cssg_system_last_times(self.h, _np_ptr(out), 2), "cssg_system_last_times")
        return {"geodesic_ms": float(out[0]), "walk_ms": float(out[1])}


# ----------------------------------------------------------------------------------------------------------------
# learned distance screen
# ----------------------------------------------------------------------------------------------------------------
def mlp_param_count() -> int:
    return int(_lib.load().cssg_mlp_param_count())


def screen_features(ctx: Context, mesh: Mesh, sigma: float, pi, pj, face, pos):
    """Pair features on the device; all inputs torch tensors on the context's device. Returns (X bf16, chord/s)."""
    torch = _torch()
    n = int(pi.numel())
    torch.cuda.current_stream(pi.device).synchronize()
    with ctx.use():
        X = torch.zeros((max(n, 1), 16), dtype=torch.bfloat16, device=pi.device)
        c = torch.zeros(max(n, 1), dtype=torch.float32, device=pi.device)
    check(_lib.load().cssg_screen_features(ctx.h, mesh.h, float(sigma), n, _P(pi.data_ptr()), _P(pj.data_ptr()),
                                           _P(face.data_ptr()), _P(pos.data_ptr()), _P(X.data_ptr()),
                                           _P(c.data_ptr())), "cssg_screen_features")
    ctx.synchronize()
    return X[:n], c[:n]


def mlp_infer(ctx: Context, X, params):
    """Tensor-core inference; X bf16 [n, 16], params float32 [P] (torch, device)."""
    torch = _torch()
    n = int(X.shape[0])
    torch.cuda.current_stream(X.device).synchronize()
    with ctx.use():
        y = torch.zeros(max(n, 1), dtype=torch.float32, device=X.device)
        err = torch.zeros(1, dtype=torch.int32, device=X.device)
    check(_lib.load().cssg_mlp_infer(ctx.h, _P(X.data_ptr()), n, _P(params.data_ptr()), _P(y.data_ptr()),
                                     _P(err.data_ptr())), "cssg_mlp_infer")
    ctx.synchronize()
    if int(err.item()):
        raise _lib.CssgError("cssg_mlp_infer: tensor-core completion wait timed out")
    return y[:n]


def mlp_grad(ctx: Context, X, y, params):
    torch = _torch()
    torch.cuda.current_stream(X.device).synchronize()
    with ctx.use():
        g = torch.zeros(mlp_param_count(), dtype=torch.float32, device=X.device)
        loss = torch.zeros(1, dtype=torch.float32, device=X.device)
    check(_lib.load().cssg_mlp_grad(ctx.h, _P(X.data_ptr()), _P(y.data_ptr()), int(X.shape[0]),
                                    _P(params.data_ptr()), _P(g.data_ptr()), _P(loss.data_ptr())), "cssg_mlp_grad")
    ctx.synchronize()
    return g, loss


def mlp_adam(ctx: Context, params, grad, m, v, batch: int, lr: float, step: int):
    check(_lib.load().cssg_mlp_adam(ctx.h, _P(params.data_ptr()), _P(grad.data_ptr()), _P(m.data_ptr()),
                                    _P(v.data_ptr()), int(batch), ctypes.c_float(lr), int(step)), "cssg_mlp_adam")
    ctx.synchronize()
