"""Benchmark of the curvedSpaceSim per-timestep hot path on GB300.

Workload (default): the plain exact GPU path with submeshing -
torus R=3, r=1 from a 200x100 grid with alternating diagonals (20,000 vertices / 40,000 faces), N=2,000 particles at
area-weighted random positions (seed 2), harmonic repulsion sigma = range = cutoff = 0.3 (k = 1/sigma^2),
Nose-Hoover NVT at T=0.05, dt=0.002, reference patches.  One step = one noseHooverNVT::performUpdate: two geodesic
walks with velocity transport, one neighbour + exact-geodesic + force pass, the chain updates.

Metric: particle-steps/s (N x steps / time).
  value : inputs resident in HBM; K steps, each one CUDA-graph replay, timed with CUDA events on the launching
          stream; L2 flushed (a 512 MB write) before every timed step.
  e2e   : the same steps through the C ABI with host buffers: per step one cssg_system_step_host call copies the
          state (face, barycentrics, velocities, forces) from pinned host memory to the device, steps, and copies it
          back; wall clock.
The reference arm (--impl reference) times the CPU oracle (the C++ restatement of the reference path; the CGAL-based
reference itself cannot be built here) with all host threads on the same workload.
Multi-GPU: one process per GPU, each an independent replica of the system (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from curvedspacesim_gb300 import meshes as ms  # noqa: E402

# algorithmic work constants of the geodesic+force kernel (roofline accounting of the propagation); the FP64 flops of
# one processed window come from the library (api.flops_per_window(), counted once in its window geometry code)
BYTES_PER_SOURCE = 4 + 24 + 24 + 24   # read face, barycentrics, R3 position; write force
BYTES_PER_CANDIDATE = 4 + 4 + 24 + 24  # read index, face, barycentrics, R3 position
BYTES_PER_FACE = 12 + 12 + 72         # patch face: vertex ids, neighbours, edge frames
# DRAM bytes (read + write) of one launch of the regular propagation pass, from a full ncu capture of that workload
# (profiles/geodesic_kernel_torus200x100_N2000_nvt.txt, geodesic_kernel_bumpy_sphere7_N20000_screen.txt and
# lane_kernel_noisy_torus1000x500_N100000_nvt.txt, each with the pass the autotuner picks there); workloads without a
# capture report null
TRAFFIC_BYTES = {"torus200x100_N2000_nvt_patch": 50_715_648 + 116_845_824,
                 "bumpy_sphere7_N20000_nve_patch_screen": 98_532_096 + 43_409_920,
                 "noisy_torus1000x500_N100000_nvt_patch": 7_921_458 + 976_500_992}


def workload_config(name):
    if name == "batch64":
        return dict(workload="batch64_uneven_nve_patch", batched=True, n_systems=64, phi=0.4, integrator="nve",
                    submesh=True, dt=0.002, T=0.1, seed=3)
    if name == "bumpy_screen":
        return dict(workload="bumpy_sphere7_N20000_nve_patch_screen", mesh=("bumpy", 7, 0), n=20000, sigma=0.02,
                    integrator="nve", submesh=True, range_=0.02, dt=0.002, T=0.1, seed=4, screen=True,
                    train_seeds=list(range(1, 9)), configs_per_seed=8, holdout_seeds=[9, 10], train_steps=3000,
                    audit_every=50)
    if name == "noisy_torus_nvt":
        return dict(workload="noisy_torus1000x500_N100000_nvt_patch", mesh=("noisy_torus", 1000, 500), n=100000,
                    phi=0.5, sigma=None, integrator="nvt", submesh=True, range_=None, dt=0.001, T=0.05, seed=5)
    if name == "mlp_infer":
        return dict(workload="mlp14x64x64x64x1_bf16_4M_pairs", pairs=1 << 22, mlp=True)
    if name == "torus_nvt":
        return dict(workload="torus200x100_N2000_nvt_patch", mesh=("torus", 200, 100), n=2000, sigma=0.3,
                    integrator="nvt", submesh=True, range_=0.3, dt=0.002, T=0.05, seed=2)
    if name == "ico_nve":
        return dict(workload="icosphere4_N100_nve_alltoall", mesh=("ico", 4), n=100, sigma=0.2, integrator="nve",
                    submesh=False, range_=0.0, dt=0.005, T=0.1, seed=1)
    raise SystemExit(f"unknown workload {name}")


def build_batch(cfg):
    """64 independent systems: each an icosphere (subdivision 3-6), a torus grid (50x25 ... 400x200) or an
    ellipsoid (scaled icosphere, axes U[0.5, 2]); N log-uniform in [50, 5000]; sigma from area fraction 0.4."""
    rng = np.random.default_rng(cfg["seed"])
    systems = []
    for _ in range(cfg["n_systems"]):
        kind = rng.integers(3)
        if kind == 0:
            V, F = ms.icosphere(int(rng.integers(3, 7)))
            name = "icosphere"
        elif kind == 1:
            nu = int(rng.choice([50, 100, 200, 400]))
            V, F = ms.torus(nu, nu // 2, 3.0, 1.0)
            name = "torus"
        else:
            V, F = ms.ellipsoid(int(rng.integers(3, 7)), rng.uniform(0.5, 2.0, size=3))
            name = "ellipsoid"
        n = int(round(math.exp(rng.uniform(math.log(50), math.log(5000)))))
        sigma = ms.sigma_for_area_fraction(ms.total_area(V, F), n, cfg["phi"])
        f, b = ms.area_weighted_positions(V, F, n, rng)
        vel = ms.tangent_velocities(V, F, f, cfg["T"], rng)
        systems.append(dict(V=V, F=F, n=n, sigma=sigma, f=f, b=b, vel=vel, kind=name))
    return systems


def build_inputs(cfg):
    if cfg["mesh"][0] == "torus":
        V, F = ms.torus(cfg["mesh"][1], cfg["mesh"][2], 3.0, 1.0)
    elif cfg["mesh"][0] == "bumpy":
        V, F = ms.bumpy_sphere(cfg["mesh"][1], amplitude=0.05, seed=cfg["mesh"][2])
    elif cfg["mesh"][0] == "noisy_torus":
        V, F = ms.noisy_torus(cfg["mesh"][1], cfg["mesh"][2], 3.0, 1.0, std=0.01, smoothing_rings=3, seed=0)
    else:
        V, F = ms.icosphere(cfg["mesh"][1])
    rng = np.random.default_rng(cfg["seed"])
    f, b = ms.area_weighted_positions(V, F, cfg["n"], rng)
    vel = ms.tangent_velocities(V, F, f, cfg["T"], rng)
    return V, F, f, b, vel


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, max clock, throttle reasons).

    start() returns once the first sample has arrived, so the sampler's own start-up stays outside the timed region;
    begin() / end() bracket that region, and stop() keeps the samples that arrived inside it (plus the first one after
    it, which covers its last interval)."""

    PERIOD_MS = 100

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.t_begin = self.t_end = None
        self.first = threading.Event()

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=10.0)
        except OSError:
            self.proc = None

    def _read(self):
        try:
            for line in self.proc.stdout:
                self.lines.append((time.perf_counter(), line.strip()))
                self.first.set()
        finally:
            self.first.set()  # nvidia-smi ended (or failed): nothing more to wait for

    def begin(self):
        self.t_begin = time.perf_counter()

    def end(self):
        self.t_end = time.perf_counter()

    def stop(self):
        if self.proc is None:
            return None
        if self.t_end is not None:  # wait for the sample that covers the end of the region
            deadline = time.perf_counter() + 3 * self.PERIOD_MS * 1e-3
            while time.perf_counter() < deadline and not any(t > self.t_end for t, _ in self.lines):
                time.sleep(0.01)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        keep = list(self.lines)
        if self.t_begin is not None and self.t_end is not None:
            inside = [x for x in keep if self.t_begin <= x[0] <= self.t_end]
            after = [x for x in keep if x[0] > self.t_end][:1]
            keep = inside + after
        sm, mx, reasons = [], [], set()
        for _, ln in keep:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for name, val in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"],
                                 p[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
               "samples": len(sm), "period_ms": self.PERIOD_MS}
        if self.t_begin is not None and self.t_end is not None:
            out["region_s"] = round(self.t_end - self.t_begin, 4)
        return out


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def systems_of(cfg):
    """The workload as a list of independent systems (one entry for the single-system workloads)."""
    if cfg.get("batched"):
        out = build_batch(cfg)
        for sy in out:
            sy["range_"] = sy["sigma"]
        return out
    V, F, f, b, vel = build_inputs(cfg)
    sigma = cfg["sigma"]
    if sigma is None:  # from the area fraction: sigma = 2 sqrt(phi A / (N pi))
        sigma = ms.sigma_for_area_fraction(ms.total_area(V, F), cfg["n"], cfg["phi"])
    rng_ = cfg["range_"] if cfg["range_"] is not None else sigma
    return [dict(V=V, F=F, n=cfg["n"], sigma=sigma, range_=rng_, f=f, b=b, vel=vel)]


def oracle_step_rate(cfg, systems, threads, budget_s, max_steps=200):
    """Oracle (CPU restatement of the reference path) on `threads` host threads: particle-steps/s over whole steps
    of every system, stopping at the first step boundary after budget_s."""
    import oracle
    oracle.build()
    kind = 0 if cfg["integrator"] == "nve" else 1
    states = []
    for sy in systems:
        OM = oracle.OracleMesh(sy["V"], sy["F"])
        sigma = sy["sigma"]
        prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sy["range_"], submesh=int(cfg["submesh"]),
                        max_dist=sigma, cutoff=sigma, dt=cfg["dt"], T=cfg["T"])
        states.append([OM, prm, (sy["f"], sy["b"], sy["vel"], np.zeros((sy["n"], 3)), OM.nvt_chain(sy["n"], prm))])
    ntot = sum(sy["n"] for sy in systems)
    steps = 0
    t0 = time.perf_counter()
    while True:
        for st in states:
            OM, prm, state = st
            out = OM.simulate(kind, 1, *state[:4], prm, chain=state[4], threads=threads)
            st[2] = out[:5]
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s or steps >= max_steps:
            break
    return ntot * steps / el, steps


def run_reference(args, cfg):
    """CPU oracle (restatement of the reference path) with all host threads, same workload."""
    world, rank, _, pg = dist_setup()
    if rank != 0:
        return
    systems = systems_of(cfg)
    threads = os.cpu_count() or 1
    oracle_step_rate(cfg, systems, threads, 0.0, max_steps=args.warmup)  # warm-up
    value, steps = oracle_step_rate(cfg, systems, threads, 1e30, max_steps=args.steps)
    line = {
        "impl": "reference", "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(sy["n"] for sy in systems) / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": cfg["workload"], "n": sum(sy["n"] for sy in systems), "systems": len(systems),
                   "integrator": cfg["integrator"], "submesh": cfg["submesh"], "l2": "cpu run"},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} full steps of the whole workload (oracle restatement; CGAL "
                                   f"reference not buildable)"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(cfg, systems, seconds_budget=20.0):
    """Bounded sample of the same workload on the host: the oracle on all threads and on one thread."""
    threads = os.cpu_count() or 1
    v_all, s_all = oracle_step_rate(cfg, systems, threads, seconds_budget / 2)
    v_one, s_one = oracle_step_rate(cfg, systems, 1, seconds_budget / 2)
    return {"value": v_all, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{s_all} whole steps of the whole workload on {threads} threads (oracle restatement; the CGAL "
                      f"reference is not buildable); single thread: {v_one:.1f} particle-steps/s over {s_one} steps"}


def run_ours(args, cfg):
    import torch
    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    from curvedspacesim_gb300 import api

    systems = systems_of(cfg)
    n = sum(sy["n"] for sy in systems)
    ctx = api.Context(local)
    meshes, params = [], []
    for sy in systems:
        M = api.Mesh(sy["V"], sy["F"], device=local)
        sigma = sy["sigma"]
        meshes.append(M)
        params.append(api.make_params(cfg["integrator"], "harmonic", k=1.0 / sigma ** 2, sigma=sigma,
                                      range_=sy["range_"], submesh=cfg["submesh"], max_dist=sigma, cutoff=sigma,
                                      dt=cfg["dt"], temperature=cfg["T"]))
    S = api.System(ctx, meshes, [sy["n"] for sy in systems], params)
    S.set_state(np.concatenate([sy["f"] for sy in systems]), np.concatenate([sy["b"] for sy in systems]),
                np.concatenate([sy["vel"] for sy in systems]), np.zeros((n, 3)))
    stream = ctx.tstream  # the library's stream: events and the L2 flush are issued on it
    with ctx.use():
        flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    # warm-up, then the autotuner (band width, CTA size, medium-pass slots) on the warmed-up state, then one more
    # step that captures the graph with the chosen configuration
    S.step(max(args.warmup, 1), graph=not args.profile)
    torch.cuda.synchronize()
    bits, cnt = S.check()
    if bits:
        raise RuntimeError(f"per-item errors during warm-up: {bits:#x} {cnt}")
    tune = None
    if args.tuning:
        _apply_tuning(S, args.tuning)
        d, w, m, cap, lpt, g, wide = _parse_tuning(args.tuning)
        tune = {"delta_scale": d, "warps_per_block": w, "mid_slots": m, "warps_per_sm": cap, "lpt_order": lpt,
                "warps_per_source": g, "wide_registers": wide, "lanes_per_warp": S.lanes(), "lane_split": S.lane_split(),
                "pass_groups": list(S.pass_groups()), "source": "--tuning"}
        S.step(1, graph=not args.profile)
        torch.cuda.synchronize()
    elif not args.no_autotune:
        tune = S.autotune(reps=3)
        S.step(1, graph=not args.profile)
        torch.cuda.synchronize()
        bits, cnt = S.check()
        if bits:
            raise RuntimeError(f"per-item errors after autotuning: {bits:#x} {cnt}")
    if args.profile:
        S.step(1, graph=False)
        torch.cuda.synchronize()
        bits, cnt = S.check()
        print(json.dumps({"profile_run": cfg["workload"], "status_bits": bits, "counters": cnt}), flush=True)
        return

    # ---- value: resident inputs, one graph replay per step, L2 flushed before each step ----
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    barrier(pg)
    torch.cuda.synchronize()
    sampler.begin()
    for k in range(args.steps):
        with ctx.use():
            flush.zero_()
        starts[k].record(stream)
        S.step(1, graph=True)
        ends[k].record(stream)
    torch.cuda.synchronize()
    sampler.end()
    clocks = sampler.stop()
    barrier(pg)
    ms_steps = [a.elapsed_time(e) for a, e in zip(starts, ends)]
    t_ms = max_over_ranks(pg, sum(ms_steps))
    bits, cnt = S.check()
    if bits:
        raise RuntimeError(f"per-item errors in the timed region: {bits:#x} {cnt}")
    value = world * n * args.steps / (t_ms * 1e-3)
    kps = S.kernels_per_step()

    # ---- kernel times (events around the geodesic and walk kernels, no graph) ----
    S.timing(True)
    S.step(args.steps, graph=False)
    torch.cuda.synchronize()
    kt = S.last_times()
    S.timing(False)
    bits, cnt2 = S.check()
    geo_ms = kt["geodesic_ms"] / args.steps
    walk_ms = kt["walk_ms"] / args.steps

    # algorithmic work of the geodesic kernel per launch (counters of the timed-kernel pass)
    windows = cnt2["windows"] / args.steps
    S.enable_pairs()
    S.compute_forces()
    _, pj, _, _ = S.pairs()
    cands = len(pj)
    faces = sum(sy["n"] * min(len(sy["F"]), 1.3 * math.pi * (sy["sigma"] + 0.0) ** 2 /
                              (ms.total_area(sy["V"], sy["F"]) / len(sy["F"]))) for sy in systems)
    geo_bytes = n * BYTES_PER_SOURCE + cands * BYTES_PER_CANDIDATE + faces * BYTES_PER_FACE
    geo_flops = windows * api.flops_per_window()
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    fp64_peak = api.fp64_peak_gflops(ctx)
    achieved_gbs = geo_bytes / (geo_ms * 1e-3) / 1e9
    achieved_fp64 = geo_flops / (geo_ms * 1e-3) / 1e9
    traffic = TRAFFIC_BYTES.get(cfg["workload"])

    # ---- e2e: host state in, step, host state out, every step ----
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    hf, hb, hv, hfo = pin((n,), torch.int32), pin((n, 3), torch.float64), pin((n, 3), torch.float64), \
        pin((n, 3), torch.float64)
    hf[:], hb[:], hv[:], hfo[:] = S.get_state()
    barrier(pg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        S.step_host(1, hf, hb, hv, hfo)  # host state in, one step, host state out: one C-ABI call
    e2e_s = max_over_ranks(pg, time.perf_counter() - t0)
    e2e = world * n * args.steps / e2e_s
    io_bytes = n * (4 + 24 + 24 + 24)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(cfg, systems)

    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cfg["workload"], "n": n, "systems": len(systems), "integrator": cfg["integrator"],
                       "submesh": cfg["submesh"], "graph": True,
                       "l2": "flushed before every timed step (512 MB write)", "parallelism": f"replicas x{world}",
                       "autotune": tune},
            "e2e": {"value": e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": io_bytes,
                    "d2h_bytes_per_step": io_bytes},
            "gpu_launches": kps * args.steps,
            "roofline": {"bound": "fp64", "achieved": achieved_fp64, "peak": fp64_peak, "unit": "GFLOP/s",
                         "frac": achieved_fp64 / fp64_peak, "traffic": int(traffic) if traffic else None,
                         "kernel": "geodesic pass", "kernel_ms": geo_ms, "flops_per_launch": geo_flops,
                         "flops_per_window": api.flops_per_window(), "windows_per_launch": windows,
                         "lanes_per_warp": tune.get("lanes_per_warp") if tune else None,
                         "peak_source": "measured FP64 FMA chain on this GPU (cssg_diag_fp64_peak); "
                                        "MEASURED_PEAKS.json has no FP64 entry",
                         "hbm": {"achieved_gbs": achieved_gbs, "peak_gbs": hbm_peak, "frac": achieved_gbs / hbm_peak,
                                 "algorithmic_bytes_per_launch": geo_bytes,
                                 "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks
                                 else "of fallback 6.8 TB/s"}},
            "kernels_ms_per_step": {"geodesic": geo_ms, "walk": walk_ms},
            "counters_per_step": {k: v / args.steps for k, v in cnt2.items()},
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)


def _timed_steps(ctx, S, steps, flush, stream, graph=True):
    """K single steps, each timed with CUDA events on the library's stream after an L2 flush; returns ms per step."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        with ctx.use():
            flush.zero_()
        starts[k].record(stream)
        S.step(1, graph=graph)
        ends[k].record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(e) for a, e in zip(starts, ends)]


def oracle_audit(V, F, sigma, state, gpu_pairs, gpu_force, threads):
    """The FP64 oracle's neighbour distances and forces on one state, against a GPU pass on the same state:
    in-range pair sets (d <= sigma), the largest relative distance error over the common pairs, and the largest
    force difference."""
    import oracle
    oracle.build()
    face, bary = state[0], state[1]
    OM = oracle.OracleMesh(V, F)
    off, idx, mc = OM.candidates(face, bary, sigma)
    d_o, _, _ = OM.neighbor_distances(face, bary, off, idx, mc, 1, sigma, sigma, threads=threads)
    src = np.repeat(np.arange(len(face)), np.diff(off))
    ref = {(int(a), int(b)): float(x) for a, b, x in zip(src, idx, d_o) if x <= sigma}
    gi, gj, gd = gpu_pairs[:3]
    got = {(int(a), int(b)): float(x) for a, b, x in zip(gi, gj, gd) if b >= 0 and x <= sigma}
    common = set(ref) & set(got)
    rel = max([abs(got[k] - ref[k]) / ref[k] for k in common if ref[k] > 0] or [0.0])
    prm = OM.params(0, k=1.0 / sigma ** 2, sigma=sigma, rng=sigma, submesh=1, max_dist=sigma, cutoff=sigma)
    f_o, _, _ = OM.forces(face, bary, prm, threads=threads)
    return {"in_range_pairs": len(ref), "missing_in_range_pairs": len(set(ref) - set(got)),
            "extra_in_range_pairs": len(set(got) - set(ref)), "pair_sets_identical": set(ref) == set(got),
            "max_rel_distance_error": rel, "max_abs_force_error": float(np.max(np.abs(gpu_force - f_o))),
            "tolerance_rel_distance": 1e-6}


def screen_bound(ctx, M, sigma, state, pairs):
    """Upper bound of any screen's saving: the exact solver's windows for every candidate pair against the windows
    when only the in-range candidates (d <= sigma, known here from the exact pass) are queried, with the same patch
    radius per source (the reference patch does not depend on the screen)."""
    from curvedspacesim_gb300 import api
    face, bary = state[0], state[1]
    n = len(face)
    i, j, d = pairs[:3]
    pos = ms.bary_to_r3(M.V, M.F, face, bary)
    chord = np.linalg.norm(pos[i] - pos[j], axis=1)
    thr = np.zeros(n)
    np.maximum.at(thr, i, chord)
    thr = np.minimum(thr, sigma)
    out = {}
    for name, keep in (("all_candidates", np.ones(len(i), dtype=bool)), ("in_range_only", d <= sigma)):
        off = np.zeros(n + 1, dtype=np.int64)
        np.add.at(off, i[keep] + 1, 1)
        off = np.cumsum(off).astype(np.int32)
        _, _, _, st = api.distance_batch(ctx, M, face, bary, off, face[j[keep]], bary[j[keep]], submesh=True,
                                         max_dist=sigma, threshold=thr, cutoff=sigma)
        if np.any(st != 0):
            raise RuntimeError(f"screen bound: per-source errors {np.unique(st)}")
        out[name] = int(api.distance_batch.last_stats[:, 0].sum())
    return {"windows_all_candidates": out["all_candidates"], "windows_in_range_only": out["in_range_only"],
            "out_of_range_candidate_pairs": int((d > sigma).sum()), "candidate_pairs": int(len(d)),
            "max_window_saving": 1.0 - out["in_range_only"] / max(out["all_candidates"], 1)}


def run_screen(args, cfg):
    """Learned distance screen against the plain exact path on the same surface and particles (the metric's
    workload: bumpy sphere, subdivision 7, N=20,000, sigma 0.02, NVE).

    The screen is trained here on exact pairs that the GPU solver produces on other surfaces (train_seeds), with the
    library's own forward/backward/Adam kernels; its skip margin is calibrated on held-out surfaces (holdout_seeds) so
    that no held-out in-range pair is skipped.  Both paths then step the evaluation surface from the same state.
    After the timed steps the screened path's pairs and forces on its final state are audited against the FP64
    oracle (the CPU restatement of the reference path), and the plain path against the screened one."""
    import torch
    from curvedspacesim_gb300 import api, screen
    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    ctx = api.Context(local)
    sub, sigma, n = cfg["mesh"][1], cfg["sigma"], cfg["n"]

    def mesh_fn(seed):
        return ms.bumpy_sphere(sub, amplitude=0.05, seed=seed)

    if args.profile:
        # minimal run for ncu: the screened path with untrained weights (the tensor-core work per pair is the same),
        # a margin that skips nothing, three steps without graph replay
        V, F, f, b, vel = build_inputs(cfg)
        M = api.Mesh(V, F, device=local)
        prm = api.make_params(cfg["integrator"], "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=cfg["range_"],
                              submesh=cfg["submesh"], max_dist=sigma, cutoff=sigma, dt=cfg["dt"],
                              temperature=cfg["T"])
        S = api.System(ctx, M, n, prm)
        S.set_screen(screen.init_params(0), 1e6)
        S.set_state(f, b, vel, np.zeros((n, 3)))
        if args.tuning:
            _apply_tuning(S, args.tuning)
        S.step(max(args.warmup, 1), graph=False)
        torch.cuda.synchronize()
        bits, cnt = S.check()
        print(json.dumps({"profile_run": cfg["workload"], "status_bits": bits, "counters": cnt,
                          "screen": S.screen_counters()}), flush=True)
        return

    t0 = time.perf_counter()
    X, y, _, _ = screen.generate(ctx, mesh_fn, cfg["train_seeds"], n, sigma, configs_per_seed=cfg["configs_per_seed"])
    params, _ = screen.train(ctx, X, y, steps=cfg["train_steps"], batch=8192, lr=3e-3)
    Xh, yh, ch, _ = screen.generate(ctx, mesh_fn, cfg["holdout_seeds"], n, sigma, configs_per_seed=2)
    margin, cal = screen.calibrate(ctx, params, Xh, yh, ch)
    skip_frac, wrong = screen.skipped_fraction(ctx, params, margin, Xh, yh, ch)
    prep_s = time.perf_counter() - t0
    n_train = int(X.shape[0])
    del X, y, Xh, yh, ch

    V, F, f, b, vel = build_inputs(cfg)
    M = api.Mesh(V, F, device=local)
    prm = api.make_params(cfg["integrator"], "harmonic", k=1.0 / sigma ** 2, sigma=sigma, range_=cfg["range_"],
                          submesh=cfg["submesh"], max_dist=sigma, cutoff=sigma, dt=cfg["dt"], temperature=cfg["T"])
    plain = api.System(ctx, M, n, prm)
    scr = api.System(ctx, M, n, prm)
    scr.set_screen(params, margin)
    if cfg.get("audit_every"):
        scr.set_screen_audit(cfg["audit_every"])
    for S in (plain, scr):
        S.set_state(f, b, vel, np.zeros((n, 3)))
    stream = ctx.tstream
    with ctx.use():
        flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    tunes = {}
    for name, S in (("plain", plain), ("screened", scr)):
        S.step(max(args.warmup, 1), graph=True)
        if args.tuning:
            _apply_tuning(S, args.tuning)
            tunes[name] = {"source": "--tuning", "value": args.tuning}
        elif not args.no_autotune:
            tunes[name] = S.autotune(reps=3)
        S.step(1, graph=True)
    torch.cuda.synchronize()
    for name, S in (("plain", plain), ("screened", scr)):
        bits, cnt = S.check()
        if bits:
            raise RuntimeError(f"{name}: per-item errors during warm-up: {bits:#x} {cnt}")
    scr.screen_counters()  # reset: the line reports the timed steps

    sampler = ClockSampler(local)
    sampler.start()
    barrier(pg)
    torch.cuda.synchronize()
    sampler.begin()
    ms_plain = _timed_steps(ctx, plain, args.steps, flush, stream)
    audits0 = scr.screen_audit_status()["audits"] if cfg.get("audit_every") else 0
    ms_scr = _timed_steps(ctx, scr, args.steps, flush, stream)
    audits_timed = (scr.screen_audit_status()["audits"] - audits0) if cfg.get("audit_every") else 0
    sampler.end()
    clocks = sampler.stop()
    barrier(pg)
    t_plain = max_over_ranks(pg, sum(ms_plain))
    t_scr = max_over_ranks(pg, sum(ms_scr))
    for name, S in (("plain", plain), ("screened", scr)):
        bits, cnt = S.check()
        if bits:
            raise RuntimeError(f"{name}: per-item errors in the timed region: {bits:#x} {cnt}")
    value = world * n * args.steps / (t_scr * 1e-3)
    value_plain = world * n * args.steps / (t_plain * 1e-3)
    sc = scr.screen_counters()

    # kernel time of the geodesic passes on both paths (CUDA events on the library's stream, no graph) and the
    # windows they processed (the kernel's counters)
    # (audit steps run two force passes, so the screened system's audits are paused for this timing pass)
    kt, win = {}, {}
    for name, S in (("plain", plain), ("screened", scr)):
        if name == "screened" and cfg.get("audit_every"):
            S.set_screen_audit(0)
        S.check()
        S.timing(True)
        S.step(args.steps, graph=False)
        torch.cuda.synchronize()
        kt[name] = S.last_times()["geodesic_ms"] / args.steps
        S.timing(False)
        win[name] = S.check()[1]["windows"] / args.steps
        if name == "screened" and cfg.get("audit_every"):
            S.set_screen_audit(cfg["audit_every"])

    # audits on the screened path's final state: screened GPU pass against the FP64 oracle, plain GPU against
    # screened GPU, and the bound on what any screen could save
    st = scr.get_state()
    pairs = {}
    for name, S in (("plain", plain), ("screened", scr)):
        S.set_state(*st)
        S.enable_pairs()
        S.compute_forces()
        pairs[name] = S.pairs()
    f_scr = scr.get_state()[3]
    f_plain = plain.get_state()[3]
    threads = os.cpu_count() or 1
    audit_oracle = oracle_audit(V, F, sigma, st, pairs["screened"], f_scr, threads) if rank == 0 else None
    missing, extra, rel = screen.audit(pairs["plain"], pairs["screened"], sigma)
    audit_plain = {"missing_in_range_pairs": len(missing), "extra_in_range_pairs": len(extra),
                   "max_rel_distance_diff": rel, "max_abs_force_diff": float(np.max(np.abs(f_plain - f_scr)))}
    bound = screen_bound(ctx, M, sigma, st, pairs["plain"])

    # FP64 roofline of the geodesic kernel (the propagation's bound) on the screened path
    fp64_peak = api.fp64_peak_gflops(ctx)
    geo_flops = win["screened"] * api.flops_per_window()
    achieved = geo_flops / (kt["screened"] * 1e-3) / 1e9
    traffic = TRAFFIC_BYTES.get(cfg["workload"])

    # e2e through the C ABI with host state, screened path
    pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
    hf, hb, hv, hfo = pin((n,), torch.int32), pin((n, 3), torch.float64), pin((n, 3), torch.float64), \
        pin((n, 3), torch.float64)
    hf[:], hb[:], hv[:], hfo[:] = scr.get_state()
    scr.step_host(1, hf, hb, hv, hfo)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        scr.step_host(1, hf, hb, hv, hfo)  # host state in, one step, host state out: one C-ABI call
    e2e = world * n * args.steps / max_over_ranks(pg, time.perf_counter() - t1)
    io_bytes = n * (4 + 24 + 24 + 24)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(cfg, [dict(V=V, F=F, n=n, sigma=sigma, range_=cfg["range_"], f=f, b=b, vel=vel)])
    if rank == 0:
        line = {
            "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_scr / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cfg["workload"], "n": n, "integrator": cfg["integrator"], "submesh": True,
                       "graph": True, "l2": "flushed before every timed step (512 MB write)",
                       "parallelism": f"replicas x{world}", "autotune": tunes or None,
                       "screen_audit_every": cfg.get("audit_every")},
            "plain": {"value": value_plain, "ms_per_step": t_plain / args.steps, "geodesic_ms": kt["plain"],
                      "windows_per_step": win["plain"]},
            "screened": {"value": value, "ms_per_step": t_scr / args.steps, "geodesic_ms": kt["screened"],
                         "windows_per_step": win["screened"], "speedup_vs_plain": value / value_plain,
                         "counters": sc},
            "screen": {"training_pairs": n_train, "train_seeds": cfg["train_seeds"],
                       "holdout_seeds": cfg["holdout_seeds"], "margin": margin, "calibration": cal,
                       "holdout_skip_fraction": skip_frac, "holdout_wrongly_skipped": wrong,
                       "prep_seconds": prep_s, "bound": bound},
            "audit_vs_oracle": audit_oracle,
            "audit_vs_plain": audit_plain,
            "e2e": {"value": e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": io_bytes,
                    "d2h_bytes_per_step": io_bytes},
            "gpu_launches": scr.kernels_per_step() * (args.steps - audits_timed)
                            + scr.kernels_per_audit_step() * audits_timed,
            "audited_steps": audits_timed,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "GFLOP/s",
                         "frac": achieved / fp64_peak, "traffic": int(traffic) if traffic else None,
                         "kernel": "geodesic (screened path)", "kernel_ms": kt["screened"],
                         "flops_per_launch": geo_flops, "flops_per_window": api.flops_per_window(),
                         "windows_per_launch": win["screened"],
                         "peak_source": "measured FP64 FMA chain on this GPU (cssg_diag_fp64_peak); "
                                        "MEASURED_PEAKS.json has no FP64 entry"},
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)


def _parse_tuning(text):
    """delta_scale,warps_per_block,mid_slots,warps_per_sm,lpt[,warps_per_source[,wide_registers[,lanes[,split[,medium,
    large]]]]]: the first seven are System.set_tuning's arguments, the eighth System.set_lanes' (0: source groups), the
    ninth System.set_lane_split's (the costliest sources that the group pass takes before the lane pass), the last two
    System.set_pass_groups' (warps per source of the medium and large passes)."""
    fields = text.split(",")
    d, w, m, cap, lpt = fields[:5]
    g = int(fields[5]) if len(fields) > 5 else 1
    wide = int(fields[6]) if len(fields) > 6 else 0
    return float(d), int(w), int(m), int(cap), bool(int(lpt)), g, wide


def _apply_tuning(S, text):
    S.set_tuning(*_parse_tuning(text))
    fields = text.split(",")
    S.set_lanes(int(fields[7]) if len(fields) > 7 else 0)
    S.set_lane_split(int(fields[8]) if len(fields) > 8 else 0)
    S.set_pass_groups(int(fields[9]) if len(fields) > 9 else 0, int(fields[10]) if len(fields) > 10 else 0)


def run_mlp(args, cfg):
    """The screen's tensor-core inference kernel on its own: 4M feature rows (BF16, 14 features padded to 16) through
    14->64->64->64->1 with GELU.  The input (128 MB) exceeds L2, so no flush is needed between launches.  Reports
    pairs/s and the tensor roofline (2 * (16*64 + 64*64 + 64*64 + 64) FLOP per pair as executed)."""
    import torch
    from curvedspacesim_gb300 import _lib, api, screen
    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    ctx = api.Context(local)
    n = cfg["pairs"]
    dev = f"cuda:{local}"
    g = torch.Generator(device="cpu").manual_seed(7)
    X = torch.randn((n, 16), generator=g).to(torch.bfloat16)
    X[:, 14:] = 0
    X = X.to(dev)
    params = torch.tensor(screen.init_params(0), device=dev)
    with ctx.use():
        y = torch.empty(n, dtype=torch.float32, device=dev)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
    L = _lib.load()
    P = _lib.ctypes.c_void_p
    torch.cuda.synchronize()

    def launch():
        rc = L.cssg_mlp_infer(ctx.h, P(X.data_ptr()), n, P(params.data_ptr()), P(y.data_ptr()), P(err.data_ptr()))
        if rc:
            raise RuntimeError(L.cssg_last_error().decode())

    for _ in range(max(args.warmup, 1)):
        launch()
    torch.cuda.synchronize()
    stream = ctx.tstream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    torch.cuda.synchronize()
    sampler.begin()
    for k in range(args.steps):
        ev[2 * k].record(stream)
        launch()
        ev[2 * k + 1].record(stream)
    torch.cuda.synchronize()
    sampler.end()
    clocks = sampler.stop()
    if int(err.item()):
        raise RuntimeError("tensor-core completion wait timed out")
    ms_each = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(args.steps)]
    t_ms = max_over_ranks(pg, sum(ms_each))
    value = world * n * args.steps / (t_ms * 1e-3)

    # ---- e2e: pinned host features in, host predictions out, through the C ABI call, every step ----
    Xh = X.cpu().pin_memory()
    yh = torch.empty(n, dtype=torch.float32).pin_memory()
    for _ in range(2):
        with torch.cuda.stream(stream):
            X.copy_(Xh, non_blocking=True)
        launch()
        with torch.cuda.stream(stream):
            yh.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    barrier(pg)
    t1 = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            X.copy_(Xh, non_blocking=True)
        launch()
        with torch.cuda.stream(stream):
            yh.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(pg, time.perf_counter() - t1)
    e2e = world * n * args.steps / e2e_s

    # ---- CPU baseline (rank 0): the oracle's FP64 forward with the kernel's BF16 roundings on a 65,536-row sample
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, ROOT)
        from oracle import mlp_ref
        Xs = X[:65536].float().cpu().numpy()
        ps = params.cpu().numpy()
        mlp_ref.forward(Xs[:1024], ps)
        reps, t2 = 0, time.perf_counter()
        while reps < 3 or time.perf_counter() - t2 < 2.0:
            mlp_ref.forward(Xs, ps)
            reps += 1
        cpu = {"value": reps * len(Xs) / (time.perf_counter() - t2), "unit": "pairs/s",
               "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{reps} passes over 65,536 of the rows (oracle/mlp_ref.forward, numpy FP64 with BF16 "
                         f"roundings; BLAS threads as numpy sets them)"}
    flops_pair = 2 * (16 * 64 + 64 * 64 + 64 * 64 + 64)
    achieved = value / world * flops_pair / 1e12
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    peak = peaks.get("bf16_tflops", 1900.0)
    if rank == 0:
        print(json.dumps({
            "metric": "screened pairs/s", "value": value, "unit": "pairs/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)", "data": "synthetic",
            "config": {"workload": cfg["workload"], "pairs_per_launch": n,
                       "l2": "inputs (128 MB) larger than L2", "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None, "kernel": "mlp_infer_tc",
                         "flops_per_pair": flops_pair,
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)" if peaks else "of fallback"},
            "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": n * 16 * 2, "d2h_bytes_per_step": n * 4},
            "cpu_baseline": cpu, "gpu_launches": args.steps, "clocks": clocks}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="bumpy_screen")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tuning (band width 1, 8 warps)")
    ap.add_argument("--tuning", default="",
                    help="explicit tuning instead of the autotuner: delta_scale,warps_per_block,mid_slots,"
                         "warps_per_sm,lpt[,warps_per_source[,wide_registers[,lanes_per_warp[,lane_split[,medium,"
                         "large]]]]] "
                         "(e.g. 4,8,0,0,1,2,0 or 2,8,0,0,0,1,1,32)")
    ap.add_argument("--profile", action="store_true",
                    help="minimal run for ncu: warm-up steps, then one step without graph replay, no other legs")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    cfg = workload_config(args.workload)
    if args.impl == "reference":
        run_reference(args, cfg)
    elif cfg.get("screen"):
        run_screen(args, cfg)
    elif cfg.get("mlp"):
        run_mlp(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()
