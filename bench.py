#!/usr/bin/env python
"""EBE-PCG benchmark of the p121 solve on GB300.

Headline workload: the 100x100x100 20-node hexahedron cube (nip=27, E=100,
v=0.3, every dof of the base face fixed, uniform top pressure with total
load -1), ~12.2M equations, synthetic (generated in memory; no dataset).

  step   = one PCG iteration over the whole mesh (element products, node
           scatter, fused updates and reductions) of the mixed-precision
           solver's inner loop (FP32 storkm, FP64 vectors and scalars);
  value  = equations x steps / device time of the K timed steps (DOF.iter/s);
  e2e    = one full mixed-precision solve to ||f-Ku||/||f|| <= 1e-8 through
           pf_solve with host buffers (load vector in, displacements out),
           DOF.iter/s over its wall time;
  time_to_1e8 = wall time of that solve and of the plain FP64 solve, and
           the displacement error of both against FP64 solved to 1e-12.

The default run also measures the other configurations of the benchmark in
the same line ("configs"): the 80^3 heterogeneous cube (mixed vs FP64 at
1e-8, errors against FP64 at 1e-12), the 60^3 cube with 16 load cases
(block solve on the tensor cores vs 16 sequential FP64 solves) and the
serving stream (continuous batching, p50/p99 latency and solves/s); the
10^3 CPU-runnable case is in the CPU baseline leg, against the CPU build.

--impl reference times the CPU build of p121's PCG (oracle/p121_cpu.c,
OpenMP on all host cores, every loop of the iteration parallel) on the same
100^3 cube.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "EBE-PCG DOF·iter/s & time-to-1e-8, mixed vs FP64 on 1 GB300; serving p50/p99 ms"
UNIT = "DOF·iter/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=100, help="elements per cube edge")
    ap.add_argument("--no-solves", action="store_true", help="skip the time-to-1e-8 solves")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-configs", action="store_true",
                    help="cube100: skip the other configurations (heterogeneous 80^3, 16 load cases at 60^3, "
                         "serving stream)")
    ap.add_argument("--serving-requests", type=int, default=500,
                    help="cube100: requests of the serving stream measured in the default line")
    ap.add_argument("--workload", default="cube100",
                    choices=["cube100", "hetero80", "serving", "multirhs60", "cube10", "shared100", "p123book",
                             "p122book"],
                    help="cube100: the headline; hetero80: per-element E and v, accuracy study; "
                         "serving: continuous batching of a Poisson request stream; shared100: one element "
                         "matrix for every element (PCG_KM); p123book: p123's book run (Laplace, 200^3 8-node "
                         "bricks); p122book: p122's book run (Mohr-Coulomb viscoplasticity, 20^3 20-node bricks, "
                         "12 load increments)")
    ap.add_argument("--requests", type=int, default=2000, help="serving: number of requests")
    ap.add_argument("--rates", default="20", help="serving: comma-separated arrival rates (requests/s); "
                                                    "0 = all requests at t=0")
    ap.add_argument("--budget-gb", type=float, default=40.0, help="serving: device-memory budget of the batch")
    ap.add_argument("--chunk", type=int, default=10, help="serving: PCG iterations per launch/sync cycle")
    ap.add_argument("--serving-prec", type=int, default=32, choices=[16, 32, 64],
                    help="serving: 32 = FP32 products with FP64 residual replacement, 16 = FP16 storkm "
                         "products with the same replacement, 64 = FP64")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--limit", type=int, default=50000, help="multirhs60: PCG iteration limit of the block solves")
    ap.add_argument("--tuning", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="cube100: force the packed-symmetric kernel configuration (0: 14x2, 1: 12x2, 2: 8x3); "
                         "-1 keeps the autotuner's choice")
    return ap.parse_args()


# ---------------------------------------------------------------------------
_BACKEND = "nccl"


def dist_init(n_gpus):
    """torch.distributed for N > 1 replicas (one process per GPU).  The
    backend is NCCL; PF_DIST_BACKEND=gloo runs the same aggregation on CPU."""
    global _BACKEND
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        _BACKEND = os.environ.get("PF_DIST_BACKEND", "nccl")
        if _BACKEND == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(_BACKEND)
        return rank, world, local, dist
    return 0, 1, 0, None


def _reduce(dist, local, v, op):
    import torch
    dev = f"cuda:{local}" if _BACKEND == "nccl" else "cpu"
    t = torch.tensor([float(v)], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=op)
    return float(t.item())


def dist_max(dist, local, v):
    """Max over ranks (the slowest replica's time)."""
    return v if dist is None else _reduce(dist, local, v, dist.ReduceOp.MAX)


def dist_sum(dist, local, v):
    """Sum over ranks (the units all replicas processed)."""
    return v if dist is None else _reduce(dist, local, v, dist.ReduceOp.SUM)


def barrier(dist):
    if dist is not None:
        dist.barrier()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel_tag, key="dram_bytes_per_launch_full_size"):
    """A DRAM figure from the committed ncu summary of that kernel, if any:
    bytes per full-size launch (the default key), or, with key
    dram_per_algorithmic_byte, the DRAM bytes per algorithmic byte of a
    smaller capture of the same kernel."""
    path = os.path.join(ROOT, "profiles", f"{kernel_tag}.md")
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


# ---------------------------------------------------------------------------
def elem_bytes(nels, nslots, storkm_bytes, result_bytes):
    """Algorithmic bytes of one element-product launch: storkm (per element),
    connectivity, the element results and the gathered vector (each slot once)."""
    return nels * (storkm_bytes + 20 * 4 + 60 * result_bytes) + nslots * 8


def cpu_build_leg(n, k_steps, warm):
    """The CPU build of p121's PCG (oracle/p121_cpu.c: OpenMP over every loop
    of the iteration, -O3 with contraction) on the n^3 cube: storkm formed on
    the host, then `warm` untimed and `k_steps` timed PCG iterations."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    c = O.CpuP121(n, n, n, 27, 100.0, 0.3)
    t_setup = time.perf_counter() - t0
    try:
        c.init()
        c.iterate(max(warm, 1))
        t1 = time.perf_counter()
        c.iterate(k_steps)
        dt = time.perf_counter() - t1
        return {"value": c.neq * k_steps / dt, "unit": UNIT, "cores": c.threads, "kind": "port", "seconds": dt,
                "setup_s": t_setup,
                "sample": f"{n}x{n}x{n} cube (neq {c.neq}, storkm {n ** 3 * 28800 / 1e9:.1f} GB FP64), nip 27, "
                          f"{k_steps} p121 PCG iterations of the CPU build (oracle/p121_cpu.c: GATHER, element "
                          f"products, node-centric SCATTER, dot products, updates and checon_par on "
                          f"{c.threads} OpenMP threads, gcc -O3 -ffp-contract=fast)"}
    finally:
        c.close()


def cpu_config1(gpu_x, gpu_iters, gpu_wall):
    """Config 1 (10^3, checon_par tol 1e-6, limit 5000) on the CPU build:
    its iterations, time and solution against the GPU drop-in's."""
    from oracle import oracle as O
    c = O.CpuP121(10, 10, 10, 27, 100.0, 0.3)
    try:
        c.init()
        t0 = time.perf_counter()
        it = c.iterate(5000, 1e-6, 0)
        dt = time.perf_counter() - t0
        x = c.x()
    finally:
        c.close()
    return {"workload": "p121 10^3 hex20 cube (the CPU-runnable case), nip 27, E 100, v 0.3, fixed base, top "
                        "pressure (total -1), checon_par tol 1e-6, limit 5000",
            "neq": int(x.size), "gpu_p121_drop_in": {"iters": gpu_iters, "solve_wall_s": gpu_wall},
            "cpu_build": {"iters": it, "solve_wall_s": dt},
            "iters_equal": gpu_iters == it,
            "rel_err_2": float(np.linalg.norm(gpu_x - x) / np.linalg.norm(x)),
            "rel_err_inf": float(np.abs(gpu_x - x).max() / np.abs(x).max()), "tolerance": 1e-6}


def oracle_cube(nxe, nye, nze):
    """Fixed-base, top-pressure cube built with the oracle's own routines."""
    from oracle import oracle as O
    L = O.lib()
    nels = nxe * nye * nze
    g_num = np.zeros((nels, 20), np.int32)
    gc = np.zeros((nels, 3, 20))
    coord = np.zeros(60)
    num = np.zeros(20, np.int32)
    for e in range(nels):
        L.orc_geometry_20bxz(e + 1, nxe, nze, 1.0, 1.0, 1.0, coord, num)
        g_num[e] = num
        gc[e] = coord.reshape(3, 20)
    nn = int(g_num.max())
    base = np.unique(g_num[:, [0, 6, 7, 8, 11, 12, 18, 19]][np.arange(nels) % (nxe * nze) >= nxe * (nze - 1)])
    rest = np.zeros((len(base) + 1, 4), np.int32)
    rest[0] = [1, 1, 1, 1]                     # keeps find_g3 inside rest
    rest[1:, 0] = base
    g_g = O.steering(g_num, rest)
    neq = int(g_g.max())
    r = np.zeros(neq + 1)
    p = 1.0 / (nxe * nye)
    top = np.nonzero(np.arange(nels) % (nxe * nze) < nxe)[0]
    for e in top:
        for a in (3, 5, 15, 17):
            r[g_g[e, 3 * a - 1]] += p / 12.0
        for a in (4, 10, 11, 16):
            r[g_g[e, 3 * a - 1]] -= p / 3.0
    return dict(g_num=g_num, gc=gc, g_g=g_g, neq=neq, r=r[1:].copy(), nn=nn)


def run_reference(args, rank):
    if rank != 0:
        return 0
    n = args.size
    leg = cpu_build_leg(n, args.steps, args.warmup)
    line = {
        "metric": METRIC, "value": leg["value"], "unit": UNIT, "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * leg["seconds"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_of(args),
        "cpu_baseline": {k: leg[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": leg["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": leg["setup_s"],
        "note": "ParaFEM's Fortran/MPI p121 cannot be built here (no Fortran compiler or MPI); the timed "
                "reference is the CPU build of its PCG in oracle/p121_cpu.c, every loop of the iteration on "
                "all host threads, as MPI p121 spreads them over ranks",
    }
    print(json.dumps(line))
    return 0


def config_of(args):
    n = args.size
    return {"workload": f"p121 cube {n}x{n}x{n} hex20, nip 27, E 100, v 0.3, fixed base, top pressure "
                        f"(total -1), mixed FP32-storkm PCG + FP64 defect correction",
            "nels": n ** 3, "global_batch": 1, "parallelism": "replicas",
            "l2": "inputs larger than L2 (storkm FP32 %.1f GB)" % (n ** 3 * 14400 / 1e9)}


def run_gb300(args, rank, world, local, dist):
    import parafem_gb300 as P
    n = args.size
    t0 = time.perf_counter()
    prob = P.cube_problem(n, n, n)
    t_host = time.perf_counter() - t0
    s = P.Solver(local)
    s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    s.set_material(100.0, 0.3)
    t1 = time.perf_counter()
    s.form_storkm(27)
    t_form = time.perf_counter() - t1
    neq = prob["neq"]
    nels = n ** 3
    r = prob["r"]
    extra = {"host_setup_s": t_host, "storkm_formation_s": t_form, "autotune": s.tuning()}
    if args.tuning >= 0:
        s.set_tuning(args.tuning)
        extra["forced_tuning"] = args.tuning

    # e2e: one full mixed solve through the C-ABI with host buffers
    solves = {}
    e2e_val = None
    if args.no_solves:
        s.solve(r, 1e-8, 1, P.MODE_MIXED)          # loads the right-hand side only
    else:
        barrier(dist)
        t2 = time.perf_counter()
        x, it_m, rel_m = s.solve(r, 1e-8, 20000, P.MODE_MIXED)
        t_mixed = time.perf_counter() - t2
        st_m = s.stats()
        t_mixed = dist_max(dist, local, t_mixed)
        e2e_val = dist_sum(dist, local, neq * it_m) / t_mixed
        solves["mixed"] = {"wall_s": t_mixed, "device_s": st_m["solve_ms"] / 1e3, "inner_iters": it_m,
                           "corrections": st_m["outer"], "relres": rel_m}
        # FP16 storkm in the inner products (PF_MODE_MIXED16); the FP16 copy is
        # packed once, before the timed solve, as a caller would after forming storkm
        s.bench_iterations(16, 1)
        barrier(dist)
        t5 = time.perf_counter()
        x16, it_16, rel_16 = s.solve(r, 1e-8, 40000, P.MODE_MIXED16)
        t_16 = dist_max(dist, local, time.perf_counter() - t5)
        st_16 = s.stats()
        solves["mixed16"] = {"wall_s": t_16, "device_s": st_16["solve_ms"] / 1e3, "inner_iters": it_16,
                             "corrections": st_16["outer"], "relres": rel_16}
        t3 = time.perf_counter()
        x64, it_64, rel_64 = s.solve(r, 1e-8, 20000, P.MODE_FP64_RES)
        t_64 = dist_max(dist, local, time.perf_counter() - t3)
        st_64 = s.stats()
        solves["fp64"] = {"wall_s": t_64, "device_s": st_64["solve_ms"] / 1e3, "iters": it_64,
                          "relres": rel_64}
        solves["mixed_over_fp64_time"] = t_mixed / t_64
        solves["mixed16_over_fp64_time"] = t_16 / t_64
        solves["mixed_vs_fp64_rel_err_2"] = float(np.linalg.norm(x - x64) / np.linalg.norm(x64))
        # accuracy: both solutions against FP64 converged to relres 1e-12
        xr, it_r, rel_r = s.solve(r, 1e-12, 50000, P.MODE_FP64_RES)
        nr_ = np.linalg.norm(xr)
        solves["fp64_1e-12"] = {"iters": it_r, "relres": rel_r, "device_s": s.stats()["solve_ms"] / 1e3}
        solves["mixed_vs_fp64_1e-12_rel_err_2"] = float(np.linalg.norm(x - xr) / nr_)
        solves["mixed_vs_fp64_1e-12_rel_err_inf"] = float(np.abs(x - xr).max() / np.abs(xr).max())
        solves["fp64_1e-8_vs_fp64_1e-12_rel_err_2"] = float(np.linalg.norm(x64 - xr) / nr_)
        solves["mixed16_vs_fp64_1e-12_rel_err_2"] = float(np.linalg.norm(x16 - xr) / nr_)
        solves["mixed16_vs_fp64_1e-12_rel_err_inf"] = float(np.abs(x16 - xr).max() / np.abs(xr).max())

    # timed steps: K iterations of the FP32-storkm PCG, device resident
    s.bench_iterations(32, max(args.warmup, 3))
    clk = Clocks(local).start() if rank == 0 else None
    l0 = s.launches()
    barrier(dist)
    ms_tot, ms_elem, ms_scat = s.bench_iterations(32, args.steps)
    barrier(dist)
    launches = s.launches() - l0
    clocks = clk.stop() if clk else None
    ms_tot = dist_max(dist, local, ms_tot)
    value = dist_sum(dist, local, neq) * args.steps / (ms_tot / 1e3)
    # FP64 steps (the plain drop-in path) and full-storage FP32 steps, for reference
    k2 = max(args.steps // 2, 3)
    s.bench_iterations(64, 3)
    ms64, ms64_elem, _ = s.bench_iterations(64, k2)
    extra["fp64_dof_iter_s"] = neq * k2 / (ms64 / 1e3)
    extra["fp64_elem_ms"] = ms64_elem / k2
    ms31, ms31_elem, _ = s.bench_iterations(31, k2)
    extra["fp32_full_dof_iter_s"] = neq * k2 / (ms31 / 1e3)
    extra["fp32_full_elem_ms"] = ms31_elem / k2
    s.bench_iterations(16, 3)
    ms16, ms16_elem, _ = s.bench_iterations(16, args.steps)
    extra["fp16_dof_iter_s"] = neq * args.steps / (ms16 / 1e3)
    extra["fp16_step_ms"] = ms16 / args.steps
    extra["fp16_elem_ms"] = ms16_elem / args.steps
    extra["fp16_autotune"] = s.tuning16()

    peak, peak_kind = measured_peaks()
    nslots = 3 * prob["nn"]
    b_launch = elem_bytes(nels, nslots, 7328, 4)
    avg_s = ms_elem / args.steps / 1e3
    achieved = b_launch / avg_s / 1e9
    roof = {"kernel": "k_elem_sym32 (packed-symmetric FP32 storkm, bulk-copy staged)", "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_launch": b_launch,
            "avg_launch_ms": avg_s * 1e3, "traffic": ncu_traffic("k_elem_sym32_cube100"),
            "scatter_avg_ms": ms_scat / args.steps}
    extra["fp64_elem_hbm_frac"] = elem_bytes(nels, nslots, 28800, 8) / (ms64_elem / k2 / 1e3) / 1e9 / peak
    extra["fp32_full_elem_hbm_frac"] = elem_bytes(nels, nslots, 14400, 4) / (ms31_elem / k2 / 1e3) / 1e9 / peak
    extra["fp16_elem_hbm_frac"] = elem_bytes(nels, nslots, 3664, 4) / (ms16_elem / args.steps / 1e3) / 1e9 / peak

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (packed-symmetric storkm) / f64 vectors and reductions", "data": "synthetic",
        "config": config_of(args),
        "e2e": None if e2e_val is None else {
            "value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(neq * 8),
            "d2h_bytes_per_step": int(neq * 8), "step": "one full mixed solve to relres 1e-8"},
        "time_to_1e8": solves, "roofline": roof, "gpu_launches": int(launches),
        "clocks": clocks, "extra": extra,
    }
    s.close()
    if not args.no_configs and world == 1:
        line["configs"] = other_configs(args, local)
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            leg = cpu_build_leg(n, 10, 2)
            line["cpu_baseline"] = {k: v for k, v in leg.items() if k not in ("seconds",)}
            x1, it1, t1 = gpu_config1(local)
            line["cpu_baseline"]["config1_vs_gpu_drop_in"] = cpu_config1(x1, it1, t1)
        except Exception as exc:  # the baseline is reported, never the target
            line["cpu_baseline"] = {"error": str(exc)}
    if rank == 0:
        print(json.dumps(line))
    return 0


def other_configs(args, local):
    """The benchmark's other configurations, measured in the default run:
    heterogeneous 80^3 (mixed and FP64 to 1e-8, errors against FP64 at
    1e-12), 16 load cases at 60^3 (tensor-core block solve against 16
    sequential FP64 solves) and the serving stream (a Poisson stream at 20
    requests/s and the same requests all at once)."""
    out = {}
    t0 = time.perf_counter()
    out["hetero80"] = hetero_solves(80, args.seed, local, ("mixed", "fp64"))
    out["hetero80"]["bench_wall_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    out["multirhs60"] = multirhs_solves(60, 16, args.seed, local, args.limit, (16,), True, strict=True)
    out["multirhs60"]["bench_wall_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    nreq = args.serving_requests
    res = serving_stream(nreq, [20.0, 0.0], args.budget_gb, args.chunk, args.serving_prec, args.seed, local)
    out["serving"] = {"workload": serving_workload(nreq, args.budget_gb, args.seed),
                      "prec": args.serving_prec, "at_20_per_s": res[0], "all_at_once": res[1],
                      "bench_wall_s": time.perf_counter() - t0}
    return out


def hetero_solves(n, seed, local, modes=("mixed", "fp64")):
    """n^3 cube with per-element E log-uniform in [1, 1000] and v uniform in
    [0.2, 0.35] (Philox4x32-10, key = seed, counter = element index): the
    given solves to relres 1e-8, and the displacement error of each against
    the FP64 solve converged to relres 1e-12."""
    import parafem_gb300 as P
    prob = P.cube_problem(n, n, n)
    nels = n ** 3
    e, v = P.random_material(nels, seed, 1.0, 1000.0, 0.2, 0.35)
    s = P.Solver(local)
    try:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(e, v)
        s.form_storkm(27)
        neq, r = prob["neq"], prob["r"]
        out = {"workload": f"heterogeneous {n}^3 hex20 cube, E log-uniform [1,1000], v uniform [0.2,0.35], "
                           f"Philox4x32-10 seed {seed}, nip 27, fixed base, top pressure, tol 1e-8",
               "nels": nels, "neq": neq}
        xr, itr, relr = s.solve(r, 1e-12, 50000, P.MODE_FP64_RES)
        out["oracle_fp64_1e-12"] = {"iters": itr, "relres": relr, "device_s": s.stats()["solve_ms"] / 1e3}
        nr = np.linalg.norm(xr)
        if "mixed16" in modes:
            s.ebe_matvec(np.zeros(neq), 16)   # packs the FP16 storkm once, outside the timed solves
        names = {"mixed": P.MODE_MIXED, "mixed16": P.MODE_MIXED16, "fp64": P.MODE_FP64_RES,
                 "mixed_restart": P.MODE_MIXED_RESTART}
        for name in modes:
            t0 = time.perf_counter()
            x, it, rel = s.solve(r, 1e-8, 50000, names[name])
            wall = time.perf_counter() - t0
            st = s.stats()
            out[name] = {"iters": it, "relres": rel, "wall_s": wall, "device_s": st["solve_ms"] / 1e3,
                         "corrections": st["outer"], "rel_err_2": float(np.linalg.norm(x - xr) / nr),
                         "rel_err_inf": float(np.abs(x - xr).max() / np.abs(xr).max())}
        if "mixed" in out and "fp64" in out:
            out["mixed_over_fp64_time"] = out["mixed"]["wall_s"] / out["fp64"]["wall_s"]
            out["mixed_dof_iter_per_s"] = neq * out["mixed"]["iters"] / out["mixed"]["device_s"]
        if "mixed16" in out and "fp64" in out:
            out["mixed16_over_fp64_time"] = out["mixed16"]["wall_s"] / out["fp64"]["wall_s"]
        return out
    finally:
        s.close()


def run_hetero(args, rank, world, local, dist):
    """The heterogeneous cube (80^3 by default) with every solve mode."""
    n = args.size if args.size != 100 else 80
    out = hetero_solves(n, args.seed, local, ("mixed", "mixed16", "fp64", "mixed_restart"))
    value = out["mixed_dof_iter_per_s"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 0,
            "ms_per_step": out["mixed"]["device_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (packed-symmetric storkm) / f64 vectors and reductions",
            "data": "synthetic",
            "config": {"workload": out["workload"], "nels": out["nels"], "neq": out["neq"]},
            "solves": out}
    if rank == 0:
        print(json.dumps(line))
    return 0


def serving_requests(n, seed):
    """The serving stream's requests (seeded): cube edges uniform in 4..40,
    E log-uniform in [10, 1000], v uniform in [0.2, 0.35], top pressure
    uniform in [0.5, 2.0]; fixed base; tol 1e-8."""
    rng = np.random.default_rng(seed)
    dims = rng.integers(4, 41, size=(n, 3))
    e = np.exp(rng.uniform(np.log(10.0), np.log(1000.0), n))
    v = rng.uniform(0.2, 0.35, n)
    pres = rng.uniform(0.5, 2.0, n)
    return dims, e, v, pres


def serving_stream(n_req, rates, budget_gb, chunk, prec, seed, local):
    """Continuous batching of a Poisson request stream (requests from
    serving_requests): one result per arrival rate (0 = every request at
    t = 0) with p50/p99 latency, solves/s and DOF.iter/s."""
    import collections
    import parafem_gb300 as P
    dims, es, vs, pres = serving_requests(n_req, seed)
    results = []
    for rate in rates:
        rng = np.random.default_rng(seed + 1)
        gaps = rng.exponential(1.0 / rate, n_req) if rate > 0 else np.zeros(n_req)
        arrivals = np.cumsum(gaps) - (gaps[0] if rate > 0 else 0.0)
        b = P.Batch(int(budget_gb * (1 << 30)), 512, local, prec=prec)
        cache = {}

        def build(i):
            if i not in cache:
                nx, ny, nz = (int(t) for t in dims[i])
                prob = P.cube_problem(nx, ny, nz, pressure=float(pres[i]))
                cache[i] = prob
            return cache[i]

        queue = collections.deque()
        sid2req, lat, iters, relres, neqs = {}, {}, {}, {}, {}
        nxt, ndone, active = 0, 0, 0
        max_neq = 0
        l0 = b.launches()
        t0 = time.perf_counter()
        while ndone < n_req:
            now = time.perf_counter() - t0
            while nxt < n_req and arrivals[nxt] <= now:
                queue.append(nxt)
                nxt += 1
            while queue:
                i = queue[0]
                prob = build(i)
                sid = b.admit(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"], es[i], vs[i],
                              prob["r"], tol=1e-8, limit=50000)
                if sid is None:
                    break
                queue.popleft()
                sid2req[sid] = i
                neqs[i] = prob["neq"]
                max_neq = max(max_neq, prob["neq"])
                del cache[i]
                active += 1
            if active:
                b.launch(chunk)
                if queue:
                    build(queue[0])          # host prepares the next request while the GPU iterates
                active, nd = b.sync()
                t_done = time.perf_counter() - t0
                for _ in range(nd):
                    sid, it, rel, _x = b.collect(max_neq)
                    i = sid2req.pop(sid)
                    lat[i] = t_done - arrivals[i]
                    iters[i], relres[i] = it, rel
                    ndone += 1
            elif nxt < n_req:
                time.sleep(max(0.0, min(0.01, arrivals[nxt] - (time.perf_counter() - t0))))
        makespan = time.perf_counter() - t0
        launches = b.launches() - l0
        b.close()
        L = np.array([lat[i] for i in range(n_req)]) * 1e3
        dof_it = sum(neqs[i] * iters[i] for i in range(n_req))
        results.append({"rate_per_s": rate, "requests": n_req, "makespan_s": makespan,
                        "solves_per_s": n_req / makespan, "p50_ms": float(np.percentile(L, 50)),
                        "p99_ms": float(np.percentile(L, 99)), "mean_ms": float(L.mean()),
                        "dof_iter_per_s": dof_it / makespan, "max_relres": float(max(relres.values())),
                        "mean_iters": float(np.mean(list(iters.values()))), "gpu_launches": launches})
    return results


def serving_workload(n_req, budget_gb, seed):
    return (f"serving stream: {n_req} Poisson-arrival requests, hex20 cubes with edges uniform in 4..40, E "
            f"log-uniform [10,1000], v uniform [0.2,0.35], fixed base, top pressure uniform [0.5,2.0], tol 1e-8, "
            f"budget {budget_gb} GB, seed {seed}")


def run_serving(args, rank, world, local, dist):
    n_req = args.requests
    results = serving_stream(n_req, [float(t) for t in args.rates.split(",")], args.budget_gb, args.chunk,
                             args.serving_prec, args.seed, local)
    best = max(results, key=lambda r: r["dof_iter_per_s"])
    line = {"metric": METRIC, "value": best["dof_iter_per_s"], "unit": UNIT, "n_gpus": world,
            "steps": n_req, "warmup": 0, "ms_per_step": best["makespan_s"] * 1e3 / n_req,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {32: "f32 storkm products + f64 residual replacement / f64 vectors",
                      16: "f16 storkm products + f64 residual replacement / f64 vectors",
                      64: "f64 storkm / f64 vectors"}[args.serving_prec], "data": "synthetic",
            "config": {"workload": serving_workload(n_req, args.budget_gb, args.seed),
                       "parallelism": "continuous batching"},
            "serving": results}
    if rank == 0:
        print(json.dumps(line))
    return 0


def multirhs_solves(n, k, seed, local, limit, precs=(16, 32), sequential=True, strict=False):
    """n^3 cube, E=100, v=0.3, k load cases of i.i.d. N(0,1) vertical forces
    on the top-face nodes (seeded): block solves (16 = tensor-core products,
    32 = FP32 CUDA-core products) against k sequential FP64 solves, all to
    relres 1e-8.  strict: also the tensor-core block solve to 1e-9 and, for
    two cases, every solution's error against FP64 solved to 1e-12."""
    import parafem_gb300 as P
    prob = P.cube_problem(n, n, n)
    s = P.Solver(local)
    try:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        neq, nels = prob["neq"], n ** 3
        R = P.random_top_loads(prob["g_g"], n, n, neq, k, seed)
        out = {"workload": f"multi-RHS {n}^3 hex20 cube, E 100, v 0.3, {k} load cases N(0,1) on top-face nodes "
                           f"(seed {seed}), nip 27, tol 1e-8", "neq": neq, "cases": k}
        sols = {}
        runs = [(prec, 1e-8) for prec in precs] + ([(16, 1e-9)] if strict and 16 in precs else [])
        for prec, tol in runs:
            name = {16: "block_tensor_cores", 32: "block_fp32_cuda_cores"}[prec] + ("" if tol == 1e-8 else "_1e-9")
            t0 = time.perf_counter()
            X, it, rel = s.solve_multi(R, tol, limit, prec)
            st = s.stats_raw()
            n_it = max(st[6], 1)
            out[name] = {"tol": tol, "wall_s": time.perf_counter() - t0, "device_s": st[2] / 1e3,
                         "max_iters": int(it.max()), "mean_iters": float(it.mean()),
                         "max_relres": float(rel.max()), "corrections": int(st[1]), "launched_iters": int(st[6]),
                         "elem_ms_per_iter": st[3] / n_it, "scatter_ms_per_iter": st[4] / n_it,
                         "iter_ms": st[5] / n_it,
                         "dof_iter_per_s": neq * k * float(it.mean()) / (st[2] / 1e3)}
            sols[name] = X
            if prec == 16 and tol == 1e-8:
                out["tensor_core_tuning"] = s.multi_tuning()
                peak, peak_kind = measured_peaks()
                # per element: the FP16 record (16,400 B), connectivity, the k FP32
                # results of its 60 dofs; the split P (8 B per value) once
                b = nels * (16400 + 80 + 60 * k * 4) + 3 * prob["nn"] * k * 8
                ms = s.multi_product_ms(R, 5)
                # DRAM traffic: the 40^3 capture's bytes per algorithmic byte
                # (the records and results grow with the elements, P with the nodes)
                ratio = ncu_traffic("k_mr_elem_h16_cube40", "dram_per_algorithmic_byte")
                out["roofline"] = {"kernel": "k_mr_elem_h16 (tcgen05 FP16x2, TMA gather4)", "bound": "hbm",
                                   "bytes_per_launch": b, "avg_launch_ms": ms,
                                   "achieved": b / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                                   "frac": b / (ms / 1e3) / 1e9 / peak, "peak_kind": f"{peak_kind} hbm_gbs",
                                   "traffic": b * ratio if ratio else None}
        first = {16: "block_tensor_cores", 32: "block_fp32_cuda_cores"}[precs[0]]
        if sequential:
            t0 = time.perf_counter()
            errs, its = [], []
            for j in range(k):
                x64, it64, rel64 = s.solve(R[:, j], 1e-8, 50000, P.MODE_FP64_RES)
                errs.append(float(np.linalg.norm(sols[first][:, j] - x64) / np.linalg.norm(x64)))
                its.append(it64)
                if strict and j in (0, k - 1):
                    sols.setdefault("fp64_1e-8", {})[j] = x64
            out["sequential_fp64"] = {"wall_s": time.perf_counter() - t0, "mean_iters": float(np.mean(its)),
                                      "max_iters": int(max(its))}
            out["block_vs_fp64_rel_err_2_max"] = max(errs)
            out["speedup_block_vs_sequential_fp64"] = out["sequential_fp64"]["wall_s"] / out[first]["wall_s"]
        if strict:
            acc = {}
            for j in (0, k - 1):
                xr, _, _ = s.solve(R[:, j], 1e-12, 50000, P.MODE_FP64_RES)
                nr = np.linalg.norm(xr)
                for name in ("block_tensor_cores", "block_tensor_cores_1e-9"):
                    if name in sols:
                        acc.setdefault(name, []).append(float(np.linalg.norm(sols[name][:, j] - xr) / nr))
                if "fp64_1e-8" in sols:
                    acc.setdefault("fp64_1e-8", []).append(float(np.linalg.norm(sols["fp64_1e-8"][j] - xr) / nr))
            out["rel_err_2_vs_fp64_1e-12_cases_0_and_last"] = acc
        return out
    finally:
        s.close()


def run_multirhs(args, rank, world, local, dist):
    """The 16-load-case cube (60^3 by default)."""
    n = args.size if args.size != 100 else 60
    out = multirhs_solves(n, 16, args.seed, local, args.limit, (16, 32), not args.no_solves)
    tc = out["block_tensor_cores"]
    line = {"metric": METRIC, "value": tc["dof_iter_per_s"], "unit": UNIT, "n_gpus": world, "steps": 1, "warmup": 0,
            "ms_per_step": tc["device_s"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "fp16x2 tensor-core products, f32 accumulation / f64 vectors and reductions",
            "data": "synthetic",
            "config": {"workload": out["workload"], "neq": out["neq"], "cases": 16},
            "multirhs": out}
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_shared(args, rank, world, local, dist):
    """The 100^3 cube of the headline with one element matrix shared by every
    element (PCG_KM): km of element 1 formed on the GPU, no per-element
    storkm.  Mixed (tensor-core products) and FP64 time to relres 1e-8,
    device-resident steps of both, and the tensor-core kernel's roofline."""
    import parafem_gb300 as P
    n = args.size
    prob = P.cube_problem(n, n, n)
    s = P.Solver(local)
    s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    s.set_material(100.0, 0.3)
    km = s.form_km(1, 27)
    s.set_shared_km(km)
    neq, nels, r = prob["neq"], n ** 3, prob["r"]
    out = {}
    if not args.no_solves:
        for name, mode in (("mixed", P.MODE_MIXED), ("fp64", P.MODE_FP64_RES)):
            t0 = time.perf_counter()
            x, it, rel = s.solve(r, 1e-8, 50000, mode)
            wall = time.perf_counter() - t0
            st = s.stats()
            out[name] = {"iters": it, "relres": rel, "wall_s": wall, "device_s": st["solve_ms"] / 1e3,
                         "corrections": st["outer"]}
            if name == "mixed":
                xm = x
        out["mixed_over_fp64_time"] = out["mixed"]["wall_s"] / out["fp64"]["wall_s"]
        out["mixed_vs_fp64_rel_err_2"] = float(np.linalg.norm(xm - x) / np.linalg.norm(x))
    else:
        s.solve(r, 1e-8, 1, P.MODE_MIXED)       # loads the right-hand side only
    s.bench_iterations(32, max(args.warmup, 3))
    clk = Clocks(local).start() if rank == 0 else None
    l0 = s.launches()
    ms_tot, ms_elem, ms_scat = s.bench_iterations(32, args.steps)
    launches = s.launches() - l0
    clocks = clk.stop() if clk else None
    k2 = max(args.steps // 4, 3)
    ms64, ms64_elem, _ = s.bench_iterations(64, k2)
    s.close()
    value = neq * args.steps / (ms_tot / 1e3)
    peak, peak_kind = measured_peaks()
    nslots = 3 * prob["nn"]
    b_launch = elem_bytes(nels, nslots, 0, 16 / 3)   # connectivity, gathered p, node-padded FP32 results
    avg_s = ms_elem / args.steps / 1e3
    achieved = b_launch / avg_s / 1e9
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16x3 tensor-core products, f32 accumulation / f64 vectors and reductions",
            "data": "synthetic",
            "config": {"workload": f"{n}^3 hex20 cube, one shared element matrix (PCG_KM), E 100, v 0.3, nip 27, "
                                   f"fixed base, top pressure", "nels": nels, "neq": neq},
            "roofline": {"kernel": "k_elem_shared_tc (shared km, tcgen05 BF16x3)", "bound": "hbm",
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_launch": b_launch,
                         "avg_launch_ms": avg_s * 1e3,
                         "traffic": ncu_traffic("k_elem_shared_tc_cube100") if n == 100 else None,
                         "scatter_avg_ms": ms_scat / args.steps},
            "fp64_step_ms": ms64 / k2, "fp64_elem_ms": ms64_elem / k2,
            "gpu_launches": int(launches), "clocks": clocks, "solves": out}
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_p123(args, rank, world, local, dist):
    """p123's book run (examples/5th_ed/p123/book/p123.mg): 200^3 8-node
    bricks of 0.005, kx = ky = kz = 2, box_bc8 restraints, load 10 at
    freedom 39801, checon_par tol 1e-5.  The reference recorded 180
    iterations and 52.4 s in the solver on 16 Cray XE6 cores."""
    import parafem_gb300 as P
    n = args.size if args.size != 100 else 200
    t0 = time.perf_counter()
    prob = P.box8_problem(n, n, n, .005, .005, .005)
    t_host = time.perf_counter() - t0
    s = P.Solver(local)
    s.setup_scalar8(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    t1 = time.perf_counter()
    s.form_storkc(8, 2.0, 2.0, 2.0)
    t_form = time.perf_counter() - t1
    neq = prob["neq"]
    s.solve(prob["r"], 1e-5, 10000, P.MODE_P121)        # warm-up
    t2 = time.perf_counter()
    x, it, rel = s.solve(prob["r"], 1e-5, 10000, P.MODE_P121)
    t_solve = time.perf_counter() - t2
    st = s.stats()
    s.bench_iterations(64, max(args.warmup, 3))
    clk = Clocks(local).start() if rank == 0 else None
    l0 = s.launches()
    ms_tot, ms_elem, ms_scat = s.bench_iterations(64, args.steps)
    launches = s.launches() - l0
    clocks = clk.stop() if clk else None
    s.close()
    nres = prob["nres"]
    peak, peak_kind = measured_peaks()
    b_launch = prob["g_num"].shape[0] * (512 + 32 + 64) + prob["nn"] * 8   # storkc, conn, results, gathered p
    avg_s = ms_elem / args.steps / 1e3
    line = {"metric": METRIC, "value": neq * args.steps / (ms_tot / 1e3), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"p123 book run: {n}^3 8-node bricks (Laplace), kx=ky=kz=2, nip 8, checon tol "
                                   f"1e-5", "nels": n ** 3, "neq": neq},
            "solve": {"iters": it, "wall_s": t_solve, "device_s": st["solve_ms"] / 1e3,
                      "dof_iter_per_s": neq * it / t_solve, "potentials": [float(v) for v in x[nres - 1:nres + 3]],
                      "reference_book": {"iters": 180, "solver_s": 52.3833, "cores": 16}},
            "roofline": {"kernel": "k_elem8 (FP64 storkc)", "bound": "hbm", "achieved": b_launch / avg_s / 1e9,
                         "peak": peak, "unit": "GB/s", "frac": b_launch / avg_s / 1e9 / peak,
                         "peak_kind": f"{peak_kind} hbm_gbs", "bytes_per_launch": b_launch,
                         "avg_launch_ms": avg_s * 1e3, "traffic": None, "scatter_avg_ms": ms_scat / args.steps},
            "host_setup_s": t_host, "storkc_formation_s": t_form, "gpu_launches": int(launches), "clocks": clocks}
    if rank == 0:
        print(json.dumps(line))
    return 0


def run_p122(args, rank, world, local, dist):
    """p122's book run (examples/5th_ed/p122/book/p122.mg): 20^3 20-node
    bricks of 0.5, E 1e4, v 0.3, Mohr-Coulomb c 100, phi = psi = 0, 12 load
    increments under load control, plastic tolerance 1e-4, PCG tolerance
    1e-5.  The reference recorded 409 s on 16 Cray XE6 cores.  The mesh,
    restraints and loads are p12meshgen's p122 case (host side)."""
    import parafem_gb300 as P
    nxe = nze = 20
    nels, aa = 8000, 0.5
    qinc = [200.0, 100.0, 50.0, 50.0, 50.0, 30.0, 20.0, 10.0, 10.0, 5.0, 5.0, 5.0]
    prob = P.cube_problem(nxe, nels // nxe // nze, nze, bc=0, pressure=0.0, aa=aa, bb=aa, cc=aa)
    ld0 = P.patch_loads(nxe, nze, prob["g_num"], prob["g_g"], prob["neq"], -aa * aa / 12.0)
    s = P.Solver(local)
    s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
    s.set_material(1.0e4, 0.3)
    s.form_storkm(8)
    l0 = s.launches()
    t0 = time.perf_counter()
    res, _ = s.p122_solve(8, 0.0, 100.0, 0.0, qinc, 1000, 1000, 1e-4, 1e-5, ld0)
    wall = time.perf_counter() - t0
    launches = s.launches() - l0
    s.close()
    cj = float(res[:, 4].sum())
    line = {"metric": METRIC, "value": prob["neq"] * cj / wall, "unit": UNIT, "n_gpus": world, "steps": int(cj),
            "warmup": 0, "ms_per_step": 1e3 * wall / cj, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "p122 book run: 20^3 20-node bricks, Mohr-Coulomb (c 100, phi 0, psi 0), E 1e4, "
                                   "v 0.3, 12 load increments", "nels": nels, "neq": prob["neq"]},
            "p122": {"wall_s": wall, "increments": [
                {"displacement": float(r[0]), "sigma_z": float(r[1]), "sigma_x": float(r[2]), "sigma_y": float(r[3]),
                 "cj_iterations": int(r[4]), "plastic_iterations": int(r[5])} for r in res],
                "reference_book": {"wall_s": 409.0, "cores": 16}},
            "gpu_launches": int(launches)}
    if rank == 0:
        print(json.dumps(line))
    return 0


def gpu_config1(local):
    """Config 1 on the GPU drop-in (PF_MODE_P121): 10^3, checon_par tol 1e-6."""
    import parafem_gb300 as P
    prob = P.cube_problem(10, 10, 10)
    with P.Solver(local) as s:
        s.setup(prob["g_num"], prob["g_g"], prob["g_coord"], prob["nn"], prob["neq"])
        s.set_material(100.0, 0.3)
        s.form_storkm(27)
        s.solve(prob["r"], 1e-6, 5000, P.MODE_P121)          # warm-up
        t1 = time.perf_counter()
        x, it, _ = s.solve(prob["r"], 1e-6, 5000, P.MODE_P121)
        return x, it, time.perf_counter() - t1


def run_cube10(args, rank, world, local, dist):
    """The reference's CPU-runnable case: 10^3 cube, nip 27, E 100, v 0.3,
    fixed base, top pressure (total -1), checon_par tol 1e-6, limit 5000.
    GPU drop-in (PF_MODE_P121) vs the CPU build of p121, same inputs."""
    x, it, t_gpu = gpu_config1(local)
    cfg = cpu_config1(x, it, t_gpu)
    neq = cfg["neq"]
    line = {"metric": METRIC, "value": neq * it / t_gpu, "unit": UNIT, "n_gpus": world, "steps": it,
            "warmup": 1, "ms_per_step": 1e3 * t_gpu / it, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": cfg["workload"], "neq": neq}, "cube10": cfg}
    if rank == 0:
        print(json.dumps(line))
    return 0


def main():
    args = parse_args()
    rank, world, local, dist = dist_init(args.gpus)
    try:
        if args.impl == "reference":
            return run_reference(args, rank)
        if args.workload == "hetero80":
            return run_hetero(args, rank, world, local, dist)
        if args.workload == "serving":
            return run_serving(args, rank, world, local, dist)
        if args.workload == "multirhs60":
            return run_multirhs(args, rank, world, local, dist)
        if args.workload == "cube10":
            return run_cube10(args, rank, world, local, dist)
        if args.workload == "shared100":
            return run_shared(args, rank, world, local, dist)
        if args.workload == "p123book":
            return run_p123(args, rank, world, local, dist)
        if args.workload == "p122book":
            return run_p122(args, rank, world, local, dist)
        return run_gb300(args, rank, world, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
