#!/usr/bin/env python3
"""Benchmark: MG-CFD multigrid V-cycles on the 8M-node synthetic mesh.

Workload: 200^3 jittered lattice (8,000,000 nodes, 23,880,000 edges, 240,000
boundary entries on level 0), 4 multigrid levels (200^3, 100^3, 50^3, 25^3),
Mach 0.8, angle of attack 3 degrees, FP64.  One step = one V-cycle
(euler3d.cpp:458-641: 6 smoothing steps, 18 edge-flux sweeps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--precision fp64|mixed] [--increment atomic|gather] [--n 200]
  python bench.py --mode batch     # 64 uneven meshes in one launch per stage
  python bench.py --mode serve     # Poisson request stream, p50/p99 latency

Prints one JSON line.  `value` is V-cycles/s with the mesh resident in HBM,
`e2e` is V-cycles/s through the host-buffer entry point mgcfd_solve (mesh
upload, setup, 25 V-cycles, download of every level's state), and `roofline`
describes the level-0 edge-flux kernel.  --impl reference times the CPU
restatement of the reference path (OpenMP, all host threads) on the same
mesh.  Under torchrun each rank runs an independent replica (the solve does
not shard across GPUs); value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "mg-cfd-app-op2_gb300"))

MACH, AOA, NLEVELS, SEED = 0.8, 3.0, 4, 20240501
E2E_CYCLES = 25


def algorithmic_flux_bytes(nnodes: int, nedges: int, precision: str = "fp64", increment: str = "atomic") -> int:
    """Bytes one level-0 flux sweep must move at least.

    FP64: 24 B weights + 8 B map per edge; 80 B state read, 40 B flux read
    and 40 B flux written per node (the reference's own model of the loop
    plus the map and the read half of the increment).
    Mixed, edge kernel: 16 B FP32 weights + 8 B map read and 20 B FP32 edge
    flux written per edge; 32 B FP32 primitives read per node.
    Mixed, fused stage (flux and time step in one node kernel): per edge the
    a-side weights + map (24 B) and the b-side copies (20 B); per node the
    FP32 primitives read (32 B), old state (40 B), 1/vol, boundary index and
    CSR offsets (20 B), state written (40 B) and next primitives written (32 B)."""
    if precision == "mixed" and increment == "fused":
        return 44 * nedges + 164 * nnodes
    if precision == "mixed":
        return 44 * nedges + 32 * nnodes
    return 32 * nedges + 120 * nnodes


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_profile(name):
    p = ROOT / "profiles" / name
    if p.exists():
        try:
            return json.loads(p.read_text())
        except json.JSONDecodeError:
            return None
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_min_mhz": min(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def pinned_levels(levels, keep):
    """Copies of a mesh's level arrays in page-locked host memory (the inputs
    of the end-to-end, batch and serve measurements); `keep` holds the
    buffers alive."""
    import numpy as np
    import torch

    import mgcfd

    def pin(a):
        if a is None:
            return None
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        keep.append(t)
        return t.numpy()

    return [mgcfd.Level(coords=pin(L.coords), edge_to_nodes=pin(L.edge_to_nodes), bnd_to_node=pin(L.bnd_to_node),
                        bnd_group=pin(L.bnd_group), edge_weights=pin(L.edge_weights), bnd_weights=pin(L.bnd_weights),
                        node_to_mg=pin(L.node_to_mg), n_axis=L.n_axis, volumes=pin(L.volumes)) for L in levels]


def run_gb300(args):
    import ctypes as C

    import numpy as np
    import torch

    import mgcfd
    from mgcfd import _lib

    from mgcfd import replicas
    world, rank, local = replicas.world()
    torch.cuda.set_device(local)
    dist = replicas.init()

    mesh = mgcfd.HostMesh.generate(args.n, NLEVELS, SEED)
    L0 = mesh.level(0)
    N, E = L0.nnodes, L0.nedges
    solver = mgcfd.Solver(mesh, MACH, AOA, precision=args.precision, increment=args.increment,
                          renumber=args.renumber, accumulation=args.accumulation, time_kernels=True)
    solver.run(args.warmup)
    if solver.synchronize() != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    st0 = solver.stats()

    def barrier():
        replicas.barrier(dist)

    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        solver.run(args.steps)
        status = solver.synchronize()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
    barrier()
    if status != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    st1 = solver.stats()
    value, elapsed = replicas.job_throughput(args.steps, t1 - t0, dist, device="cuda")
    flux_ms = (st1.flux_ms_l0 - st0.flux_ms_l0) / max(1, st1.flux_sweeps_l0 - st0.flux_sweeps_l0)
    launches = int(st1.kernel_launches - st0.kernel_launches)
    precision_error = None
    if args.precision == "mixed":
        # Final level-0 state against an FP64 solve of the same cycles:
        # per-variable max and L2 relative error (density, 3 momenta, energy).
        got = solver.fetch(0)
        ref_solver = mgcfd.Solver(mesh, MACH, AOA, precision="fp64", renumber=args.renumber)
        ref_solver.run(args.warmup + args.steps)
        if ref_solver.synchronize() != 0:
            raise RuntimeError(_lib.load().mgcfd_last_error().decode())
        ref = ref_solver.fetch(0)
        ref_solver.close()
        d = got - ref
        precision_error = {
            "variables": ["rho", "rho_u", "rho_v", "rho_w", "rho_E"],
            "max_rel": [float(np.max(np.abs(d[:, k])) / np.max(np.abs(ref[:, k]))) for k in range(5)],
            "l2_rel": [float(np.linalg.norm(d[:, k]) / np.linalg.norm(ref[:, k])) for k in range(5)],
            "cycles": args.warmup + args.steps, "against": "FP64 solve of the same mesh and cycles"}
    solver.close()

    # End to end through the host-buffer entry point, pinned host memory.
    levels = mesh.levels()
    pinned = []
    hl = pinned_levels(levels, pinned)
    outs = [torch.empty((L.nnodes, 5), dtype=torch.float64).pin_memory() for L in levels]
    views = mgcfd.level_views_from_arrays(hl)
    out_ptrs = (_lib.c_double_p * len(outs))(*[C.cast(o.data_ptr(), _lib.c_double_p) for o in outs])
    opts = mgcfd.options(precision=args.precision, increment=args.increment, renumber=args.renumber,
                         accumulation=args.accumulation)
    lib = _lib.load()
    h2d = sum(a.nbytes for L in hl for a in (L.coords, L.edge_to_nodes, L.bnd_to_node, L.bnd_group, L.edge_weights,
                                              L.bnd_weights) + ((L.node_to_mg,) if L.node_to_mg is not None else ()))
    d2h = sum(o.numel() * 8 for o in outs)
    _lib.check(lib.mgcfd_solve(len(hl), views, MACH, AOA, 1, C.byref(opts), out_ptrs))  # warm-up
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    barrier()
    te0 = time.perf_counter()
    for _ in range(e2e_steps):
        _lib.check(lib.mgcfd_solve(len(hl), views, MACH, AOA, E2E_CYCLES, C.byref(opts), out_ptrs))
    te1 = time.perf_counter()
    barrier()
    e2e_value, e2e_elapsed = replicas.job_throughput(e2e_steps * E2E_CYCLES, te1 - te0, dist, device="cuda")

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(levels, args.cpu_cycles)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak, peak_kind = measured_peaks()
    inc = args.increment if args.increment != "auto" else ("fused" if args.precision == "mixed" else "atomic")
    bytes_per_sweep = algorithmic_flux_bytes(N, E, args.precision, inc)
    achieved = bytes_per_sweep / (flux_ms * 1e-3) / 1e9
    prof = committed_profile(f"flux_edge_{args.precision}_{inc}.json") or {}
    traffic = prof.get("dram_bytes_per_launch_scaled_to_bench") if args.n == 200 else None
    fp64_roof = None
    if prof.get("fp64"):
        # The FP64 flux sweep is bound by FP64 issue, not HBM: the same launch
        # against the measured FP64 FMA rate.
        f = prof["fp64"]
        per_edge = "ops_per_edge" in f
        ach = (f["ops_per_edge"] * E if per_edge else f["ops_per_node"] * N) / (flux_ms * 1e-3) / 1e9
        fp64_roof = {"bound": "fp64", "achieved": round(ach, 1), "peak": f["peak_gops"], "unit": "G FP64 op/s",
                     "frac": round(ach / f["peak_gops"], 4),
                     ("ops_per_edge" if per_edge else "ops_per_node"): f["ops_per_edge" if per_edge else "ops_per_node"],
                     "peak_source": f["peak_source"], "ncu_fp64_pipe_busy": f["pipe_busy_ncu"]}
    line = {
        "metric": "MG V-cycles/s at 8M nodes (200^3, 4 levels)",
        "value": round(value, 3),
        "unit": "cycles/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * elapsed / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32-flux/f64-accumulate",
        "data": "synthetic: seeded jittered 200^3 lattice, permuted ids",
        "config": {"workload": f"{args.n}^3 jittered lattice, {NLEVELS} levels, Mach {MACH}, AoA {AOA} deg, "
                               f"{N} nodes / {E} edges on level 0",
                   "precision": args.precision, "increment": inc, "renumber": args.renumber,
                   "accumulation": args.accumulation if args.precision == "mixed" else "fp64",
                   "l2": "inputs larger than L2 (level-0 state and edges ~2.4 GB), no flush",
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": ("k_update fused stage (level-0 edge fluxes + time step)" if inc == "fused"
                                else "k_flux (level-0 edge flux sweep)"), "flux_ms_per_launch": round(flux_ms, 4),
                     "algorithmic_bytes_per_launch": bytes_per_sweep, "peak_source": peak_kind,
                     "fp64": fp64_roof},
        "e2e": {"value": round(e2e_value, 3), "unit": "cycles/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step": f"mgcfd_solve: upload mesh, setup, {E2E_CYCLES} V-cycles, download all levels",
                "steps": e2e_steps},
        "gpu_launches": launches,
        "precision_error": precision_error,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def cpu_baseline(levels, cycles):
    """The oracle restatement with OpenMP on every host core, timed on a
    bounded sample (a few V-cycles of the same mesh)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    threads = os.cpu_count() or 1
    run = O.OracleRun(levels)
    run.run(MACH, AOA, 1, nthreads=threads)  # warm-up: colouring, page faults
    st, secs = run.run(MACH, AOA, cycles, nthreads=threads)
    # The sequential form (the reference's OP2 seq order, one core), one V-cycle.
    st1, secs1 = run.run(MACH, AOA, 1, nthreads=1)
    run.close()
    return {"value": round(cycles / secs, 4), "unit": "cycles/s", "cores": threads, "kind": "port",
            "sample": f"{cycles} V-cycles of the same 8M-node 4-level mesh, OpenMP over coloured edges",
            "seq_1core": {"value": round(1.0 / secs1, 4), "unit": "cycles/s", "cores": 1,
                          "sample": "1 V-cycle, sequential edge order"}}


def run_reference(args):
    from mgcfd import replicas
    world, rank, local = replicas.world()
    if rank != 0:
        return
    import mgcfd
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    mesh = mgcfd.HostMesh.generate(args.n, NLEVELS, SEED)
    levels = mesh.levels()
    threads = os.cpu_count() or 1
    run = O.OracleRun(levels)
    run.run(MACH, AOA, args.warmup, nthreads=threads)
    st, secs = run.run(MACH, AOA, args.steps, nthreads=threads)
    value = args.steps / secs
    L0 = levels[0]
    line = {
        "impl": "reference",
        "metric": "MG V-cycles/s at 8M nodes (200^3, 4 levels)",
        "value": round(value, 4), "unit": "cycles/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded jittered 200^3 lattice, permuted ids",
        "config": {"workload": f"{args.n}^3 jittered lattice, {NLEVELS} levels, Mach {MACH}, AoA {AOA} deg, "
                               f"{L0.nnodes} nodes / {L0.nedges} edges on level 0",
                   "implementation": "CPU restatement of the reference path (oracle/mgcfd_oracle.c), OpenMP"},
        "cpu_baseline": {"value": round(value, 4), "unit": "cycles/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} V-cycles after {args.warmup} warm-up cycles"},
        "e2e": {"value": round(value, 4), "unit": "cycles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "status": st,
    }
    print(json.dumps(line), flush=True)


def run_batch(args):
    """Batched solves: 64 meshes (lattice edge log-uniform 16..96, Mach U(0.3, 0.8),
    AoA U(0, 6) degrees, 3 levels, 20 V-cycles) solved in one batch against 64
    sequential plain solves.  Every solve is timed through the host-buffer API
    from page-locked host buffers: upload, device setup, the V-cycles and the
    download of level 0."""
    import numpy as np
    import torch  # noqa: F401  (CUDA context for the timers below)

    import mgcfd
    from mgcfd import autotune
    rng = np.random.default_rng(3)
    nm = args.batch_meshes
    sizes = np.exp(rng.uniform(np.log(16), np.log(96), nm)).round().astype(int)
    machs = rng.uniform(0.3, 0.8, nm).tolist()
    aoas = rng.uniform(0.0, 6.0, nm).tolist()
    host_meshes = [mgcfd.HostMesh.generate(int(n), 3, 1000 + i) for i, n in enumerate(sizes)]
    keep = []
    meshes = [pinned_levels(m.levels(), keep) for m in host_meshes]  # inputs in page-locked host memory
    cycles = 20
    total_nodes = sum(m[0].nnodes for m in meshes)

    def solve_batch(**o):
        b = mgcfd.Batch(meshes, machs, aoas, **o)
        b.run(cycles)
        assert b.synchronize() == 0
        outs = b.fetch_meshes(0)
        b.close()
        return outs

    def solve_sequential(**o):
        outs = []
        for m in range(nm):
            s = mgcfd.Solver(meshes[m], machs[m], aoas[m], **o)
            s.run(cycles)
            assert s.synchronize() == 0
            outs.append(s.fetch(0))
            s.close()
        return outs

    line = {"metric": f"batched solves/s ({nm} meshes, 16^3-96^3 lattices, 3 levels, {cycles} V-cycles)",
            "unit": "solves/s", "higher_is_better": True, "n_gpus": 1, "data": "synthetic: seeded lattices",
            "config": {"workload": f"{nm} meshes, {total_nodes} level-0 nodes in total, sizes {sizes.min()}^3.."
                                   f"{sizes.max()}^3", "inputs": "page-locked host memory"}}
    def timed(fn, **o):  # median wall time of `repeats` runs, and the last run's results
        ts = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            outs = fn(**o)
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts), outs

    repeats = 3
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as sampler:
        t0 = time.perf_counter()
        solve_sequential(precision="fp64")  # warm-up pass (pool, graphs, clocks)
        line["warmup_s"] = round(time.perf_counter() - t0, 3)
        line["timing"] = f"median wall time of {repeats} runs, each from host meshes to level-0 results on the host"
        t_seq, seq = timed(solve_sequential, precision="fp64")
        results = {"sequential_fp64": nm / t_seq}
        for prec in ("fp64", "mixed"):
            t0 = time.perf_counter()
            best, timings = autotune.tune_batch(meshes, machs, aoas, precision=prec)
            t_tune = time.perf_counter() - t0
            solve_batch(**best)
            dt, outs = timed(solve_batch, **best)
            results[f"batched_{prec}"] = nm / dt
            err = max(float(np.max(np.abs(a - b) / np.maximum(np.abs(b).max(axis=0), 1e-300)))
                      for a, b in zip(outs, seq))
            line[f"batched_{prec}_tuning"] = {"chosen": best, "ms_per_cycle": {f"{k[0]}/{k[1]}": round(v, 3)
                                                                               for k, v in timings.items()},
                                              "tuning_s": round(t_tune, 3), "max_rel_err_vs_fp64_sequential": err}
            if prec == "mixed":  # the same batch with compensated FP32-pair node sums
                pair = dict(best, accumulation="pair32")
                solve_batch(**pair)
                dt, outs = timed(solve_batch, **pair)
                results["batched_mixed_pair32"] = nm / dt
                line["batched_mixed_pair32_max_rel_err_vs_fp64_sequential"] = max(
                    float(np.max(np.abs(a - b) / np.maximum(np.abs(b).max(axis=0), 1e-300))) for a, b in zip(outs, seq))
    line["clocks"] = sampler.summary()
    line["value"] = round(results["batched_fp64"], 3)
    line["results_solves_per_s"] = {k: round(v, 3) for k, v in results.items()}
    line["speedup_batched_fp64_vs_sequential"] = round(results["batched_fp64"] / results["sequential_fp64"], 3)
    line["speedup_batched_mixed_vs_sequential_fp64"] = round(results["batched_mixed"] / results["sequential_fp64"], 3)
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving: a Poisson stream of requests, each a seeded lattice mesh with
    node count log-uniform in 20K..4M (a pool of distinct meshes drawn per
    request), Mach U(0.3, 0.85), AoA U(0, 6) degrees, 3 or 4 levels, run until
    the level-0 density residual falls to 1e-6 of its first value or 50
    V-cycles, under a 150 GB HBM budget.  Three forms serve the same stream:
      plain_fp64    one FP64 solve at a time (the plain path),
      served_fp64   FP64, up to --serve-slots requests overlapping,
      served_mixed  mixed precision, up to --serve-slots requests overlapping.
    Capacity is solves/s with every request queued at once; then each form
    serves Poisson arrivals at rates that are multiples of the plain path's
    capacity, reporting p50/p99 latency (submit to result) and solves/s."""
    import threading

    import numpy as np

    import mgcfd
    rng = np.random.default_rng(11)
    pool, keep = [], []
    for i in range(args.serve_pool):
        nodes = float(np.exp(rng.uniform(np.log(20e3), np.log(4e6))))
        n = max(8, int(round(nodes ** (1.0 / 3.0))))
        m = mgcfd.HostMesh.generate(n, int(rng.integers(3, 5)), 500 + i)
        pool.append(pinned_levels(m.levels(), keep))  # requests arrive in page-locked host memory
    R = args.serve_requests
    picks = rng.integers(0, len(pool), R)
    machs = rng.uniform(0.3, 0.85, R)
    aoas = rng.uniform(0.0, 6.0, R)
    gaps = rng.exponential(1.0, R)  # unit-rate inter-arrival times, scaled per rate
    # plain_fp64 is the plain path: one FP64 solve at a time, each uploading and
    # setting up its mesh.  The served forms overlap requests and keep meshes
    # resident between requests (same pool mesh = same mesh key).
    forms = {"plain_fp64": dict(max_active=1, precision="fp64"),
             "served_fp64": dict(max_active=args.serve_slots, precision="fp64"),
             "served_mixed": dict(max_active=args.serve_slots, precision="mixed"),
             "served_mixed_pair32": dict(max_active=args.serve_slots, precision="mixed", accumulation="pair32")}
    resident = {"plain_fp64": False, "served_fp64": True, "served_mixed": True, "served_mixed_pair32": True}

    def serve(form, rate):
        srv = mgcfd.Server(hbm_budget_gb=150.0, max_cycles=50, residual_drop=1e-6, **forms[form])
        t_start = time.perf_counter()
        arrivals = np.cumsum(gaps / rate) if rate else np.zeros(R)

        def feeder():
            for k in range(R):
                delay = t_start + arrivals[k] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                key = int(picks[k]) + 1 if resident[form] else None  # same pool mesh = same resident mesh
                srv.submit(pool[picks[k]], float(machs[k]), float(aoas[k]), mesh_key=key, resident=resident[form])

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        srv.drain(3600)
        t_end = time.perf_counter()
        res = [r for r, _ in srv.poll()]
        st = srv.stats()
        srv.close()
        lat = np.array([r["finish_s"] - r["submit_s"] for r in res])
        ok = sum(1 for r in res if r["status"] == 0)
        return {"rate_per_s": round(rate, 3) if rate else "all at once",
                "solves_per_s": round(len(res) / (t_end - t_start), 3),
                "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
                "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2), "ok": ok, "failed": len(res) - ok,
                "mean_cycles": round(float(np.mean([r["cycles"] for r in res])), 2),
                "peak_active": int(st["peak_active"]), "peak_budget_gb": round(st["peak_bytes"] / 2 ** 30, 2),
                "resident_mesh_hits": int(st["cache_hits"])}

    serve("served_mixed", 0)  # warm-up: CUDA context, memory pool, module load
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as sampler:
        capacity = {f: serve(f, 0) for f in forms}
        plain_cap = capacity["plain_fp64"]["solves_per_s"]
        rates = [f * plain_cap for f in args.serve_rate_multiples]
        sweep = {f: [serve(f, r) for r in rates] for f in forms}
    cap = {f: capacity[f]["solves_per_s"] for f in forms}
    line = {"metric": "served solves/s and p50/p99 latency (Poisson stream), vs the plain FP64 path",
            "unit": "solves/s", "higher_is_better": True, "n_gpus": 1,
            "data": "synthetic: seeded jittered lattices",
            "config": {"workload": f"{R} requests over a pool of {len(pool)} meshes "
                                   f"({min(m[0].nnodes for m in pool)}..{max(m[0].nnodes for m in pool)} "
                                   "level-0 nodes, 3-4 levels), 50 V-cycles or residual drop 1e-6, "
                                   "HBM budget 150 GB",
                       "slots": args.serve_slots, "rate_multiples_of_plain_capacity": args.serve_rate_multiples,
                       "inputs": "page-locked host memory"},
            "value": cap["served_mixed"], "capacity_solves_per_s": cap,
            "speedup_served_mixed_vs_plain_fp64": round(cap["served_mixed"] / cap["plain_fp64"], 3),
            "speedup_served_mixed_pair32_vs_plain_fp64": round(cap["served_mixed_pair32"] / cap["plain_fp64"], 3),
            "speedup_served_fp64_vs_plain_fp64": round(cap["served_fp64"] / cap["plain_fp64"], 3),
            "capacity_runs": capacity, "sweep": sweep, "clocks": sampler.summary()}
    print(json.dumps(line), flush=True)


def run_rates(args):
    """Issue rates of the arithmetic the kernels are built from (FP64/FP32
    FMA, reciprocal, square root, rsqrt, format conversions, FP64 atomics,
    device copy), measured on this GPU: the denominators of the FP64 cost
    model the kernels are designed against."""
    from mgcfd import _build
    src = ROOT / "tests" / "native" / "fp64_rates.cu"  # a probe, not part of the library
    exe = _build.OBJ / "fp64_rates"
    exe.parent.mkdir(parents=True, exist_ok=True)
    subprocess.run([_build._nvcc(), *_build.ARCH, "-O3", "-std=c++17", f"-I{_build.CSRC}", str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    d = json.loads(out)
    print(json.dumps({"metric": "arithmetic issue rates", "unit": "G/s", "n_gpus": 1, "rates": d}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--increment", default="auto", choices=["auto", "atomic", "gather", "fused"],
                    help="auto: FP64 atomics for fp64, the fused node-centric stage for mixed")
    ap.add_argument("--renumber", default="spatial", choices=["none", "spatial", "rcm"])
    ap.add_argument("--accumulation", default="fp64", choices=["fp64", "pair32"],
                    help="mixed precision node sums: FP64 adds, or compensated FP32 pairs")
    ap.add_argument("--n", type=int, default=200)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-cycles", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="plain", choices=["plain", "batch", "serve", "rates"])
    ap.add_argument("--batch-meshes", type=int, default=64)
    ap.add_argument("--serve-requests", type=int, default=240)
    ap.add_argument("--serve-pool", type=int, default=24)
    ap.add_argument("--serve-rate-multiples", type=float, nargs="*", default=[0.5, 0.9, 2.0],
                    help="Poisson rates as multiples of the plain path's capacity (none: capacity only)")
    ap.add_argument("--serve-slots", type=int, default=16)
    args = ap.parse_args()
    if args.warmup < 0 or args.steps < 1:
        ap.error("need --steps >= 1 and --warmup >= 0")
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "batch":
        run_batch(args)
    elif args.mode == "serve":
        run_serve(args)
    elif args.mode == "rates":
        run_rates(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
