#!/usr/bin/env python3
"""Benchmark: MG-CFD multigrid V-cycles on the 8M-node synthetic mesh.

Workload: 200^3 jittered lattice (8,000,000 nodes, 23,880,000 edges, 240,000
boundary entries on level 0), 4 multigrid levels (200^3, 100^3, 50^3, 25^3),
Mach 0.8, angle of attack 3 degrees, FP64.  One step = one V-cycle
(euler3d.cpp:458-641: 6 smoothing steps, 18 edge-flux sweeps).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--precision fp64|mixed|dw] [--increment atomic|gather|fused] [--n 200]
  python bench.py --mode batch     # 64 uneven meshes in one launch per stage
  python bench.py --mode serve     # Poisson request stream, p50/p99 latency
  python bench.py --mode loops     # the V-cycle through the per-loop entry points

Prints one JSON line.  `value` is V-cycles/s with the mesh resident in HBM
(the default CUDA-graph path, timed with CUDA events on the solver's stream),
`e2e` is V-cycles/s through the host-buffer entry point mgcfd_solve (mesh
upload, setup, 25 V-cycles, download of every level's state), and `roofline`
describes the level-0 edge-flux kernel.  The same line carries the
double-word form (FP64 state, float-float edge flux and primitives, held to
the FP64 bar: `dw`) and the mixed-precision workload (`mixed`) on the same
mesh, and served solves on a fresh-mesh request stream against the plain
FP64 path (`served`).  --impl reference times the CPU
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
MIXED_CYCLES = 25  # the mixed-precision workload's cycle count


def algorithmic_flux_bytes(nnodes: int, nedges: int, precision: str = "fp64", increment: str = "atomic") -> int:
    """Bytes one level-0 flux sweep must move at least.

    FP64: 24 B weights + 8 B map per edge; 80 B state read, 40 B flux read
    and 40 B flux written per node (the reference's own model of the loop
    plus the map and the read half of the increment).
    Mixed, edge kernel: 16 B FP32 weights + 8 B map read and 20 B FP32 edge
    flux written per edge; 32 B FP32 primitives read per node.
    Mixed, fused stage (flux and time step in one node kernel), the mean over
    a step's three stages: per edge the a-side weights + map (24 B) and the
    b-side copies (20 B); per node the FP32 primitives read (32 B), old state
    (40 B), 1/vol, boundary index and CSR offsets (20 B), then in the first two
    stages the next primitives written (32 B; the state is written for boundary
    nodes only) and in the last the state and the residual written (80 B):
    124 and 172 B, 140 B per node on average.
    DW (double-word flux): 32 B weights as pair words + 8 B map per edge; 64 B
    primitives as pair words read, 40 B flux read and 40 B written per node.
    DW, fused stage, the mean over a step's three stages: per edge both ends'
    table entries (neighbour and edge index, 2 x 8 B) and the weights as pair
    words (32 B); per node the primitives read (64 B), old state (40 B), 1/vol,
    boundary index and table offset (16 B), then the next primitives written
    (64 B) in the first two stages and the state and residual (80 B) in the
    last: 184 and 200 B, 568/3 B per node on average."""
    if precision == "dw" and increment == "fused":
        return 48 * nedges + (568 * nnodes) // 3
    if precision == "dw":
        return 40 * nedges + 144 * nnodes
    if precision == "mixed" and increment == "fused":
        return 44 * nedges + 140 * nnodes
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


def flux_roofline(precision, increment, n, N, E, flux_ms):
    """Roofline of the level-0 edge-flux kernel (the fused stage for mixed
    precision): algorithmic bytes per launch over the CUDA-event launch time,
    against the measured HBM copy rate, plus the FP64-pipe roofline where the
    committed ncu profile gives the FP64 work per unit."""
    peak, peak_kind = measured_peaks()
    bytes_per_sweep = algorithmic_flux_bytes(N, E, precision, increment)
    achieved = bytes_per_sweep / (flux_ms * 1e-3) / 1e9
    prof = committed_profile(f"flux_edge_{precision}_{increment}.json") or {}
    traffic = prof.get("dram_bytes_per_launch_scaled_to_bench") if n == 200 else None
    fp64_roof = None
    if prof.get("fp64"):
        # FP64 kernels are bound by FP64 issue, not HBM: the same launch
        # against the measured FP64 FMA rate.
        f = prof["fp64"]
        key = "ops_per_edge" if "ops_per_edge" in f else "ops_per_node"
        ach = f[key] * (E if key == "ops_per_edge" else N) / (flux_ms * 1e-3) / 1e9
        fp64_roof = {"bound": "fp64", "achieved": round(ach, 1), "peak": f["peak_gops"], "unit": "G FP64 op/s",
                     "frac": round(ach / f["peak_gops"], 4), key: f[key], "peak_source": f["peak_source"],
                     "ncu_fp64_pipe_busy": f["pipe_busy_ncu"]}
    kernel = ("k_update fused stage (level-0 edge fluxes + time step)" if increment == "fused"
              else "k_flux (level-0 edge flux sweep)")
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "kernel": kernel,
            "flux_ms_per_launch": round(flux_ms, 4), "algorithmic_bytes_per_launch": bytes_per_sweep,
            "peak_source": peak_kind, "fp64": fp64_roof}


def timed_cycles(solver, stream, cycles):
    """Device time of `cycles` V-cycles (CUDA-graph replays) enqueued on the
    solver's own stream, between two CUDA events recorded on that stream."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.run(cycles)
    e1.record(stream)
    status = solver.synchronize()
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3, status


def kernel_times(mesh, cycles, **opts):
    """Mean CUDA-event time of a level-0 edge-flux launch (the fused stage in
    mixed precision).  A separate solver records events around those launches,
    which takes it off the CUDA-graph path, so this pass is not the timed one."""
    import mgcfd
    from mgcfd import _lib
    s = mgcfd.Solver(mesh, MACH, AOA, time_kernels=True, **opts)
    s.run(3)
    if s.synchronize() != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    st0 = s.stats()
    s.run(cycles)
    if s.synchronize() != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    st1 = s.stats()
    s.close()
    return (st1.flux_ms_l0 - st0.flux_ms_l0) / max(1, st1.flux_sweeps_l0 - st0.flux_sweeps_l0)


def run_gb300(args):
    import ctypes as C

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
    inc = args.increment if args.increment != "auto" else ("fused" if args.precision in ("mixed", "dw") else "atomic")
    variant = dict(precision=args.precision, increment=args.increment, renumber=args.renumber,
                   accumulation=args.accumulation, stage_neighbour_ids=args.stage_ids,
                   edge_parallel_stage=args.edge_parallel)
    # The timed region: the production path, one CUDA graph per V-cycle on
    # the solver's stream, timed with CUDA events on that stream.
    stream = torch.cuda.Stream()
    solver = mgcfd.Solver(mesh, MACH, AOA, stream=stream.cuda_stream, **variant)
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
        secs, status = timed_cycles(solver, stream, args.steps)
        t1 = time.perf_counter()
    barrier()
    if status != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    st1 = solver.stats()
    value, elapsed = replicas.job_throughput(args.steps, secs, dist, device="cuda")
    launches = int(st1.kernel_launches - st0.kernel_launches)
    solver.close()
    # Per-kernel events in their own pass (off the graph path).
    flux_ms = kernel_times(mesh, args.kernel_cycles, **variant)

    # End to end through the host-buffer entry point, pinned host memory.
    levels = mesh.levels()
    pinned = []
    hl = pinned_levels(levels, pinned)
    outs = [torch.empty((L.nnodes, 5), dtype=torch.float64).pin_memory() for L in levels]
    views = mgcfd.level_views_from_arrays(hl)
    out_ptrs = (_lib.c_double_p * len(outs))(*[C.cast(o.data_ptr(), _lib.c_double_p) for o in outs])
    opts = mgcfd.options(**variant)
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
    dw_e2e = None
    if rank == 0 and not args.no_extra_forms:
        # The same end-to-end step with the double-word form.
        dopts = mgcfd.options(precision="dw", increment="fused", renumber=args.renumber)
        _lib.check(lib.mgcfd_solve(len(hl), views, MACH, AOA, 1, C.byref(dopts), out_ptrs))  # warm-up
        td0 = time.perf_counter()
        for _ in range(e2e_steps):
            _lib.check(lib.mgcfd_solve(len(hl), views, MACH, AOA, E2E_CYCLES, C.byref(dopts), out_ptrs))
        td1 = time.perf_counter()
        dw_e2e = {"value": round(e2e_steps * E2E_CYCLES / (td1 - td0), 3), "unit": "cycles/s",
                  "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps}
    del pinned, hl, outs

    mixed = dw = served = cpu = None
    if rank == 0 and not args.no_extra_forms:
        want = fp64_reference(mesh, stream, MIXED_CYCLES)
        fp64_value = value if args.precision == "fp64" else None
        dw = dw_section(mesh, args, N, E, stream, fp64_value, want)
        dw["e2e"] = dw_e2e
        mixed = mixed_section(mesh, args, N, E, stream, fp64_value, want)
        served = served_section(args)
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(levels, args.cpu_cycles)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    line = {
        "metric": metric_name(args, N),
        "value": round(value, 3),
        "unit": "cycles/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * elapsed / args.steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fp64": "f64", "mixed": "f32-flux/f64-accumulate", "dw": "f32x2-flux/f64"}[args.precision],
        "data": data_words(args),
        "config": line_config(args, N, E),
        "variant": {"increment": inc, "renumber": args.renumber,
                    "accumulation": args.accumulation if args.precision == "mixed" else "fp64",
                    "parallelism": f"replicas x{world}"},
        "timing": "CUDA events on the solver's stream around the timed V-cycles, each one CUDA-graph replay "
                  f"(the default path); wall clock {round(t1 - t0, 4)} s for the same region",
        "roofline": dict(flux_roofline(args.precision, inc, args.n, N, E, flux_ms),
                         timing=f"mean CUDA-event time of the level-0 launches over {args.kernel_cycles} V-cycles "
                                "of a second solver that records events around them (no CUDA graph)"),
        "e2e": {"value": round(e2e_value, 3), "unit": "cycles/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step": f"mgcfd_solve: upload mesh, setup, {E2E_CYCLES} V-cycles, download all levels",
                "steps": e2e_steps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "dw": dw,
        "mixed": mixed,
        "served": served,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


L2_BYTES = 129e6  # GB300 L2


def line_config(args, N, E):
    """The config both arms print for the same workload.  The L2 note counts
    the level-0 arrays an FP64 V-cycle touches (per node: state and
    primitives, old state, residual, increments, volume terms, maps and
    offsets, about 252 B; per edge: map and weights, 40 B)."""
    level0 = 252 * N + 40 * E
    if level0 > 2 * L2_BYTES:
        l2 = f"inputs larger than L2 (level-0 arrays ~{level0 / 1e9:.2f} GB), no flush"
    else:
        l2 = f"level-0 arrays ~{level0 / 1e6:.0f} MB fit in L2 ({L2_BYTES / 1e6:.0f} MB): L2-warm timings, not HBM"
    return {"workload": f"{args.n}^3 jittered lattice, {NLEVELS} levels, Mach {MACH}, AoA {AOA} deg, "
                        f"{N} nodes / {E} edges on level 0",
            "precision": args.precision, "l2": l2}


def node_count_words(N):
    """8000000 -> "8M"; other counts with thousands separators."""
    return f"{N // 10**6}M" if N >= 10**6 and N % 10**6 == 0 else f"{N:,}"


def metric_name(args, N, where=None):
    """The line's metric: "MG V-cycles/s at 8M nodes (200^3, 4 levels)" for the default workload."""
    base = f"MG V-cycles/s at {node_count_words(N)} nodes"
    return f"{base} ({args.n}^3, {NLEVELS} levels)" if where is None else f"{base} {where}"


def data_words(args):
    return f"synthetic: seeded jittered {args.n}^3 lattice, permuted ids"


def fp64_reference(mesh, stream, cycles):
    """Every level's state after `cycles` V-cycles of the FP64 solver."""
    import mgcfd
    from mgcfd import _lib
    ref = mgcfd.Solver(mesh, MACH, AOA, stream=stream.cuda_stream)
    ref.run(cycles)
    if ref.synchronize() != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    want = [ref.fetch(l) for l in range(NLEVELS)]
    ref.close()
    return want


def timed_form(mesh, args, stream, cycles, want, **opts):
    """V-cycles/s of one solver form on the CUDA-graph path, then its final
    state after `cycles` V-cycles from the start against `want`: each
    variable's max and L2 relative error at level 0, the worst max relative
    error over all levels, and the FP64 parity metric (largest error relative
    to each value, or to a thousandth of its variable's scale)."""
    import numpy as np

    import mgcfd
    from mgcfd import _lib
    sys.path.insert(0, str(ROOT / "tests"))
    from parity import state_error
    s = mgcfd.Solver(mesh, MACH, AOA, stream=stream.cuda_stream, **opts)
    s.run(args.warmup)
    if s.synchronize() != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    secs, st = timed_cycles(s, stream, args.steps)
    if st != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    s.reset()
    s.run(cycles)
    if s.synchronize() != 0:
        raise RuntimeError(_lib.load().mgcfd_last_error().decode())
    got = [s.fetch(l) for l in range(NLEVELS)]
    s.close()
    mx = np.abs(got[0] - want[0]).max(axis=0) / np.abs(want[0]).max(axis=0)
    l2 = np.linalg.norm(got[0] - want[0], axis=0) / np.linalg.norm(want[0], axis=0)
    worst = max(float((np.abs(g - w).max(axis=0) / np.abs(w).max(axis=0)).max()) for g, w in zip(got, want))
    parity = max(state_error(g, w) for g, w in zip(got, want))
    return args.steps / secs, {"max_rel_l0": [float(f"{x:.3e}") for x in mx],
                               "l2_rel_l0": [float(f"{x:.3e}") for x in l2],
                               "max_rel_all_levels": float(f"{worst:.3e}"),
                               "state_error_all_levels": float(f"{parity:.3e}")}


def dw_section(mesh, args, N, E, stream, fp64_value, want):
    """The double-word form on the same mesh: state, node sums, time step and
    norms in FP64, edge fluxes and node primitives in float-float arithmetic on
    the FP32 pipes, fused node-centric stage.  Held to the FP64 path's 1e-10
    bar; its state after 25 V-cycles is compared with the FP64 solve's."""
    opts = dict(precision="dw", increment="fused", renumber=args.renumber)
    rate, err = timed_form(mesh, args, stream, MIXED_CYCLES, want, **opts)
    return {"workload": f"{args.n}^3 lattice, {NLEVELS} levels, Mach {MACH}, AoA {AOA} deg, fused node-centric stage",
            "dtype": "f32x2-flux/f64", "value": round(rate, 3), "unit": "cycles/s",
            "speedup_vs_fp64_value": round(rate / fp64_value, 3) if fp64_value else None,
            "error_against": f"FP64 solve of the same mesh after {MIXED_CYCLES} V-cycles",
            "variables": ["rho", "rho_u", "rho_v", "rho_w", "rho_E"], **err,
            "roofline": flux_roofline("dw", "fused", args.n, N, E, kernel_times(mesh, args.kernel_cycles, **opts))}


def mixed_section(mesh, args, N, E, stream, fp64_value, want):
    """The mixed-precision workload on the same mesh: edge-flux arithmetic and
    geometry in FP32, node sums, time step and norms in FP64 (FP64 node sums,
    or compensated FP32-pair sums).  V-cycles/s on the CUDA-graph path, the
    fused stage's roofline, and each variable's max and L2 relative error of
    the final state after 25 V-cycles against the FP64 solve."""
    cycles = MIXED_CYCLES
    out = {"workload": f"{args.n}^3 lattice, {NLEVELS} levels, Mach {MACH}, AoA {AOA} deg, fused node-centric stage",
           "error_against": f"FP64 solve of the same mesh after {cycles} V-cycles",
           "variables": ["rho", "rho_u", "rho_v", "rho_w", "rho_E"]}
    for acc in ("fp64", "pair32"):
        opts = dict(precision="mixed", increment="fused", renumber=args.renumber, accumulation=acc)
        rate, err = timed_form(mesh, args, stream, cycles, want, **opts)
        out[f"accumulation_{acc}"] = {
            "value": round(rate, 3), "unit": "cycles/s",
            "speedup_vs_fp64_value": round(rate / fp64_value, 3) if fp64_value else None, **err,
            "roofline": flux_roofline("mixed", "fused", args.n, N, E, kernel_times(mesh, args.kernel_cycles, **opts))}
    return out


def generate_pool(specs, keep):
    """Seeded lattice meshes (n, levels, seed) generated on host threads (the
    generator releases the interpreter lock) and copied to page-locked memory."""
    import concurrent.futures as cf

    import mgcfd

    def one(spec):
        n, nl, seed = spec
        return mgcfd.HostMesh.generate(n, nl, seed)

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        meshes = list(ex.map(one, specs))
    return [pinned_levels(m.levels(), keep) for m in meshes]


def serve_specs(count, rng, seed0):
    """Request meshes as the serving workload draws them: node count
    log-uniform in 20K..4M (a cubic lattice of that size), 3 or 4 levels."""
    import numpy as np
    out = []
    for i in range(count):
        nodes = float(np.exp(rng.uniform(np.log(20e3), np.log(4e6))))
        out.append((max(8, int(round(nodes ** (1.0 / 3.0)))), int(rng.integers(3, 5)), seed0 + i))
    return out


# Served forms: slots=1 serves one request at a time; the others overlap up
# to --serve-slots requests.  The *_cohorts forms also admit requests of at
# most COHORT_NODES level-0 nodes that wait together as one batched solver
# (up to 16 per cohort, one launch per stage).
COHORT_NODES = 262144
SERVE_FORMS = {"plain_fp64": dict(slots=1, precision="fp64"),
               "serial_mixed": dict(slots=1, precision="mixed"),
               "served_fp64": dict(precision="fp64"),
               "served_mixed": dict(precision="mixed"),
               "served_mixed_pair32": dict(precision="mixed", accumulation="pair32"),
               "served_mixed_cohorts": dict(precision="mixed", batch_max_meshes=16, batch_max_nodes=COHORT_NODES),
               "served_mixed_pair32_cohorts": dict(precision="mixed", accumulation="pair32", batch_max_meshes=16,
                                                   batch_max_nodes=COHORT_NODES),
               "served_dw": dict(precision="dw"),
               "served_dw_cohorts": dict(precision="dw", batch_max_meshes=16, batch_max_nodes=COHORT_NODES)}
RATE_FORMS = ("plain_fp64", "served_mixed", "served_mixed_pair32", "served_mixed_cohorts",
              "served_mixed_pair32_cohorts", "served_dw")
ERROR_FORMS = ("served_mixed", "served_mixed_pair32", "served_mixed_cohorts", "served_mixed_pair32_cohorts",
               "served_dw", "served_dw_cohorts")


def serve_stream(pool, picks, machs, aoas, gaps, form, rate, slots, reuse, want_results=False):
    """Serve one request stream with one form; returns (summary, results).
    rate = 0 queues every request at once (capacity).  With reuse, requests on
    the same pool mesh share a resident mesh key; without it every request
    uploads and sets up its mesh (a fresh mesh as far as the server knows)."""
    import threading

    import numpy as np

    import mgcfd
    o = dict(SERVE_FORMS[form])
    active = o.pop("slots", slots)
    srv = mgcfd.Server(hbm_budget_gb=150.0, max_active=active, max_cycles=50, residual_drop=1e-6, **o)
    R = len(picks)
    t_start = time.perf_counter()
    arrivals = np.cumsum(gaps / rate) if rate else np.zeros(R)
    ids = {}

    def feeder():
        for k in range(R):
            delay = t_start + arrivals[k] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            key = int(picks[k]) + 1 if (reuse and form != "plain_fp64") else 0
            rid = srv.submit(pool[picks[k]], float(machs[k]), float(aoas[k]), mesh_key=key,
                             resident=key != 0, want_result=want_results)
            ids[rid] = k

    th = threading.Thread(target=feeder)
    th.start()
    th.join()
    srv.drain(3600)
    t_end = time.perf_counter()
    polled = srv.poll()
    st = srv.stats()
    srv.close()
    res = [r for r, _ in polled]
    results = {ids[r["id"]]: (r, v) for r, v in polled}
    lat = np.array([r["finish_s"] - r["submit_s"] for r in res])
    ok = sum(1 for r in res if r["status"] == 0)
    return {"rate_per_s": round(rate, 3) if rate else "all at once",
            "solves_per_s": round(len(res) / (t_end - t_start), 3),
            "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
            "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2), "ok": ok, "failed": len(res) - ok,
            "mean_cycles": round(float(np.mean([r["cycles"] for r in res])), 2),
            "peak_active": int(st["peak_active"]), "peak_budget_gb": round(st["peak_bytes"] / 2 ** 30, 2),
            "resident_mesh_hits": int(st["cache_hits"]), "cohorts": int(st["cohorts"]),
            "cohort_requests": int(st["cohort_requests"])}, results


def served_section(args):
    """Served solves on a fresh-mesh stream: every request is its own seeded
    mesh (the pool is as large as the request count), so no form reuses a
    resident mesh.  The plain FP64 path (one solve at a time) against the
    served forms (up to --serve-slots overlapping requests), at capacity and
    at one Poisson rate below the plain path's capacity."""
    import numpy as np
    rng = np.random.default_rng(29)
    R = args.line_serve_requests
    keep = []
    pool = generate_pool(serve_specs(R, rng, 7000), keep)
    picks = np.arange(R)
    machs = rng.uniform(0.3, 0.85, R)
    aoas = rng.uniform(0.0, 6.0, R)
    gaps = rng.exponential(1.0, R)
    serve_stream(pool, picks[:4], machs, aoas, gaps, "served_mixed", 0, args.serve_slots, False)  # warm-up
    cap, results = {}, {}
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as sampler:
        for f in SERVE_FORMS:
            cap[f], results[f] = serve_stream(pool, picks, machs, aoas, gaps, f, 0, args.serve_slots, False,
                                              want_results=f == "plain_fp64" or f in ERROR_FORMS)
        rate = args.line_serve_rate * cap["plain_fp64"]["solves_per_s"]
        at_rate = {f: serve_stream(pool, picks, machs, aoas, gaps, f, rate, args.serve_slots, False)[0]
                   for f in RATE_FORMS}
    err = {}
    for f in ERROR_FORMS:
        worst, same = 0.0, 0
        for k, (r, v) in results[f].items():
            rp, vp = results["plain_fp64"][k]
            if r["status"] == rp["status"] == 0 and r["cycles"] == rp["cycles"]:
                same += 1
                worst = max(worst, float((np.abs(v - vp).max(axis=0) / np.abs(vp).max(axis=0)).max()))
        err[f] = {"max_rel_vs_plain_fp64": float(f"{worst:.3e}"), "requests_compared": same}
    sizes = [L[0].nnodes for L in pool]
    c = {f: cap[f]["solves_per_s"] for f in cap}
    return {"metric": "served solves/s and p50/p99 latency, fresh mesh per request, vs the plain FP64 path",
            "workload": f"{R} requests, each its own seeded lattice mesh ({min(sizes)}..{max(sizes)} level-0 nodes, "
                        "3-4 levels), Mach U(0.3,0.85), AoA U(0,6) deg, 50 V-cycles or residual drop 1e-6, "
                        "HBM budget 150 GB, inputs in page-locked host memory; no mesh stays resident",
            "slots": args.serve_slots, "capacity_solves_per_s": c,
            "speedup_served_mixed_vs_plain_fp64": round(c["served_mixed"] / c["plain_fp64"], 3),
            "speedup_served_mixed_pair32_vs_plain_fp64": round(c["served_mixed_pair32"] / c["plain_fp64"], 3),
            "speedup_served_fp64_vs_plain_fp64": round(c["served_fp64"] / c["plain_fp64"], 3),
            "speedup_served_mixed_cohorts_vs_plain_fp64": round(c["served_mixed_cohorts"] / c["plain_fp64"], 3),
            "speedup_served_mixed_pair32_cohorts_vs_plain_fp64": round(c["served_mixed_pair32_cohorts"] /
                                                                       c["plain_fp64"], 3),
            "speedup_served_dw_vs_plain_fp64": round(c["served_dw"] / c["plain_fp64"], 3),
            "speedup_served_dw_cohorts_vs_plain_fp64": round(c["served_dw_cohorts"] / c["plain_fp64"], 3),
            "cohort_rule": f"requests of at most {COHORT_NODES} level-0 nodes waiting together share one batched "
                           "solver (up to 16)",
            "poisson": {"rate_multiple_of_plain_capacity": args.line_serve_rate, "runs": at_rate},
            "final_state_error": err, "capacity_runs": cap, "clocks": sampler.summary()}


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
        "metric": metric_name(args, L0.nnodes),
        "value": round(value, 4), "unit": "cycles/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * secs / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": data_words(args),
        "config": line_config(args, L0.nnodes, L0.nedges),
        "implementation": "CPU restatement of the reference path (oracle/mgcfd_oracle.c), OpenMP over coloured edges",
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
        for prec in ("fp64", "mixed", "dw"):
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
    line["speedup_batched_dw_vs_sequential_fp64"] = round(results["batched_dw"] / results["sequential_fp64"], 3)
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving: a Poisson stream of requests, each a seeded lattice mesh with
    node count log-uniform in 20K..4M, Mach U(0.3, 0.85), AoA U(0, 6)
    degrees, 3 or 4 levels, run until the level-0 density residual falls to
    1e-6 of its first value or 50 V-cycles, under a 150 GB HBM budget.  Four
    forms serve the same stream:
      plain_fp64           one FP64 solve at a time (the plain path),
      served_fp64          FP64, up to --serve-slots requests overlapping,
      served_mixed         mixed precision, overlapping,
      served_mixed_pair32  mixed precision with compensated FP32-pair sums.
    Requests draw their meshes from a pool of --serve-pool distinct meshes
    (default: one per request, at most 128, to bound host memory).  Without
    --serve-reuse no form keeps a mesh resident, so every request uploads and
    sets up its mesh, as a fresh mesh would; with it the served forms also
    report a labelled variant that keeps pool meshes resident between
    requests.  Capacity is solves/s with every request queued at once; then
    each form serves Poisson arrivals at rates that are multiples of the plain
    path's capacity, reporting p50/p99 latency (submit to result)."""
    import numpy as np
    rng = np.random.default_rng(11)
    R = args.serve_requests
    P = args.serve_pool or min(R, 128)
    keep = []
    pool = generate_pool(serve_specs(P, rng, 500), keep)
    picks = np.arange(R) % P if P >= R else rng.integers(0, P, R)
    machs = rng.uniform(0.3, 0.85, R)
    aoas = rng.uniform(0.0, 6.0, R)
    gaps = rng.exponential(1.0, R)  # unit-rate inter-arrival times, scaled per rate
    serve_stream(pool, picks[:4], machs, aoas, gaps, "served_mixed", 0, args.serve_slots, False)  # warm-up
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as sampler:
        capacity = {f: serve_stream(pool, picks, machs, aoas, gaps, f, 0, args.serve_slots, False)[0]
                    for f in SERVE_FORMS}
        reuse = ({f"{f}_resident": serve_stream(pool, picks, machs, aoas, gaps, f, 0, args.serve_slots, True)[0]
                  for f in ("served_fp64", "served_mixed", "served_mixed_pair32")} if args.serve_reuse else {})
        plain_cap = capacity["plain_fp64"]["solves_per_s"]
        rates = [f * plain_cap for f in args.serve_rate_multiples]
        sweep = {f: [serve_stream(pool, picks, machs, aoas, gaps, f, r, args.serve_slots, False)[0] for r in rates]
                 for f in RATE_FORMS}
    cap = {f: capacity[f]["solves_per_s"] for f in SERVE_FORMS}
    sizes = [L[0].nnodes for L in pool]
    line = {"metric": "served solves/s and p50/p99 latency (Poisson stream), vs the plain FP64 path",
            "unit": "solves/s", "higher_is_better": True, "n_gpus": 1,
            "data": "synthetic: seeded jittered lattices",
            "config": {"workload": f"{R} requests over {P} distinct meshes ({min(sizes)}..{max(sizes)} "
                                   "level-0 nodes, 3-4 levels), 50 V-cycles or residual drop 1e-6, "
                                   "HBM budget 150 GB; no mesh kept resident in the headline forms",
                       "slots": args.serve_slots, "rate_multiples_of_plain_capacity": args.serve_rate_multiples,
                       "inputs": "page-locked host memory"},
            "value": cap["served_mixed"], "capacity_solves_per_s": cap,
            "speedup_served_mixed_vs_plain_fp64": round(cap["served_mixed"] / cap["plain_fp64"], 3),
            "speedup_served_mixed_pair32_vs_plain_fp64": round(cap["served_mixed_pair32"] / cap["plain_fp64"], 3),
            "speedup_served_fp64_vs_plain_fp64": round(cap["served_fp64"] / cap["plain_fp64"], 3),
            "speedup_served_mixed_cohorts_vs_plain_fp64": round(cap["served_mixed_cohorts"] / cap["plain_fp64"], 3),
            "capacity_runs": capacity, "resident_mesh_variant": reuse or None, "sweep": sweep,
            "clocks": sampler.summary()}
    print(json.dumps(line), flush=True)


def run_loops(args):
    """The reference's V-cycle driven loop by loop through the per-loop entry
    points (mgcfd.LoopSolver: every op_par_loop of euler3d.cpp:413-641 one
    mgcfd_op_* call on device dats in OP2 layout, as an OP2 host stub bound to
    this library would issue them), on the same 8M-node mesh:
      file_order  the mesh's own numbering (node ids randomly permuted): the
                  edge-flux plan reorders the nodes (Cuthill-McKee on the GPU)
      renumbered  the mesh after the renumbering tool (Morton order): the
                  plan keeps the caller's order
      plan_free   file order with plans off (the naive per-loop kernels), a
                  few cycles, for contrast
      *_dw        the same with the flux calls in the DW form
                  (mgcfd_op_flux_precision: double-word primitives and fluxes
                  through the plans, node-centric, no atomics)
    V-cycles/s from CUDA events on the driver's stream; the level-0 edge-flux
    call (primitives, flux, scatter) timed alone with events; the first cycle
    (upload, set-up loops, plan builds) reported separately; the final state
    checked against the device-resident solver after the same cycles."""
    import numpy as np
    import torch

    import mgcfd
    from mgcfd import ops
    mesh = mgcfd.HostMesh.generate(args.n, NLEVELS, SEED)
    L0 = mesh.level(0)
    N, E = L0.nnodes, L0.nedges
    total = 1 + args.warmup + args.steps
    ref = mgcfd.Solver(mesh, MACH, AOA)
    ref.run(total)
    assert ref.synchronize() == 0
    want = ref.fetch(0)
    ref.close()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.Stream()
    ref = mgcfd.Solver(mesh, MACH, AOA, stream=stream.cuda_stream)
    ref.run(args.warmup)
    ref.synchronize()
    secs, _ = timed_cycles(ref, stream, args.steps)
    solver_value = args.steps / secs
    ref.close()
    peak, peak_kind = measured_peaks()
    renumbered = mesh.renumber("spatial")
    forms = {"file_order": ("auto", mesh, "fp64"), "renumbered": ("auto", renumbered, "fp64"),
             "file_order_dw": ("auto", mesh, "dw"), "renumbered_dw": ("auto", renumbered, "dw")}
    chosen = set(args.loops_forms.split(","))
    forms = {k: v for k, v in forms.items() if k in chosen}
    out = {}
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as sampler:
        for name, (mode, m, prec) in forms.items():
            ops.plans_mode(mode)
            ops.flux_precision(prec)
            t0 = time.perf_counter()
            s = mgcfd.LoopSolver(m, MACH, AOA, stream=stream)
            s.run(1)
            st, _ = s.synchronize()
            first = time.perf_counter() - t0
            s.run(args.warmup)
            s.synchronize()
            e0.record(stream)
            s.run(args.steps)
            e1.record(stream)
            st, rms = s.synchronize()
            secs = e0.elapsed_time(e1) * 1e-3
            got = s.fetch(0)
            if name.startswith("renumbered"):  # back to the file order of the reference solution
                perm = np.empty(N, np.int64)
                perm[:] = mgcfd.renumber_nodes("spatial", L0.coords)
                back = np.empty_like(got)
                back[perm] = got
                got = back
            err = float((np.abs(got - want).max(axis=0) / np.abs(want).max(axis=0)).max())
            d = s.L[0]
            reps = 10
            e0.record(stream)
            for _ in range(reps):
                ops.compute_flux_edge(E, N, d["e2n"].data_ptr(), d["var"].data_ptr(), d["ewt"].data_ptr(),
                                      s.ff.smoothing_coefficient, d["flux"].data_ptr(), s.s)
            e1.record(stream)
            stream.synchronize()
            flux_ms = e0.elapsed_time(e1) / reps
            info = ops.plans_info()
            s.close()
            ops.plans_release()  # each form builds its own plans
            ops.flux_precision("fp64")
            byt = algorithmic_flux_bytes(N, E)
            out[name] = {"value": round(args.steps / secs, 3), "unit": "cycles/s", "status": st,
                         "first_cycle_s": round(first, 3), "plans": info,
                         "max_rel_vs_solver": float(f"{err:.3e}"),
                         "flux_call_ms": round(flux_ms, 4),
                         "flux_call_vs_solver_flux": None,
                         "roofline": {"bound": "hbm", "achieved": round(byt / (flux_ms * 1e-3) / 1e9, 1), "peak": peak,
                                      "unit": "GB/s", "frac": round(byt / (flux_ms * 1e-3) / 1e9 / peak, 4),
                                      "algorithmic_bytes_per_launch": byt, "peak_source": peak_kind}}
        if "plan_free" in chosen:
            ops.plans_mode("off")
            s = mgcfd.LoopSolver(mesh, MACH, AOA, stream=stream)
            s.run(1)
            s.synchronize()
            e0.record(stream)
            s.run(args.loops_plan_free_cycles)
            e1.record(stream)
            st, _ = s.synchronize()
            out["plan_free"] = {"value": round(args.loops_plan_free_cycles / (e0.elapsed_time(e1) * 1e-3), 3),
                                "unit": "cycles/s", "status": st, "cycles": args.loops_plan_free_cycles}
            s.close()
            ops.plans_mode("auto")
    solver_flux_ms = kernel_times(mesh, args.kernel_cycles)
    for name in forms:
        out[name]["flux_call_vs_solver_flux"] = round(out[name]["flux_call_ms"] / solver_flux_ms, 3)
    line = {"metric": metric_name(args, N, "through the per-loop entry points (OP2 dat layout)"),
            "unit": "cycles/s", "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "data": data_words(args),
            "config": line_config(args, N, E),
            "value": out.get("file_order", {}).get("value"), "forms": out,
            "device_solver": {"value": round(solver_value, 3), "unit": "cycles/s",
                              "flux_ms_per_launch": round(solver_flux_ms, 4)},
            "timing": "CUDA events on the driver's stream; globals stay on the device (no host wait per loop)",
            "clocks": sampler.summary()}
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
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "dw"])
    ap.add_argument("--increment", default="auto", choices=["auto", "atomic", "gather", "fused", "coloured"],
                    help="auto: FP64 atomics for fp64, the fused node-centric stage for mixed")
    ap.add_argument("--renumber", default="spatial", choices=["none", "spatial", "rcm"])
    ap.add_argument("--accumulation", default="fp64", choices=["fp64", "pair32"],
                    help="mixed precision node sums: FP64 adds, or compensated FP32 pairs")
    ap.add_argument("--n", type=int, default=200)
    ap.add_argument("--stage-ids", action="store_true",
                    help="fused mixed stage: stage neighbour ids in shared memory with cp.async (measured slower)")
    ap.add_argument("--edge-parallel", action="store_true",
                    help="fused mixed stage: edge-parallel form (all edge ends of a block at once, then per-node sums)")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-cycles", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="plain", choices=["plain", "batch", "serve", "rates", "loops"])
    ap.add_argument("--loops-plan-free-cycles", type=int, default=2)
    ap.add_argument("--batch-meshes", type=int, default=64)
    ap.add_argument("--serve-requests", type=int, default=240)
    ap.add_argument("--serve-pool", type=int, default=0,
                    help="distinct meshes the requests draw from (0: one per request, at most 128)")
    ap.add_argument("--serve-reuse", action="store_true",
                    help="also report the served forms with pool meshes kept resident between requests")
    ap.add_argument("--serve-rate-multiples", type=float, nargs="*", default=[0.5, 0.9, 2.0],
                    help="Poisson rates as multiples of the plain path's capacity (none: capacity only)")
    ap.add_argument("--serve-slots", type=int, default=16)
    ap.add_argument("--loops-forms", default="file_order,renumbered,file_order_dw,renumbered_dw,plan_free",
                    help="--mode loops: which forms to run (comma-separated)")
    ap.add_argument("--kernel-cycles", type=int, default=5,
                    help="V-cycles of the separate per-kernel event pass behind the roofline")
    ap.add_argument("--no-extra-forms", action="store_true",
                    help="plain line only: skip the mixed-precision and served sections")
    ap.add_argument("--line-serve-requests", type=int, default=64,
                    help="requests (each its own mesh) of the served section of the plain line")
    ap.add_argument("--line-serve-rate", type=float, default=0.8,
                    help="Poisson rate of the served section, as a multiple of the plain path's capacity")
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
    elif args.mode == "loops":
        run_loops(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
