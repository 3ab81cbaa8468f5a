"""The reference's multigrid driver loop run loop by loop through the per-loop
entry points (mgcfd_op_* in include/mgcfd_gb300.h).

This is what an OP2 application sees when its op_par_loop calls are bound to
this library (through a host stub that passes each dat's and map's device
pointer to the matching entry point): every dat is a device array
in OP2's layout ([set size][dim], row-major, in the mesh file's numbering),
every map a 0-based int32 array, and each loop of euler3d.cpp is one call:

  set-up  euler3d.cpp:413-441  initialize_variables, zero_5d (fluxes),
                               zero_1d + calculate_cell_volumes (volumes,
                               re-oriented weights), dampen_ewt (edge and
                               boundary weights)
  cycle   euler3d.cpp:458-641  copy_double, calculate_dt, get_min_dt,
                               compute_step_factor, 3 x {compute_flux_edge,
                               compute_bnd_node_flux, time_step}, residual,
                               calc_rms + count_bad_vals on level 0, then
                               up_pre/up/up_post or down

Globals stay on the device: get_min_dt writes its minimum to a device scalar
that compute_step_factor reads, so no call waits for the host.  Each
smoothing step writes min_dt, the level-0 rms and the NaN/Inf count to its
own slot; synchronize() reads them and reports what the reference would have
stopped on (min_dt < 0, euler3d.cpp:480-484; bad values, :539-548).
The edge flux and the restriction build their execution plans on their first
call (plans.cu), so the first V-cycle includes that set-up.
"""
from __future__ import annotations

import numpy as np

from . import _lib, ops
from .mesh import HostMesh, freestream

_OK, _NEG_DT, _BAD = 0, _lib.ERR_NEGATIVE_DT, _lib.ERR_BAD_VALUES


class LoopSolver:
    """Device dats of a multigrid mesh in OP2 layout and the V-cycle of
    euler3d.cpp driven through mgcfd_op_* calls on one stream."""

    def __init__(self, mesh, mach: float, aoa_deg: float, stream=None, measure_mem_bound: bool = False):
        import torch
        self.torch = torch
        levels = mesh.levels() if isinstance(mesh, HostMesh) else mesh
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.s = self.stream.cuda_stream
        self.ff = freestream(mach, aoa_deg)
        self.measure_mem_bound = measure_mem_bound
        self.L = []
        dev = torch.device("cuda")
        with torch.cuda.stream(self.stream):
            for lv in levels:
                d = {"n": lv.nnodes, "ne": lv.nedges, "nb": lv.nbnd}

                def up(a, dtype):
                    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).to(dev, non_blocking=False)

                d["coords"] = up(lv.coords, np.float64)
                d["e2n"] = up(lv.edge_to_nodes, np.int32)
                d["b2n"] = up(lv.bnd_to_node, np.int32)
                d["grp"] = up(lv.bnd_group, np.int32)
                d["ewt"] = up(lv.edge_weights, np.float64)
                d["bwt"] = up(lv.bnd_weights, np.float64)
                d["n2mg"] = up(lv.node_to_mg, np.int32) if lv.node_to_mg is not None else None
                legacy = getattr(lv, "volumes", None) is not None
                d["vol"] = up(lv.volumes, np.float64) if legacy else torch.empty(lv.nnodes, dtype=torch.float64,
                                                                                   device=dev)
                d["legacy"] = legacy
                for name in ("var", "old", "flux", "res"):
                    d[name] = torch.empty((lv.nnodes, 5), dtype=torch.float64, device=dev)
                d["sf"] = torch.empty(lv.nnodes, dtype=torch.float64, device=dev)
                d["dummy"] = torch.empty((lv.nnodes, 5), dtype=torch.float64, device=dev) if measure_mem_bound else None
                d["scratch"] = torch.empty(lv.nnodes, dtype=torch.int32, device=dev)
                self.L.append(d)
        torch.cuda.synchronize()
        self._setup()
        self.level, self.up, self.cycle = 0, True, 0
        self._slots = None

    def _p(self, t):
        return t.data_ptr() if t is not None else 0

    # euler3d.cpp:413-441
    def _setup(self):
        s = self.s
        for d in self.L:
            ops.initialize_variables(d["n"], self.ff, self._p(d["var"]), s)
            ops.zero(d["n"], 5, self._p(d["flux"]), s)
            if self.measure_mem_bound:
                ops.zero(d["n"], 5, self._p(d["dummy"]), s)
            if not d["legacy"]:
                ops.zero(d["n"], 1, self._p(d["vol"]), s)
                ops.calculate_cell_volumes(d["ne"], d["n"], self._p(d["e2n"]), self._p(d["coords"]),
                                           self._p(d["ewt"]), self._p(d["vol"]), s)
        for d in self.L:
            ops.dampen_ewt(d["ne"], self._p(d["ewt"]), s)
            ops.dampen_ewt(d["nb"], self._p(d["bwt"]), s)

    def _alloc_slots(self, steps: int):
        torch = self.torch
        self._slots = {"min_dt": torch.zeros(steps, dtype=torch.float64, device="cuda"),
                       "rms": torch.zeros(steps, dtype=torch.float64, device="cuda"),
                       "bad": torch.zeros(steps, dtype=torch.int32, device="cuda"),
                       "level": [], "next": 0}

    # euler3d.cpp:467-550 at the current level
    def _smooth(self):
        d, s, l = self.L[self.level], self.s, self.level
        k = self._slots["next"]
        self._slots["next"] += 1
        self._slots["level"].append(l)
        min_dt = self._slots["min_dt"][k:].data_ptr()
        n = d["n"]
        P = self._p
        ops.copy_double(n, P(d["var"]), P(d["old"]), s)
        ops.calculate_dt(n, P(d["var"]), P(d["vol"]), P(d["sf"]), s)
        ops.get_min_dt(n, P(d["sf"]), min_dt, s)
        ops.compute_step_factor(n, P(d["var"]), P(d["vol"]), min_dt, P(d["sf"]), s)
        for rk in range(3):
            ops.compute_flux_edge(d["ne"], n, P(d["e2n"]), P(d["var"]), P(d["ewt"]), self.ff.smoothing_coefficient,
                                  P(d["flux"]), s)
            ops.compute_bnd_node_flux(d["nb"], n, P(d["b2n"]), P(d["grp"]), P(d["bwt"]), P(d["var"]), self.ff,
                                      P(d["flux"]), s)
            ops.time_step(n, rk, P(d["sf"]), P(d["flux"]), P(d["old"]), P(d["var"]), s)
            if self.measure_mem_bound:
                ops.unstructured_stream(d["ne"], n, P(d["e2n"]), P(d["var"]), P(d["ewt"]), P(d["dummy"]), s)
        ops.residual(n, P(d["old"]), P(d["var"]), P(d["res"]), s)
        if l == 0:
            ops.calc_rms(n, P(d["res"]), self._slots["rms"][k:].data_ptr(), s)
            ops.count_bad_vals(n, P(d["var"]), self._slots["bad"][k:].data_ptr(), s)

    # euler3d.cpp:573-640
    def _transfer(self):
        s, P = self.s, self._p
        nl = len(self.L)
        if nl <= 1:
            self.cycle += 1
            return
        if self.up:
            self.level += 1
            f, c = self.L[self.level - 1], self.L[self.level]
            ops.up_pre(f["n"], c["n"], P(f["n2mg"]), P(c["var"]), P(c["scratch"]), s)
            ops.up(f["n"], c["n"], P(f["n2mg"]), P(f["var"]), P(c["var"]), P(c["scratch"]), s)
            ops.up_post(c["n"], P(c["var"]), P(c["scratch"]), s)
            if self.level == nl - 1:
                self.up = False
        else:
            self.level -= 1
            f, c = self.L[self.level], self.L[self.level + 1]
            ops.down(f["n"], c["n"], P(f["n2mg"]), P(f["var"]), P(f["res"]), P(f["coords"]), P(c["res"]),
                     P(c["coords"]), s)
            if self.level == 0:
                self.up = True
                self.cycle += 1

    def steps_per_cycle(self) -> int:
        return 1 if len(self.L) <= 1 else 2 * len(self.L) - 2

    def run(self, ncycles: int) -> None:
        """Enqueue `ncycles` V-cycles (asynchronous)."""
        self._alloc_slots(max(1, ncycles * self.steps_per_cycle()))
        target = self.cycle + ncycles
        while self.cycle < target:
            self._smooth()
            self._transfer()

    def synchronize(self):
        """Waits; returns (status, level-0 rms of the last level-0 step).
        status is what the reference would have stopped on."""
        self.stream.synchronize()
        if not self._slots or not self._slots["level"]:
            return _OK, 0.0
        used = self._slots["next"]
        mins = self._slots["min_dt"][:used].cpu().numpy()
        rms = self._slots["rms"][:used].cpu().numpy()
        bad = self._slots["bad"][:used].cpu().numpy()
        lv = np.array(self._slots["level"])
        last_rms = 0.0
        for k in range(used):
            if mins[k] < 0.0:
                return _NEG_DT, last_rms
            if lv[k] == 0:
                last_rms = float(np.sqrt(rms[k] / self.L[0]["n"]))  # euler3d.cpp:537
                if bad[k] > 0:
                    return _BAD, last_rms
        return _OK, last_rms

    def fetch(self, level: int, what: str = "var") -> np.ndarray:
        self.stream.synchronize()
        return self.L[level][what].cpu().numpy()

    def close(self):
        """Release the plans built from this mesh's maps and volume dats, then
        the dats."""
        if not self.L:
            return
        self.stream.synchronize()
        for d in self.L:
            for m in ("e2n", "n2mg", "vol"):
                if d.get(m) is not None:
                    ops.plan_release(d[m].data_ptr())
        self.L = []

