#!/usr/bin/env python3
"""Regenerate the golden fixtures in this directory from the reference itself.

Needs the reference sources (it builds oracle/_ref/euler3d_ref: the unmodified
reference euler3d.cpp against the sequential OP2 stand-in).  For each case it
generates the synthetic mesh, writes it in the reference's HDF5 layout, runs
the reference binary with --output-variables --output-step-factors, and stores
what the reference wrote:

  <case>.npz   full per-level variables and step factors (small meshes), or
               per-level statistics plus 1024 sampled rows (the 48^3 case),
               and a SHA-256 of every generated mesh array (pins the generator).

Usage: python tests/golden/make_golden.py
"""
import hashlib
import json
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "mg-cfd-app-op2_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))

import mgcfd  # noqa: E402
import oracle as O  # noqa: E402

# name: (n, levels, seed, mach, aoa_deg, cycles, full_arrays)
CASES = {
    "lattice8_l3_c4": (8, 3, 1234, 0.5, 3.0, 4, True),
    "lattice9_l3_c3": (9, 3, 77, 0.8, 3.0, 3, True),
    "lattice6_l1_c5": (6, 1, 5, 0.3, 6.0, 5, True),
    "lattice12_l2_c3_m12": (12, 2, 99, 1.2, 0.0, 3, True),
    "lattice20_l4_c2": (20, 4, 2024, 0.8, 3.0, 2, True),
    "config0_48_l3_c10": (48, 3, 1234, 0.5, 3.0, 10, False),
}
SAMPLES = 1024


def mesh_digest(levels):
    d = {}
    for l, L in enumerate(levels):
        for name in ("coords", "edge_to_nodes", "bnd_to_node", "bnd_group", "edge_weights", "bnd_weights",
                     "node_to_mg"):
            a = getattr(L, name)
            if a is not None:
                d[f"L{l}.{name}"] = hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    return d


def sample_rows(n, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(SAMPLES, n), replace=False)).astype(np.int64)


def main():
    for name, (n, nl, seed, mach, aoa, cycles, full) in CASES.items():
        mesh = mgcfd.HostMesh.generate(n, nl, seed)
        levels = mesh.levels()
        out = {"meta": json.dumps(dict(n=n, levels=nl, seed=seed, mach=mach, aoa=aoa, cycles=cycles, full=full,
                                       mesh_sha256=mesh_digest(levels)))}
        with tempfile.TemporaryDirectory() as d:
            mesh.write(d, "mesh_")
            r = O.run_reference_binary(d, cycles, mach, aoa)
            if r.returncode != 0:
                raise SystemExit(f"{name}: reference failed\n{r.stdout}\n{r.stderr}")
            for l in range(nl):
                var = mgcfd.h5_read(f"{d}/solution.variables.L{l}.cycles={cycles}.h5", f"p_variables_result_L{l}")
                sf = mgcfd.h5_read(f"{d}/solution.step_factors.L{l}.cycles={cycles}.h5",
                                   f"p_step_factors_result_L{l}").reshape(-1)
                if full:
                    out[f"variables_L{l}"] = var
                    out[f"step_factors_L{l}"] = sf
                else:
                    idx = sample_rows(var.shape[0], seed + l)
                    out[f"rows_L{l}"] = idx
                    out[f"variables_rows_L{l}"] = var[idx]
                    out[f"step_factors_rows_L{l}"] = sf[idx]
                    out[f"stats_L{l}"] = np.stack([var.sum(axis=0), (var * var).sum(axis=0), var.min(axis=0),
                                                   var.max(axis=0)])
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, "written")


if __name__ == "__main__":
    main()
