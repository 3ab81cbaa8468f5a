"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

Build recipe of the checkers under oracle/ (oracle/recipe.py):
  oracle/_build/liboracle.so   the C restatement of the reference path
                               (mgcfd_oracle.c), with OpenMP for the timed
                               CPU baseline
  oracle/_ref/euler3d_ref      the reference's own euler3d.cpp and headers,
                               compiled unmodified against the sequential
                               OP2 stand-in in op2shim/ (only where the
                               reference sources are present)

This recipe is the one place that reads the reference sources where they lie:
MGCFD_REFERENCE_DIR, or /root/reference when that is unset.  Nothing is
copied out of that tree; the binary goes to oracle/_ref/ (git-ignored).

Both are compiled with -ffp-contract=off so their arithmetic is plain IEEE
binary64 in source order on x86_64 and aarch64 alike.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT / "mg-cfd-app-op2_gb300"))
from mgcfd import _build as B  # noqa: E402  (shared compile helpers; h5lite sources)

ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_BIN = HERE / "_ref" / "euler3d_ref"
DEFAULT_REFERENCE_DIR = "/root/reference"


def build_oracle(force: bool = False) -> Path:
    """Compile the C restatement into liboracle.so."""
    src, hdr = HERE / "mgcfd_oracle.c", HERE / "mgcfd_oracle.h"
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    force = force or not B._stamp_ok(ORACLE_LIB.parent)
    if force or B._stale(ORACLE_LIB, [src, hdr]):
        B._run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                "-o", str(ORACLE_LIB), str(src), "-lm"])
    B._write_stamp(ORACLE_LIB.parent)
    return ORACLE_LIB


def reference_dir() -> Path | None:
    p = Path(os.environ.get("MGCFD_REFERENCE_DIR", DEFAULT_REFERENCE_DIR))
    return p if (p / "euler3d.cpp").exists() else None


def build_reference(force: bool = False) -> Path | None:
    """Compile the unmodified reference driver against the OP2 stand-in.

    Returns None where the reference sources are absent (the GPU host)."""
    ref = reference_dir()
    if ref is None:
        return None
    shim = HERE / "op2shim"
    deps = [HERE / "ref_main.cpp", shim / "op2shim.cpp", shim / "op_seq.h", shim / "op_hdf5.h",
            B.CSRC / "h5lite.cpp", B.CSRC / "h5lite.h"]
    deps += sorted(ref.glob("*.h")) + [ref / "euler3d.cpp"]
    if force or not B._stamp_ok(REF_BIN.parent) or B._stale(REF_BIN, deps):
        REF_BIN.parent.mkdir(parents=True, exist_ok=True)
        B._run(["g++", "-O2", "-std=c++14", "-ffp-contract=off", "-w", f"-I{shim}", f"-I{B.CSRC}", f"-I{ref}",
                "-o", str(REF_BIN), str(HERE / "ref_main.cpp"), str(shim / "op2shim.cpp"), str(B.CSRC / "h5lite.cpp")])
        B._write_stamp(REF_BIN.parent)
    return REF_BIN


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_reference(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
