"""Build recipes for the mgcfd_gb300 native code.

Outputs (all git-ignored, rebuilt when a source is newer than the output):
  mg-cfd-app-op2_gb300/lib/libmgcfd_gb300.so   the product: CUDA kernels + C ABI
  mg-cfd-app-op2_gb300/bin/euler3d_gb300        euler3d-compatible command line driver
  mg-cfd-app-op2_gb300/bin/mgcfd_renumber       standalone mesh renumbering tool
(The checkers under oracle/ have their own recipe, oracle/recipe.py.)

CUDA code is compiled for sm_103a only.  Host C/C++ is compiled with
-ffp-contract=off so results are identical on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent.parent          # mg-cfd-app-op2_gb300/
ROOT = PKG.parent                                      # repository root
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB = PKG / "lib" / "libmgcfd_gb300.so"
CLI = PKG / "bin" / "euler3d_gb300"
RENUMBER_CLI = PKG / "bin" / "mgcfd_renumber"
TOOLS = {"euler3d_gb300.cpp": CLI, "mgcfd_renumber.cpp": RENUMBER_CLI}
OBJ = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                     f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mgcfd_gb300")


def _stamp_ok(directory: Path) -> bool:
    """True when `directory` holds outputs built on this host architecture."""
    stamp = directory / ".host"
    return stamp.exists() and stamp.read_text().strip() == platform.machine()


def _write_stamp(directory: Path) -> None:
    directory.mkdir(parents=True, exist_ok=True)
    (directory / ".host").write_text(platform.machine() + "\n")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def _headers():
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h")))


def library_sources():
    return sorted(CSRC.glob("*.cu")), sorted(p for p in CSRC.glob("*.cpp") if p.name not in TOOLS)


def build_library(force: bool = False, jobs: int | None = None) -> Path:
    """Compile every .cu/.cpp under csrc/ and link libmgcfd_gb300.so."""
    cu, cpp = library_sources()
    OBJ.mkdir(parents=True, exist_ok=True)
    force = force or not _stamp_ok(OBJ)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    hdrs = _headers()
    nvcc = _nvcc()
    jobs_list = []
    objs = []
    for src in cu:
        obj = OBJ / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs_list.append([nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = OBJ / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs_list.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, c) for c in jobs_list]:
                f.result()
    if force or jobs_list or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"])
    cuda = Path(nvcc).resolve().parent.parent  # the toolkit: the CLI allocates its --per-loop dats itself
    for name, exe in TOOLS.items():
        src = CSRC / name
        if src.exists() and (force or _stale(exe, [src, LIB] + hdrs)):
            exe.parent.mkdir(parents=True, exist_ok=True)
            _run(["g++", *CXX_FLAGS, f"-I{cuda / 'include'}", str(src), "-o", str(exe), f"-L{LIB.parent}",
                  "-lmgcfd_gb300", f"-L{cuda / 'lib64'}", "-lcudart", f"-Wl,-rpath,{LIB.parent}",
                  "-Wl,-rpath,$ORIGIN/../lib"])
    _write_stamp(OBJ)
    return LIB


def build_all(force: bool = False) -> None:
    build_library(force)
