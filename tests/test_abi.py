"""The C ABI library loads and exports every function include/mgcfd_gb300.h
declares, and the ctypes table binds exactly those functions (CPU only: no
compute call is made)."""
import ctypes as C
import re
from pathlib import Path

import mgcfd
from mgcfd import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "mgcfd_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return set(re.findall(r"\b(mgcfd_[a-z0-9_]+)\s*\(", text))


def test_every_declared_symbol_is_exported():
    lib = C.CDLL(str(_lib.lib_path()))
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_table_matches_header():
    assert set(_lib.SIGNATURES) == declared_functions()


def test_host_only_calls_work_without_gpu():
    lib = _lib.load()
    assert lib.mgcfd_abi_version() == 1
    assert lib.mgcfd_status_string(_lib.ERR_NEGATIVE_DT).decode().startswith("negative time step")
    ff = mgcfd.freestream(1.2, 0.0)    # const.h defaults
    assert ff.ff_variable[0] == 1.4
    assert ff.smoothing_coefficient == float(C.c_float(0.2).value)


def test_freestream_matches_oracle_bits():
    import oracle as O
    for mach, aoa in [(1.2, 0.0), (0.5, 3.0), (0.8, 3.0), (0.3, 6.0)]:
        a, b = mgcfd.freestream(mach, aoa), O.freestream(mach, aoa)
        for f in ("ff_variable", "ff_flux_contribution_momentum_x", "ff_flux_contribution_momentum_y",
                  "ff_flux_contribution_momentum_z", "ff_flux_contribution_density_energy"):
            assert list(getattr(a, f)) == list(getattr(b, f)), (mach, aoa, f)
