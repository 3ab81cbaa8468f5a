"""The DW precision form: double-word (float-float) edge-flux arithmetic on the
FP32 pipes, FP64 state, sums, time step and norms.  Held to the FP64 path's
bar: within 1e-10 relative of the oracle (GPU).

The building blocks are checked first: the binary64 -> pair split gives
h = round(d) and l = round(d - h) bit for bit (numpy's IEEE conversions), and
the DW edge flux is within 2^-42 of the exact flux relative to the sum of its
terms' magnitudes (an extended-precision numpy evaluation of the same
formula), where the FP64 flux is within 2^-48."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

import mgcfd
import oracle as O
from irregular import irregular_levels
from mgcfd import _build
from parity import DELTA_TOL, STATE_TOL, delta_error, state_error

pytestmark = pytest.mark.gpu
HERE = Path(__file__).resolve().parent
GOLDEN = HERE / "golden"


@pytest.fixture(scope="module")
def dwlib():
    out = HERE / "_build" / "libdw_check.so"
    out.parent.mkdir(exist_ok=True)
    src = HERE / "native" / "dw_check.cu"
    subprocess.run([_build._nvcc(), *_build.ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                    f"-I{_build.CSRC}", str(src), "-o", str(out)], check=True, capture_output=True)
    lib = C.CDLL(str(out))
    lib.dw_check_split.restype = C.c_int
    lib.dw_check_flux.restype = C.c_int
    lib.dw_check_node.restype = C.c_int
    return lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_split_is_round_then_round_of_the_rest(dwlib):
    rng = np.random.default_rng(3)
    n = 300_000
    # every binade binary32 can hold, plus the special and edge classes
    mag = np.ldexp(rng.random(n) + 0.5, rng.integers(-160, 140, n))
    d = np.where(rng.random(n) < 0.5, -mag, mag)
    f = rng.integers(1, 0x7f7fffff, 50_000, dtype=np.int64).astype(np.uint32).view(np.float32).astype(np.float64)
    up = np.nextafter(f.astype(np.float32), np.float32(np.inf)).astype(np.float64)
    mid = f + (up - f) / 2  # halfway between two floats: ties to even
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, 2.0 - 2 ** -52, 2.0 ** 127, 2.0 ** 127 * (2 - 2 ** -52),
                      2.0 ** 128, 2.0 ** -74, 2.0 ** -74 * (1 - 2 ** -53), 2.0 ** -126, 1e-45, 5e-324, 1.7e308,
                      3.4028235677973366e38, 1.0 + 2 ** -24, 1.0 + 2 ** -24 + 2 ** -52, 1.0 - 2 ** -25])
    d = np.concatenate([d, f, mid, np.nextafter(mid, np.inf), np.nextafter(mid, -np.inf), edges, -edges])
    h = np.empty(len(d), np.float32)
    lo = np.empty(len(d), np.float32)
    assert dwlib.dw_check_split(C.c_int64(len(d)), _p(d), _p(h), _p(lo)) == 0
    with np.errstate(over="ignore", invalid="ignore"):
        want_h = d.astype(np.float32)
        rest = np.where(np.isfinite(want_h), d - want_h.astype(np.float64), 0.0)
        want_l = rest.astype(np.float32)
    nan = np.isnan(d)
    assert np.array_equal(h.view(np.uint32)[~nan], want_h.view(np.uint32)[~nan])
    assert np.isnan(h[nan]).all()
    assert np.array_equal(lo.view(np.uint32)[~nan], want_l.view(np.uint32)[~nan])
    # the pair holds d to 2^-48 relative wherever l is a normal binary32 number
    ok = np.isfinite(want_h) & (np.abs(d) >= 2.0 ** -100) & (np.abs(d) < 2.0 ** 127)
    err = np.abs((h[ok].astype(np.longdouble) + lo[ok]) - d[ok]) / np.abs(d[ok])
    assert err.max() <= 2.0 ** -48


def _flux_ref(a, b, w):
    """edge_flux's formula (device_math.cuh) in numpy long double, and the same
    formula on absolute values (the sum of the terms' magnitudes)."""
    def formula(a, b, w, sub):
        rho, mx, my, mz, E, p, s, ri = (a[:, k] for k in range(8))
        rb, mxb, myb, mzb, Eb, pb, sb, rib = (b[:, k] for k in range(8))
        hx, hy, hz, wf = (w[:, k] for k in range(4))
        uha = (mx * hx + my * hy + mz * hz) * ri
        uhb = (mxb * hx + myb * hy + mzb * hz) * rib
        fac = wf * (s + sb)
        ga, gb = uha + fac, sub(uhb, fac)
        pp = p + pb
        return np.stack([rho * ga + rb * gb, mx * ga + mxb * gb + pp * hx, my * ga + myb * gb + pp * hy,
                         mz * ga + mzb * gb + pp * hz, E * ga + Eb * gb + p * uha + pb * uhb], axis=1)
    L = np.longdouble
    exact = formula(a.astype(L), b.astype(L), w.astype(L), lambda x, y: x - y)
    mag = formula(np.abs(a).astype(L), np.abs(b).astype(L), np.abs(w).astype(L), lambda x, y: x + y)
    return exact, mag


def test_edge_flux_error_bound(dwlib):
    rng = np.random.default_rng(8)
    n = 200_000

    def prims(n):
        rho = rng.uniform(0.2, 3.0, n)
        m = rng.uniform(-2.0, 2.0, (n, 3)) * rho[:, None]
        E = rng.uniform(1.5, 5.0, n)
        p = 0.4 * (E - 0.5 * (m ** 2).sum(1) / rho)
        s = np.sqrt((m ** 2).sum(1)) / rho + np.sqrt(1.4 * np.abs(p) / rho)
        x = np.column_stack([rho, m, E, p, s, 1.0 / rho])
        # rescale whole rows by powers of two over a wide range, some rows near-equal to their partner
        return x * np.ldexp(1.0, rng.integers(-30, 30, n))[:, None]
    a = prims(n)
    b = np.where(rng.random((n, 1)) < 0.2, a * (1 + rng.uniform(-1e-6, 1e-6, (n, 8))), prims(n))
    w = np.column_stack([rng.uniform(-1, 1, (n, 3)), -rng.uniform(0, 1, n)])
    w *= np.ldexp(1.0, rng.integers(-40, 0, n))[:, None]
    w[:100] = 0.0  # edges of zero weight
    a, b, w = (np.ascontiguousarray(x) for x in (a, b, w))
    f64 = np.empty((n, 5))
    fdw = np.empty((n, 5))
    assert dwlib.dw_check_flux(C.c_int64(n), _p(a), _p(b), _p(w), _p(f64), _p(fdw)) == 0
    exact, mag = _flux_ref(a, b, w)
    mag = np.where(mag == 0, 1.0, mag)
    e64 = (np.abs(f64 - exact) / mag).astype(np.float64)
    edw = (np.abs(fdw - exact) / mag).astype(np.float64)
    assert np.isfinite(fdw).all()
    assert e64.max() <= 2.0 ** -48, e64.max()
    assert edw.max() <= 2.0 ** -42, edw.max()
    assert np.all(fdw[:100] == 0.0)


def _prims_ld(x):
    """node_prim's formula in long double: rho, m, E, p, |u|+c, 1/rho."""
    L = np.longdouble
    rho, mx, my, mz, E = (x[:, k].astype(L) for k in range(5))
    ri = 1 / rho
    m2 = mx * mx + my * my + mz * mz
    p = (L(1.4) - 1) * (E - m2 * ri / 2)
    s = np.sqrt(m2) * ri + np.sqrt(L(1.4) * p * ri)
    return np.stack([rho, mx, my, mz, E, p, s, ri], axis=1)


def test_node_primitives_and_factored_node_sum(dwlib):
    """node_prim_dw (the primitives in pairs, no FP64 instruction) against
    node_prim and long double; node_flux_dw (each node's edge-flux sum in the
    factored form the fused stage uses) against the long-double sum of the
    same edges' fluxes, relative to the sum of the terms' magnitudes."""
    rng = np.random.default_rng(21)
    n, K = 50_000, 6

    def states(shape):
        rho = rng.uniform(0.3, 2.5, shape)
        u = rng.uniform(-0.9, 0.9, shape + (3,))
        p = rng.uniform(0.2, 2.0, shape)
        E = p / 0.4 + 0.5 * rho * (u ** 2).sum(-1)
        return np.concatenate([rho[..., None], rho[..., None] * u, E[..., None]], axis=-1)
    me = np.ascontiguousarray(states((n,)))
    nb = np.ascontiguousarray(states((n, K)))
    nb[: n // 5] = me[: n // 5, None, :] * (1 + rng.uniform(-1e-7, 1e-7, (n // 5, K, 5)))  # near-uniform flow
    w = np.concatenate([rng.uniform(-1, 1, (n, K, 3)), -rng.uniform(0, 1, (n, K, 1))], axis=-1)
    w = np.ascontiguousarray(w * np.ldexp(1.0, rng.integers(-30, 0, (n, K, 1))))
    out, pdw, p64 = np.empty((n, 5)), np.empty((n, 8)), np.empty((n, 8))
    assert dwlib.dw_check_node(C.c_int64(n), C.c_int32(K), _p(me), _p(nb), _p(w), _p(out), _p(pdw), _p(p64)) == 0
    ref = _prims_ld(me)
    # p = 0.4 (E - rho|u|^2/2) cancels by up to 40x for these states: judged
    # against the magnitude of its terms, 0.4|E|; c and so s inherit at most
    # half of that amplification.
    den = np.abs(ref)
    den[:, 5] = 0.4 * np.abs(ref[:, 4])
    err_dw = (np.abs(pdw - ref) / den).astype(np.float64)
    err_64 = (np.abs(p64 - ref) / den).astype(np.float64)
    assert err_dw.max() <= 2.0 ** -40, err_dw.max(axis=0)
    assert err_64.max() <= 2.0 ** -46, err_64.max(axis=0)
    # The node sum: every edge with the node as end a (weights already oriented).
    a = np.repeat(_prims_ld(me).astype(np.float64), K, axis=0)
    b = _prims_ld(nb.reshape(-1, 5)).astype(np.float64)
    exact, mag = _flux_ref(a, b, w.reshape(-1, 4))
    exact = exact.reshape(n, K, 5).sum(axis=1)
    mag = mag.reshape(n, K, 5).sum(axis=1)
    err = (np.abs(out - exact) / np.where(mag == 0, 1, mag)).astype(np.float64)
    assert np.isfinite(out).all() and err.max() <= 2.0 ** -40, err.max()


def _oracle(levels, mach, aoa, cycles):
    run = O.OracleRun(levels)
    st, _ = run.run(mach, aoa, cycles)
    assert st == 0
    return run


def _check(s, ref, nl, mach, aoa):
    x0 = np.array(O.freestream(mach, aoa).ff_variable[:])
    for l in range(nl):
        r = ref.get(l, O.Q_VARIABLES) if hasattr(ref, "get") else ref[l]
        x = s.fetch(l)
        assert state_error(x, r) <= STATE_TOL, (l, state_error(x, r))
        assert delta_error(x, r, x0) <= DELTA_TOL, (l, delta_error(x, r, x0))


@pytest.mark.parametrize("n,nl,cycles", [(6, 1, 3), (8, 2, 3), (9, 3, 2), (16, 3, 4), (20, 4, 2)])
@pytest.mark.parametrize("increment", ["atomic", "gather", "fused"])
def test_small_meshes_dw(n, nl, cycles, increment):
    mesh = mgcfd.HostMesh.generate(n, nl, 1000 + n)
    mach, aoa = 0.5, 3.0
    ref = _oracle(mesh.levels(), mach, aoa, cycles)
    s = mgcfd.Solver(mesh, mach, aoa, precision="dw", increment=increment)
    s.run(cycles)
    assert s.synchronize() == 0
    _check(s, ref, nl, mach, aoa)
    for l in range(nl):
        np.testing.assert_allclose(s.fetch(l, mgcfd.Q_STEP_FACTORS), ref.get(l, O.Q_STEP_FACTORS), rtol=1e-12)
    s.close()


@pytest.mark.parametrize("renumber,host_setup,increment", [("spatial", False, "atomic"), ("none", False, "fused"),
                                                            ("rcm", True, "fused"), ("spatial", False, "fused")])
def test_config0_mesh_dw(renumber, host_setup, increment):
    """48^3, 3 levels, 10 V-cycles, Mach 0.5, 3 degrees."""
    mesh = mgcfd.HostMesh.generate(48, 3, 1234)
    mach, aoa, cycles = 0.5, 3.0, 10
    ref = _oracle(mesh.levels(), mach, aoa, cycles)
    s = mgcfd.Solver(mesh, mach, aoa, precision="dw", renumber=renumber, host_setup=host_setup, increment=increment)
    s.run(cycles)
    assert s.synchronize() == 0
    _check(s, ref, 3, mach, aoa)
    s.close()


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("*.npz")))
@pytest.mark.parametrize("increment", ["atomic", "fused"])
def test_dw_matches_reference_fixture(name, increment):
    import json
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    mesh = mgcfd.HostMesh.generate(meta["n"], meta["levels"], meta["seed"])
    s = mgcfd.Solver(mesh, meta["mach"], meta["aoa"], precision="dw", increment=increment)
    s.run(meta["cycles"])
    assert s.synchronize() == 0
    x0 = np.array(mgcfd.freestream(meta["mach"], meta["aoa"]).ff_variable[:])
    for l in range(meta["levels"]):
        var = s.fetch(l)
        if meta["full"]:
            ref = z[f"variables_L{l}"]
        else:
            var, ref = var[z[f"rows_L{l}"]], z[f"variables_rows_L{l}"]
        assert state_error(var, ref) <= STATE_TOL, (l, state_error(var, ref))
        assert delta_error(var, ref, x0) <= DELTA_TOL
    s.close()


def test_irregular_mesh_dw():
    levels = irregular_levels(3000, 3, seed=11)
    mach, aoa, cycles = 0.6, 2.0, 3
    ref = _oracle(levels, mach, aoa, cycles)
    for opts in (dict(increment="atomic"), dict(increment="gather", renumber="rcm"), dict(increment="fused"),
                 dict(increment="fused", renumber="none", host_setup=True)):
        s = mgcfd.Solver(levels, mach, aoa, precision="dw", **opts)
        s.run(cycles)
        assert s.synchronize() == 0
        _check(s, ref, 3, mach, aoa)
        s.close()


@pytest.mark.parametrize("increment", ["gather", "fused"])
def test_dw_batch_equals_solo_and_oracle(increment):
    meshes = [mgcfd.HostMesh.generate(n, 3, 50 + n) for n in (10, 17, 23)]
    machs, aoas, cycles = [0.4, 0.6, 0.75], [1.0, 3.0, 5.0], 3
    b = mgcfd.Batch(meshes, machs, aoas, precision="dw", increment=increment)
    b.run(cycles)
    assert b.synchronize() == 0
    for m, (mesh, mach, aoa) in enumerate(zip(meshes, machs, aoas)):
        s = mgcfd.Solver(mesh, mach, aoa, precision="dw", increment=increment)
        s.run(cycles)
        assert s.synchronize() == 0
        ref = _oracle(mesh.levels(), mach, aoa, cycles)
        for l in range(3):
            np.testing.assert_array_equal(b.fetch_mesh(m, l), s.fetch(l))  # deterministic increments
        _check(s, ref, 3, mach, aoa)
        s.close()
    b.close()


@pytest.mark.parametrize("increment", ["gather", "fused"])
def test_dw_repeats_bitwise(increment):
    mesh = mgcfd.HostMesh.generate(20, 3, 9)
    out = []
    for _ in range(2):
        s = mgcfd.Solver(mesh, 0.7, 2.0, precision="dw", increment=increment)
        s.run(3)
        assert s.synchronize() == 0
        out.append([s.fetch(l) for l in range(3)])
        s.close()
    for x, y in zip(*out):
        np.testing.assert_array_equal(x, y)


def test_dw_refuses_coloured_and_mixed_stage_variants():
    mesh = mgcfd.HostMesh.generate(8, 2, 1)
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.Solver(mesh, 0.5, 3.0, precision="dw", increment="coloured")
    for variant in ("stage_neighbour_ids", "edge_parallel_stage"):
        with pytest.raises(mgcfd._lib.MgcfdError):
            mgcfd.Solver(mesh, 0.5, 3.0, precision="dw", increment="fused", **{variant: True})


@pytest.mark.parametrize("increment", ["atomic", "fused"])
def test_dw_nan_weight_reports_bad_values(increment):
    mesh = mgcfd.HostMesh.generate(8, 2, 3)
    bad = [mgcfd.Level(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in L.__dict__.items()
                          if k != "owner"}) for L in mesh.levels()]
    bad[0].edge_weights[0, :] = np.nan  # a NaN weight splits into a NaN pair and poisons two nodes' fluxes
    s = mgcfd.Solver(bad, 0.5, 3.0, precision="dw", increment=increment)
    s.run(2)
    assert s.synchronize() == mgcfd._lib.ERR_BAD_VALUES
    with pytest.raises(mgcfd._lib.MgcfdError):
        s.run(1)


def test_dw_refuses_weights_outside_its_range():
    """The pairs have binary32's exponent range: edge weights below 2^-70 (or
    at and above 2^70) are refused at set-up; FP64 takes the same mesh."""
    mesh = mgcfd.HostMesh.generate(8, 2, 3)
    scaled = [mgcfd.Level(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in L.__dict__.items()
                             if k != "owner"}) for L in mesh.levels()]
    scaled[1].edge_weights *= 2.0 ** -80
    with pytest.raises(mgcfd._lib.MgcfdError, match="range"):
        mgcfd.Solver(scaled, 0.5, 3.0, precision="dw")
    s = mgcfd.Solver(scaled, 0.5, 3.0)
    s.close()
    mgcfd.Solver(mesh, 0.5, 3.0, precision="dw").close()  # the unscaled mesh is fine
