"""The oracle restatement (oracle/rg_oracle.c) against the reference's own
outputs recorded in tests/golden/ (bit-exact: same arithmetic, same order)."""

import ctypes as C

import numpy as np
import pytest

import golden_io
import oracle

FIXTURES = ["channel_tiny.npz", "channel_1000.npz"]


def _iters(g):
    return [int(k) for k in g["keep"]]


@pytest.mark.parametrize("name", FIXTURES)
def test_assembly_bit_exact(name):
    g = golden_io.load(name)
    for k in _iters(g):
        st = golden_io.state(g, k)
        m = golden_io.oracle_model(st)
        A, B = oracle.assemble(m, st["ptr"], st["index"], np.float32)
        assert np.array_equal(A, st["A"]), f"A differs at iteration {k}"
        assert np.array_equal(B, st["B"]), f"B differs at iteration {k}"


@pytest.mark.parametrize("name", FIXTURES)
def test_scale_factor_bicgstab_bit_exact(name):
    g = golden_io.load(name)
    for k in _iters(g):
        st = golden_io.state(g, k)
        A = st["A"].copy()
        B = st["B"].copy()
        s = oracle.scale_l2(st["ptr"], A, B)
        assert s == g["scales"][k]
        rc, ILU = oracle.ilu0_factor(st["ptr"], st["index"], A)
        assert rc == 0
        ok, X, its, _ = oracle.bicgstab(st["ptr"], st["index"], A, ILU, B)
        assert ok and its == g["iters"][k]
        assert np.array_equal(X, st["X"])


class _Cfg(C.Structure):
    _fields_ = [("np_model", C.c_int), ("model_nodes", C.c_void_p), ("ne_region", C.c_int),
                ("region_nodes", C.c_void_p), ("region_flag", C.c_void_p), ("maxDeltaUV", C.c_double),
                ("maxDeltaS", C.c_double), ("maxUs", C.c_double), ("dryLimit", C.c_double),
                ("relaxMethod", C.c_int), ("dryRewMethod", C.c_int)]


def oracle_update(st, X):
    P = oracle._p
    mn = np.ascontiguousarray(st["model_nodes"], np.int32)
    rn = np.ascontiguousarray(st["region_nodes"], np.int32)
    rf = np.ascontiguousarray(st["region_flag"], np.int32)
    cfg = _Cfg(len(mn), P(mn), len(rf), P(rn), P(rf), 0.5, 0.5, 100.0, 0.01, 2, 2)
    U, V, S, z = (st[k].copy() for k in ("U", "V", "S", "z"))
    eqno = np.ascontiguousarray(st["eqno"])
    rot = np.ascontiguousarray(st["rot4"])
    stats = np.zeros(9)
    oracle.lib().orc_newton_update(C.byref(cfg), P(eqno), P(np.ascontiguousarray(st["flag"], np.int32)),
                                   P(rot), P(np.ascontiguousarray(X)), P(U), P(V), P(S), P(z),
                                   P(np.ascontiguousarray(st["zor"])), C.c_double(float(st["hmin"])), P(stats))
    return U, V, S, z, stats


def test_newton_update_bit_exact():
    g = golden_io.load("channel_tiny.npz")
    n = int(g["n_newton"])
    for k in range(n):
        st = golden_io.state(g, k)
        nxt = golden_io.state(g, k + 1 if k + 1 < n else "final")
        U, V, S, z, _ = oracle_update(st, st["X"])
        for a, b in ((U, "U"), (V, "V"), (S, "S"), (z, "z")):
            assert np.array_equal(a, nxt[b]), f"{b} differs after iteration {k}"


def test_friction_bit_exact():
    g = golden_io.load("channel_tiny.npz")
    n = int(g["n_newton"])
    for k in range(1, n):
        st = golden_io.state(g, k)
        rn = np.ascontiguousarray(st["region_nodes"], np.int32)
        nnd = np.where(rn[:, 3] >= 0, 6, 3).astype(np.int32)
        cf = np.zeros(len(st["x"]))
        P = oracle._p
        oracle.lib().orc_friction(C.c_int(len(cf)), C.c_int(len(rn)), P(rn), P(nnd),
                                  P(np.ascontiguousarray(st["region_n"])),
                                  P(np.ascontiguousarray(st["region_areafact"])), P(st["U"]), P(st["V"]),
                                  P(st["S"]), P(st["z"]), C.c_double(float(st["hmin"])),
                                  C.c_double(float(st["g"])), P(cf))
        assert np.array_equal(cf, st["cf"])


def test_zero_pivot_repair_runs():
    """A planted zero pivot is repaired by adding the row with the largest
    entry in the pivot column (Preco_ilu0.cpp:95-133)."""
    g = golden_io.load("channel_tiny.npz")
    st = golden_io.state(g, 0)
    A = st["A"].astype(np.float64).copy()
    ptr, idx = st["ptr"], st["index"]
    A[ptr[5]] = 0.0                      # diagonal of equation 5
    rc, ILU = oracle.ilu0_factor(ptr, idx, A)
    assert rc == 0
    assert abs(ILU[ptr[5]]) > 1e-20


@pytest.mark.parametrize("name", ["meander_tiny.npz", "braided_small.npz"])
def test_unsteady_dry_wet_assembly_and_solve_bit_exact(name):
    """Unsteady flow with dry flood plains (meander) and with the braided river's dry bars
    and anabranch banks (a 200 m window at the benchmark's resolution): the oracle
    reproduces the reference's assembled system and correction at the kept iterations."""
    g = golden_io.load(name)
    for k in [int(v) for v in g["keep"]]:
        st = golden_io.state(g, k)
        m = golden_io.oracle_model(st)
        A, B = oracle.assemble(m, st["ptr"], st["index"], np.float32)
        assert np.array_equal(A, st["A"]) and np.array_equal(B, st["B"])
        s = oracle.scale_l2(st["ptr"], A, B)
        assert s == g["scales"][k]
        rc, ILU = oracle.ilu0_factor(st["ptr"], st["index"], A)
        ok, X, its, _ = oracle.bicgstab(st["ptr"], st["index"], A, ILU, B)
        assert its == g["iters"][k] and np.array_equal(X, st["X"])


@pytest.mark.parametrize("name", ["channel_tiny.npz", "channel_1000.npz", "meander_tiny.npz", "braided_small.npz"])
def test_oracle_pattern_matches_reference(name):
    """The oracle's CRS pattern builder reproduces EQS::SetIndexMat's width and index
    arrays bit for bit from the reference's own equation numbers and element list."""
    g = golden_io.load(name)
    st = golden_io.state(g, 0)
    six = st["elem_nnd"] == 6
    ptr, idx = oracle.pattern(len(st["x"]), st["elem_nodes"][six], st["eqno"], len(st["width"]))
    assert np.array_equal(np.diff(ptr), st["width"])
    assert np.array_equal(idx, st["index"])
