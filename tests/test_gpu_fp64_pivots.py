"""ILU(0) factorisation of the mixed precision path with FP64 near-dry rows.

The factorisation follows PRECO_ILU0::Factor (Preco_ilu0.cpp:160-185): for a
row, its L entries in column order, multiplier = -entry / pivot of the pivot
row, then the pivot row's U entries subtracted into the row's pattern.  In the
mixed path the rows of nodes shallower than the FP64-pivot depth run this in
double (from the FP32 pivot rows) and are stored in FP32; all other rows run in
FP32.  The NumPy statement below does exactly that, row by row, and must match
the GPU factors bit for bit -- with no rows, half the rows and all rows in FP64.
With no FP64 rows it is the oracle's FP32 factorisation (checked on the CPU)."""

import numpy as np
import pytest

import golden_io
import oracle
from rismo2d_gb300 import _lib


def factor_statement(ptr, idx, A, fp64):
    n = len(ptr) - 1
    LU = A.astype(np.float32).copy()
    pos = [dict((int(c), int(ptr[i] + k)) for k, c in enumerate(idx[ptr[i]:ptr[i + 1]])) for i in range(n)]
    for i in range(n):
        b, e = int(ptr[i]), int(ptr[i + 1])
        row = LU[b:e].astype(np.float64) if fp64[i] else LU[b:e].copy()
        for kcol in sorted(int(c) for c in idx[b + 1:e] if c < i):
            pk = pos[i][kcol] - b
            piv = LU[ptr[kcol]]
            f = -row[pk] / np.float64(piv) if fp64[i] else np.float32(-row[pk]) / piv
            row[pk] = f
            for t in range(int(ptr[kcol]) + 1, int(ptr[kcol + 1])):
                c = int(idx[t])
                if c > kcol and c in pos[i]:
                    q = pos[i][c] - b
                    if fp64[i]:
                        row[q] = row[q] + f * np.float64(LU[t])
                    else:
                        row[q] = np.float32(row[q] + np.float32(f * LU[t]))
        LU[b:e] = row.astype(np.float32)
    return LU


def test_statement_without_fp64_rows_is_the_oracle():
    g = golden_io.load("meander_tiny.npz")
    st = golden_io.state(g, 0)
    ref = factor_statement(st["ptr"], st["index"], st["A"], np.zeros(len(st["width"]), bool))
    _rc, LU = oracle.ilu0_factor(st["ptr"], st["index"], st["A"].astype(np.float32))
    assert np.array_equal(ref, LU)


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["none", "half", "all"])
def test_mixed_factor_with_fp64_rows_matches_statement(which):
    g = golden_io.load("meander_tiny.npz")
    st = golden_io.state(g, 0)
    H = st["S"] - st["z"]
    wet = st["eqno"][:, 0] >= 0
    depth = {"none": 0.0, "half": float(np.median(H[wet])), "all": 1e9}[which]
    ctx = golden_io.gpu_context(st, _lib.PREC_MIXED)
    ctx.set_fp64_pivots(depth)
    ctx.load_system(st["A"], st["B"])
    LU = ctx.ilu0_factor(want_LU=True)
    n = len(st["width"])
    shallow = H < depth
    fp64 = np.zeros(n, bool)
    for j in range(3):
        e = st["eqno"][:, j]
        ok = e >= 0
        fp64[e[ok]] = shallow[ok]
    if which == "half":
        assert 0 < fp64.sum() < n          # a mix of FP64 and FP32 rows
    ref = factor_statement(st["ptr"], st["index"], st["A"], fp64)
    assert np.array_equal(LU, ref), int(np.sum(LU != ref))
    ctx.close()
