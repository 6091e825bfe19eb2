"""CUDA path against the oracle and the reference's golden outputs, through
the C ABI.  Tolerances:
  * residual B: 1e-12 of the step's initial residual norm ||B_0|| (B is a sum
    of element terms of size ~||B_0|| that cancel towards convergence, so its
    rounding error does not shrink with it);
  * float matrix: 2e-6 of the row's largest entry (a few float ulps: the GPU
    accumulates element contributions in colour order and contracts products);
    5e-5 for the mixed path, whose Jacobian is computed in FP32;
  * Krylov solution: the true relative residual ||B - A X|| / ||B|| below
    1e-7 (solver target 1e-8); X within 1e-6 of max|X| of the reference's
    solution when the preconditioner is the reference's (float ILU), 1e-4 when
    it differs (FP64 or mixed), since two runs that both stop at a 1e-8
    residual can differ by the condition number times that."""

import numpy as np
import pytest

import golden_io
import oracle

pytestmark = pytest.mark.gpu

FIXTURES = ["channel_tiny.npz", "channel_1000.npz"]


def _rowscale(st, A):
    ptr = st["ptr"]
    s = np.maximum.reduceat(np.abs(A.astype(np.float64)), ptr[:-1])
    return np.repeat(s, np.diff(ptr))


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_assembly_matches_reference(name, prec):
    g = golden_io.load(name)
    for k in [int(v) for v in g["keep"]]:
        st = golden_io.state(g, k)
        ctx = golden_io.gpu_context(st, prec)
        A, B = ctx.assemble()
        ref_A = st["A"].astype(np.float64)
        scale = _rowscale(st, st["A"])
        tolA = 2e-6 if prec != 2 else 5e-5
        assert np.max(np.abs(A - ref_A) / scale) < tolA
        assert np.max(np.abs(B - st["B"])) <= 1e-12 * g["scales"][0]
        ctx.close()


@pytest.mark.parametrize("name", FIXTURES)
def test_scale_and_factor_match_oracle(name):
    g = golden_io.load(name)
    k = int(g["keep"][0])
    st = golden_io.state(g, k)
    ctx = golden_io.gpu_context(st, 1)
    ctx.load_system(st["A"], st["B"])
    s = ctx.scale()
    assert abs(s - g["scales"][k]) <= 1e-13 * g["scales"][k]
    A = st["A"].copy()
    B = st["B"].copy()
    oracle.scale_l2(st["ptr"], A, B)
    rc, ILU = oracle.ilu0_factor(st["ptr"], st["index"], A)
    LU = ctx.ilu0_factor(want_LU=True)
    # same operations in the same order per entry: bit-identical factors
    assert np.array_equal(LU, ILU)
    ctx.close()


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("prec", [0, 1])
def test_spmv_ilu_apply_match_oracle(name, prec):
    g = golden_io.load(name)
    st = golden_io.state(g, int(g["keep"][0]))
    ctx = golden_io.gpu_context(st, prec)
    A = st["A"].astype(np.float32 if prec == 1 else np.float64)
    ctx.load_system(A, st["B"])
    rng = np.random.default_rng(3)
    x = rng.standard_normal(ctx.neq)
    r = ctx.spmv(x)
    r_ref = oracle.spmv(st["ptr"], st["index"], A, x)
    assert np.max(np.abs(r - r_ref)) <= 1e-12 * np.max(np.abs(r_ref))
    ctx.ilu0_factor()
    _, ILU = oracle.ilu0_factor(st["ptr"], st["index"], A)
    y = ctx.ilu0_apply(x)
    y_ref = oracle.ilu0_solve(st["ptr"], st["index"], ILU, x)
    if prec == 1:
        # reference storage: the reference's summation order, separately rounded -- bit-identical
        assert np.array_equal(y, y_ref)
    elif prec == 0:
        # FP64: the reference's order with fused multiply-adds
        assert np.max(np.abs(y - y_ref)) <= 1e-13 * np.max(np.abs(y_ref))
    else:
        assert np.max(np.abs(y - y_ref)) <= 1e-9 * np.max(np.abs(y_ref))
    ctx.close()


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_bicgstab_matches_reference(name, prec):
    g = golden_io.load(name)
    for k in [int(v) for v in g["keep"]]:
        st = golden_io.state(g, k)
        ctx = golden_io.gpu_context(st, prec)
        ctx.load_system(st["A"], st["B"])
        ctx.scale()
        ctx.ilu0_factor()
        ok, X, its, acc = ctx.bicgstab(1000, 1e-8)
        assert ok
        # the context scales in its own storage precision (float division for
        # float storage, CRSMat.cpp:340; double for the FP64 path)
        A = st["A"].astype(np.float64 if prec == 0 else np.float32)
        B = st["B"].copy()
        oracle.scale_l2(st["ptr"], A, B)
        r = B - oracle.spmv(st["ptr"], st["index"], A, X)
        assert np.linalg.norm(r) <= 1e-7 * np.linalg.norm(B)
        ref = st["X"]
        tol = 1e-6 if prec == 1 else 1e-4
        assert np.max(np.abs(X - ref)) <= tol * np.max(np.abs(ref))
        if prec == 1:
            assert abs(its - int(g["iters"][k])) <= max(3, int(0.15 * g["iters"][k]))
        ctx.close()


def test_solve_and_update_chain_channel_tiny():
    """Every Newton iteration of the small channel through rg_solve and
    rg_newton_update, fed the reference's boundary data per iteration; the
    state after each update matches the reference's next state."""
    g = golden_io.load("channel_tiny.npz")
    n = int(g["n_newton"])
    st0 = golden_io.state(g, 0)
    ctx = golden_io.gpu_context(st0, 1)
    ctx.set_update_lists(st0["model_nodes"], st0["region_nodes"], st0["zor"])
    for k in range(n):
        st = golden_io.state(g, k)
        golden_io.load_iteration(ctx, st)
        ok, X, scale, its = ctx.solve(1000, 1e-8)
        assert ok
        assert abs(scale - g["scales"][k]) <= 1e-12 * g["scales"][0]
        ctx.newton_update(relax_method=2, max_delta_uv=0.5, max_delta_s=0.5, max_us=100.0,
                          dry_limit=0.01, dryrew_method=2)
        nxt = golden_io.state(g, k + 1 if k + 1 < n else "final")
        got = ctx.get_state()
        for v in ("U", "V", "S"):
            ref = nxt[v]
            err = np.max(np.abs(got[v] - ref))
            assert err <= 1e-6 * max(1.0, np.max(np.abs(ref))), (k, v, err)
    ctx.close()


def test_friction_matches_reference():
    g = golden_io.load("channel_tiny.npz")
    st = golden_io.state(g, 1)
    ctx = golden_io.gpu_context(st, 0)
    ctx.set_update_lists(st["model_nodes"], st["region_nodes"], st["zor"])
    ctx.set_friction(st["region_n"], st["region_areafact"])
    cf = ctx.friction()
    assert np.max(np.abs(cf - st["cf"])) <= 1e-14 * np.max(np.abs(st["cf"]))
    ctx.close()


def _random_system(n, seed):
    """Structurally symmetric, diagonally dominant sparse system in the
    reference's row layout (diagonal first, other columns shuffled)."""
    rng = np.random.default_rng(seed)
    cols = [set([i]) for i in range(n)]
    for i in range(n):
        for j in rng.integers(0, n, size=min(n, 6)):
            if j != i and abs(int(j) - i) < 40:
                cols[i].add(int(j))
                cols[int(j)].add(i)
    width, index, A = [], [], []
    for i in range(n):
        others = [c for c in cols[i] if c != i]
        rng.shuffle(others)
        row = [i] + others
        width.append(len(row))
        index.extend(row)
        A.extend([len(row) * 2.0 + rng.random()] + list(rng.uniform(-1, 1, len(others))))
    width = np.array(width, np.int32)
    ptr = np.zeros(n + 1, np.int64)
    ptr[1:] = np.cumsum(width)
    return width, np.array(index, np.int32), ptr, np.array(A, np.float32), rng.standard_normal(n)


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 257, 1001])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_ragged_sizes_linear_algebra(n, prec):
    """Odd and tiny equation counts (a half-filled last warp in every kernel)."""
    g = golden_io.load("channel_tiny.npz")
    st = golden_io.state(g, 0)
    ctx = golden_io.gpu_context(st, prec)
    width, index, ptr, A, b = _random_system(n, n)
    ctx.set_pattern(width, index, -np.ones((len(st["x"]), 3), np.int32))
    A_in = A.astype(np.float64) if prec == 0 else A
    ctx.load_system(A_in, b)
    x = np.linspace(-1.0, 1.0, n)
    r = ctx.spmv(x)
    r_ref = oracle.spmv(ptr, index, A_in, x)
    assert np.max(np.abs(r - r_ref)) <= 1e-12 * max(1.0, np.max(np.abs(r_ref)))
    ctx.ilu0_factor()
    _, ILU = oracle.ilu0_factor(ptr, index, A_in)
    y = ctx.ilu0_apply(x)
    y_ref = oracle.ilu0_solve(ptr, index, ILU, x)
    assert np.max(np.abs(y - y_ref)) <= 1e-5 * max(1.0, np.max(np.abs(y_ref)))
    ok, X, its, _ = ctx.bicgstab(500, 1e-8)
    assert ok
    res = b - oracle.spmv(ptr, index, A_in, X)
    assert np.linalg.norm(res) <= 1e-6 * np.linalg.norm(b)
    ctx.close()
