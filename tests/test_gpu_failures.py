"""Failure paths on the GPU, made on the host (no fault, trap or hang of the GPU):

* a planted zero pivot: the level-scheduled factorisation flags it and the
  dependency-driven kernel repairs it as PRECO_ILU0::Factor does
  (Preco_ilu0.cpp:95-138) -- factors bit-identical to the oracle's repair;
* a NaN planted in the right-hand side: BiCGStab stops with RG_ERR_NONFINITE
  instead of iterating (the reference has no such test; Bicgstab.cpp:174-199
  only restarts on a vanishing (r0, r));
* a polling limit short enough that the bounded device waits of the
  dependency-driven triangular solves give up: RG_ERR_DEVICE_WAIT with the
  kernel and rows in the message, and the same context then solves correctly;
* a deliberately bad warm start (the water level 1 m too high) is rejected:
  the step reaches the plain start's state with the plain start's Newton count.
"""

import numpy as np
import pytest

import golden_io
import oracle
from rismo2d_gb300 import _lib, meshgen

pytestmark = pytest.mark.gpu


def test_planted_zero_pivot_repaired_like_the_oracle():
    g = golden_io.load("channel_tiny.npz")
    st = golden_io.state(g, 0)
    ptr, idx = st["ptr"], st["index"]
    A = st["A"].astype(np.float32).copy()
    A[ptr[5]] = 0.0                                  # diagonal of equation 5
    rc, LU_ref = oracle.ilu0_factor(ptr, idx, A)
    assert rc == 0 and abs(LU_ref[ptr[5]]) > 1e-20  # the oracle repaired it
    ctx = golden_io.gpu_context(st, _lib.PREC_REF32)
    ctx.load_system(A, st["B"])
    LU = ctx.ilu0_factor(want_LU=True)
    assert np.array_equal(LU, LU_ref)
    ctx.close()


@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_nan_in_rhs_reports_nonfinite(prec):
    g = golden_io.load("channel_1000.npz")
    st = golden_io.state(g, 0)
    ctx = golden_io.gpu_context(st, prec)
    B = st["B"].copy()
    B[17] = np.nan
    ctx.load_system(st["A"], B)
    ctx.ilu0_factor()
    with pytest.raises(_lib.RgError) as ei:
        ctx.bicgstab(1000, 1e-8)
    assert ei.value.status == _lib.RG_ERR_NONFINITE
    # the context recovers: the clean system solves
    ctx.load_system(st["A"], st["B"])
    ctx.scale()
    ctx.ilu0_factor()
    ok, X, its, acc = ctx.bicgstab(1000, 1e-8)
    assert ok and np.all(np.isfinite(X))
    ctx.close()


def test_device_wait_limit_runs_out_and_context_recovers(monkeypatch):
    # the dependency-driven triangular solves (the ones with polled waits)
    monkeypatch.setenv("RG_NO_WAVE", "1")
    g = golden_io.load("channel_1000.npz")
    st = golden_io.state(g, 0)
    ctx = golden_io.gpu_context(st, _lib.PREC_REF32)
    ctx.load_system(st["A"], st["B"])
    LU = ctx.ilu0_factor(want_LU=True)
    b = np.random.default_rng(3).standard_normal(len(st["B"]))
    ref = oracle.ilu0_solve(st["ptr"], st["index"], LU, b)
    ctx.set_wait_limit(1)                              # every wait gives up after one poll
    with pytest.raises(_lib.RgError) as ei:
        for _ in range(20):                            # a row that must wait exists in every solve
            ctx.ilu0_apply(b)
    assert ei.value.status == _lib.RG_ERR_DEVICE_WAIT
    assert "waited for" in str(ei.value)
    ctx.set_wait_limit(0)
    x = ctx.ilu0_apply(b)
    # the dependency-driven solves sum in their own order: equal to rounding
    assert np.max(np.abs(x - ref)) <= 1e-12 * np.max(np.abs(ref))
    ctx.close()


def test_bad_warm_start_is_rejected():
    from golden.make_golden import MEANDER_TINY, meander_hydrograph
    from rismo2d_gb300.sim import RG_CRIT_RESIDUAL, Params, Simulation
    mesh = meshgen.meander(**MEANDER_TINY)
    runs = {}
    for mode in ("plain", "bad"):
        sim = Simulation(mesh, Params(), hydrograph=meander_hydrograph(), precision=_lib.PREC_MIXED)
        sim.set_state(mesh.U0, mesh.V0, mesh.S0)
        sim.step(0.0, 10.0, criterion=RG_CRIT_RESIDUAL, residual_tol=1e-8)
        if mode == "bad":
            s = sim.get_state()
            sim.set_warm_start(s["U"], s["V"], s["S"] + 1.0)
        rep = sim.step(10.0, 10.0, criterion=RG_CRIT_RESIDUAL, residual_tol=1e-8)
        runs[mode] = (rep, sim.get_state())
        sim.close()
    rep_b, st_b = runs["bad"]
    rep_p, st_p = runs["plain"]
    assert rep_b["warm_start"] == 0 and rep_b["residual_warm"] > rep_b["residual_first"]
    assert rep_b["newton_iterations"] == rep_p["newton_iterations"]
    for v in ("U", "V", "S"):
        scale = max(1.0, float(np.max(np.abs(st_p[v]))))
        assert np.max(np.abs(st_b[v] - st_p[v])) <= 1e-12 * scale, v
    assert np.array_equal(st_b["flag"], st_p["flag"])
