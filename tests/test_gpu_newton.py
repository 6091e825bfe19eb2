"""Whole time steps through the standalone stepper (rg_sim_step) against the
reference's converged states.  Tolerances follow the acceptance bar: H, U, V
within 1e-6 of the field's maximum for the FP64 and reference-precision paths,
1e-5 for the mixed path; dry/wet flags identical."""

import numpy as np
import pytest

import golden_io
from golden.make_golden import MEANDER_TINY, meander_hydrograph
from rismo2d_gb300 import _lib, meshgen
from rismo2d_gb300.sim import RG_CRIT_CORRECTION, RG_CRIT_RESIDUAL, Params, Simulation

pytestmark = pytest.mark.gpu

CHANNELS = {
    "channel_tiny.npz": dict(nx=6, ny=2, length=120.0, width=40.0, nbumps=3, Q=40.0),
    "channel_1000.npz": dict(),
}
TOL = {_lib.PREC_FP64: 1e-6, _lib.PREC_REF32: 1e-6, _lib.PREC_MIXED: 1e-5}
DRY = 64


def _compare(got, ref_U, ref_V, ref_S, ref_z, tol):
    H, Hr = got["S"] - got["z"], ref_S - ref_z
    for a, b in ((got["U"], ref_U), (got["V"], ref_V), (H, Hr)):
        scale = max(np.max(np.abs(b)), 1e-3)
        assert np.max(np.abs(a - b)) <= tol * scale, np.max(np.abs(a - b)) / scale


@pytest.mark.parametrize("name", list(CHANNELS))
@pytest.mark.parametrize("prec", [0, 1, 2])
@pytest.mark.parametrize("criterion", [RG_CRIT_CORRECTION, RG_CRIT_RESIDUAL])
def test_steady_channel_step(name, prec, criterion):
    g = golden_io.load(name)
    mesh = meshgen.channel(**CHANNELS[name])
    sim = Simulation(mesh, Params(), precision=prec)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    rep = sim.step(0.0, 3600.0, steady=True, criterion=criterion, residual_tol=1e-8)
    assert rep["converged"]
    if criterion == RG_CRIT_RESIDUAL:
        assert rep["residual_ratio"] <= 1e-8
    got = sim.get_state()
    _compare(got, g["final_U"], g["final_V"], g["final_S"], g["final_z"], TOL[prec])
    assert np.array_equal(got["flag"] & DRY, g["final_flag"] & DRY)
    sim.close()


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_unsteady_meander_three_steps(prec):
    """Unsteady flow with dry flood plains and dry/rewet every 10 iterations;
    40 Newton iterations per step as the reference ran them (the mixed path
    within its 1e-5 bar)."""
    g = golden_io.load("meander_tiny.npz")
    mesh = meshgen.meander(**MEANDER_TINY)
    sim = Simulation(mesh, Params(max_newton=40), hydrograph=meander_hydrograph(), precision=prec)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    for i in range(int(g["n_steps"])):
        sim.step(10.0 * i, 10.0, steady=False, criterion=RG_CRIT_CORRECTION)
        got = sim.get_state()
        assert np.array_equal(got["flag"] & DRY, g[f"step{i}_flag"] & DRY), f"dry flags differ after step {i}"
        _compare(got, g[f"step{i}_U"], g[f"step{i}_V"], g[f"step{i}_S"], g[f"step{i}_z"], TOL[prec])
    sim.close()


@pytest.mark.parametrize("name", list(CHANNELS))
@pytest.mark.parametrize("prec", [0, 2])
@pytest.mark.parametrize("forcing,reuse", [(0.5, 64), (0.1, 0), (0.0, 1000)])
def test_steady_channel_inexact_newton(name, prec, forcing, reuse):
    """Inexact Newton (BiCGStab to the forcing term) and reused ILU(0) factors
    change only the path to the solution.  From the cold start of a steady run
    ||B_0|| is large, so the step is iterated to ||B||/||B_0|| <= 1e-11 (the
    final state then no longer depends on the path) and must reach the
    reference's converged state within the acceptance tolerance."""
    g = golden_io.load(name)
    mesh = meshgen.channel(**CHANNELS[name])
    sim = Simulation(mesh, Params(max_newton=400), precision=prec)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    rep = sim.step(0.0, 3600.0, steady=True, criterion=RG_CRIT_RESIDUAL, residual_tol=1e-11,
                   linear_forcing=forcing, ilu_reuse=reuse)
    assert rep["converged"] and rep["residual_ratio"] <= 1e-11
    got = sim.get_state()
    _compare(got, g["final_U"], g["final_V"], g["final_S"], g["final_z"], TOL[prec])
    assert np.array_equal(got["flag"] & DRY, g["final_flag"] & DRY)
    stages = sim.stage_ms()
    assert stages["krylov"] > 0.0 and stages["assemble"] > 0.0
    sim.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_lake_at_rest_on_the_gpu(prec):
    """Known answer: a lake at rest over a bumpy bed (no flow, no inflow, outlet at the lake
    level) is an exact solution -- the GPU's first Newton residual vanishes to rounding and
    the step leaves the lake as it was."""
    from rismo2d_gb300 import deck
    mesh = meshgen.channel(nx=20, ny=4, length=400.0, width=50.0, nbumps=6, seed=5, Q=10.0)
    S_lake = float(np.max(mesh.z)) + 2.0
    bcs = [("QINLET", 1, [(0.0, S_lake)]), ("OUTLET", 2, [(S_lake,)])]
    sim = Simulation(mesh, Params(max_newton=2), precision=prec, line_bcs=bcs)
    zero = np.zeros(mesh.np)
    sim.set_state(zero, zero, np.full(mesh.np, S_lake))
    rep = sim.step(0.0, 3600.0, steady=True, criterion=RG_CRIT_CORRECTION)
    H = S_lake - deck.bed_zor(mesh)
    scale = 9.81 * float(np.max(H)) ** 2 * 400.0
    assert rep["residual_first"] <= 1e-10 * scale
    got = sim.get_state()
    assert np.max(np.abs(got["U"])) <= 1e-9 and np.max(np.abs(got["V"])) <= 1e-9
    assert np.max(np.abs(got["S"] - S_lake)) <= 1e-9
    sim.close()
