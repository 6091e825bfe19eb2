"""Parity on the benchmark-size meander (200,028 six-node triangles, 402,747
nodes, dry flood plains, dt = 10 s, hydrograph Q(t) = 300 + 500 sin^2(pi t /
7200)) against the compiled reference's own end states of five unsteady time
steps (tests/golden/meander200k.npz, made by tests/golden/make_golden_large.py).

The fixture holds U, V, S, z at 60,000 seeded wet nodes and the dry flag of
every node.  Acceptance bar: H, U, V within 1e-6 of the field's maximum for
the FP64 path, 1e-5 for the mixed path (with every option the benchmark
uses), dry/wet flags of all nodes bit-identical."""

import numpy as np
import pytest

import golden_io
from rismo2d_gb300 import _lib, meshgen
from rismo2d_gb300.sim import RG_CRIT_CORRECTION, RG_CRIT_RESIDUAL, Params, Simulation

pytestmark = pytest.mark.gpu

DRY = 64
DT = 10.0


def _check(got, g, k, tol):
    s = g["sample"]
    H, Hr = got["S"][s] - got["z"][s], g[f"S_{k}"] - g[f"z_{k}"]
    errs = {}
    for name, a, b in (("U", got["U"][s], g[f"U_{k}"]), ("V", got["V"][s], g[f"V_{k}"]), ("H", H, Hr)):
        scale = max(float(np.max(np.abs(b))), 1e-3)
        errs[name] = float(np.max(np.abs(a - b))) / scale
    dry = np.unpackbits(g[f"dry_{k}"])[: int(g["np"])].astype(bool)
    assert np.array_equal((got["flag"] & DRY) != 0, dry), f"dry flags differ after step {k}"
    assert max(errs.values()) <= tol, (k, errs)
    return errs


def test_fp64_steps_match_reference():
    """The reference's algorithm on the GPU in FP64, stopped by the reference's own
    correction test, reproduces its five end states and dry flags."""
    g = golden_io.load("meander200k.npz")
    mesh = meshgen.meander()
    sim = Simulation(mesh, Params(), hydrograph=meshgen.sin2_hydrograph(), precision=_lib.PREC_FP64)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    for k in range(int(g["steps"])):
        rep = sim.step(DT * k, DT, criterion=RG_CRIT_CORRECTION)
        _check(sim.get_state(), g, k, 1e-6)
        # same algorithm: the Newton count follows the reference's (rounding may shift the
        # last correction across convUV)
        assert abs(rep["newton_iterations"] - int(g["newton"][k])) <= 3, (rep["newton_iterations"], g["newton"][k])
    sim.close()


def test_mixed_benchmark_options_match_reference():
    """The benchmark's arm -- FP32 Krylov / ILU(0) in FP64 refinement, inexact Newton
    (forcing 0.5), ILU(0) reuse 64, the friction-depth Jacobian, the learned warm start
    -- iterated to ||B||/||B_0|| <= 1e-8 ends every step at the reference's state."""
    from rismo2d_gb300 import warmstart as ws
    g = golden_io.load("meander200k.npz")
    mesh = meshgen.meander()
    kw = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=1e-8, linear_forcing=0.5, ilu_reuse=64,
              friction_jacobian=True)
    # a small network trained on another hydrograph (the prediction only has to be usable)
    train_hyd = meshgen.sin2_hydrograph(Q0=250.0, dQ=700.0, period=5400.0)
    sim = Simulation(mesh, Params(), hydrograph=train_hyd, precision=_lib.PREC_MIXED)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    states, times, _ = ws.collect_trajectory(sim, train_hyd, 0.0, DT, 5, **kw)
    sim.close()
    net = ws.WarmStartNet(mesh, seed=7)
    net.set_scales((4.0, 1.0, 1.0), *ws.trajectory_scales(states))
    ws.add_trajectory(net, states, times, train_hyd, DT)
    net.train(epochs=10, batch=8192, lr=1e-3, seed=3)

    hyd = meshgen.sin2_hydrograph()
    sim = Simulation(mesh, Params(), hydrograph=hyd, precision=_lib.PREC_MIXED)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    hist = [sim.get_state()]
    for k in range(int(g["steps"])):
        if len(hist) >= 2:
            sim.set_warm_start(*ws.predict_next(net, hist[-2], hist[-1], DT * k, hyd, DT))
        rep = sim.step(DT * k, DT, **kw)
        assert rep["converged"] and rep["residual_ratio"] <= 1e-8
        got = sim.get_state()
        _check(got, g, k, 1e-5)
        hist = [hist[-1], got]
    sim.close()
    net.close()


def test_mixed_options_without_friction_term_match_reference():
    """Inexact Newton and ILU(0) reuse with the reference's own Jacobian (no friction-depth
    term), cold-started: the converged state of every step is still the reference's."""
    g = golden_io.load("meander200k.npz")
    mesh = meshgen.meander()
    kw = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=1e-8, linear_forcing=0.5, ilu_reuse=64,
              friction_jacobian=False)
    sim = Simulation(mesh, Params(), hydrograph=meshgen.sin2_hydrograph(), precision=_lib.PREC_MIXED)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    for k in range(int(g["steps"])):
        rep = sim.step(DT * k, DT, **kw)
        assert rep["converged"] and rep["residual_ratio"] <= 1e-8
        _check(sim.get_state(), g, k, 1e-5)
    sim.close()
