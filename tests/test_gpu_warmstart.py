"""What the learned warm start gains.  The network is trained on the GPU on a
trajectory of the plain solver under one inflow hydrograph; held-out time
steps under another hydrograph then run twice from the same state -- plain,
and with the network's prediction as the Newton starting point.

Both runs must reach the same solution: identical dry/wet flags, U and V
within 1e-5 of the largest speed, S within 1e-5 of the largest water level
(two Newton paths stopped at ||B||/||B_0|| <= 1e-8 differ by far less).

- Straight channel, all wet: Newton converges quadratically here, so a
  closer start saves little; the prediction must start closer than the last
  time level (smaller residual) in most steps.
- The meander valley with dry flood plains (200,028 triangles): Newton
  converges linearly (about 0.55 per iteration after the first), so the
  closer start saves iterations; the warm-started steps must need at least
  5% fewer Newton iterations in total."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = 10.0


def _same_solution(a, b):
    assert np.array_equal(a["flag"], b["flag"])
    uv_scale = max(1.0, float(np.max(np.hypot(a["U"], a["V"]))))
    s_scale = max(1.0, float(np.max(np.abs(a["S"]))))
    for v, scale in (("U", uv_scale), ("V", uv_scale), ("S", s_scale)):
        assert np.max(np.abs(a[v] - b[v])) <= 1e-5 * scale, v


def _held_out(mesh, params, hyd, net, start, nsteps, **kw):
    """`start` plain steps, then `nsteps` steps plain and warm-started from the same state."""
    from rismo2d_gb300 import _lib
    from rismo2d_gb300 import warmstart as ws
    from rismo2d_gb300.sim import Simulation
    runs = {}
    for mode in ("plain", "warm"):
        sim = Simulation(mesh, params, hydrograph=hyd, precision=_lib.PREC_MIXED)
        sim.set_state(mesh.U0, mesh.V0, mesh.S0)
        hist, times, _ = ws.collect_trajectory(sim, hyd, 0.0, DT, start, **kw)
        newton, accepted, closer = 0, 0, 0
        t = times[-1]
        for _ in range(nsteps):
            if mode == "warm":
                sim.set_warm_start(*ws.predict_next(net, hist[-2], hist[-1], t, hyd, DT))
            rep = sim.step(t, DT, **kw)
            assert rep["converged"]
            newton += rep["newton_iterations"]
            accepted += rep["warm_start"]
            closer += int(0.0 <= rep["residual_warm"] < rep["residual_first"])
            t += DT
            hist.append(sim.get_state())
        runs[mode] = dict(state=hist[-1], newton=newton, accepted=accepted, closer=closer)
        sim.close()
    return runs


def _train(mesh, params, hyd, nsteps, skip, epochs, batch, **kw):
    from rismo2d_gb300 import _lib
    from rismo2d_gb300 import warmstart as ws
    from rismo2d_gb300.sim import Simulation
    sim = Simulation(mesh, params, hydrograph=hyd, precision=_lib.PREC_MIXED)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    states, times, reps = ws.collect_trajectory(sim, hyd, 0.0, DT, nsteps, **kw)
    sim.close()
    assert all(r["converged"] for r in reps[skip:])
    net = ws.WarmStartNet(mesh, seed=7)
    net.set_scales((4.0, 1.0, 1.0), *ws.trajectory_scales(states[skip:]))
    assert ws.add_trajectory(net, states[skip:], times[skip:], hyd, DT) > 0
    losses = net.train(epochs=epochs, batch=batch, lr=1e-3, seed=3)
    assert losses[-1] < 0.5 * losses[0]
    return net


def test_warm_start_channel_same_solution_closer_start():
    from rismo2d_gb300 import meshgen
    from rismo2d_gb300.sim import Params, RG_CRIT_RESIDUAL
    kw = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=1e-8)
    mesh = meshgen.channel(nx=100, ny=10, length=2000.0, width=100.0, nbumps=12, seed=3, Q=200.0)
    params = Params(max_newton=60)
    train_hyd = meshgen.sin2_hydrograph(Q0=150.0, dQ=200.0, period=900.0, t_end=1800.0, every=30.0, S=3.0)
    test_hyd = meshgen.sin2_hydrograph(Q0=180.0, dQ=150.0, period=700.0, t_end=1800.0, every=30.0, S=3.0)
    net = _train(mesh, params, train_hyd, 40, 5, 60, 4096, **kw)
    nsteps = 12
    runs = _held_out(mesh, params, test_hyd, net, 8, nsteps, **kw)
    _same_solution(runs["plain"]["state"], runs["warm"]["state"])
    print(f"\nchannel, {nsteps} held-out steps: Newton plain {runs['plain']['newton']}, warm start "
          f"{runs['warm']['newton']} ({runs['warm']['accepted']} accepted, {runs['warm']['closer']} closer)")
    assert runs["warm"]["closer"] >= nsteps // 2
    net.close()


def test_warm_start_meander_saves_newton_iterations():
    from rismo2d_gb300 import meshgen
    from rismo2d_gb300.sim import Params, RG_CRIT_RESIDUAL
    kw = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=1e-8)
    mesh = meshgen.meander()
    params = Params()
    train_hyd = meshgen.sin2_hydrograph(Q0=250.0, dQ=700.0, period=5400.0, t_end=7200.0)
    test_hyd = meshgen.sin2_hydrograph()
    net = _train(mesh, params, train_hyd, 12, 0, 30, 8192, **kw)
    nsteps = 6
    runs = _held_out(mesh, params, test_hyd, net, 2, nsteps, **kw)
    _same_solution(runs["plain"]["state"], runs["warm"]["state"])
    print(f"\nmeander, {nsteps} held-out steps: Newton plain {runs['plain']['newton']}, warm start "
          f"{runs['warm']['newton']} ({runs['warm']['accepted']} accepted, {runs['warm']['closer']} closer)")
    assert runs["warm"]["accepted"] == nsteps
    assert runs["warm"]["newton"] <= 0.95 * runs["plain"]["newton"]
    net.close()
