"""Discharge through control sections (MODEL::Continuity, Contin.cpp:43-170):
the FP64 mass-balance check of the precision pattern.

CPU: the oracle's restatement integrates a uniform flow exactly.
GPU: rg_continuity in FP64 equals the oracle on the same state after FP64 and
mixed-precision steps, and a converged steady channel passes its inflow through
the outlet."""

import numpy as np
import pytest

import oracle
from rismo2d_gb300 import _lib, meshgen


def _lines(mesh):
    segs, sect = [], []
    for no, seg in sorted(mesh.lines.items()):
        for s in seg:
            segs.append(s)
            sect.append(no)
    return np.asarray(segs, np.int32), np.asarray(sect, np.int32)


def test_oracle_uniform_flow_known_answer():
    """Uniform U = 0.8 m/s, V = 0.3 m/s, depth 2 m: the discharge through the
    inlet line (x = 0, 40 m long, normal +x) is U*H*40 exactly; the y part is 0."""
    mesh = meshgen.channel(nx=6, ny=4, length=120.0, width=40.0, nbumps=3)
    segs, sect = _lines(mesh)
    U = np.full(mesh.np, 0.8)
    V = np.full(mesh.np, 0.3)
    S = mesh.z + 2.0
    qx, qy = oracle.continuity(segs, sect, 2, mesh.x, mesh.y, U, V, S, mesh.z)
    assert abs(qx[0] - 0.8 * 2.0 * 40.0) <= 1e-12 * 64.0
    assert abs(qx[1] - 0.8 * 2.0 * 40.0) <= 1e-12 * 64.0
    assert abs(qy[0]) <= 1e-12 and abs(qy[1]) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [_lib.PREC_FP64, _lib.PREC_MIXED])
def test_gpu_continuity_matches_oracle(prec):
    from golden.make_golden import MEANDER_TINY, meander_hydrograph
    from rismo2d_gb300.sim import RG_CRIT_RESIDUAL, Params, Simulation
    mesh = meshgen.meander(**MEANDER_TINY)
    sim = Simulation(mesh, Params(), hydrograph=meander_hydrograph(), precision=prec)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    segs, sect = _lines(mesh)
    for k in range(2):
        sim.step(10.0 * k, 10.0, criterion=RG_CRIT_RESIDUAL, residual_tol=1e-8)
        got = sim.continuity()
        st = sim.get_state()
        qx, qy = oracle.continuity(segs, sect, 2, mesh.x, mesh.y, st["U"], st["V"], st["S"], st["z"])
        scale = max(1.0, float(np.max(np.abs(qx + qy))))
        assert np.max(np.abs(got["Qx"] - qx)) <= 1e-12 * scale
        assert np.max(np.abs(got["Qy"] - qy)) <= 1e-12 * scale
    sim.close()


@pytest.mark.gpu
def test_steady_channel_mass_balance():
    """A converged steady channel (1000 triangles, Q = 200 m^3/s) passes its inflow
    through the outlet: |Q_out / Q_in - 1| <= 1e-3."""
    from rismo2d_gb300.sim import RG_CRIT_RESIDUAL, Params, Simulation
    mesh = meshgen.channel()
    sim = Simulation(mesh, Params(), precision=_lib.PREC_FP64)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    rep = sim.step(0.0, 3600.0, steady=True, criterion=RG_CRIT_RESIDUAL, residual_tol=1e-10)
    assert rep["converged"]
    q = sim.continuity()["Q"]
    assert abs(q[0] - 200.0) <= 1e-3 * 200.0, q
    assert abs(q[1] / q[0] - 1.0) <= 1e-3, q
    sim.close()
