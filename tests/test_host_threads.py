"""The host passes of the time stepper (dry/rewet, connectivity counts) run on
a pool of host threads; their results must not depend on the thread count.
Two host-only simulations of the meander, one thread and eight, go through
the same sequence of dry/rewet passes with perturbed water levels (nodes
drying and rewetting, marsh elements) and must agree bit for bit."""

import os

import numpy as np


def _run(mesh, threads: str, noise):
    from rismo2d_gb300 import meshgen
    from rismo2d_gb300.sim import Simulation, Params, RG_DEVICE_NONE
    old = os.environ.get("RG_HOST_THREADS")
    os.environ["RG_HOST_THREADS"] = threads
    try:
        sim = Simulation(mesh, Params(), hydrograph=meshgen.sin2_hydrograph(), device=RG_DEVICE_NONE)
    finally:
        if old is None:
            del os.environ["RG_HOST_THREADS"]
        else:
            os.environ["RG_HOST_THREADS"] = old
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    out = []
    for dS in noise:
        out.append((sim.dry_rewet_pass(), sim.get_state()))
        st = out[-1][1]
        sim.set_state(st["U"] + 0.01, st["V"], np.maximum(st["S"] + dS, st["z"]))
        out.append((sim.dry_rewet_pass(), sim.get_state()))
        out.append((sim.dry_rewet_pass(), sim.get_state()))
    sim.close()
    return out


def test_dry_rewet_independent_of_thread_count():
    from rismo2d_gb300 import meshgen
    mesh = meshgen.meander(nx=400, ny=40, length=3000.0)
    rng = np.random.default_rng(1)
    noise = [rng.normal(0.0, 0.3, mesh.np) for _ in range(3)]
    a = _run(mesh, "1", noise)
    b = _run(mesh, "8", noise)
    changes = 0
    for (ca, sa), (cb, sb) in zip(a, b):
        assert ca == cb
        changes += sum(ca)
        for key in ("U", "V", "S", "z", "flag"):
            assert np.array_equal(sa[key], sb[key]), key
    assert changes > 0   # the passes did dry and rewet elements
