"""The library's own host model (rg_sim, no GPU) against the reference's model
set-up recorded in the golden fixtures: equation numbers, CRS pattern, node
flags, boundary kinds and rotations must be identical (integers bit-exact,
rotation entries and inlet discharges to rounding)."""

import numpy as np
import pytest

import golden_io
from rismo2d_gb300 import meshgen
from rismo2d_gb300.sim import RG_DEVICE_NONE, Params, Simulation

CASES = {
    "channel_tiny.npz": dict(nx=6, ny=2, length=120.0, width=40.0, nbumps=3, Q=40.0),
    "channel_1000.npz": dict(),
}


@pytest.mark.parametrize("name", list(CASES))
def test_numbering_and_boundary_match_reference(name):
    g = golden_io.load(name)
    mesh = meshgen.channel(**CASES[name])
    k = int(g["keep"][0])
    st = golden_io.state(g, k)
    corners = np.unique(mesh.elems[:, :3])
    assert np.array_equal(mesh.x, st["x"]) and np.array_equal(mesh.z[corners], st["zor"][corners])
    sim = Simulation(mesh, Params(), device=RG_DEVICE_NONE)
    sim.set_state(mesh.U0, mesh.V0, st["S"])
    sim.prepare_iteration(float(st["time"] + st["dt"]), st["cf"])
    num = sim.numbering()
    assert num["neq"] == len(st["width"])
    assert np.array_equal(num["eqno"], st["eqno"])
    assert np.array_equal(num["width"], st["width"])
    assert np.array_equal(num["index"], st["index"])
    bnd = sim.boundary()
    assert np.array_equal(bnd["nflag"], st["flag"])
    assert np.array_equal(bnd["bckind"], st["bckind"])
    assert np.max(np.abs(bnd["rot4"] - st["rot4"])) < 1e-12
    assert np.max(np.abs(bnd["bcU"] - st["bcU"])) <= 1e-12 * max(1.0, np.max(np.abs(st["bcU"])))
    assert np.array_equal(bnd["bcS"], st["bcS"])
    sim.close()


def test_meander_host_model_first_iteration():
    """Dry flood plains: after the first dry/rewet pass the wet model, numbering
    and pattern equal the reference's."""
    from golden.make_golden import MEANDER_TINY, meander_hydrograph
    g = golden_io.load("meander_tiny.npz")
    st = golden_io.state(g, 0)
    mesh = meshgen.meander(**MEANDER_TINY)
    sim = Simulation(mesh, Params(), hydrograph=meander_hydrograph(), device=RG_DEVICE_NONE)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    sim.dry_rewet_pass()
    sim.prepare_iteration(float(st["time"] + st["dt"]), st["cf"])
    num = sim.numbering()
    assert np.array_equal(num["eqno"], st["eqno"])
    assert np.array_equal(num["width"], st["width"])
    assert np.array_equal(num["index"], st["index"])
    bnd = sim.boundary()
    assert np.array_equal(bnd["nflag"], st["flag"])
    assert np.array_equal(bnd["bckind"], st["bckind"])
    state = sim.get_state()
    assert np.array_equal(state["S"], st["S"]) and np.array_equal(state["z"], st["z"])
    sim.close()


def test_braided_host_model_first_iteration():
    """The braided river's dry bars and anabranch banks (a 200 m window at the benchmark's
    resolution): after the first dry/rewet pass the wet model, numbering, pattern and node
    flags equal the reference's."""
    from golden.make_golden import BRAIDED_SMALL
    g = golden_io.load("braided_small.npz")
    st = golden_io.state(g, 0)
    mesh = meshgen.braided(**BRAIDED_SMALL)
    sim = Simulation(mesh, Params(), hydrograph=meshgen.braided_hydrograph(S=mesh.meta["S_in"]),
                     device=RG_DEVICE_NONE)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    sim.dry_rewet_pass()
    sim.prepare_iteration(float(st["time"] + st["dt"]), st["cf"])
    num = sim.numbering()
    assert np.array_equal(num["eqno"], st["eqno"])
    assert np.array_equal(num["width"], st["width"])
    assert np.array_equal(num["index"], st["index"])
    bnd = sim.boundary()
    assert np.array_equal(bnd["nflag"], st["flag"])
    assert np.array_equal(bnd["bckind"], st["bckind"])
    sim.close()
