"""Reference-format deck I/O (rismo2d_gb300/deck.py): a deck written in the
reference's formats reads back to the same mesh, parameters, boundary
conditions and initial state; a simulation built from the read deck sets up
the same host model (numbering, pattern, boundary data) as one built from the
mesh; the ASCII restart file round-trips; and -- where the reference binary
was built here (oracle/_ref) -- the reference's own restart output reads back
to the reference's converged state of the golden fixture."""

import os
import subprocess

import numpy as np
import pytest

from rismo2d_gb300 import deck, meshgen
from rismo2d_gb300.sim import Params, Simulation, RG_DEVICE_NONE

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
HERE = os.path.dirname(os.path.abspath(__file__))


def _meander_deck(tmp_path):
    mesh = meshgen.meander(nx=24, ny=8, length=600.0, nbands=3, seed=4)
    hyd = [(t, 300.0 + 50.0 * t / 600.0, 4.0) for t in (0.0, 600.0, 1200.0)]
    main = deck.write_deck(mesh, str(tmp_path), steady=False, dt=10.0, nsteps=3, theta=0.8, maxiter=40,
                           hydrograph=hyd, solver_maxiter=500, solver_maxdiff=1e-9, conv_uv=1e-7, conv_s=2e-7,
                           relax=(2, 0.001, 0.1, 0.4, 0.3, 0.1), dryrew=(2, 7, 0.02, 0.03, 100, 4))
    return mesh, hyd, main


def test_deck_round_trip(tmp_path):
    mesh, hyd, main = _meander_deck(tmp_path)
    run = deck.read_deck(main)
    m = run.mesh
    for k in ("x", "y", "z", "S0", "U0", "V0"):
        assert np.array_equal(getattr(m, k), getattr(mesh, k)), k
    assert np.array_equal(m.elems, mesh.elems) and np.array_equal(m.elem_type, mesh.elem_type)
    assert sorted(m.lines) == sorted(mesh.lines)
    for no in mesh.lines:
        assert np.array_equal(m.lines[no], np.asarray(mesh.lines[no]))
    assert m.materials == sorted(mesh.materials)
    p = run.params
    assert (p.solver_maxiter, p.solver_maxdiff, p.conv_uv, p.conv_s) == (500, 1e-9, 1e-7, 2e-7)
    assert (p.relax_method, p.max_delta_uv, p.max_delta_s) == (2, 0.4, 0.3)
    assert (p.dryrew_method, p.dryrew_freq, p.dry_limit, p.rewet_limit, p.countdown) == (2, 7, 0.02, 0.03, 4)
    assert (p.theta, p.max_newton, run.max_newton) == (0.8, 40, 40)
    assert (run.steady, run.dt, run.first_step, run.last_step) == (False, 10.0, 1, 3)
    bcs = {k: (no, rows) for k, no, rows in run.line_bcs}
    assert bcs["QTINLET"] == (1, [(t, q, s) for t, q, s in hyd])
    assert bcs["OUTLET"][0] == 2 and bcs["OUTLET"][1][0][0] == mesh.meta["S_out"]
    assert run.time0 == 0.0


def test_host_model_from_deck_matches_mesh(tmp_path):
    mesh, hyd, main = _meander_deck(tmp_path)
    run = deck.read_deck(main)
    a = Simulation(mesh, run.params, hydrograph=hyd, device=RG_DEVICE_NONE)
    b = Simulation(run.mesh, run.params, line_bcs=run.line_bcs, device=RG_DEVICE_NONE)
    for sim, m in ((a, mesh), (b, run.mesh)):
        sim.set_state(m.U0, m.V0, m.S0)
        sim.dry_rewet_pass()
        sim.prepare_iteration(10.0)
    na, nb = a.numbering(), b.numbering()
    for k in na:
        assert np.array_equal(np.asarray(na[k]), np.asarray(nb[k])), k
    ba, bb = a.boundary(), b.boundary()
    for k in ba:
        assert np.array_equal(np.asarray(ba[k]), np.asarray(bb[k])), k
    a.close()
    b.close()


def test_restart_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    n = 57
    st = {k: rng.normal(0.0, 1.0, n) for k in ("U", "V", "S", "dUdt", "dVdt", "dSdt", "z")}
    path = str(tmp_path / "restart.dat")
    deck.write_restart(path, 93784.5, st)
    got = deck.read_initial(path)
    assert got["time"] == 93784.5 and got["release"] == 40700
    for k in ("U", "V", "S", "dUdt", "dVdt", "dSdt"):
        assert np.array_equal(got[k], st[k]), k
    assert np.array_equal(got["Zb"], st["z"])
    assert got["K"] is not None and not np.any(got["K"])


def test_time_strings():
    assert deck.parse_time("3600") == 3600.0
    assert deck.parse_time("10:30.5") == 630.5
    assert deck.parse_time("01:00:00.000000") == 3600.0
    assert deck.parse_time("2:01:00:00") == 2 * 86400.0 + 3600.0
    assert deck.parse_time("1T02:03:04.500000") == 93784.5
    for s in (0.0, 59.25, 3600.0, 93784.5):
        assert deck.parse_time(deck.format_time(s)) == s


@pytest.mark.skipif(not os.path.exists(os.path.join(REPO, "oracle", "_ref", "rismo2d")),
                    reason="the reference binary is built only where its sources are (oracle/Makefile)")
def test_reads_the_references_restart_output(tmp_path):
    """The reference's own ASCII restart file after the golden channel_tiny run."""
    mesh = meshgen.channel(nx=6, ny=2, length=120.0, width=40.0, nbumps=3, Q=40.0)
    main = deck.write_deck(mesh, str(tmp_path), restart_file="restart.dat")
    exe = os.path.join(REPO, "oracle", "_ref", "rismo2d")
    subprocess.run([exe, os.path.basename(main)], cwd=str(tmp_path), capture_output=True, text=True, timeout=300)
    got = deck.read_initial(str(tmp_path / "restart.dat"))
    g = np.load(os.path.join(HERE, "golden", "channel_tiny.npz"))
    for k in ("U", "V", "S"):
        ref = g[f"final_{k}"]
        assert np.max(np.abs(got[k] - ref)) <= 1e-6 * max(np.max(np.abs(ref)), 1e-3), k
    # the reference writes its bed NODE::zor as Zb: the region file's elevation at the
    # corners, the mean of the two corners at the mid-side nodes
    zor = deck.bed_zor(mesh)
    assert np.max(np.abs(got["Zb"] - zor)) <= 1e-6 * np.max(np.abs(zor))
