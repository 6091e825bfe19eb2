"""The drop-in binding (rismo2d_gb300/shim/rg300_eqs_solve.cpp) compiles against
the reference's own headers and links into the reference's objects with
EQS::Solve rerouted to librg300 (oracle/Makefile target `shim`).  Needs the
reference sources, so it is skipped where they are absent."""

import os
import subprocess

import oracle
import pytest

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
REFSRC = oracle.reference_sources()


@pytest.mark.skipif(not REFSRC or not os.path.isdir(REFSRC), reason="reference sources not present")
def test_shim_links_into_reference():
    lib = os.path.join(REPO, "rismo2d_gb300", "librg300.so")
    if not os.path.exists(lib):
        pytest.skip("librg300.so not built")
    subprocess.check_call(["make", "-s", "-j8", "shim", f"REFSRC={REFSRC}"], cwd=os.path.join(REPO, "oracle"))
    exe = os.path.join(REPO, "oracle", "_ref", "rismo2d_rg300")
    assert os.path.exists(exe)
    syms = subprocess.run(["nm", exe], capture_output=True, text=True).stdout
    assert "__wrap__ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi" in syms
    assert " U rg_solve" in syms


def _run_deck(exe, workdir, mesh, **deck_kw):
    from rismo2d_gb300 import deck
    os.makedirs(workdir, exist_ok=True)
    main = deck.write_deck(mesh, workdir, restart_file="restart.dat", **deck_kw)
    out = subprocess.run([exe, os.path.basename(main)], cwd=workdir, capture_output=True, text=True, timeout=600)
    report = open(os.path.join(workdir, "report.txt")).read()
    assert "normal program termination" in report, (out.stdout + out.stderr)[-2000:]
    return deck.read_initial(os.path.join(workdir, "restart.dat")), out.stdout


@pytest.mark.skipif(not REFSRC or not os.path.isdir(REFSRC), reason="reference sources not present")
@pytest.mark.parametrize("case", ["channel_tiny", "meander_tiny"])
def test_shim_runs_the_reference_on_cpu(tmp_path, case):
    """The drop-in binding run end to end: the reference's own Newton loop with every
    EQS::Solve going through rg300_eqs_solve.cpp, here into a CPU stand-in of the library
    calls it makes (oracle/shim_cpu_double.c over the oracle's restatement, the
    reference's float storage).  Its restart output must equal the unmodified
    reference's on the same deck: the binding hands over the reference's numbering,
    pattern, node state, boundary data and relaxation factors unchanged, through the
    renumbering after dry/rewet on the meander."""
    import numpy as np
    from golden.make_golden import MEANDER_TINY, meander_hydrograph
    from rismo2d_gb300 import meshgen
    subprocess.check_call(["make", "-s", "-j8", "all", "shim_cpu", f"REFSRC={REFSRC}"],
                          cwd=os.path.join(REPO, "oracle"))
    if case == "channel_tiny":
        mesh, kw = meshgen.channel(nx=6, ny=2, length=120.0, width=40.0, nbumps=3, Q=40.0), {}
    else:
        mesh = meshgen.meander(**MEANDER_TINY)
        kw = dict(steady=False, dt=10.0, nsteps=3, hydrograph=meander_hydrograph(), maxiter=40)
    ref, _ = _run_deck(os.path.join(REPO, "oracle", "_ref", "rismo2d"), str(tmp_path / "ref"), mesh, **kw)
    got, log = _run_deck(os.path.join(REPO, "oracle", "_ref", "rismo2d_rg300_cpu"), str(tmp_path / "shim"),
                         mesh, **kw)
    solves = [int(ln.split()[3]) for ln in log.splitlines() if ln.startswith("rg300 CPU stand-in:")]
    assert solves and solves[-1] > 0, "EQS::Solve was not rerouted through the binding"
    for k in ("U", "V", "S", "Zb"):
        assert np.array_equal(got[k], ref[k]), (k, float(np.max(np.abs(got[k] - ref[k]))))
