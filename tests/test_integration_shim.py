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
