"""The reference arm's ingredients on the CPU (oracle/refarm.py): the compiled
reference's own iteration counts to ||B||/||B_0|| <= 1e-8 read from the golden
fixtures, and the time-step estimate built from them."""

import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import refarm  # noqa: E402


def test_reference_counts_from_the_recorded_runs():
    b = refarm.reference_counts("braided4m")
    assert b["fixture"] == "braided_tile.npz" and b["steps"] == 2 and b["tol_reached"]
    assert b["newton_per_step"] == 14.5 and b["krylov_per_step"] == 1188.5
    m = refarm.reference_counts("meander200k")
    assert m["fixture"] == "meander200k.npz" and m["steps"] == 5 and m["tol_reached"]
    assert m["newton_per_step"] == 34.6 and m["krylov_per_step"] == 825.0
    # a looser tolerance needs fewer iterations
    loose = refarm.reference_counts("braided4m", tol=1e-4)
    assert loose["newton_per_step"] < b["newton_per_step"] and loose["krylov_per_step"] < b["krylov_per_step"]


def test_counts_stop_at_the_first_iteration_below_the_tolerance():
    """Restated with a plain loop: a step takes k Newton solves when ||B_k|| / ||B_0|| is the
    first residual ratio at or below the tolerance, and the BiCGStab iterations of exactly
    those k solves."""
    g = np.load(os.path.join(refarm.GOLDEN, "braided_tile.npz"))
    newton, krylov = [], []
    for s in range(int(g["steps"])):
        sc, kr = g[f"scales_{s}"], g[f"krylov_{s}"]
        k = 1
        while sc[k] / sc[0] > 1e-8:
            k += 1
        newton.append(k)
        krylov.append(int(sum(kr[:k])))
    got = refarm.reference_counts("braided4m")
    assert got["newton_per_step"] == np.mean(newton) and got["krylov_per_step"] == np.mean(krylov)


def test_time_step_estimate():
    parts = {"assemble_s": 4.0, "scale_s": 0.1, "factor_s": 9.5}
    counts = {"newton_per_step": 14.5, "krylov_per_step": 1188.5}
    assert abs(refarm.estimate(parts, 0.388, counts) - (14.5 * 13.6 + 1188.5 * 0.388)) < 1e-9


def test_host_cpu_names_the_machine():
    import platform
    assert platform.machine() in refarm.host_cpu()
