"""Generate the golden fixtures under tests/golden/ from the reference solver.

Builds the reference from its sources (oracle/Makefile -> oracle/_ref), writes
seeded synthetic decks with rismo2d_gb300.deck, runs the dump-instrumented
reference binary and stores, per selected Newton iteration, the node/element
state the hot path reads, the assembled CRS system, ||B||, the BiCGStab count
and the correction X -- plus the converged state.

Run in a container that has the reference sources:

    python tests/golden/make_golden.py [--reference DIR]   (default: $RG_REFERENCE_SOURCES,
                                                           else oracle/Makefile's REFSRC)

The fixtures are the reference's own outputs; the oracle (oracle/rg_oracle.c)
and the CUDA path are checked against them.
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle  # noqa: E402
import refdump  # noqa: E402
from rismo2d_gb300 import deck, meshgen  # noqa: E402

STATE_KEYS = (["x", "y", "z", "zor", "U", "V", "S", "dUdt", "dVdt", "dSdt", "oU", "oV", "oS",
               "odUdt", "odVdt", "odSdt", "cf", "cfw", "vt", "uu", "uv", "vv",
               "r00", "r01", "r10", "r11", "niox", "nioy", "nx", "ny", "bcU", "bcV", "bcS",
               "flag", "bckind", "rot", "countdown", "eq0", "eq1", "eq2",
               "elem_flag", "elem_type", "elem_nnd", "elem_areafact", "elem_nodes",
               "region_flag", "region_type", "region_areafact", "region_nodes", "model_nodes",
               "materials"]
              + refdump.SCALARS)


def run_reference(mesh, workdir: str, refsrc: str, **deck_kw) -> list:
    subprocess.check_call(["make", "-s", "-j8", f"REFSRC={refsrc}"], cwd=os.path.join(REPO, "oracle"))
    main = deck.write_deck(mesh, workdir, **deck_kw)
    env = dict(os.environ, RG_DUMP=os.path.join(workdir, "dump.bin"))
    exe = os.path.join(REPO, "oracle", "_ref", "rismo2d_dump")
    out = subprocess.run([exe, os.path.basename(main)], cwd=workdir, env=env,
                         capture_output=True, text=True)
    log = out.stdout + out.stderr
    # REPORT::Error exits with status 0 (Report.cpp:87-126); teardown always prints a
    # harmless MEMORY::Delete(1) notice (Memory.cpp:250,282), which is whitelisted.
    errors = [ln for ln in log.splitlines()
              if "=== ERROR" in ln and "MEMORY::Delete(1)" not in ln]
    report = open(os.path.join(workdir, "report.txt")).read()
    if errors or "normal program termination" not in report:
        raise RuntimeError("reference run failed:\n" + log[-2000:])
    return refdump.newton_iterations(refdump.read_dump(os.path.join(workdir, "dump.bin")))


MEANDER_TINY = dict(nx=32, ny=10, length=800.0, nbands=4, seed=2, depth_out=3.5)
# a 200 m x 200 m window of the braided river at the benchmark's resolution (5 m x 4 m
# quads): anabranch, bars and their dry fringes
BRAIDED_SMALL = dict(nx=40, ny=50, length=200.0, width=200.0)


def meander_hydrograph():
    """Q(t) = 300 + 500 sin^2(pi t / 7200) sampled every 600 s, inlet level 4 m."""
    return [(t, 300.0 + 500.0 * np.sin(np.pi * t / 7200.0) ** 2, 4.0) for t in np.arange(0.0, 7201.0, 600.0)]


def pack(its: list, keep: list) -> dict:
    out = {}
    newton = [it for it in its if "state" in it]
    finals = [it["final"] for it in its if "final" in it]
    out["n_newton"] = np.int32(len(newton))
    out["scales"] = np.array([it["scale"] for it in newton])
    out["iters"] = np.array([it["x"]["iters"] for it in newton], np.int32)
    c0 = newton[0]["crs"]
    out["crs_width"] = c0["width"].astype(np.int32)
    out["crs_index"] = c0["index"].astype(np.int32)
    for k in keep:
        it = newton[k]
        if not np.array_equal(it["crs"]["index"], c0["index"]):
            # the wet model changed (dry/rewet): keep this iteration's own pattern
            out[f"it{k}_crs_width"] = it["crs"]["width"].astype(np.int32)
            out[f"it{k}_crs_index"] = it["crs"]["index"].astype(np.int32)
        for key in STATE_KEYS:
            out[f"it{k}_{key}"] = np.asarray(it["state"][key])
        out[f"it{k}_A"] = it["crs"]["A"]
        out[f"it{k}_B"] = it["crs"]["B"]
        out[f"it{k}_X"] = it["x"]["X"]
    for key in STATE_KEYS:
        out[f"final_{key}"] = np.asarray(finals[-1][key])
    # end-of-step states of every time step (U, V, S, z and the node flags)
    out["n_steps"] = np.int32(len(finals))
    for i, f in enumerate(finals):
        for key in ("U", "V", "S", "z", "flag", "dUdt", "dVdt", "dSdt"):
            out[f"step{i}_{key}"] = np.asarray(f[key])
    # Newton iterations per time step
    per_step, cnt = [], 0
    for it in its:
        if "state" in it:
            cnt += 1
        elif "final" in it:
            per_step.append(cnt)
            cnt = 0
    out["newton_per_step"] = np.array(per_step, np.int32)
    out["keep"] = np.array(keep, np.int32)
    return out


def write_braided_small(tmp: str, refsrc: str):
    """One unsteady 20 s step of the braided window from its dry start: the first and the
    last Newton iterations kept."""
    m = meshgen.braided(**BRAIDED_SMALL)
    its = run_reference(m, os.path.join(tmp, "braided"), refsrc, steady=False, dt=20.0, nsteps=1,
                        hydrograph=meshgen.braided_hydrograph(S=m.meta["S_in"]), maxiter=40)
    n = len([i for i in its if "state" in i])
    np.savez_compressed(os.path.join(HERE, "braided_small.npz"), **pack(its, [0, n - 1]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=oracle.reference_sources())
    ap.add_argument("--only", choices=("braided_small",), default=None,
                    help="write only this fixture (the others are left as they are)")
    args = ap.parse_args()
    if args.only == "braided_small":
        with tempfile.TemporaryDirectory() as tmp:
            write_braided_small(tmp, args.reference)
        return
    with tempfile.TemporaryDirectory() as tmp:
        # small steady channel: every Newton iteration kept
        m = meshgen.channel(nx=6, ny=2, length=120.0, width=40.0, nbumps=3, Q=40.0)
        its = run_reference(m, os.path.join(tmp, "tiny"), args.reference)
        n = len([i for i in its if "state" in i])
        np.savez_compressed(os.path.join(HERE, "channel_tiny.npz"), **pack(its, list(range(n))))
        # the 1000-triangle steady channel: first and a late iteration kept
        m = meshgen.channel()
        its = run_reference(m, os.path.join(tmp, "cfg1"), args.reference)
        n = len([i for i in its if "state" in i])
        np.savez_compressed(os.path.join(HERE, "channel_1000.npz"), **pack(its, [0, n - 2]))
        # unsteady meander with flood plains that dry and rewet: three 10 s steps
        m = meshgen.meander(**MEANDER_TINY)
        its = run_reference(m, os.path.join(tmp, "meander"), args.reference, steady=False, dt=10.0,
                            nsteps=3, hydrograph=meander_hydrograph(), maxiter=40)
        n = len([i for i in its if "state" in i])
        np.savez_compressed(os.path.join(HERE, "meander_tiny.npz"), **pack(its, [0, 1, n - 1]))
        write_braided_small(tmp, args.reference)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
