"""Reference end states of whole time steps on the benchmark-size meshes.

Writes the deck of a named workload with rismo2d_gb300.deck, runs the compiled
reference (oracle/_ref/rismo2d_dump, built from the reference's sources by
oracle/Makefile) with light dump records (RG_DUMP_LIGHT=1: residual norms,
BiCGStab counts, timings and the end state of every time step) and stores a
compact fixture under tests/golden/:

    <case>.npz
      steps, newton[k], krylov[k], step_s[k]      per time step k
      scales_k                                    ||B|| of every Newton iteration of step k
      krylov_k, solve_s_k, assemble_s_k           its BiCGStab count, EQS::Solve and assembly seconds
      sample                                      node indices of the stored values
      U_k, V_k, S_k, z_k                          end-of-step values at those nodes
      dry_k                                       packed bits of NODE::kDry for ALL nodes
      np                                          node count

Nodes are sampled (all wet nodes up to `--max-sample`, seeded) so that the
fixture stays small; the dry flags are stored for every node.

Run where the reference sources are (default: $RG_REFERENCE_SOURCES, else
oracle/Makefile's REFSRC):

    python tests/golden/make_golden_large.py meander200k
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle  # noqa: E402
import refdump  # noqa: E402
from rismo2d_gb300 import deck, meshgen  # noqa: E402

DRY = 64   # NODE::kDry


def case_meander200k():
    """The 200,028-triangle meander with flood plains (the `--workload meander200k` case), dt 10 s."""
    mesh = meshgen.meander()
    return mesh, meshgen.sin2_hydrograph(), dict(dt=10.0, maxiter=60)


def case_braided(nx: int, ny: int, length: float, width: float):
    mesh = meshgen.braided(nx=nx, ny=ny, length=length, width=width)
    return mesh, meshgen.braided_hydrograph(S=mesh.meta["S_in"]), dict(dt=20.0, maxiter=60)


CASES = {
    "meander200k": case_meander200k,
    "braided4m": lambda: case_braided(4000, 500, 20000.0, 2000.0),
    "braided_tile": lambda: case_braided(400, 500, 2000.0, 2000.0),
}


def run(case: str, nsteps: int, workdir: str, max_sample: int, seed: int) -> dict:
    subprocess.check_call(["make", "-s", "-j8", f"REFSRC={oracle.reference_sources()}"],
                          cwd=os.path.join(REPO, "oracle"))
    mesh, hyd, kw = CASES[case]()
    deck.write_deck(mesh, workdir, steady=False, dt=kw["dt"], nsteps=nsteps, hydrograph=hyd,
                    maxiter=kw["maxiter"])
    env = dict(os.environ, RG_DUMP=os.path.join(workdir, "dump.bin"), RG_DUMP_LIGHT="1")
    t0 = time.time()
    out = subprocess.run([os.path.join(REPO, "oracle", "_ref", "rismo2d_dump"), "main.inp"], cwd=workdir,
                         env=env, capture_output=True, text=True)
    wall = time.time() - t0
    log = out.stdout + out.stderr
    # REPORT::Error exits with status 0 (Report.cpp:87-126); the teardown notice of
    # MEMORY::Delete(1) (Memory.cpp:250,282) is harmless
    errors = [ln for ln in log.splitlines() if "=== ERROR" in ln and "MEMORY::Delete(1)" not in ln]
    if errors:
        raise RuntimeError("reference run failed:\n" + log[-2000:])
    steps = refdump.light_steps(refdump.read_dump(os.path.join(workdir, "dump.bin")))
    rng = np.random.default_rng(seed)
    out = {"np": np.int32(mesh.np), "steps": np.int32(len(steps)), "dt": np.float64(kw["dt"]),
           "wall_s": np.float64(wall)}
    wet0 = (steps[0]["flag"] & DRY) == 0
    cand = np.nonzero(wet0)[0]
    sample = np.sort(rng.choice(cand, size=min(max_sample, len(cand)), replace=False)) if len(cand) > max_sample \
        else cand
    out["sample"] = sample.astype(np.int32)
    newton, krylov, step_s = [], [], []
    for k, s in enumerate(steps):
        newton.append(len(s["scales"]))
        krylov.append(int(sum(s["iters"])))
        step_s.append(float(s["seconds"]))
        out[f"scales_{k}"] = np.asarray(s["scales"], np.float64)
        out[f"krylov_{k}"] = np.asarray(s["iters"], np.int32)
        out[f"solve_s_{k}"] = np.asarray(s["solve_s"], np.float64)        # EQS::Solve wall time per iteration
        out[f"assemble_s_{k}"] = np.asarray(s["assemble_s"], np.float64)  # assembly wall time per iteration
        for v in ("U", "V", "S", "z"):
            out[f"{v}_{k}"] = np.asarray(s[v])[sample]
        out[f"dry_{k}"] = np.packbits(((s["flag"] & DRY) != 0).astype(np.uint8))
    out["newton"] = np.asarray(newton, np.int32)
    out["krylov"] = np.asarray(krylov, np.int32)
    out["step_s"] = np.asarray(step_s, np.float64)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--workdir", default=None)
    ap.add_argument("--max-sample", type=int, default=60000)
    ap.add_argument("--seed", type=int, default=11)
    args = ap.parse_args()
    workdir = args.workdir or os.path.join("/tmp", f"rg_golden_{args.case}")
    out = run(args.case, args.steps, workdir, args.max_sample, args.seed)
    path = os.path.join(HERE, f"{args.case}.npz")
    np.savez_compressed(path, **out)
    print(json.dumps({"fixture": path, "bytes": os.path.getsize(path), "newton": out["newton"].tolist(),
                      "krylov": out["krylov"].tolist(), "step_s": out["step_s"].tolist()}))


if __name__ == "__main__":
    main()
