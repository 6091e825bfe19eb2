#!/usr/bin/env python3
"""Seconds per shallow-water time step on one GB300, Newton iterated to 1e-8.

Default workload (the metric's configuration, synthetic and seeded): the
braided river of rismo2d_gb300.meshgen.braided -- 20 km x 2 km valley, five
intersecting sinuous anabranches (80-160 m wide, bed 3 m below the valley line
with +-0.3 m gradient-noise roughness) between bars whose bed is three octaves
of gradient noise 1 to 3 m above the valley line, 4,000,000 six-node triangles
/ 8,009,001 nodes, Manning n = 1/30, constant eddy viscosity 0.5 m^2/s (the
k-epsilon closure is not built), no sediment.  Unsteady, dt = 20 s, theta = 1,
flood hydrograph Q(t) = 500 + 2500 sin^2(pi t / 86400) m^3/s at the inlet,
outlet level fixed, dry/rewet method 2 every 10 Newton iterations (71% of the
nodes start dry on the bars).  Every time step runs Newton until the scaled
residual ||B_k|| / ||B_0|| <= 1e-8.
`--workload meander200k` selects the 200,028-triangle meander (dt = 10 s).

A "step" is one such time step.  Headline arm (`value`): the mixed-precision
solver (FP32 Krylov / SpMV / ILU(0) inside FP64 iterative refinement, FP64
residual and update) started from the learned warm start, as an inexact Newton
iteration (BiCGStab to relative residual 0.5, ILU(0) factors reused for up to
64 Newton iterations) with the friction-depth term in the Jacobian; the
Newton convergence test is the same ||B_k|| / ||B_0|| <= 1e-8.  The network
is trained on the GPU before the timed region, on a trajectory of the plain
mixed solver under a different flood wave; the timed steps are held out, and
each includes its prediction (features + forward pass, host copies in and out).

Comparison arms run the first time steps of the same run (from the same
initial state) and are set against the headline arm's own times for those
steps: the plain FP64 GPU path (the reference's algorithm: ILU(0) factored
and BiCGStab to maxDiff every iteration, the reference's Jacobian), the FP64
path with the headline's Newton-Krylov options, the mixed path with the
reference's algorithm, and the mixed path cold-started.  `--impl reference`
times the CPU restatement of the reference's solver (oracle/refarm.py).
One JSON line on stdout.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

RESIDUAL_TOL = 1.0e-8
METRIC = "s per time step at 1e-8 Newton residual: mixed+learned vs plain FP64, 1 GB300"
PEAKS_FILE = os.path.join(REPO, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# Newton-Krylov options of the headline arm
LINEAR_FORCING = 0.5
ILU_REUSE = 64
TRAIN_EPOCHS = 30
TRAIN_BATCH = 8192
# per-launch DRAM bytes of the dominant kernel from the ncu capture summarised in
# profiles/ (read at run time from the summary's "traffic_bytes_per_launch" line)
TRAFFIC_FILE = os.path.join(REPO, "profiles", "k_trsv_traffic.json")


def workloads():
    from rismo2d_gb300 import meshgen
    return {
        "braided4m": dict(
            mesh=lambda: meshgen.braided(),
            hyd=lambda m: meshgen.braided_hydrograph(S=m.meta["S_in"]),
            train_hyd=lambda m: meshgen.braided_hydrograph(Q0=400.0, Qpeak=2400.0, duration=64800.0,
                                                           S=m.meta["S_in"]),
            dt=20.0, train_steps=6,
            desc=("braided river 20 km x 2 km, 4,000,000 P2 triangles (8,009,001 nodes), 5 anabranches between "
                  "fractal bars (3 octaves, 2 m relief), unsteady dt=20 s, Q(t)=500+2500 sin^2(pi t/86400), "
                  "dry/rewet on, Newton to ||B||/||B0||<=1e-8")),
        "braided_tile": dict(
            mesh=lambda: meshgen.braided(nx=400, ny=500, length=2000.0, width=2000.0),
            hyd=lambda m: meshgen.braided_hydrograph(S=m.meta["S_in"]),
            train_hyd=lambda m: meshgen.braided_hydrograph(Q0=400.0, Qpeak=2400.0, duration=64800.0,
                                                           S=m.meta["S_in"]),
            dt=20.0, train_steps=6,
            desc=("2 km x 2 km window of the braided river at full resolution, 400,000 P2 triangles (801,801 "
                  "nodes), unsteady dt=20 s, Q(t)=500+2500 sin^2(pi t/86400), dry/rewet on, Newton to "
                  "||B||/||B0||<=1e-8")),
        "meander200k": dict(
            mesh=lambda: meshgen.meander(),
            hyd=lambda m: meshgen.sin2_hydrograph(),
            train_hyd=lambda m: meshgen.sin2_hydrograph(Q0=250.0, dQ=700.0, period=5400.0),
            dt=10.0, train_steps=12,
            desc=("meander 10 km x 620 m, 200,028 P2 triangles (402,747 nodes), unsteady dt=10 s, "
                  "Q(t)=300+500 sin^2(pi t/7200), dry/rewet on, Newton to ||B||/||B0||<=1e-8")),
    }


# ---- distributed setup: replicas only (the ILU(0) chain does not shard) ----

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Dist:
    def __init__(self, backend: str):
        self.world, self.rank, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        dev = f"cuda:{self.local}" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---- clocks sampled during the timed region ---------------------------------

class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, local_rank: int):
        self.proc = None
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v for v in vis.split(",") if v.strip()]
        self.index = ids[local_rank] if local_rank < len(ids) else str(local_rank)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.index, f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out = self.proc.communicate(timeout=10)[0]
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out = self.proc.communicate()[0]
        sm, smax, reasons = [], [], set()
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(self.NAMES, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- GPU arms -----------------------------------------------------------------

def l2_flush(buf):
    import torch
    buf.zero_()
    torch.cuda.synchronize()


def train_net(wl, mesh, params, device: int, opts: dict):
    """The warm-start network of the workload's mesh, trained on the GPU on the plain mixed
    solver's trajectory under the training flood wave (not the timed one)."""
    from rismo2d_gb300 import _lib
    from rismo2d_gb300 import warmstart as ws
    from rismo2d_gb300.sim import Simulation, RG_CRIT_RESIDUAL
    hyd = wl["train_hyd"](mesh)
    dt = wl["dt"]
    t0 = time.perf_counter()
    sim = Simulation(mesh, params, hydrograph=hyd, precision=_lib.PREC_MIXED, device=device)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    states, times, reps = ws.collect_trajectory(sim, hyd, 0.0, dt, wl["train_steps"], criterion=RG_CRIT_RESIDUAL,
                                                residual_tol=RESIDUAL_TOL, **opts)
    sim.close()
    t1 = time.perf_counter()
    net = ws.WarmStartNet(mesh, device=device, seed=7)
    net.set_scales((4.0, 1.0, 1.0), *ws.trajectory_scales(states))
    nsamp = ws.add_trajectory(net, states, times, hyd, dt)
    losses = net.train(epochs=TRAIN_EPOCHS, batch=TRAIN_BATCH, lr=1e-3, seed=3)
    t2 = time.perf_counter()
    info = {"hydrograph": "a different flood wave from rest (held out from the timed steps)",
            "trajectory_steps": wl["train_steps"], "samples": int(nsamp), "epochs": TRAIN_EPOCHS,
            "batch": TRAIN_BATCH, "loss_first_last": [round(float(losses[0]), 4), round(float(losses[-1]), 4)],
            "trajectory_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2),
            "converged": all(r["converged"] for r in reps)}
    return net, info


def run_gpu(wl, mesh, params, prec: int, nsteps: int, device: int, flush_buf, *, timed_from: int = 0,
            profile: bool = False, clocks=None, dist=None, net=None, opts=None, keep_states: int = 0,
            continuity: bool = False):
    """`nsteps` time steps from the initial state through Simulation.step; steps from
    `timed_from` on are the timed region (barrier, profiler range, clocks).  Per step:
    device time by CUDA events on the library's stream (plus the prediction's wall time),
    host wall time of step + state download (e2e), the step report.  With `net`, every
    step that has two earlier levels starts from the network's prediction."""
    import torch
    from rismo2d_gb300 import warmstart as ws
    from rismo2d_gb300.sim import Simulation, RG_CRIT_RESIDUAL
    opts = dict(opts or {})
    hyd = wl["hyd"](mesh)
    dt = wl["dt"]
    sim = Simulation(mesh, params, hydrograph=hyd, precision=prec, device=device)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    hist = [sim.get_state()] if net else []
    kw = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=RESIDUAL_TOL, **opts)
    out = dict(dev_ms=[], e2e_ms=[], reps=[], states=[], h2d=0, d2h=0, launches=0, continuity=[])
    t = 0.0
    st0 = None
    for k in range(nsteps):
        if k == timed_from:
            st0 = sim.stats()
            sim.stage_ms(reset=True)
            if profile:
                sim.profile(True, reset=True)
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            if clocks:
                clocks.start()
            if profile:
                torch.cuda.profiler.start()
        l2_flush(flush_buf)
        h0 = time.perf_counter()
        pred_ms, bi, bo = 0.0, 0, 0
        if net is not None and len(hist) >= 2:
            p0 = time.perf_counter()
            sim.set_warm_start(*ws.predict_next(net, hist[-2], hist[-1], t, hyd, dt))
            nwet = int(np.count_nonzero(ws.wet(hist[-1])))
            pred_ms = (time.perf_counter() - p0) * 1e3
            bi, bo = 6 * 8 * mesh.np + 4 * nwet, 16 * nwet     # network copies in and out
        sim.event_record(0)
        rep = sim.step(t, dt, **kw)
        sim.event_record(1)
        state = sim.get_state()                              # result to host memory (numpy)
        h1 = time.perf_counter()
        if net is not None:
            hist = [hist[-1], state]
        out["dev_ms"].append(sim.event_elapsed(0, 1) + pred_ms)
        out["e2e_ms"].append((h1 - h0) * 1e3)
        out["reps"].append(rep)
        if k >= timed_from:
            out["h2d"] += bi
            out["d2h"] += bo
            out["launches"] += 2 if bi else 0
        if k < keep_states:
            out["states"].append({v: state[v] for v in ("U", "V", "S", "flag")})
        t += dt
    torch.cuda.synchronize()
    if profile:
        torch.cuda.profiler.stop()
    if dist:
        dist.barrier()
    out["clocks"] = clocks.stop() if clocks else None
    st1 = sim.stats()
    timed = max(1, nsteps - timed_from)
    out["stage"] = {k: round(v / timed, 2) for k, v in sim.stage_ms().items()}
    out["prof"] = sim.profile_read() if profile else None
    if profile:
        sim.profile(False)
    if st0 is not None:
        out["h2d"] += int(st1[12] - st0[12])
        out["d2h"] += int(st1[13] - st0[13])
        out["launches"] += int(st1[14] - st0[14])
    out["stats"] = st1.tolist()
    mod = sim.model()
    out["wet_tri"] = int(np.count_nonzero(np.asarray(mod["elem_nnd"]) == 6))
    last = sim.get_state()
    out["wet_nodes"] = int(np.count_nonzero((last["flag"] & 64) == 0))
    if continuity:
        out["continuity"] = sim.continuity()
    sim.close()
    return out


def arm_summary(run, steps):
    sel = [run["reps"][k] for k in steps]
    secs = [run["dev_ms"][k] / 1e3 for k in steps]
    return {"s_per_step": round(sum(secs) / len(secs), 4), "steps": [k + 1 for k in steps],
            "newton_per_step": round(statistics.mean(r["newton_iterations"] for r in sel), 2),
            "krylov_per_step": round(statistics.mean(r["krylov_iterations"] for r in sel), 2),
            "converged": all(r["converged"] for r in sel),
            "residual_ratio_max": max(r["residual_ratio"] for r in sel)}


def rel_errs(sa, sb):
    errs = []
    for a, b in zip(sa, sb):
        wet = (b["flag"] & 64) == 0               # NODE::kDry
        rel = {v: float(np.max(np.abs(a[v][wet] - b[v][wet])) / max(1e-30, np.max(np.abs(b[v][wet]))))
               for v in ("U", "V", "S")}
        rel["flags_identical"] = bool(np.array_equal(a["flag"], b["flag"]))
        errs.append(rel)
    return errs


# ---- roofline -----------------------------------------------------------------------

def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def per_launch_bytes(neq: int, nnz: int, tri: int, nodes: int, w: int, wx: int) -> dict:
    """Algorithmic bytes per launch: SpMV z(w+4) + 4(n+1) + 2n wx; one triangular solve half of
    the ILU(0) apply z(w+4) + 4(n+1) + 3n wx; factor 2zw + 4z + 4(n+1); assembly zw + 8n + 120N +
    24T + 900T (T wet triangles, N wet nodes)."""
    return {"spmv": nnz * (w + 4) + 4 * (neq + 1) + 2 * neq * wx,
            "trsv": (nnz * (w + 4) + 4 * (neq + 1) + 3 * neq * wx) / 2.0,
            "factor": 2 * nnz * w + 4 * nnz + 4 * (neq + 1),
            "assemble": nnz * w + 8 * neq + 120 * nodes + 24 * tri + 900 * tri}


def class_rooflines(prof, neq, nnz, tri, nodes, w, wx):
    peak, kind = hbm_peak()
    per = per_launch_bytes(neq, nnz, tri, nodes, w, wx)
    out = {}
    for cls, (launches, ms) in prof.items():
        if cls not in per or launches == 0 or ms <= 0:
            continue
        gbs = per[cls] * launches / (ms / 1e3) / 1e9
        out[cls] = {"launches": launches, "avg_launch_ms": round(ms / launches, 4),
                    "algorithmic_bytes_per_launch": int(per[cls]), "achieved_gbs": round(gbs, 2),
                    "frac": round(gbs / peak, 5)}
    return {"peak_gbs": peak, "peak_kind": kind, "classes": out}


def trsv_roofline(prof, neq, nnz, tri, nodes, dev_ms_total):
    launches, ms = prof["trsv"]
    if launches == 0 or ms <= 0:
        return None
    per = per_launch_bytes(neq, nnz, tri, nodes, 4, 4)["trsv"]
    achieved = per / (ms / launches / 1e3) / 1e9
    peak, kind = hbm_peak()
    traffic = None
    try:
        with open(TRAFFIC_FILE) as f:
            tr = json.load(f)
        if tr.get("neq") and tr.get("bytes_per_launch"):
            # the capture's DRAM bytes scaled to this system by the equation count
            traffic = float(tr["bytes_per_launch"]) * neq / float(tr["neq"])
    except (OSError, ValueError, KeyError):
        traffic = None
    return {"bound": "hbm", "kernel": "ILU(0) triangular solves, FP32 (L and U launches)",
            "achieved": round(achieved, 2), "peak": peak, "peak_kind": kind, "unit": "GB/s",
            "frac": round(achieved / peak, 5), "traffic": traffic, "algorithmic_bytes_per_launch": per,
            "launches": launches, "avg_launch_ms": round(ms / launches, 4),
            "share_of_step_device_time": round(ms / dev_ms_total, 4) if dev_ms_total > 0 else None}


# ---- main ---------------------------------------------------------------------------

def _step_timed(sim, t, dt, kw):
    import torch
    torch.cuda.synchronize()
    a = time.perf_counter()
    rep = sim.step(t, dt, **kw)
    return rep, time.perf_counter() - a


def _state_errs(sa, sb, z):
    """Max errors of state `sa` against `sb`: U and V relative to the field's maximum
    magnitude, depth H = S - z relative to the maximum depth (over nodes wet in both),
    and the number of nodes whose dry flag differs."""
    wa, wb = (sa["flag"] & 64) == 0, (sb["flag"] & 64) == 0
    w = wa & wb
    out = {}
    for v in ("U", "V"):
        den = max(float(np.max(np.abs(sb[v][w]))), 1e-30)
        out[v] = float(np.max(np.abs(sa[v][w] - sb[v][w]))) / den
    hb = sb["S"][w] - z[w]
    out["H"] = float(np.max(np.abs(sa["S"][w] - sb["S"][w]))) / max(float(np.max(hb)), 1e-30)
    out["dry_flags_differing"] = int(np.count_nonzero(wa != wb))
    return out


def study_precision(nsteps: int, ref_steps: int) -> dict:
    """The precision configuration: the meander refined to 1,002,174 triangles, unsteady
    (dt = 10 s, Q(t) = 300 + 500 sin^2(pi t / 7200)), `nsteps` time steps of the mixed path
    and of the FP64 path run side by side from the same initial state, both with the
    headline's Newton-Krylov options and Newton to ||B||/||B_0|| <= 1e-8; per step the
    mixed state's error against the FP64 state.  The first `ref_steps` steps are also run
    with the plain FP64 reference algorithm (exact linear solves, factor every iteration,
    the reference's Jacobian) to show that the options leave the converged state alone."""
    from rismo2d_gb300 import _lib, meshgen
    from rismo2d_gb300.sim import Params, Simulation, RG_CRIT_RESIDUAL
    mesh = meshgen.meander(nx=2831, ny=177)
    hyd = meshgen.sin2_hydrograph()
    dt = 10.0
    opts = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=RESIDUAL_TOL, linear_forcing=LINEAR_FORCING,
                ilu_reuse=ILU_REUSE, friction_jacobian=True)
    ref = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=RESIDUAL_TOL)
    sims = {"mixed": Simulation(mesh, Params(), hydrograph=hyd, precision=_lib.PREC_MIXED),
            "fp64": Simulation(mesh, Params(), hydrograph=hyd, precision=_lib.PREC_FP64)}
    if ref_steps > 0:
        sims["fp64_reference_algorithm"] = Simulation(mesh, Params(), hydrograph=hyd, precision=_lib.PREC_FP64)
    for sim in sims.values():
        sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    rows, t = [], 0.0
    for k in range(nsteps):
        row = {"step": k}
        st = {}
        for name, sim in sims.items():
            if name == "fp64_reference_algorithm" and k >= ref_steps:
                continue
            rep, secs = _step_timed(sim, t, dt, ref if name == "fp64_reference_algorithm" else opts)
            st[name] = sim.get_state()
            row[name] = {"s": round(secs, 3), "newton": rep["newton_iterations"], "krylov": rep["krylov_iterations"],
                         "converged": bool(rep["converged"])}
        row["mixed_vs_fp64"] = _state_errs(st["mixed"], st["fp64"], mesh.z)
        if "fp64_reference_algorithm" in st:
            row["fp64_vs_fp64_reference_algorithm"] = _state_errs(st["fp64"], st["fp64_reference_algorithm"], mesh.z)
        rows.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
        t += dt
    for sim in sims.values():
        sim.close()
    worst = {v: max(r["mixed_vs_fp64"][v] for r in rows) for v in ("U", "V", "H")}
    worst["dry_flags_differing"] = max(r["mixed_vs_fp64"]["dry_flags_differing"] for r in rows)
    mean = lambda arm, key: round(float(np.mean([r[arm][key] for r in rows if arm in r])), 3)
    return {"study": "precision1m", "mesh": {"triangles": int(mesh.ne), "nodes": int(mesh.np)},
            "steps": nsteps, "dt": dt, "worst_mixed_vs_fp64": worst,
            "per_step_mean": {arm: {"s": mean(arm, "s"), "newton": mean(arm, "newton"), "krylov": mean(arm, "krylov")}
                              for arm in sims},
            "all_converged": all(r[a]["converged"] for r in rows for a in sims if a in r),
            "rows": rows}


def study_learned(train_steps: int, test_steps: int, every: int) -> dict:
    """The learned configuration: the meander at 1,002,174 triangles with seeded random
    bump fields.  Training: 4 flood waves (peaks U(400, 1200) m^3/s, seeds 10-13, each on
    its own bump field of the same seed), `train_steps` steps each of the mixed solver with
    the headline options from rest; every `every`-th time-level triple becomes training
    samples.  Held out: 2 flood waves (seeds 20, 21) on their own bump fields, run cold and
    with the learned warm start for `test_steps` steps; Newton, Krylov and seconds per step
    and the final states' difference."""
    from rismo2d_gb300 import _lib, meshgen
    from rismo2d_gb300 import warmstart as ws
    from rismo2d_gb300.sim import Params, Simulation, RG_CRIT_RESIDUAL
    dt, period = 10.0, 2000.0
    opts = dict(criterion=RG_CRIT_RESIDUAL, residual_tol=RESIDUAL_TOL, linear_forcing=LINEAR_FORCING,
                ilu_reuse=ILU_REUSE, friction_jacobian=True)

    def case(seed):
        mesh = meshgen.meander(nx=2831, ny=177, bumps=400, bump_seed=seed, bump_amp=(0.05, 0.25))
        peak = float(np.random.default_rng(seed).uniform(400.0, 1200.0))
        hyd = meshgen.sin2_hydrograph(Q0=300.0, dQ=peak - 300.0, period=period, t_end=period, every=100.0)
        return mesh, hyd, peak

    net = None
    info = {"train": [], "held_out": []}
    t0 = time.perf_counter()
    nsamp = 0
    for seed in (10, 11, 12, 13):
        mesh, hyd, peak = case(seed)
        sim = Simulation(mesh, Params(), hydrograph=hyd, precision=_lib.PREC_MIXED)
        sim.set_state(mesh.U0, mesh.V0, mesh.S0)
        states, times, reps = ws.collect_trajectory(sim, hyd, 0.0, dt, train_steps, **opts)
        sim.close()
        if net is None:
            net = ws.WarmStartNet(mesh, seed=7)
            net.set_scales((4.0, 1.0, 1.0), *ws.trajectory_scales(states))
        else:
            net.set_bed(mesh)
        for k in range(2, len(states), every):
            qn, qp = ws.discharge_ratios(hyd, times[k - 1], dt)
            nsamp += net.add_triple(states[k - 2], states[k - 1], states[k], qn, qp)
        info["train"].append({"seed": seed, "peak": round(peak, 1), "steps": train_steps,
                              "newton_per_step": round(float(np.mean([r["newton_iterations"] for r in reps])), 2),
                              "converged": all(r["converged"] for r in reps)})
        print(json.dumps(info["train"][-1]), file=sys.stderr, flush=True)
    t1 = time.perf_counter()
    losses = net.train(epochs=TRAIN_EPOCHS, batch=TRAIN_BATCH, lr=1e-3, seed=3)
    t2 = time.perf_counter()
    info.update(samples=int(nsamp), epochs=TRAIN_EPOCHS, loss_first_last=[round(float(losses[0]), 4),
                                                                          round(float(losses[-1]), 4)],
                trajectory_s=round(t1 - t0, 1), train_s=round(t2 - t1, 1))
    for seed in (20, 21):
        mesh, hyd, peak = case(seed)
        net.set_bed(mesh)
        res = {"seed": seed, "peak": round(peak, 1), "steps": test_steps}
        finals = {}
        for arm in ("cold", "learned"):
            sim = Simulation(mesh, Params(), hydrograph=hyd, precision=_lib.PREC_MIXED)
            sim.set_state(mesh.U0, mesh.V0, mesh.S0)
            hist = [sim.get_state()]
            newton, krylov, secs, conv, t = [], [], [], [], 0.0
            for k in range(test_steps):
                a = time.perf_counter()
                if arm == "learned" and len(hist) >= 2:
                    sim.set_warm_start(*ws.predict_next(net, hist[-2], hist[-1], t, hyd, dt))
                rep = sim.step(t, dt, **opts)
                st = sim.get_state()
                secs.append(time.perf_counter() - a)
                hist = [hist[-1], st]
                newton.append(rep["newton_iterations"])
                krylov.append(rep["krylov_iterations"])
                conv.append(bool(rep["converged"]))
                t += dt
            finals[arm] = hist[-1]
            sim.close()
            sl = slice(2, None)   # the first two steps have no prediction
            res[arm] = {"newton_per_step": round(float(np.mean(newton[sl])), 2),
                        "krylov_per_step": round(float(np.mean(krylov[sl])), 2),
                        "s_per_step": round(float(np.mean(secs[sl])), 3), "converged": all(conv)}
        res["learned_speedup"] = round(res["cold"]["s_per_step"] / res["learned"]["s_per_step"], 3)
        res["learned_vs_cold_final"] = _state_errs(finals["learned"], finals["cold"], mesh.z)
        info["held_out"].append(res)
        print(json.dumps(res), file=sys.stderr, flush=True)
    net.close()
    return {"study": "learned1m", "dt": dt, "hydrograph": f"Q(t) = 300 + (peak - 300) sin^2(pi t / {period:.0f})",
            "bed": "meander + 400 Gaussian bumps (0.05-0.25 m, sigma 30 m) per seed", **info}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--workload", choices=("braided4m", "braided_tile", "meander200k"), default="braided4m")
    ap.add_argument("--probe", type=int, default=0,
                    help="only run this many cold time steps of the headline solver and print their "
                         "reports and device time per kernel class (for profiler runs)")
    ap.add_argument("--fp64-steps", type=int, default=1,
                    help="time steps of the plain FP64 arm and the other comparison arms (0: skip)")
    ap.add_argument("--cold-steps", type=int, default=2, help="timed steps of the cold-started mixed arm (0: skip)")
    ap.add_argument("--mixed-ref-steps", type=int, default=0,
                    help="time steps of the mixed path with the reference's algorithm (0: skip)")
    ap.add_argument("--linear-forcing", type=float, default=LINEAR_FORCING)
    ap.add_argument("--ilu-reuse", type=int, default=ILU_REUSE)
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU solver sampling (0: skip)")
    ap.add_argument("--study", choices=("precision1m", "learned1m"), default=None,
                    help="run a study at 1M triangles instead of the benchmark (one JSON line)")
    ap.add_argument("--study-steps", type=int, default=50)
    ap.add_argument("--study-ref-steps", type=int, default=2)
    ap.add_argument("--study-train-steps", type=int, default=100)
    ap.add_argument("--study-test-steps", type=int, default=30)
    ap.add_argument("--study-every", type=int, default=2)
    args = ap.parse_args()
    warmup = max(3, args.warmup)
    wl = workloads()[args.workload]
    if args.study == "precision1m":
        print(json.dumps(study_precision(args.study_steps, args.study_ref_steps)), flush=True)
        return 0
    if args.probe > 0:
        import torch
        from rismo2d_gb300 import _lib
        from rismo2d_gb300.sim import Params
        torch.cuda.set_device(0)
        flush_buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda:0")
        mesh = wl["mesh"]()
        opts = dict(linear_forcing=args.linear_forcing, ilu_reuse=args.ilu_reuse, friction_jacobian=True)
        run = run_gpu(wl, mesh, Params(), _lib.PREC_MIXED, args.probe, 0, flush_buf, profile=True, opts=opts)
        print(json.dumps({"probe": args.workload, "steps": args.probe,
                          "s_per_step": [round(v / 1e3, 3) for v in run["dev_ms"]],
                          "newton": [r["newton_iterations"] for r in run["reps"]],
                          "krylov": [r["krylov_iterations"] for r in run["reps"]],
                          "neq": int(run["stats"][0]), "nnz": int(run["stats"][1]),
                          "device_ms_by_kernel_class": {c: [n, round(ms, 3)] for c, (n, ms) in run["prof"].items()}}),
              flush=True)
        return 0
    if args.study == "learned1m":
        print(json.dumps(study_learned(args.study_train_steps, args.study_test_steps, args.study_every)), flush=True)
        return 0

    if args.impl == "reference":
        world, rank, _local = dist_env()
        if rank != 0:
            return 0
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import refarm
        line = refarm.bench_line(args.workload, wl, args.steps, warmup, METRIC)
        line["n_gpus"] = args.gpus
        print(json.dumps(line), flush=True)
        return 0

    import torch
    from rismo2d_gb300 import _lib
    from rismo2d_gb300.sim import Params
    dist = Dist("nccl")
    device = dist.local
    torch.cuda.set_device(device)
    flush_buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{device}")   # 256 MiB > L2
    mesh = wl["mesh"]()
    params = Params()
    clocks = Clocks(device)
    opts = dict(linear_forcing=args.linear_forcing, ilu_reuse=args.ilu_reuse, friction_jacobian=True)
    ref_opts = dict(linear_forcing=0.0, ilu_reuse=0, friction_jacobian=False)
    kf = max(0, min(args.fp64_steps, warmup + args.steps))
    net, learned_info = train_net(wl, mesh, params, device, opts)
    k = args.steps
    head = run_gpu(wl, mesh, params, _lib.PREC_MIXED, warmup + k, device, flush_buf, timed_from=warmup,
                   profile=True, clocks=clocks, dist=dist, net=net, opts=opts, keep_states=kf, continuity=True)
    net.close()
    timed = list(range(warmup, warmup + k))
    dev_s = sum(head["dev_ms"][i] for i in timed) / 1e3
    dev_s_max = dist.max(dev_s)
    value = dev_s_max / (k * dist.world)                         # whole-job seconds per time step
    e2e_s = dist.max(sum(head["e2e_ms"][i] for i in timed) / 1e3) / (k * dist.world)
    head_sum = arm_summary(head, timed)
    first = list(range(kf))

    arms = {}
    if kf > 0:
        arms["headline_first_steps"] = arm_summary(head, first)
        fp = run_gpu(wl, mesh, params, _lib.PREC_FP64, kf, device, flush_buf, profile=True, opts=ref_opts,
                     keep_states=kf)
        arms["fp64_reference_algorithm"] = arm_summary(fp, first)
        arms["fp64_reference_algorithm"]["roofline_by_kernel_class"] = class_rooflines(
            fp["prof"], int(fp["stats"][0]), int(fp["stats"][1]), fp["wet_tri"], fp["wet_nodes"], 8, 8)
        arms["fp64_reference_algorithm"]["host_stage_ms_per_step"] = fp["stage"]
        arms["headline_vs_fp64_max_rel_err"] = rel_errs(head["states"][:kf], fp["states"])
        fo = run_gpu(wl, mesh, params, _lib.PREC_FP64, kf, device, flush_buf, opts=opts)
        arms["fp64_headline_options"] = arm_summary(fo, first)
        h, f = arms["headline_first_steps"]["s_per_step"], arms["fp64_reference_algorithm"]["s_per_step"]
        arms["speedup_vs_fp64_same_steps"] = round(f / h, 3) if h > 0 else None
        arms["speedup_split"] = {
            "newton_krylov_options_in_fp64": round(f / arms["fp64_headline_options"]["s_per_step"], 3),
            "precision_and_learned_start_with_headline_options":
                round(arms["fp64_headline_options"]["s_per_step"] / h, 3)}
        km = max(0, min(args.mixed_ref_steps, kf))
        if km > 0:
            mr = run_gpu(wl, mesh, params, _lib.PREC_MIXED, km, device, flush_buf, opts=ref_opts)
            arms["mixed_reference_algorithm"] = arm_summary(mr, list(range(km)))
            fs = sum(fp["dev_ms"][:km]) / 1e3 / km
            arms["speedup_split"]["precision_with_reference_algorithm"] = round(
                fs / arms["mixed_reference_algorithm"]["s_per_step"], 3)
    if args.cold_steps > 0:
        kc = min(args.cold_steps, k)
        c = run_gpu(wl, mesh, params, _lib.PREC_MIXED, warmup + kc, device, flush_buf, timed_from=warmup, opts=opts)
        csteps = list(range(warmup, warmup + kc))
        arms["mixed_cold_start"] = arm_summary(c, csteps)
        hs = sum(head["dev_ms"][i] for i in csteps)
        arms["mixed_cold_start"]["learned_speedup"] = round(sum(c["dev_ms"][i] for i in csteps) / hs, 3)

    cpu = None
    if dist.rank == 0 and args.cpu_budget > 0:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import refarm
        cpu = refarm.cpu_baseline(args.workload, wl, args.cpu_budget)
    st = head["stats"]
    neq, nnz = int(st[0]), int(st[1])
    roof = trsv_roofline(head["prof"], neq, nnz, head["wet_tri"], head["wet_nodes"], dev_s * 1e3)
    if dist.rank == 0:
        q = head["continuity"]
        line = {"metric": METRIC, "value": round(value, 4), "unit": "s/step", "n_gpus": dist.world, "steps": k,
                "warmup": warmup, "ms_per_step": round(1e3 * dev_s_max / k, 2), "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 Krylov/ILU(0) + f64 refinement",
                "data": "synthetic (seeded mesh and bed, no external dataset)",
                "config": {"workload": wl["desc"], "workload_name": args.workload,
                           "solver": "mixed: FP32 BiCGStab/ILU(0)/SpMV in FP64 iterative refinement, started from "
                                     "the learned warm start (prediction inside each timed step); inexact Newton "
                                     f"(BiCGStab to {args.linear_forcing:g}); ILU(0) reused up to {args.ilu_reuse} "
                                     "Newton iterations; friction-depth term in the Jacobian; the Newton test "
                                     "stays ||B_k||/||B_0|| <= 1e-8",
                           "precision_arm": "mixed+learned", "linear_forcing": args.linear_forcing,
                           "ilu_reuse": args.ilu_reuse, "friction_jacobian": True,
                           "parallelism": "replicas only" if dist.world > 1 else "1 GPU",
                           "l2": "256 MiB buffer written before every step; the system exceeds L2 at 4M triangles",
                           "neq": neq, "nnz": nnz, "wet_triangles": head["wet_tri"], "wet_nodes": head["wet_nodes"]},
                "newton_per_step": head_sum["newton_per_step"], "krylov_per_step": head_sum["krylov_per_step"],
                "converged": head_sum["converged"], "residual_ratio_max": head_sum["residual_ratio_max"],
                "warm_start_accepted": sum(head["reps"][i]["warm_start"] for i in timed),
                "learned": learned_info, "arms": arms,
                "continuity_last_step": {"Q_inlet": float(q["Q"][0]), "Q_outlet": float(q["Q"][1]),
                                         "kernel": "k_continuity (FP64, MODEL::Continuity)"} if q else None,
                "host_stage_ms_per_step": head["stage"], "clocks": head["clocks"],
                "e2e": {"value": round(e2e_s, 4), "unit": "s/step",
                        "h2d_bytes_per_step": head["h2d"] // k, "d2h_bytes_per_step": head["d2h"] // k,
                        "api": "Simulation.step + get_state (host numpy state out)"},
                "gpu_launches": head["launches"],
                "device_ms_by_kernel_class": {kk: [v[0], round(v[1], 2)] for kk, v in head["prof"].items()},
                "roofline": roof,
                "roofline_by_kernel_class": class_rooflines(head["prof"], neq, nnz, head["wet_tri"],
                                                            head["wet_nodes"], 4, 4),
                "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
