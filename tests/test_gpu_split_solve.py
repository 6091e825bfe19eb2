"""The FP32 ILU(0) apply of the mixed path on a system whose triangular solves
have far sources (the 200k meander's first Newton system: sources more than
the shared-memory ring's reach behind their rows).  In the split layout those
entries are summed by helper blocks into the right-hand side before the
wavefront block solves the chunk; the result must agree with the oracle's
PRECO_ILU0::Solve (Preco_ilu0.cpp:497-980) on the same FP32 factors (double
arithmetic) to FP32 accuracy, and with the unsplit FP32 layout (far sources
read from global memory by the wavefront block).  The pinned-slot table is
turned off so that this system has far entries at all."""

import ctypes as C

import numpy as np
import pytest

import oracle
from rismo2d_gb300 import _lib, meshgen
from rismo2d_gb300.sim import RG_DEVICE_NONE, Params, Simulation

pytestmark = pytest.mark.gpu


def _system():
    mesh = meshgen.meander()
    sim = Simulation(mesh, Params(), hydrograph=meshgen.sin2_hydrograph(), device=RG_DEVICE_NONE)
    sim.set_state(mesh.U0, mesh.V0, mesh.S0)
    sim.dry_rewet_pass()
    sim.prepare_iteration(10.0)
    out = dict(mesh=mesh, num=sim.numbering(), mod=sim.model(), bnd=sim.boundary(), st=sim.get_state())
    sim.close()
    return out


def _factored_context(d, precision=_lib.PREC_MIXED):
    m, num, mod, bnd, st = d["mesh"], d["num"], d["mod"], d["bnd"], d["st"]
    ctx = _lib.Context(m.x, m.y, mod["elem_nodes"], mod["elem_nnd"], mod["elem_flag"], mod["elem_vt"], 9.81, 0.005,
                       Params().vk, precision=precision)
    ctx.set_pattern(num["width"], num["index"], num["eqno"])
    ctx.set_boundary(bnd["nflag"], bnd["bckind"], bnd["rot4"], mod["niox"], mod["nioy"], bnd["bcU"], bnd["bcS"])
    z0 = np.zeros(m.np)
    ctx.set_state(U=st["U"], V=st["V"], S=st["S"], dUdt=z0, dVdt=z0, dSdt=z0, z=st["z"], cf=np.full(m.np, 0.01),
                  cfw=z0)
    ctx.set_relax(0.1, 0.1)
    ctx.assemble(want_A=False)
    ctx.scale()
    LU = ctx.ilu0_factor(want_LU=True)
    stats = np.zeros(15, np.int64)
    ctx.lib.rg_get_stats(ctx.ptr, stats.ctypes.data_as(C.c_void_p), C.c_int(15))
    return ctx, LU, stats


def test_split_fp32_apply_matches_oracle_and_unsplit(monkeypatch):
    # no pinned slots, so that the far sources of this 200k system are not all pinned
    monkeypatch.setenv("RG_WAVE_PIN", "0")
    d = _system()
    n = d["num"]["neq"]
    ptr = np.zeros(n + 1, np.int64)
    ptr[1:] = np.cumsum(d["num"]["width"])
    idx = d["num"]["index"]
    ctx, LU, stats = _factored_context(d)
    assert stats[8] > 0 and stats[9] > 0            # far entries in both triangular solves
    rng = np.random.default_rng(5)
    monkeypatch.setenv("RG_WAVE_SPLIT", "0")
    ctx0, LU0, stats0 = _factored_context(d)
    assert np.array_equal(LU0, LU)
    for _ in range(3):                               # repeated solves: fresh epochs of the helper flags
        b = rng.standard_normal(n).astype(np.float32)
        x = ctx.ilu0_apply_f32(b).astype(np.float64)
        ref = oracle.ilu0_solve(ptr, idx, LU, b.astype(np.float64))
        x0 = ctx0.ilu0_apply_f32(b).astype(np.float64)
        scale = float(np.max(np.abs(ref)))
        assert np.max(np.abs(x - ref)) <= 1e-4 * scale
        assert np.max(np.abs(x - x0)) <= 1e-4 * scale
    ctx.close()
    ctx0.close()


def test_split_fp64_apply_matches_oracle(monkeypatch):
    """The FP64 path splits too (its summation order is free; only the reference-
    storage mode keeps the reference's order): equal to the oracle's FP64 solve to
    rounding."""
    monkeypatch.setenv("RG_WAVE_PIN", "0")
    d = _system()
    n = d["num"]["neq"]
    ptr = np.zeros(n + 1, np.int64)
    ptr[1:] = np.cumsum(d["num"]["width"])
    ctx, LU, stats = _factored_context(d, _lib.PREC_FP64)
    assert stats[8] > 0 and stats[9] > 0
    rng = np.random.default_rng(6)
    for _ in range(2):
        b = rng.standard_normal(n)
        x = ctx.ilu0_apply(b)
        ref = oracle.ilu0_solve(ptr, d["num"]["index"], LU, b)
        assert np.max(np.abs(x - ref)) <= 1e-11 * np.max(np.abs(ref))
    ctx.close()
