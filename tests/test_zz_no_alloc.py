"""rg_ilu0_apply_dev_noalloc: ILU(0) apply on device vectors with the fixed
file-scope scratch, against the existing rg_ilu0_apply on the same factors,
two calls in a row; and the rejection of a system larger than the scratch."""

import ctypes as C

import numpy as np
import pytest

import golden_io


def _lib():
    from rismo2d_gb300 import _lib
    return _lib


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_noalloc_apply_matches_ilu0_apply(precision):
    torch = pytest.importorskip("torch")
    lib = _lib()
    st = golden_io.state(golden_io.load("channel_1000.npz"), 0)
    ctx = golden_io.gpu_context(st, precision)
    ctx.assemble(want_A=False)
    ctx.scale()
    ctx.ilu0_factor()
    rng = np.random.default_rng(11 + precision)
    for _call in range(2):
        b = rng.standard_normal(ctx.neq)
        x_ref = ctx.ilu0_apply(b)
        b_dev = torch.from_numpy(b).to("cuda:0")
        x_dev = torch.full_like(b_dev, 12345.0)
        torch.cuda.synchronize()
        rc = ctx.lib.rg_ilu0_apply_dev_noalloc(ctx.ptr, C.c_void_p(b_dev.data_ptr()), C.c_void_p(x_dev.data_ptr()))
        assert rc == lib.RG_OK, ctx.lib.rg_last_error(ctx.ptr)
        x = x_dev.cpu().numpy()
        assert np.array_equal(x, x_ref)
    ctx.close()


@pytest.mark.gpu
def test_noalloc_rejects_oversized_system():
    torch = pytest.importorskip("torch")
    lib = _lib()
    st = golden_io.state(golden_io.load("channel_tiny.npz"), 0)
    ctx = lib.Context(st["x"], st["y"], st["elem_nodes"], st["elem_nnd"], st["elem_flag"], st["elem_vt"],
                      float(st["g"]), float(st["hmin"]), float(st["vk"]), precision=lib.PREC_FP64)
    max_eq = 1 << 18
    n = max_eq + 1                       # a diagonal-only pattern one row past the scratch
    width = np.ones(n, np.int32)
    index = np.arange(n, dtype=np.int32)
    eqno = np.full((len(st["x"]), 3), -1, np.int32)
    ctx.set_pattern(width, index, eqno)
    v = torch.zeros(4, dtype=torch.float64, device="cuda:0")
    rc = ctx.lib.rg_ilu0_apply_dev_noalloc(ctx.ptr, C.c_void_p(v.data_ptr()), C.c_void_p(v.data_ptr()))
    assert rc == lib.RG_ERR_ARG
    assert b"exceed the fixed scratch" in ctx.lib.rg_last_error(ctx.ptr)
    ctx.close()


@pytest.mark.gpu
def test_noalloc_rejects_overlapping_vectors():
    """The solves fill x before they read b: an x that overlaps b is refused."""
    torch = pytest.importorskip("torch")
    lib = _lib()
    st = golden_io.state(golden_io.load("channel_tiny.npz"), 0)
    ctx = golden_io.gpu_context(st, lib.PREC_MIXED)
    ctx.assemble(want_A=False)
    ctx.scale()
    ctx.ilu0_factor()
    v = torch.zeros(2 * ctx.neq, dtype=torch.float64, device="cuda:0")
    p0 = v.data_ptr()
    rc = ctx.lib.rg_ilu0_apply_dev_noalloc(ctx.ptr, C.c_void_p(p0), C.c_void_p(p0 + 8 * (ctx.neq // 2)))
    assert rc == lib.RG_ERR_ARG
    assert b"overlap" in ctx.lib.rg_last_error(ctx.ptr)
    ctx.close()
