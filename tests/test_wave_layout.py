"""The host layout of the wavefront triangular solves, emulated on the CPU
(tests/cpp/wave_emulate.cpp): alignment and capacity invariants of the TMA
bulk copies and the shared-memory ring slots, for many sizes and bands,
including rings and stages small enough to force ring misses and level
splitting."""

import os
import subprocess

REPO = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def test_wave_layout_emulation(tmp_path):
    exe = tmp_path / "wave_emulate"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I/usr/local/cuda/include",
                           os.path.join(REPO, "tests", "cpp", "wave_emulate.cpp"),
                           os.path.join(REPO, "rismo2d_gb300", "csrc", "rg_wave_layout.cpp"),
                           "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-3000:]
