"""Learned Newton warm start (include/rg300_mlp.h) from Python.

`WarmStartNet` wraps the GPU network: stencils from the mesh, training
samples from time-level triples of the plain solver, training on the GPU, and
the prediction of the next time level that `Simulation.set_warm_start` hands
to the next step.  `collect_trajectory` runs the plain solver to produce the
training data.  The plain Newton / BiCGStab iteration still decides
convergence, and a step falls back to the last time level whenever the
prediction starts with the larger residual.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import p

NODE_DRY = 64   # NODE::kDry (Node.h)
NPARAM = 3 * (128 * 128 + 128) + 3 * 128 + 3


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


def wet(state: dict) -> np.ndarray:
    return np.ascontiguousarray(((state["flag"] & NODE_DRY) == 0).astype(np.int32))


def hydrograph_q(hydrograph, t: float) -> float:
    h = np.asarray(hydrograph, np.float64)
    return float(np.interp(t, h[:, 0], h[:, 1]))


class WarmStartNet:
    """The per-node network of one mesh on one GPU."""

    def __init__(self, mesh, device: int = 0, seed: int = 0):
        self.lib = _lib.load()
        self.lib.rg_mlp_last_error.restype = C.c_char_p
        self.ptr = C.c_void_p()
        st = self.lib.rg_mlp_create(C.c_int(device), C.c_uint(seed), C.byref(self.ptr))
        if st != _lib.RG_OK:
            raise _lib.RgError(st, "rg_mlp_create")
        self.np = int(mesh.np)
        x, y, z = _f64(mesh.x), _f64(mesh.y), _f64(mesh.z)
        en = np.ascontiguousarray(mesh.elems, np.int32).reshape(-1)
        self._check(self.lib.rg_mlp_set_mesh(self.ptr, C.c_int(self.np), p(x), p(y), p(z),
                                             C.c_int(len(en) // 6), p(en)), "rg_mlp_set_mesh")
        self.step_scale = (0.01, 0.01, 0.001)
        self.out_scale = (0.002, 0.002, 0.0002)

    def set_bed(self, mesh):
        """Another mesh of the same node set (a different bed): later samples and
        predictions use its geometry and bed; samples already added are kept."""
        if int(mesh.np) != self.np:
            raise ValueError("set_bed: the mesh has a different node count")
        x, y, z = _f64(mesh.x), _f64(mesh.y), _f64(mesh.z)
        en = np.ascontiguousarray(mesh.elems, np.int32).reshape(-1)
        self._check(self.lib.rg_mlp_set_mesh(self.ptr, C.c_int(self.np), p(x), p(y), p(z),
                                             C.c_int(len(en) // 6), p(en)), "rg_mlp_set_mesh")

    def _check(self, st, what):
        if st != _lib.RG_OK:
            raise _lib.RgError(st, f"{what}: {self.lib.rg_mlp_last_error(self.ptr).decode()}")

    def close(self):
        if self.ptr:
            self.lib.rg_mlp_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scales(self, in_ref=(4.0, 1.0, 1.0), step_scale=(0.01, 0.01, 0.001), out_scale=(0.002, 0.002, 0.0002)):
        self._check(self.lib.rg_mlp_set_scales(self.ptr, p(_f32(in_ref)), p(_f32(step_scale)), p(_f32(out_scale))),
                    "rg_mlp_set_scales")
        self.step_scale = tuple(float(v) for v in step_scale)
        self.out_scale = tuple(float(v) for v in out_scale)

    def params(self) -> np.ndarray:
        out = np.zeros(NPARAM, np.float32)
        self._check(self.lib.rg_mlp_get_params(self.ptr, p(out)), "rg_mlp_get_params")
        return out

    def set_params(self, params):
        self._check(self.lib.rg_mlp_set_params(self.ptr, p(_f32(params))), "rg_mlp_set_params")

    def features(self, nodes, s1: dict, s2: dict, q_next: float, q_prev: float) -> np.ndarray:
        nodes = np.ascontiguousarray(nodes, np.int32)
        out = np.zeros((len(nodes), 128), np.float32)
        self._check(self.lib.rg_mlp_features(self.ptr, C.c_int(len(nodes)), p(nodes), p(_f64(s1["U"])),
                                             p(_f64(s1["V"])), p(_f64(s1["S"])), p(_f64(s2["U"])),
                                             p(_f64(s2["V"])), p(_f64(s2["S"])), C.c_double(q_next),
                                             C.c_double(q_prev), p(out)), "rg_mlp_features")
        return out

    def add_triple(self, s2: dict, s1: dict, s0: dict, q_next: float, q_prev: float) -> int:
        added = C.c_longlong()
        self._check(self.lib.rg_mlp_add_samples(
            self.ptr, p(_f64(s2["U"])), p(_f64(s2["V"])), p(_f64(s2["S"])), p(_f64(s1["U"])), p(_f64(s1["V"])),
            p(_f64(s1["S"])), p(_f64(s0["U"])), p(_f64(s0["V"])), p(_f64(s0["S"])), p(wet(s2)), p(wet(s1)),
            p(wet(s0)), C.c_double(q_next), C.c_double(q_prev), C.byref(added)), "rg_mlp_add_samples")
        return added.value

    def clear_samples(self):
        self._check(self.lib.rg_mlp_clear_samples(self.ptr), "rg_mlp_clear_samples")

    def train(self, epochs: int = 20, batch: int = 8192, lr: float = 1e-3, seed: int = 0) -> np.ndarray:
        losses = np.zeros(max(epochs, 1))
        self._check(self.lib.rg_mlp_train(self.ptr, C.c_int(epochs), C.c_int(batch), C.c_float(lr), C.c_uint(seed),
                                          p(losses)), "rg_mlp_train")
        return losses[:epochs]

    def loss_grad(self, X, T, mask):
        X, T, mask = _f32(X), _f32(T), _f32(mask)
        n = X.shape[0]
        loss = C.c_double()
        y = np.zeros((n, 3), np.float32)
        g = np.zeros(NPARAM, np.float32)
        self._check(self.lib.rg_mlp_loss_grad(self.ptr, C.c_int(n), p(X), p(T), p(mask), C.byref(loss), p(y), p(g)),
                    "rg_mlp_loss_grad")
        return loss.value, y, g

    def predict(self, s2: dict, s1: dict, q_next: float, q_prev: float):
        U, V, S = (np.zeros(self.np) for _ in range(3))
        self._check(self.lib.rg_mlp_predict(self.ptr, p(_f64(s2["U"])), p(_f64(s2["V"])), p(_f64(s2["S"])),
                                            p(_f64(s1["U"])), p(_f64(s1["V"])), p(_f64(s1["S"])), p(wet(s2)),
                                            p(wet(s1)), C.c_double(q_next), C.c_double(q_prev), p(U), p(V), p(S)),
                    "rg_mlp_predict")
        return U, V, S


def trajectory_scales(states: list) -> tuple:
    """(step_scale, out_scale) of a trajectory: the RMS over its wet nodes of one
    step's change of U, V, S, and of the next level's deviation from the linear
    extrapolation of the last two."""
    d = {v: [] for v in ("U", "V", "S")}
    e = {v: [] for v in ("U", "V", "S")}
    for a, b in zip(states[:-1], states[1:]):
        w = (wet(a) & wet(b)).astype(bool)
        for v in d:
            d[v].append(b[v][w] - a[v][w])
    for a, b, c in zip(states[:-2], states[1:-1], states[2:]):
        w = (wet(a) & wet(b) & wet(c)).astype(bool)
        for v in e:
            e[v].append(c[v][w] - 2.0 * b[v][w] + a[v][w])
    rms = lambda xs, floor: max(float(np.sqrt(np.mean(np.square(np.concatenate(xs))))), floor)
    return (tuple(rms(d[v], 1e-6) for v in ("U", "V", "S")), tuple(rms(e[v], 1e-7) for v in ("U", "V", "S")))


def collect_trajectory(sim, hydrograph, t0: float, dt: float, nsteps: int, **step_kw) -> tuple:
    """Run `nsteps` plain steps from the simulation's current state; returns the
    states (the first entry the starting state), their times and the step reports."""
    states = [sim.get_state()]
    times = [t0]
    reps = []
    t = t0
    for _ in range(nsteps):
        reps.append(sim.step(t, dt, **step_kw))
        t += dt
        states.append(sim.get_state())
        times.append(t)
    return states, times, reps


def discharge_ratios(hydrograph, t1: float, dt: float) -> tuple:
    q1 = hydrograph_q(hydrograph, t1)
    return hydrograph_q(hydrograph, t1 + dt) / q1, q1 / hydrograph_q(hydrograph, t1 - dt)


def add_trajectory(net: WarmStartNet, states: list, times: list, hydrograph, dt: float) -> int:
    n = 0
    for k in range(2, len(states)):
        qn, qp = discharge_ratios(hydrograph, times[k - 1], dt)
        n += net.add_triple(states[k - 2], states[k - 1], states[k], qn, qp)
    return n


def predict_next(net: WarmStartNet, s2: dict, s1: dict, t1: float, hydrograph, dt: float):
    qn, qp = discharge_ratios(hydrograph, t1, dt)
    return net.predict(s2, s1, qn, qp)
