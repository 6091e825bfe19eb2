"""The warm-start network's GPU kernels against the CPU statement of the same
arithmetic (oracle/mlp_oracle.py): forward outputs, loss and every parameter
gradient on a ragged batch with a partial mask; stencil features; training
targets and the prediction's extrapolation base; training lowers the loss.

Tolerances: the GPU sums in fp32 and rounds activations to bf16 exactly like
the oracle, but a product that lands on a bf16 rounding boundary can round
the other way, which moves single activations by one bf16 ulp (2^-8
relative), and the tensor-core backward rounds the upstream gradient to bf16
(2^-9 relative per element); outputs are compared to 2e-2 of their magnitude,
the loss to 1e-2 relative and each gradient block to 3e-2 in relative 2-norm."""

import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu

BLOCKS = ["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"]
SHAPES = {"W1": (128, 128), "b1": (128,), "W2": (128, 128), "b2": (128,), "W3": (128, 128), "b3": (128,),
          "W4": (3, 128), "b4": (3,)}


def unpack(flat):
    out, o = {}, 0
    for k in BLOCKS:
        n = int(np.prod(SHAPES[k]))
        out[k] = flat[o:o + n].reshape(SHAPES[k])
        o += n
    assert o == len(flat)
    return out


def tiny_mesh():
    from rismo2d_gb300 import meshgen
    return meshgen.channel(nx=6, ny=2, length=120.0, width=40.0, nbumps=3, Q=40.0)


def test_forward_backward_match_oracle():
    from rismo2d_gb300.warmstart import WarmStartNet
    net = WarmStartNet(tiny_mesh(), seed=3)
    rng = np.random.default_rng(5)
    params = net.params()
    params[mo.D_H * mo.D_IN:mo.D_H * mo.D_IN + 128] = rng.normal(0, 0.1, 128)   # nonzero b1
    params[-3:] = rng.normal(0, 0.1, 3)
    net.set_params(params)
    n = 77                                        # ragged against the 64-row tiles
    X = rng.normal(0.0, 1.0, (n, 128)).astype(np.float32)
    T = rng.normal(0.0, 0.5, (n, 3)).astype(np.float32)
    m = (rng.random(n) > 0.2).astype(np.float32)
    loss, y, g = net.loss_grad(X, T, m)
    P = unpack(params.astype(np.float64))
    ref_loss, ref_y, ref_g = mo.loss_and_grads(P, X, T.astype(np.float64), m.astype(np.float64))
    assert np.max(np.abs(y - ref_y)) <= 2e-2 * np.max(np.abs(ref_y))
    assert abs(loss - ref_loss) <= 1e-2 * abs(ref_loss)
    G = unpack(g.astype(np.float64))
    for k in BLOCKS:
        err = np.linalg.norm(G[k] - ref_g[k]) / max(np.linalg.norm(ref_g[k]), 1e-30)
        assert err <= 3e-2, (k, err)
    net.close()


def test_features_of_the_node_itself():
    from rismo2d_gb300.warmstart import WarmStartNet
    mesh = tiny_mesh()
    net = WarmStartNet(mesh, seed=1)
    net.set_scales((4.0, 1.0, 1.0), (0.02, 0.03, 0.004), (0.01, 0.01, 0.001))
    rng = np.random.default_rng(2)
    s1 = {"U": rng.normal(0, 0.5, mesh.np), "V": rng.normal(0, 0.5, mesh.np), "S": mesh.z + 2.0 + rng.random(mesh.np)}
    s2 = {"U": s1["U"] - 0.01, "V": s1["V"] + 0.02, "S": s1["S"] - 0.003}
    nodes = np.arange(mesh.np, dtype=np.int32)
    X = net.features(nodes, s1, s2, 1.05, 0.98)
    # slot 0 is the node: dz = 0, H, U, V, dS, dU, dV, distance 0; then the discharge ratios
    assert np.all(X[:, 0] == 0.0)
    assert np.allclose(X[:, 1], mo.bf16(((s1["S"] - mesh.z) / 4.0).astype(np.float32)))
    assert np.allclose(X[:, 2], mo.bf16(s1["U"].astype(np.float32)))
    assert np.allclose(X[:, 4], 0.003 / 0.004, rtol=1e-2)
    assert np.allclose(X[:, 5], 0.01 / 0.02, rtol=1e-2)
    assert np.allclose(X[:, 6], -0.02 / 0.03, rtol=1e-2)
    assert np.all(X[:, 7] == 0.0)
    assert np.allclose(X[:, 120], 0.5, rtol=1e-2) and np.allclose(X[:, 121], -0.2, rtol=1e-2)
    assert np.all(X[:, 122:] == 0.0)
    # every other slot is a neighbour at relative distance in [0, 1]
    d = X[:, 15:120:8]
    assert np.all((d >= 0.0) & (d <= 1.0))
    net.close()


def _synthetic_trajectory(mesh, nlev=12, seed=9):
    """Time levels whose step change is a smooth function of the state, so the
    deviation from linear extrapolation is a smooth function of level 1 and of
    its change from level 2 -- what the features hold."""
    rng = np.random.default_rng(seed)
    U = rng.normal(0, 0.3, mesh.np)
    V = rng.normal(0, 0.3, mesh.np)
    S = mesh.z + 2.0
    flag = np.zeros(mesh.np, np.int32)
    states = []
    for _ in range(nlev):
        states.append({"U": U.copy(), "V": V.copy(), "S": S.copy(), "flag": flag})
        U, V, S = U + 0.01 * np.sin(3.0 * V), V + 0.01 * np.cos(2.0 * U), S + 0.001 * U
    return states


def test_targets_and_prediction_base():
    """With every parameter zero the network outputs 0: the prediction is the
    linear extrapolation 2 L1 - L2 (L1 where the node was dry at level 2), and
    the first training loss is the mean squared target (L0 - extrapolation) /
    output scale, both computed here on the host."""
    from rismo2d_gb300.warmstart import WarmStartNet, NPARAM, wet, NODE_DRY
    mesh = tiny_mesh()
    net = WarmStartNet(mesh, seed=2)
    net.set_params(np.zeros(NPARAM, np.float32))
    os_ = (0.003, 0.004, 0.0005)
    net.set_scales((4.0, 1.0, 1.0), (0.01, 0.01, 0.001), os_)
    s2, s1, s0 = _synthetic_trajectory(mesh, 3)
    s2 = dict(s2, flag=np.where(np.arange(mesh.np) % 5 == 0, NODE_DRY, 0).astype(np.int32))
    U, V, S = net.predict(s2, s1, 1.0, 1.0)
    w2 = wet(s2).astype(bool)
    base = {v: np.where(w2, 2.0 * s1[v] - s2[v], s1[v]) for v in ("U", "V", "S")}
    assert np.array_equal(U, base["U"]) and np.array_equal(V, base["V"]) and np.array_equal(S, base["S"])
    n = net.add_triple(s2, s1, s0, 1.0, 1.0)
    assert n == mesh.np
    losses = net.train(epochs=1, batch=1 << 20, lr=1e-12, seed=0)
    T = np.stack([(s0[v] - base[v]) / np.float32(o) for v, o in zip(("U", "V", "S"), os_)], axis=1)
    ref = float(np.mean(np.sum(T.astype(np.float32).astype(np.float64) ** 2, axis=1)))
    assert abs(losses[0] - ref) <= 1e-5 * ref, (losses[0], ref)
    net.close()


def test_training_lowers_the_loss():
    """Samples through the public path (time-level triples of a smooth
    synthetic dynamics): Adam on the GPU brings the training loss well below
    where it started."""
    from rismo2d_gb300.warmstart import WarmStartNet, trajectory_scales
    mesh = tiny_mesh()
    net = WarmStartNet(mesh, seed=4)
    states = _synthetic_trajectory(mesh)
    net.set_scales((4.0, 1.0, 1.0), *trajectory_scales(states))
    for k in range(2, len(states)):
        net.add_triple(states[k - 2], states[k - 1], states[k], 1.0, 1.0)
    losses = net.train(epochs=100, batch=256, lr=2e-3, seed=1)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.3 * losses[0], losses
    net.close()
