"""The CPU statement of the warm-start network (oracle/mlp_oracle.py) against
torch on the CPU: its bf16 rounding against torch's float32 -> bfloat16
conversion (round to nearest, ties to even), and its hand-derived gradients
against torch autograd in float64 on the same function (bf16 roundings of
weights and activations as straight-through identities)."""

import numpy as np
import pytest

import mlp_oracle as mo

torch = pytest.importorskip("torch")

SHAPES = {"W1": (128, 128), "b1": (128,), "W2": (128, 128), "b2": (128,), "W3": (128, 128), "b3": (128,),
          "W4": (3, 128), "b4": (3,)}


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    a = np.concatenate([rng.normal(0, 3, 20000), rng.normal(0, 1e-30, 100), [0.0, -0.0, 1.0, -1.0, 65504.0,
                                                                              3.0e38, -3.0e38, 1e-40]])
    a = a.astype(np.float32)
    # exact ties: the low 16 bits are 0x8000, both parities of the kept bit
    ties = (np.arange(1, 200, dtype=np.uint32) << 16 | 0x8000).view(np.float32)
    a = np.concatenate([a, ties, -ties])
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(mo.bf16(a).view(np.uint32), ref.view(np.uint32))


def _torch_loss(P, x, t, m):
    ste = lambda v: v + (torch.from_numpy(mo.bf16(v.detach().numpy().astype(np.float32))).double() - v).detach()
    h = torch.from_numpy(mo.bf16(x)).double()
    for l in (1, 2, 3):
        z = h @ ste(P[f"W{l}"]).T + P[f"b{l}"]
        g = 0.5 * z * (1.0 + torch.erf(z / np.sqrt(2.0)))
        h = ste(g)
    y = h @ ste(P["W4"]).T + P["b4"]
    return torch.sum(m[:, None] * (y - t) ** 2) / torch.clamp(torch.sum(m), min=1.0)


def test_oracle_gradients_match_torch_autograd():
    rng = np.random.default_rng(3)
    params = {k: rng.uniform(-1.0, 1.0, s).astype(np.float32) / np.sqrt(128.0) for k, s in SHAPES.items()}
    n = 37
    x = rng.normal(0, 1, (n, 128)).astype(np.float32)
    t = rng.normal(0, 0.5, (n, 3))
    m = (rng.random(n) > 0.3).astype(np.float64)
    loss, _y, g = mo.loss_and_grads({k: v.astype(np.float64) for k, v in params.items()}, x, t, m)
    P = {k: torch.tensor(v.astype(np.float64), requires_grad=True) for k, v in params.items()}
    tl = _torch_loss(P, x, torch.from_numpy(t), torch.from_numpy(m))
    tl.backward()
    assert abs(float(tl.detach()) - loss) <= 1e-12 * abs(loss)
    for k in SHAPES:
        ref = P[k].grad.numpy()
        assert np.allclose(g[k], ref, rtol=1e-9, atol=1e-12 * np.max(np.abs(ref))), k
