"""The surrogate MLP on the GPU (BF16 tensor-core mma.sync, FP32 accumulation) against the CPU
check on the same BF16 rounding points (oracle/mlp_ref.py)."""
import numpy as np
import pytest

from oracle import mlp_ref as MR

pytestmark = pytest.mark.gpu


def make(dims, seed=1):
    from esmgb.surrogate import MLP
    net = MLP(dims, batch_max=256, seed=seed)
    return net, [net.get_layer(l) for l in range(len(dims) - 1)]


def relnorm(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (np.linalg.norm(b) + 1e-30)


@pytest.mark.parametrize("dims,B", [([40, 64, 64, 24], 100), ([220, 512, 512, 512, 212], 256)])
def test_forward_and_gradients(dims, B):
    net, layers = make(dims)
    rng = np.random.Generator(np.random.PCG64(5))
    x = rng.standard_normal((B, dims[0])).astype(np.float32)
    t = rng.standard_normal((B, dims[-1])).astype(np.float32)
    y = net.forward(x)
    zs, _ = MR.forward(layers, x)
    assert relnorm(y, zs[-1]) < 2e-3
    loss, g = net.train_step(x, t, lr=0.0, grads=True)
    loss0, g0 = MR.grads(layers, x, t)
    assert abs(loss - loss0) < 1e-3 * abs(loss0)
    for l in range(len(dims) - 1):
        assert relnorm(g[l][0], g0[l][0]) < 1e-2, l
        assert relnorm(g[l][1], g0[l][1]) < 1e-2, l


def test_training_reduces_loss():
    dims = [16, 64, 64, 8]
    net, _ = make(dims, seed=2)
    rng = np.random.Generator(np.random.PCG64(7))
    A = rng.standard_normal((16, 8)) / 4
    losses = []
    for it in range(300):
        x = rng.standard_normal((128, 16)).astype(np.float32)
        t = np.tanh(x @ A).astype(np.float32)
        losses.append(net.train_step(x, t, lr=3e-3))
    assert np.mean(losses[-20:]) < 0.2 * np.mean(losses[:5])
