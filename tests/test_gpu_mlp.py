"""The surrogate MLP on the GPU (BF16 tensor cores, FP32 accumulation: the tcgen05 kernel with its
accumulator in tensor memory, and the warp-level mma.sync kernel) against the CPU check on the same
BF16 rounding points (oracle/mlp_ref.py), and the two kernels against each other."""
import numpy as np
import pytest

from oracle import mlp_ref as MR

pytestmark = pytest.mark.gpu


def make(dims, seed=1, kind=1, batch_max=256):
    from esmgb.surrogate import MLP
    net = MLP(dims, batch_max=batch_max, seed=seed)
    net.set_gemm(kind)
    return net, [net.get_layer(l) for l in range(len(dims) - 1)]


def relnorm(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / (np.linalg.norm(b) + 1e-30)


@pytest.mark.parametrize("kind", [1, 0])
@pytest.mark.parametrize("dims,B", [([40, 64, 64, 24], 100), ([220, 512, 512, 512, 212], 256)])
def test_forward_and_gradients(dims, B, kind):
    net, layers = make(dims, kind=kind)
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


def test_tcgen05_matches_mma_sync():
    """The tcgen05 and mma.sync GEMMs on the same BF16 operands (ragged sizes: every dimension off
    the 128 x 64 x 64 tiles): outputs and gradients agree to FP32 summation order; then the
    training step of the full-form surrogate (5 hidden layers of 1024, minibatch 1024) timed with
    either kernel."""
    import time
    dims, B = [221, 300, 129, 77], 197
    a, _ = make(dims, seed=3, kind=1)
    b, _ = make(dims, seed=3, kind=0)
    rng = np.random.Generator(np.random.PCG64(9))
    x = rng.standard_normal((B, dims[0])).astype(np.float32)
    t = rng.standard_normal((B, dims[-1])).astype(np.float32)
    assert relnorm(a.forward(x), b.forward(x)) < 1e-5
    la, ga = a.train_step(x, t, lr=0.0, grads=True)
    lb, gb = b.train_step(x, t, lr=0.0, grads=True)
    assert abs(la - lb) <= 1e-5 * abs(lb)
    for l in range(len(dims) - 1):
        assert relnorm(ga[l][0], gb[l][0]) < 1e-4, l
        assert relnorm(ga[l][1], gb[l][1]) < 1e-4, l
    dims = [1365, 1024, 1024, 1024, 1024, 1024, 1357]
    flops = 3 * 2 * 1024 * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
    x = rng.standard_normal((1024, dims[0])).astype(np.float32)
    t = rng.standard_normal((1024, dims[-1])).astype(np.float32)
    for kind in (1, 0):
        net, _ = make(dims, seed=1, kind=kind, batch_max=1024)
        for _ in range(3):
            net.train_step(x, t, 1e-3)
        t0 = time.perf_counter()
        for _ in range(10):
            net.train_step(x, t, 1e-3)
        dt = (time.perf_counter() - t0) / 10
        print(f"5 x 1024 surrogate training step, {'tcgen05' if kind else 'mma.sync'}: {1e3 * dt:.2f} ms, "
              f"{flops / dt / 1e12:.1f} TFLOP/s (host copies of the minibatch included)")
        net.close()
