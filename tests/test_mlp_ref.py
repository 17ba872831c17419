"""The CPU check of the surrogate MLP: its gradient formulas against finite differences."""
import numpy as np

from oracle import mlp_ref as MR


def test_reference_gradients_against_finite_differences():
    rng = np.random.Generator(np.random.PCG64(3))
    dims = [7, 11, 9, 5]
    layers = [(rng.standard_normal((dims[l + 1], dims[l])) * 0.5, rng.standard_normal(dims[l + 1]) * 0.1)
              for l in range(3)]
    x = rng.standard_normal((13, 7))
    t = rng.standard_normal((13, 5))
    loss, g = MR.grads_exact(layers, x, t)
    h = 1e-6
    for l in range(3):
        W, b = layers[l]
        for (i, j) in ((0, 0), (dims[l + 1] - 1, dims[l] - 1), (2, 3)):
            Wp = W.copy(); Wp[i, j] += h
            Wm = W.copy(); Wm[i, j] -= h
            lp = MR.grads_exact([*layers[:l], (Wp, b), *layers[l + 1:]], x, t)[0]
            lm = MR.grads_exact([*layers[:l], (Wm, b), *layers[l + 1:]], x, t)[0]
            assert abs((lp - lm) / (2 * h) - g[l][0][i, j]) < 1e-6 * (1 + abs(g[l][0][i, j]))
        bp = b.copy(); bp[1] += h
        bm = b.copy(); bm[1] -= h
        lp = MR.grads_exact([*layers[:l], (W, bp), *layers[l + 1:]], x, t)[0]
        lm = MR.grads_exact([*layers[:l], (W, bm), *layers[l + 1:]], x, t)[0]
        assert abs((lp - lm) / (2 * h) - g[l][1][1]) < 1e-6 * (1 + abs(g[l][1][1]))


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.0078125, -3.14159, 65504.0, 1e-3], np.float32)
    r = MR.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125     # ties to even
    assert abs(r[3] + 3.140625) < 1e-9
