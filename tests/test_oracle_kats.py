"""Known-answer tests of the CPU oracle and of the host logic, with the exact inputs and expected
values of the reference's data-free tests (test/test_local.jl:43-58, test/test_replicas.jl:17-99)."""
import math

import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("g,L", [(3.0, 0.7), (-2.0, 1.3), (1e-12, 2.0), (-40.0, 0.5)])
def test_logseg_and_trexp_offset(g, L):
    # test/test_local.jl:43-58: log mass against quadrature (atol 1e-4), offset mean within 0.01 L
    xs = np.linspace(0, L, 200001)
    num = math.log(np.sum(np.exp(-g * xs)) * (xs[1] - xs[0]))
    assert abs(O.logseg(L, g * L) - num) < 1e-4
    rng = np.random.Generator(np.random.PCG64(12))
    u = rng.random(200000)
    s = np.array([O.trexp_offset(x, g, L) for x in u])
    w = np.exp(-g * xs)
    mu = np.sum(xs * w) / np.sum(w)
    assert np.all((s >= 0) & (s <= L))
    assert abs(s.mean() - mu) < 0.01 * L


def test_langevin_update_kat():
    # test/test_replicas.jl:62-99
    k = np.array([0.0, 50.0, 1000.0, 5000.0])
    g = np.array([1e-3, -2e-3, 5e-4, 0.0])
    ks, eta = 100.0, 1e-3
    xi = np.array([0.1, -0.2, 0.3, -0.4])
    k1, nc = O.langevin_update(k, g, xi, eta, ks, 1.0)
    w = np.log(k + ks)
    w1 = w + eta * ((k + ks) * g + 1) + math.sqrt(2 * eta) * xi
    wmin = math.log(1.0 + ks)
    w1 = np.where(w1 < wmin, 2 * wmin - w1, w1)
    np.testing.assert_allclose(k1, np.exp(w1) - ks, rtol=1e-14)
    assert nc == 0 and np.all(k1 >= 1.0 - 1e-12)
    # reflection at kappa_min
    kr, _ = O.langevin_update([2.0], [0.0], [-50.0], eta, ks, 1.0)
    x = math.log(2.0 + ks) + eta - math.sqrt(2 * eta) * 50
    assert math.isclose(math.log(kr[0] + ks), 2 * wmin - x, rel_tol=1e-14)
    # clip: |drift| > clip counted and clamped
    kc, nc = O.langevin_update([1000.0, 1000.0], [1.0, -1.0], [0.0, 0.0], eta, ks, 1.0, clip=0.02)
    assert nc == 2
    np.testing.assert_allclose(np.log(kc + ks), math.log(1000.0 + ks) + np.array([0.02, -0.02]), rtol=1e-14)
    # reflection at the box when crossing it from below, none from above
    hi = np.array([1100.0, 1100.0])
    kb, _ = O.langevin_update([1090.0, 1200.0], [0.0, 0.0], [5.0, 5.0], eta, ks, 1.0, hi=hi)
    wmax = math.log(1100.0 + ks)
    x1 = math.log(1090.0 + ks) + eta + math.sqrt(2 * eta) * 5
    assert math.isclose(math.log(kb[0] + ks), 2 * wmax - x1, rel_tol=1e-14) and kb[0] < 1100
    assert math.isclose(math.log(kb[1] + ks), math.log(1200.0 + ks) + eta + math.sqrt(2 * eta) * 5, rel_tol=1e-14)


def test_philox_known_answers():
    # Philox4x32-10 known-answer vectors of the Random123 distribution (kat_vectors), from
    # tests/golden/known_answers.json
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")) as f:
        cases = json.load(f)["philox4x32_10"]["cases"]
    assert len(cases) == 3
    for c in cases:
        assert O.philox4(*c["in"]) == c["out"]
