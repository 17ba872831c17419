"""Host logic of the replica sampler against the reference's known answers
(test/test_replicas.jl:17-60) and the convergence diagnostics (test/test_convergence.jl)."""
import math

import numpy as np
import pytest

from esmgb import replicas as RP
from esmgb import convergence as CV


def _golden():
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")) as f:
        return json.load(f)


def test_schedule_gate_weights_adaptation():
    """The known answers of test/test_replicas.jl:17-56 (tests/golden/known_answers.json)."""
    G = _golden()
    ws = G["weather_schedule"]
    ctl = RP.ReplicaCtl(M=ws["ctl"]["M"], burst_every=ws["ctl"]["burst_every"], phi=ws["ctl"]["phi"],
                        gate_min=G["gate"]["ctl"]["gate_min"], gate_max=5, gate_win=G["gate"]["ctl"]["gate_win"],
                        gate_tol=G["gate"]["ctl"]["gate_tol"], eta_w=list(G["adapt_step"]["eta0"]),
                        kappa_s=[100.0, 100.0], probe_avg=G["adapt_step"]["ctl"]["probe_avg"])
    assert [[it for it in range(1, 17) if RP.weather_schedule(ctl, it, j)[1]] for j in range(1, 5)] == \
        ws["burst_steps_1_to_16"]
    assert RP.weather_schedule(ctl, 8, 1) == (ws["angle_at_8_replica_1"], True)
    assert RP.weather_schedule(ctl, 7, 1) == (ws["angle_at_7_replica_1"], False)
    ctl.theta = 0.1                      # a continuous angle composed with the burst (:23-24)
    assert math.isclose(RP.weather_schedule(ctl, 8, 1)[0], math.acos(math.cos(0.1) * math.cos(0.3)))
    assert RP.weather_schedule(ctl, 7, 1)[0] == 0.1
    ctl.theta = 0.0
    c = G["categorical"]
    assert [RP.categorical(c["p"], u) for u in c["u"]] == c["want"]
    ri = G["relaxation_indicator"]
    assert RP.relaxation_indicator(ri["gbuf"][:1], ri["win"]) == math.inf
    assert math.isclose(RP.relaxation_indicator(ri["gbuf"], ri["win"]), ri["want"])
    R = RP.ReplicaSet(M=1, eta_w=ctl.eta_w, since=[0], window=[False], active=[False])
    gr = G["gate"]["relaxing"]
    ctl.gate_max = gr["gate_max"]
    acts = []
    for g in gr["g"]:
        acts.append(RP.update_gate(R, 0, g, ctl))
        R.since[0] += 1
    assert acts == gr["want"]
    gn = G["gate"]["never_relaxed"]
    ctl.gate_max = gn["gate_max"]
    R.since[0] = 0
    R.active[0] = False
    R.gbuf[0].clear()
    acts = []
    for it in range(1, 8):
        acts.append(RP.update_gate(R, 0, [float(it) * gn["g_first"][0], gn["g_first"][1]], ctl))
        R.since[0] += 1
    assert acts == gn["want"]
    w8 = G["weights"]
    assert list(RP.tilt_weights(0.0, w8["Phi"], w8["active"])) == list(RP.uniform_weights(w8["active"])) == \
        w8["uniform"]
    w = RP.tilt_weights(w8["lam"], w8["Phi"], w8["active"])
    assert math.isclose(w.sum(), 1) and w[1] == 0
    assert math.isclose(w[3] / w[0], math.exp(w8["lam"] * (w8["Phi"][3] - w8["Phi"][0])))
    assert list(RP.uniform_weights([False] * 4)) == w8["none_active"]
    ad = G["adapt_step"]
    R.eta_w = list(ad["eta0"])
    assert [RP.adapt_step(R, g, ctl) for g in ad["gaps"]] == ad["want_adapted"]
    np.testing.assert_allclose(R.eta_w, ad["want_eta"])
    assert not R.gaps


def test_convergence_diagnostics():
    rng = np.random.Generator(np.random.PCG64(1))

    def ar(n, phi):
        x = np.zeros(n)
        x[0] = rng.standard_normal() / math.sqrt(1 - phi ** 2)
        e = rng.standard_normal(n)
        for t in range(1, n):
            x[t] = phi * x[t - 1] + e[t]
        return x
    iid = [rng.standard_normal(1000) for _ in range(4)]
    assert CV.rhat_rank(iid) < 1.01 and 3000 < CV.ess_bulk(iid) < 5000
    a9 = [ar(2000, 0.9) for _ in range(4)]
    assert 250 < CV.ess_bulk(a9) < 700
    assert CV.rhat_rank([rng.standard_normal(1000) + (0.5 if k == 0 else 0.0) for k in range(4)]) > 1.01
    assert CV.rhat_rank([rng.standard_normal(1000) * (2.0 if k == 0 else 1.0) for k in range(4)]) > 1.01
    rw = [np.cumsum(rng.standard_normal(1000)) for _ in range(4)]
    assert CV.rhat_rank(rw) > 1.01 or CV.ess_bulk(rw) < 400


def test_probe_candidate_hist_and_gap():
    """probe_candidate / record_hist / lag_probe of src/replicas.jl:690-750 on the host, with a
    fake device whose probe returns fixed equilibrium scores."""
    ctl = RP.ReplicaCtl(M=4, probe_win=3, probe_len=5, probe_tail=2)
    R = RP.ReplicaSet(M=4, eta_w=[1e-3])
    R.active = [True, True, False, True]
    R.since = [5, 9, 12, 9]
    for q in range(4):
        for j in range(4):
            RP.record_hist(R, j, [float(q)] * 3, ctl)
    assert [len(h) for h in R.hist] == [3, 3, 0, 3]   # the inactive replica keeps no window
    assert R.hist[0][0][0] == 1.0                      # the oldest record left the window
    assert RP.probe_candidate(R, ctl) == 1             # longest since its burst; first on ties
    R.hist[1] = R.hist[1][:2]
    assert RP.probe_candidate(R, ctl) == 3
    R.active = [False] * 4
    assert RP.probe_candidate(R, ctl) is None

    class FakeDev:
        def lag_probe(self, j, n, tail, sweep0):
            assert (j, n, tail, sweep0) == (3, 5, 2, 40 * 5)
            return np.array([1.0, 2.0, 4.0]), np.array([0.5, 0.5, 9.0])

    k = np.array([100.0, 200.0, 10.0])                # the third unit is below 50 MW: not interior
    hi = np.full(3, 20000.0)
    hist = [np.array([3.0, 5.0, 7.0]), np.array([5.0, 7.0, 9.0])]
    pr = RP.lag_probe(FakeDev(), 3, hist, ctl, 2.0, k, hi, 40)
    # rs_in = mean(4, 6) = 5, rs_eq = 2 * mean(1, 2) = 3, fk = 0.5
    assert pr["gap"][0] == pytest.approx((5.0 - 3.0) / 0.5)
    assert pr["rs_in"][0] == pytest.approx(5.0) and pr["rs_eq"][0] == pytest.approx(3.0)
