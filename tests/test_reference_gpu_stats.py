"""The engine against the reference's own GPU kernels, statistically (GPU).

tests/golden/ref_gpu_stats.json holds what the reference's CUDA backend,
compiled for this GPU from the reference sources, did on three networks built
by the same C++ source (oracle/ref_cases.inc) through the reference's API
(tests/golden/make_ref_gpu_stats.py, oracle/ref_gpu_run.cpp).  The reference
orders its float ring additions by atomics and draws its Poisson inputs from
cuRAND, so its runs are one realization of each network, not a bit pattern.
Here the same networks, built by this library's front end (the same
connectivity: the rand() stream is the reference's), run on the engine, whose
float path the oracle matches bit for bit (the parity tests), for the same
simulated time; several Poisson streams give the engine's own spread.

Bounds (stated here, checked per network):
* population rate, whole run and second half: within 10 % of the reference's;
* mean ISI CV (neurons with at least three spikes): within 0.10;
* plastic network: L1 distance of the 20-bin E->E weight histograms on
  [0, w_max] within 0.10, mean weight within 5 %.
"""
import json
import os

import numpy as np
import pytest

from spike_gb300 import desc_arrays, networks
from spike_gb300.model import STDPParams

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_stats.json")
RATE_TOL, CV_TOL, HIST_TOL, WMEAN_TOL = 0.10, 0.10, 0.10, 0.05


def _gold():
    if not os.path.exists(GOLD):
        pytest.skip("no reference GPU statistics recorded")
    with open(GOLD) as f:
        return json.load(f)


def _stats(ids, times, n, seconds):
    order = np.lexsort((times, ids))
    ids, times = ids[order], times[order]
    late = times >= seconds / 2
    starts = np.searchsorted(ids, np.arange(n + 1))
    cvs = []
    for k in range(n):
        t = times[starts[k]:starts[k + 1]].astype(np.float64)
        if len(t) >= 3:
            isi = np.diff(t)
            if isi.mean() > 0:
                cvs.append(isi.std() / isi.mean())
    return dict(rate_hz=len(ids) / (n * seconds), rate_late_hz=int(late.sum()) / (n * seconds / 2),
                cv_isi=float(np.mean(cvs)))


def _check(ours: list, ref: dict, tag: str):
    rate = np.mean([s["rate_hz"] for s in ours])
    late = np.mean([s["rate_late_hz"] for s in ours])
    cv = np.mean([s["cv_isi"] for s in ours])
    msg = f"{tag}: engine rate {rate:.3f} / {late:.3f} Hz, CV {cv:.3f}; reference {ref['rate_hz']:.3f} / " \
          f"{ref['rate_late_hz']:.3f} Hz, CV {ref['cv_isi']:.3f}"
    assert abs(rate - ref["rate_hz"]) <= RATE_TOL * ref["rate_hz"], msg
    assert abs(late - ref["rate_late_hz"]) <= RATE_TOL * ref["rate_late_hz"], msg
    assert abs(cv - ref["cv_isi"]) <= CV_TOL, msg


def test_vogels_abbott_against_reference_gpu():
    ref = _gold()["va"]
    m = networks.vogels_abbott(v_init=False)
    assert m.counts()[2] == ref["synapses"]
    net = m.finalise()
    m.run(ref["seconds"])
    assert net.synchronize() == 0
    ids, t = m.spikes()
    _check([_stats(ids, t, 4000, ref["seconds"])], ref, "va")


def test_brunel_against_reference_gpu():
    ref = _gold()["brunel_cfg2"]
    runs = []
    for seed in (42, 43, 44):
        m = networks.brunel(philox_seed=seed)
        assert m.counts()[2] == ref["synapses"]
        net = m.finalise()
        m.run(ref["seconds"])
        assert net.synchronize() == 0
        ids, t = m.spikes()
        runs.append(_stats(ids, t, 12500, ref["seconds"]))
    _check(runs, ref, "brunel")


def test_plastic_brunel_against_reference_gpu():
    ref = _gold()["brunel_cfg2_plastic"]
    wr = ref["weights"]
    stdp = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0,
                      w_max=wr["w_max"])
    runs, hists, means = [], [], []
    for seed in (42, 43):
        m = networks.brunel(plastic=True, stdp=stdp, philox_seed=seed)
        assert m.counts()[2] == ref["synapses"]
        net = m.finalise()
        m.run(ref["seconds"])
        assert net.synchronize() == 0
        ids, t = m.spikes()
        runs.append(_stats(ids, t, 12500, ref["seconds"]))
        d = m.desc()
        plastic = desc_arrays(d)["plastic"].astype(bool)  # the E->E group
        w = net.weights(d.n_synapses)[plastic]
        assert len(w) == wr["count"]
        h, _ = np.histogram(np.clip(w, 0.0, wr["w_max"]), bins=20, range=(0.0, wr["w_max"]))
        hists.append(h / len(w))
        means.append(float(w.mean()))
    _check(runs, ref, "brunel plastic")
    l1 = float(np.abs(np.mean(hists, axis=0) - np.asarray(wr["hist"])).sum())
    assert l1 <= HIST_TOL, f"weight histogram L1 {l1:.3f}"
    assert abs(np.mean(means) - wr["mean"]) <= WMEAN_TOL * wr["mean"], (np.mean(means), wr["mean"])
