"""Accuracy of the float32 engine against a host FP64 integration of the same
equations: the oracle's double twin, run from the same descriptor (GPU).

Over a short horizon, while the spike rasters agree, the float32 state must
stay within the stated tolerances of the FP64 state.  Past it, single spikes
drift apart (both networks are chaotic), so only population statistics are
compared: the firing rate, the ISI CV and, for plastic networks, the weight
histogram.  Each test prints its measured errors as one JSON line.
"""
import json

import numpy as np
import pytest

from oracle import OracleNet
from oracle.binding import generate_synapses
from spike_gb300 import Net, networks
from spike_gb300 import _native as N

pytestmark = pytest.mark.gpu

DT = 1e-4
# Stated bounds.  Within the horizon:
V_TOL = 1e-4       # |V - V64| relative to the threshold-reset gap
G_TOL = 1e-4       # |g - g64| relative to the largest |g64|
W_TOL = 1e-5       # |w - w64| for weights in [0, 1]
HORIZON = 200      # timesteps (20 ms): the rasters agree and the state errors are measured
# Past the horizon, where one realization of a chaotic network stands for
# another (the spread between two such realizations is of this size):
RATE_TOL = 0.10    # relative difference of the population rate
CV_TOL = 0.10      # absolute difference of the mean ISI CV
HIST_TOL = 0.05    # L1 distance of the normalised weight histograms (20 bins on [0, w_max])


def raster(x, pop=N.SPK_POP_NEURONS):
    ids, t = x.spikes(pop)
    return ids.astype(np.int64), np.rint(np.asarray(t, np.float64) / DT).astype(np.int64)


def isi_cv(ids, steps, n):
    cvs = []
    order = np.lexsort((steps, ids))
    ids, steps = ids[order], steps[order]
    bounds = np.searchsorted(ids, np.arange(n + 1))
    for q in range(n):
        s = steps[bounds[q]:bounds[q + 1]]
        if len(s) >= 3:
            isi = np.diff(s).astype(np.float64)
            cvs.append(isi.std() / isi.mean())
    return float(np.mean(cvs)) if cvs else 0.0, len(cvs)


def same_rasters(net, o):
    for pop in (N.SPK_POP_NEURONS, N.SPK_POP_INPUTS):
        gi, gs = raster(net, pop)
        oi, os_ = raster(o, pop)
        if len(gi) != len(oi) or not (np.array_equal(gi, oi) and np.array_equal(gs, os_)):
            return False
    return True


def horizon_and_errors(net, o, n, gap, n_labels, plastic, n_syn, chunk=10, limit=3000):
    """Advance both HORIZON timesteps (their rasters, neurons and inputs, must
    agree) and take the state errors there; then go on in chunks while the
    rasters agree, up to `limit`, for the step where single spikes part."""
    net.run_steps(HORIZON)
    o.run_steps(HORIZON)
    assert net.synchronize() == 0
    assert same_rasters(net, o)
    v = np.abs(net.state(N.SPK_FIELD_V, n).astype(np.float64) - o.state(N.SPK_FIELD_V, n)).max() / gap
    err = {"steps": HORIZON, "v": float(v)}
    if n_labels:
        g64 = o.state(N.SPK_FIELD_SYN_TRACE, n * n_labels).astype(np.float64)
        gg = net.state(N.SPK_FIELD_SYN_TRACE, n * n_labels).astype(np.float64)
        err["g"] = float(np.abs(gg - g64).max() / max(np.abs(g64).max(), 1e-30))
    if plastic:
        err["w"] = float(np.abs(net.weights(n_syn).astype(np.float64) - o.weights()).max())
    done = HORIZON
    while done < limit:
        net.run_steps(chunk)
        o.run_steps(chunk)
        assert net.synchronize() == 0
        if not same_rasters(net, o):
            break
        done += chunk
    return done, err


def test_conductance_network_against_fp64():
    """The 4,000-neuron conductance network (3,200 E + 800 I, 2 % connectivity)
    for 1 s."""
    m = networks.vogels_abbott()
    d = m.desc()
    n = 4000
    net = Net.from_desc(d)
    o = OracleNet(d, 64)
    h, err = horizon_and_errors(net, o, n, 10e-3, 2, False, 0)
    assert err["v"] <= V_TOL and err["g"] <= G_TOL, err
    rest = 10000 - h
    net.run_steps(rest)
    o.run_steps(rest)
    assert net.synchronize() == 0
    gi, gs = raster(net)
    oi, os_ = raster(o)
    rate_g, rate_o = len(gi) / (n * 1.0), len(oi) / (n * 1.0)
    cv_g, ng = isi_cv(gi, gs, n)
    cv_o, no = isi_cv(oi, os_, n)
    print(json.dumps({"case": "conductance_4000_1s", "rasters_agree_steps": h, "errors_at_horizon": err,
                      "rate_hz": [rate_g, rate_o], "isi_cv": [cv_g, cv_o], "neurons_with_isi": [ng, no]}))
    assert abs(rate_g - rate_o) <= RATE_TOL * rate_o
    assert abs(cv_g - cv_o) <= CV_TOL


@pytest.mark.parametrize("rule", ["weight_dependent", "evans", "weight_dependent_normalised"])
def test_plastic_network_against_fp64(rule):
    """600 voltage-synapse neurons (480 E, 120 I) with 300 Poisson inputs whose
    synapses are plastic (weights U(0, 1) at scale 5 mV), for 0.5 s, under
    weight-dependent STDP, the Evans rule, or weight-dependent STDP with the
    weight normalisation after it."""
    from test_generate import STDP, desc_from_oracle, small_gen
    from spike_gb300.networks import EVANS_STDP
    if rule == "evans":
        gen = small_gen(rule=N.SPK_STDP_EVANS, stdp_params=EVANS_STDP)
    else:
        gen = small_gen()
    arrays = generate_synapses(gen.desc)
    d = desc_from_oracle(gen, arrays)
    if rule == "weight_dependent_normalised":
        d.desc.weight_norm = N.SPK_NORM_AFTER_RULE
    n = 600
    net = Net.from_desc(d.desc)
    o = OracleNet(d.desc, 64)
    S = o.n_synapses
    h, err = horizon_and_errors(net, o, n, 0.02, 0, True, S)
    assert err["v"] <= V_TOL and err["w"] <= W_TOL, err
    rest = 5000 - h
    net.run_steps(rest)
    o.run_steps(rest)
    assert net.synchronize() == 0
    gi, gs = raster(net)
    oi, os_ = raster(o)
    rate_g, rate_o = len(gi) / (n * 0.5), len(oi) / (n * 0.5)
    cv_g, _ = isi_cv(gi, gs, n)
    cv_o, _ = isi_cv(oi, os_, n)
    plastic = np.asarray(arrays["plastic"], bool)
    wg = net.weights(S)
    wo = o.weights()
    # weights come back in creation order from both
    hg, _ = np.histogram(wg[plastic], bins=20, range=(0.0, STDP.w_max))
    ho, _ = np.histogram(wo[plastic], bins=20, range=(0.0, STDP.w_max))
    l1 = float(np.abs(hg / hg.sum() - ho / ho.sum()).sum())
    print(json.dumps({"case": f"plastic_voltage_600_0.5s_{rule}", "rasters_agree_steps": h, "errors_at_horizon": err,
                      "rate_hz": [rate_g, rate_o], "isi_cv": [cv_g, cv_o], "weight_hist_l1": l1,
                      "mean_weight": [float(wg[plastic].mean()), float(wo[plastic].mean())]}))
    assert abs(rate_g - rate_o) <= RATE_TOL * rate_o
    assert abs(cv_g - cv_o) <= CV_TOL
    assert l1 <= HIST_TOL
