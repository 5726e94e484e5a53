"""Networks generated on the GPU (spk_net_generate) against the oracle's
restatement of the generator (GPU, bit-exact).

The oracle draws the same (pre, post) pairs, weights and delays on the host
and returns the synapses in creation order; a network created from those
arrays through spk_net_create must be the generated network synapse for
synapse (weights read back bit for bit) and must run identically, spikes,
state and plastic weights included.  The generated network must also be the
same under every schedule.
"""
import numpy as np
import pytest

import descs
from engine_checks import assert_same
from oracle import OracleNet
from oracle.binding import generate_synapses
from spike_gb300 import GenNetwork, Net, Projection, schedule
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams

pytestmark = pytest.mark.gpu

STDP = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0)
GROUPS = [dict(count=480, tau_m=0.02, R=1e8, v0=0.0, vreset=0.0, theta=0.02, v_init_lo=0.0, v_init_hi=0.015),
          dict(count=120, tau_m=0.01, R=1e8, v0=0.0, vreset=0.002, theta=0.018)]
N_IN, RATE = 300, 30.0


def small_gen(stdp=True, seed=11, rule=N.SPK_STDP_WEIGHT_DEPENDENT, stdp_params=STDP):
    rates = np.random.default_rng(seed).uniform(0.5 * RATE, 1.5 * RATE, N_IN).astype(np.float32)
    projs = [
        Projection(N.SPK_POP_INPUTS, 0, N_IN, 0, 600, 0.05, weight=(0.0, 1.0), scale=5e-3, delay=(1, 3),
                   plastic=stdp),
        Projection(N.SPK_POP_NEURONS, 0, 480, 480, 120, 0.04, weight=(0.5, 1.0), scale=1e-3, delay=(1, 8)),
        Projection(N.SPK_POP_NEURONS, 0, 480, 0, 480, 0.06, weight=(0.5, 1.0), scale=1e-3, delay=(1, 8)),
        Projection(N.SPK_POP_NEURONS, 480, 120, 0, 600, 0.05, weight=(-1.0, -0.5), scale=4e-3, delay=(1, 5)),
    ]
    return GenNetwork(groups=GROUPS, projections=projs, n_inputs=N_IN, rates=rates,
                      stdp=stdp_params if stdp else None, seed=seed + 1, connectivity_seed=seed + 2,
                      record_inputs=True, stdp_rule=rule)


def desc_from_oracle(gen: GenNetwork, arrays: dict) -> descs.Desc:
    d = gen.desc
    rates = np.ctypeslib.as_array(d.input_rates, (N_IN,)).copy()
    return descs.Desc(kind=d.synapse_kind, groups=GROUPS, n_inputs=N_IN, rates=rates,
                      pre=arrays["pre"], post=arrays["post"], weight=arrays["weight"], scale=arrays["scale"],
                      delay=arrays["delay"], label=arrays["label"],
                      plastic=arrays["plastic"] if d.has_stdp else None,
                      stdp=d.stdp if d.has_stdp else None, seed=d.seed, record_inputs=True, stdp_rule=d.stdp_rule)


def delivered(arrays: dict, stdp: bool) -> np.ndarray:
    """The value each synapse delivers: w*scale (static) or w (plastic)."""
    w, s = arrays["weight"], arrays["scale"]
    plastic = arrays["plastic"].astype(bool) & stdp
    return np.where(plastic, w, (w * s).astype(np.float32)).astype(np.float32)


@pytest.mark.parametrize("sched", [None, schedule(4, 32, 5, 0), schedule(2, 64, 0, 300)])
def test_generated_network_matches_oracle_synapses_and_run(sched):
    gen = small_gen()
    arrays = generate_synapses(gen.desc)
    S = len(arrays["pre"])
    assert abs(S - gen.expected_synapses()) < 6 * np.sqrt(gen.expected_synapses())
    g = Net.generate(gen, sched)
    assert g.synapse_count() == S
    np.testing.assert_array_equal(g.weights(S).view(np.uint32), delivered(arrays, True).view(np.uint32))
    ref_desc = desc_from_oracle(gen, arrays)
    ref = Net.from_desc(ref_desc.desc, sched)
    o = OracleNet(ref_desc.desc)
    for plastic, steps in ((True, 400), (False, 200), (True, 400)):
        g.run_steps(steps, plastic)
        ref.run_steps(steps, plastic)
        o.run_steps(steps, plastic)
    assert g.synchronize() == 0 and ref.synchronize() == 0
    assert_same(g, o, 600, N_IN, 1, tag=f"generated {sched}")
    # plastic weights: generated values are w for plastic synapses
    w_gen = g.weights(S)
    w_ref = ref.weights(S)
    plastic = arrays["plastic"].astype(bool)
    np.testing.assert_array_equal(w_gen[plastic].view(np.uint32), w_ref[plastic].view(np.uint32))
    assert len(o.spikes()[0]) > 300


def test_generated_network_with_a_trace_rule_matches_oracle():
    """A generated network whose plastic synapses follow the Evans rule: the
    afferent records get their delays on the device, and the run matches
    the oracle on the same synapses."""
    from spike_gb300.networks import EVANS_STDP
    gen = small_gen(rule=N.SPK_STDP_EVANS, stdp_params=EVANS_STDP, seed=13)
    arrays = generate_synapses(gen.desc)
    S = len(arrays["pre"])
    g = Net.generate(gen)
    ref_desc = desc_from_oracle(gen, arrays)
    o = OracleNet(ref_desc.desc)
    for plastic, steps in ((True, 400), (False, 100), (True, 300)):
        g.run_steps(steps, plastic)
        o.run_steps(steps, plastic)
    assert g.synchronize() == 0
    assert_same(g, o, 600, N_IN, 1, tag="generated evans")
    plastic = arrays["plastic"].astype(bool)
    w = g.weights(S)
    np.testing.assert_array_equal(w[plastic].view(np.uint32), o.weights()[plastic].view(np.uint32))
    assert (w[plastic] != arrays["weight"][plastic]).sum() > 100
    assert g.plastic_synapse_count() == int(plastic.sum())


def test_generated_network_is_schedule_independent():
    gen = small_gen(stdp=False, seed=23)
    nets = [Net.generate(gen, s) for s in (schedule(1, 608, 1, 0), schedule(8, 32, 3, 0), schedule(4, 96, 2, 0))]
    S = nets[0].synapse_count()
    w0 = nets[0].weights(S)
    for n in nets:
        assert n.synapse_count() == S
        np.testing.assert_array_equal(n.weights(S).view(np.uint32), w0.view(np.uint32))
        n.run_steps(500, False)
    ids0, t0 = nets[0].spikes()
    for n in nets[1:]:
        assert n.synchronize() == 0
        ids, t = n.spikes()
        np.testing.assert_array_equal(ids, ids0)
        np.testing.assert_array_equal(t.view(np.uint32), t0.view(np.uint32))


def test_generated_large_network_statistics():
    """A 40,000-neuron network (about 4.8e7 synapses): synapse count within
    binomial bounds, delays and weights within their ranges, and the same
    raster under two schedules."""
    n_e, n_i, n_in = 32000, 8000, 20000
    groups = [dict(count=n_e, theta=0.02), dict(count=n_i, theta=0.02)]
    p = 0.025
    projs = [Projection(N.SPK_POP_INPUTS, 0, n_in, 0, n_e + n_i, p, weight=(0.0, 1.0), scale=1e-3, delay=(1, 10)),
             Projection(N.SPK_POP_NEURONS, 0, n_e, 0, n_e + n_i, p, weight=(0.0, 1.0), scale=1e-4, delay=(1, 10)),
             Projection(N.SPK_POP_NEURONS, n_e, n_i, 0, n_e + n_i, p, weight=(-1.0, 0.0), scale=5e-4,
                        delay=(1, 10))]
    gen = GenNetwork(groups=groups, projections=projs, n_inputs=n_in, rates=np.full(n_in, 20.0, np.float32),
                     seed=5, connectivity_seed=6)
    a = Net.generate(gen)
    b = Net.generate(gen, schedule(8, 128, 0, 0))
    S = a.synapse_count()
    mu = gen.expected_synapses()
    assert abs(S - mu) < 6 * np.sqrt(mu), (S, mu)
    assert b.synapse_count() == S
    wa, wb = a.weights(S), b.weights(S)
    np.testing.assert_array_equal(wa.view(np.uint32), wb.view(np.uint32))
    assert (np.abs(wa) <= 1e-3).all()
    for n in (a, b):
        n.run_steps(300, False)
        assert n.synchronize() == 0
    ia, ta = a.spikes()
    ib, tb = b.spikes()
    assert len(ia) > 1000
    np.testing.assert_array_equal(ia, ib)
    np.testing.assert_array_equal(ta.view(np.uint32), tb.view(np.uint32))
    assert a.events() == b.events()


def desc_from_gen(gen: GenNetwork, arrays: dict) -> descs.Desc:
    """The generated network as an explicit descriptor: the generator's
    constants with the oracle's synapses."""
    dd = gen.desc
    groups = [dict(count=g.count, tau_m=g.tau_m, R=g.R, v0=g.v0, vreset=g.vreset, theta=g.theta,
                   v_init_lo=g.v_init_lo, v_init_hi=g.v_init_hi) for g in (dd.groups[i] for i in range(dd.n_groups))]
    rates = np.ctypeslib.as_array(dd.input_rates, (dd.n_inputs,)).copy() if dd.n_inputs else None
    return descs.Desc(kind=dd.synapse_kind, groups=groups, refractory=dd.refractory_period,
                      i_bg=dd.background_current, n_inputs=dd.n_inputs, rates=rates, pre=arrays["pre"],
                      post=arrays["post"], weight=arrays["weight"], scale=arrays["scale"], delay=arrays["delay"],
                      label=arrays["label"], plastic=arrays["plastic"] if dd.has_stdp else None,
                      stdp=dd.stdp if dd.has_stdp else None, seed=dd.seed, record_inputs=bool(dd.record_inputs),
                      stdp_rule=dd.stdp_rule)


@pytest.mark.parametrize("seed", range(12))
def test_random_generated_networks(seed):
    """Seeded random generator inputs: 40-1,500 neurons in one or two groups,
    0-400 inputs, projections from the inputs and each group onto two post
    ranges (some left out) with p from 0.001 to 1, delay ranges per projection
    (the smallest low delay sets the timestep grouping), plastic input
    synapses under the event-driven or the Evans rule, planner, tile or
    post-range schedules.  The synapses equal the oracle's restatement of the
    generator, and runs equal the oracle on those synapses."""
    from spike_gb300.networks import EVANS_STDP
    rng = np.random.default_rng(7000 + seed)
    n = int(rng.integers(40, 1500))
    n_in = int(rng.choice([0, int(rng.integers(1, 400))]))
    n_exc = int(rng.integers(max(1, n // 2), n + 1))
    lif = dict(tau_m=float(rng.uniform(0.01, 0.03)), R=1e8, v0=0.0, vreset=0.0, theta=0.02, v_init_lo=0.0,
               v_init_hi=0.019)
    groups = [dict(count=n_exc, **lif)] + ([dict(count=n - n_exc, **lif)] if n > n_exc else [])
    d_min = int(rng.choice([1, 1, 2, 3]))
    d_max = d_min + int(rng.integers(0, 12))
    plastic = d_min == 1 and n_in > 0 and rng.random() < 0.6
    rule = N.SPK_STDP_EVANS if plastic and rng.random() < 0.5 else N.SPK_STDP_WEIGHT_DEPENDENT
    cut = int(rng.integers(1, n)) if n > 1 else 1
    projs = []
    sources = [(N.SPK_POP_INPUTS, 0, n_in, (0.0, 1.0), 4e-4), (N.SPK_POP_NEURONS, 0, n_exc, (0.0, 1.0), 5e-4),
               (N.SPK_POP_NEURONS, n_exc, n - n_exc, (-1.0, -0.2), 2e-3)]
    for pop, start, count, w, scale in sources:
        if count == 0:
            continue
        for ps, pc in ((0, cut), (cut, n - cut)):
            if pc == 0 or rng.random() < 0.2:
                continue
            p = float(rng.choice([rng.uniform(0.001, 0.02), rng.uniform(0.02, 0.2), 1.0]))
            # the first projection's low delay is d_min (plasticity needs grouping 1)
            lo = int(rng.integers(d_min, d_max + 1)) if projs else d_min
            projs.append(Projection(pop, start, count, ps, pc, p, weight=w, scale=scale,
                                    delay=(lo, int(rng.integers(lo, d_max + 1))),
                                    plastic=plastic and pop == N.SPK_POP_INPUTS))
    if not projs:
        projs.append(Projection(N.SPK_POP_NEURONS, 0, n_exc, 0, n, 0.05, weight=(0.0, 1.0), scale=5e-4,
                                delay=(d_min, d_max)))
    rates = rng.uniform(5, 60, n_in).astype(np.float32) if n_in else None
    stdp = (EVANS_STDP if rule == N.SPK_STDP_EVANS else STDP) if plastic else None
    gen = GenNetwork(groups=groups, projections=projs, n_inputs=n_in, rates=rates, stdp=stdp,
                     i_bg=float(rng.uniform(0.019, 0.03)), seed=seed + 1, connectivity_seed=seed + 2,
                     record_inputs=bool(rng.integers(0, 2)), stdp_rule=rule)
    sched = [None, schedule(4, 32, 0, 0), schedule(8, 64, 0, 0), schedule(1, 512, 0, 0)][int(rng.integers(0, 4))]
    arrays = generate_synapses(gen.desc)
    S = len(arrays["pre"])
    g = Net.generate(gen, sched)
    assert g.synapse_count() == S
    np.testing.assert_array_equal(g.weights(S).view(np.uint32), delivered(arrays, plastic).view(np.uint32))
    ref = desc_from_gen(gen, arrays)  # owns the arrays its descriptor points into
    o = OracleNet(ref.desc)
    G = o.timestep_grouping()
    assert g.timestep_grouping() == G
    for on, k in ((True, 150), (False, 60), (True, 120)):
        g.run_steps(G * k, on)
        o.run_steps(G * k, on)
    assert g.synchronize() == 0
    assert_same(g, o, n, n_in, 1, tag=f"seed {seed} n {n} n_in {n_in} G {G} {sched}")
    # a generated network reads back the value each synapse delivers: the
    # plastic weights as the oracle holds them, w * scale for static synapses
    pl = arrays["plastic"].astype(bool) & plastic
    w = g.weights(S)
    np.testing.assert_array_equal(w[pl].view(np.uint32), o.weights()[pl].view(np.uint32))
    np.testing.assert_array_equal(w[~pl].view(np.uint32), delivered(arrays, plastic)[~pl].view(np.uint32))
