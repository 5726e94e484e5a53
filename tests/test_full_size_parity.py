"""The benchmark networks at (or near) their full sizes against the oracle,
bit for bit (GPU).

The other parity tests use networks of a few hundred to a few thousand
neurons; these run the shapes the throughput numbers are measured on:

* the Brunel network of Examples/Brunel10K.cpp at its full size (10,000
  excitatory + 2,500 inhibitory voltage-jump LIF neurons, 10,000 Poisson
  inputs, in-degree 0.1, delays 1-20 steps, 28.1 M synapses) for its full
  2 s (20,000 timesteps), built by the host front end (the reference's
  rand() order);
* the plastic feed-forward network at a quarter of its size (12,500 Poisson
  inputs with log-normal rates onto 50,000 LIF neurons, 1,000 afferents each,
  5.0e7 synapses of which 4.5e7 follow weight-dependent STDP) for 500
  timesteps, with every weight compared; its weights are scaled to 0.4 mV
  (the benchmark network's 0.2 mV leaves the neurons below threshold for
  the first 50 ms, so no weight would change);
* instance 31 of the 256-instance sweep (44,032 neurons, p = 0.0249, STDP on
  its input synapses, 8.7e7 synapses drawn on the GPU) in bulk mode, under
  the sweep's tile schedule and under post ranges of 512, 2,048 and 4,096 posts
  per CTA, for 400 timesteps, against the oracle run on the synapses of the
  oracle's own restatement of the generator.

The oracle runs on every host core (post-range threads give the sequential
result bit for bit).
"""
import os

import numpy as np
import pytest

from engine_checks import assert_same, bits
from oracle import OracleNet
from oracle.binding import generate_synapses
from spike_gb300 import Batch, Net, networks, schedule
from spike_gb300 import _native as N
from test_generate import delivered

pytestmark = pytest.mark.gpu

THREADS = max(1, min(os.cpu_count() or 1, 32))


def test_brunel_full_size_two_seconds():
    m = networks.brunel()
    d = m.desc()
    assert d.n_synapses == 28_125_000
    net = Net.from_desc(d)
    o = OracleNet(d, threads=THREADS)
    for seconds in (0.07, 0.53, 1.4):
        net.run(seconds)
        o.run(seconds)
    assert net.synchronize() == 0
    assert net.current_time() == o.current_time()
    assert_same(net, o, 12500, 10000, 1, tag="brunel full")
    ids, _ = o.spikes()
    assert len(ids) > 500_000, len(ids)


def test_plastic_feed_forward_quarter_size_500_steps():
    m = networks.plastic_ff(n_in=12500, n_neurons=50000, ff=900, rec=100, w_scale=4.0e-4)
    d = m.desc()
    assert d.n_synapses == 49_950_000
    net = Net.from_desc(d)
    o = OracleNet(d, threads=THREADS)
    for plastic, steps in ((True, 300), (False, 50), (True, 150)):
        net.run_steps(steps, plastic)
        o.run_steps(steps, plastic)
    assert net.synchronize() == 0
    assert_same(net, o, 50000, 12500, 1, weights=True, tag="plastic_ff quarter")
    w0 = np.ctypeslib.as_array(d.weight, (d.n_synapses,))
    changed = int((net.weights(d.n_synapses) != w0).sum())
    assert changed > 1_000_000, changed


def _sweep_instance(k: int):
    rng = np.random.default_rng(42)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(50000), 256)).astype(int)
    ps = rng.uniform(0.01, 0.05, 256)
    gs = rng.uniform(3.0, 7.0, 256)
    return networks.sweep_instance(int(sizes[k]), float(ps[k]), float(gs[k]), k < 128, seed=1000 + 7 * k)


@pytest.fixture(scope="module")
def sweep31():
    gen = _sweep_instance(31)
    assert gen.desc.n_neurons == 44032 and gen.desc.has_stdp
    arrays = generate_synapses(gen.desc)
    import descs
    dd = gen.desc
    groups = [dict(count=g.count, tau_m=g.tau_m, R=g.R, v0=g.v0, vreset=g.vreset, theta=g.theta,
                   v_init_lo=g.v_init_lo, v_init_hi=g.v_init_hi) for g in (dd.groups[i] for i in range(dd.n_groups))]
    rates = np.ctypeslib.as_array(dd.input_rates, (dd.n_inputs,)).copy()
    ref = descs.Desc(kind=dd.synapse_kind, groups=groups, refractory=dd.refractory_period, i_bg=dd.background_current,
                     n_inputs=dd.n_inputs, rates=rates, pre=arrays["pre"], post=arrays["post"],
                     weight=arrays["weight"], scale=arrays["scale"], delay=arrays["delay"], label=arrays["label"],
                     plastic=arrays["plastic"], stdp=dd.stdp, seed=dd.seed, stdp_rule=dd.stdp_rule)
    o = OracleNet(ref.desc, threads=THREADS)
    steps = 400
    o.run_steps(steps)
    return gen, arrays, o, steps


@pytest.mark.parametrize("sched", [schedule(8, 64, 0, 100), schedule(1, 512, 0, 100), schedule(1, 2048, 0, 100),
                                   schedule(1, 4096, 0, 100)],
                         ids=["tiles8x64", "range512", "range2048", "range4096"])
def test_sweep_instance_44k_bulk_mode_with_stdp(sweep31, sched):
    gen, arrays, o, steps = sweep31
    S = len(arrays["pre"])
    g = Net.generate(gen, sched)
    assert g.synapse_count() == S
    b = Batch([g], schedule(0, 0, 0, 100))
    b.set_mode(N.SPK_BATCH_BULK)
    b.run_steps(steps)
    assert b.synchronize() == 0
    n, n_in = gen.desc.n_neurons, gen.desc.n_inputs
    assert_same(g, o, n, n_in, 1, tag=f"sweep31 {sched.warps_per_cta}x{sched.tile_posts}")
    plastic = arrays["plastic"].astype(bool)
    w = g.weights(S)
    np.testing.assert_array_equal(bits(w[plastic]), bits(o.weights()[plastic]))
    assert (w[plastic] != delivered(arrays, True)[plastic]).sum() > 100_000
    assert len(o.spikes()[0]) > 10_000
