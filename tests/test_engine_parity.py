"""The CUDA engine against the oracle, bit for bit (GPU).

Every comparison below is exact: spike ids and float times, membrane
potentials, synaptic traces, ring buffer, input next-spike times, STDP traces
and weights.  The engine runs with -fmad=false and ordered accumulation, the
oracle with -ffp-contract=off in the canonical order, so any difference is a
bug.  Schedules are varied to exercise the one-CTA and multi-CTA paths, tile
sizes that split rows differently, and launches that cut runs into blocks.
"""
import numpy as np
import pytest

import cases
import descs
from engine_checks import assert_same, bits, ring_depth  # noqa: F401
from oracle import OracleNet
from spike_gb300 import Batch, Net, schedule
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams

pytestmark = pytest.mark.gpu

STDP = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0)


def test_vogels_abbott_small_mixed_delays():
    m = cases.ref_va(True)
    d = m.desc()
    o = OracleNet(d)
    net = Net.from_desc(d)
    for _ in range(3):
        net.run(0.02)
        o.run(0.02)
    assert net.synchronize() == 0
    assert_same(net, o, 400, 0, 2, tag="va_mix")
    assert len(o.spikes()[0]) > 100


@pytest.mark.parametrize("sched", [None, schedule(8, 32, 0, 0), schedule(4, 64, 0, 7), schedule(2, 32, 6, 50)])
def test_random_voltage_net_with_stdp_across_schedules(sched):
    d = descs.random_voltage_net(n=300, n_in=200, plastic=True, stdp=STDP)
    o = OracleNet(d.desc)
    net = Net.from_desc(d.desc, sched)
    net.run(0.03)
    o.run(0.03)
    net.run(0.02, plasticity_on=False)
    o.run(0.02, plasticity_on=False)
    net.run(0.02)
    o.run(0.02)
    assert net.synchronize() == 0
    assert_same(net, o, 300, 200, 1, weights=True, tag=str(net.schedule()))
    pre_g = net.state(N.SPK_FIELD_PRE_TRACE, 500)
    post_g = net.state(N.SPK_FIELD_POST_TRACE, 300)
    pre_o = o.state(N.SPK_FIELD_PRE_TRACE, 500)
    post_o = o.state(N.SPK_FIELD_POST_TRACE, 300)
    # oracle reports traces only for neurons that carry plastic synapses
    mp = pre_o != 0
    np.testing.assert_array_equal(bits(pre_g[mp]), bits(pre_o[mp]))
    mq = post_o != 0
    np.testing.assert_array_equal(bits(post_g[mq]), bits(post_o[mq]))
    assert not np.array_equal(net.weights(o.n_synapses), d.arrays["weight"])


def test_reference_brunel_case_with_stdp():
    m = cases.ref_brunel()
    d = m.desc()
    o = OracleNet(d)
    net = Net.from_desc(d)
    net.run(0.1)
    o.run(0.1)
    assert net.synchronize() == 0
    assert_same(net, o, 200, 150, 1, weights=True, tag="brunel")


def test_current_synapses_two_labels():
    rng = np.random.default_rng(3)
    n, S = 120, 3000
    pre = rng.integers(-50, n, S)
    post = rng.integers(0, n, S)
    d = descs.Desc(kind=N.SPK_SYN_CURRENT, n_labels=2, label_tau=[0.003, 0.008],
                   groups=[dict(count=n, tau_m=0.02, R=1e8, v0=-0.07, vreset=-0.07, theta=-0.055)],
                   refractory=0.002, i_bg=0.0, n_inputs=50, rates=rng.uniform(5, 60, 50),
                   pre=pre, post=post, weight=rng.uniform(0, 3e-10, S), scale=np.ones(S),
                   delay=np.maximum(1, rng.integers(0, 9, S)), label=(pre < 0).astype(int) + 0,
                   record_inputs=True)
    o = OracleNet(d.desc)
    net = Net.from_desc(d.desc, schedule(2, 32, 0, 0))
    net.run(0.08)
    o.run(0.08)
    assert_same(net, o, n, 50, 2, tag="current")


def test_run_semantics_reset_and_stimulus():
    m = cases.ref_shapes()
    d = m.desc()
    o = OracleNet(d)
    net = Net.from_desc(d)
    for sec in (0.013, 0.0071, 0.05):
        net.run(sec)
        o.run(sec)
    assert net.current_time() == o.current_time()
    net.reset_state()
    o.reset_state()
    net.run(0.02)
    o.run(0.02)
    net.reset_time()
    o.reset_time()
    net.run_steps(37)
    o.run_steps(37)
    assert_same(net, o, 32, 20, 1, tag="shapes")


def test_batch_equals_each_network_alone():
    ds = [descs.random_voltage_net(n=n, n_in=ni, seed=s, plastic=(s % 2 == 0), stdp=STDP)
          for n, ni, s in ((150, 100, 1), (420, 90, 2), (64, 300, 3), (700, 50, 4))]
    nets = [Net.from_desc(x.desc, schedule(4, 0, 0, 0)) for x in ds]
    orcs = [OracleNet(x.desc) for x in ds]
    b = Batch(nets)
    b.run_steps(333)
    assert b.synchronize() == 0
    for x, net, o in zip(ds, nets, orcs):
        o.run_steps(333)
        assert_same(net, o, x.desc.n_neurons, x.desc.n_inputs, 1, weights=True, tag="batch")


def test_full_vogels_abbott_one_second():
    from spike_gb300 import networks
    m = networks.vogels_abbott()
    d = m.desc()
    o = OracleNet(d)
    net = Net.from_desc(d)
    net.run(1.0)
    o.run(1.0)
    assert net.synchronize() == 0
    assert_same(net, o, 4000, 0, 2, tag="va_full")
