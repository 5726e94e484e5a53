"""STDP rules with two traces per plastic synapse (GPU): the Evans rule
(Spike/Backend/CUDA/Plasticity/EvansSTDPPlasticity.cu), the inhibitory
rule of Vogels et al. 2011 (Spike/Backend/CUDA/Plasticity/
InhibitorySTDPPlasticity.cu) and the custom rule (Spike/Backend/CUDA/
Plasticity/CustomSTDPPlasticity.cu), with accumulating and nearest-spike
traces.  All update every plastic synapse every timestep and see a presynaptic
spike when it arrives; the engine runs them in bulk mode.  Checked against the
oracle bit for bit (spikes, state, ring, weights), across runs with plasticity
off, in a batch beside a network with the event-driven rule, and through a
snapshot; the front end's descriptor mapping is checked on the CPU."""
import numpy as np
import pytest

import descs
from engine_checks import assert_same, bits
from oracle import OracleNet
from restated_rules import rasters_of, restated_rule
from spike_gb300 import Batch, Net, schedule
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams


# Evans: a_plus = alpha_C, a_minus = alpha_D, tau_plus = tau_C, tau_minus = tau_D
EVANS = STDPParams(a_plus=0.5, a_minus=0.5, tau_plus=0.004, tau_minus=0.005, lambda_=0.0, alpha=0.0, w_max=1.0)
# inhibitory: tau_plus = tau_istdp, lambda = learningrate, alpha = targetrate
VOGELS = STDPParams(a_plus=0.0, a_minus=0.0, tau_plus=0.02, tau_minus=0.02, lambda_=0.0004, alpha=10.0, w_max=1.0)
# custom: lambda = learning_rate, alpha = a_star, clip_upper = nearest_spike_only
CUSTOM = STDPParams(a_plus=1.0, a_minus=0.8, tau_plus=0.02, tau_minus=0.03, lambda_=1.0e-5, alpha=0.1, w_max=2.0e-3)
CUSTOM_NEAREST = STDPParams(a_plus=1.0, a_minus=0.8, tau_plus=0.02, tau_minus=0.03, lambda_=2.0e-5, alpha=0.1,
                            w_max=2.0e-3, clip_upper=True)
RULES = [(N.SPK_STDP_EVANS, EVANS), (N.SPK_STDP_INHIBITORY, VOGELS), (N.SPK_STDP_CUSTOM, CUSTOM),
         (N.SPK_STDP_CUSTOM, CUSTOM_NEAREST)]
gpu = pytest.mark.gpu


@pytest.mark.parametrize("rule,sp", RULES)
def test_oracle_rules_follow_the_reference_kernels(rule, sp):
    """The oracle's rule restatement against a second one written from the
    reference's kernels, driven by the oracle's own rasters (CPU)."""
    n, n_in, steps = 300, 200, 700
    d = descs.random_voltage_net(n=n, n_in=n_in, plastic=True, stdp=sp, stdp_rule=rule, seed=21)
    o = OracleNet(d.desc)
    o.run_steps(steps, True)
    rasters = rasters_of(o, d, steps, n, n_in)
    assert rasters[0].sum() > 20 and rasters[1].sum() > 100
    want = restated_rule(rule, sp, d, rasters, rasters[0], steps, int(0.8 * n))
    got = o.weights()
    assert (want != d.arrays["weight"]).sum() > 50  # the rule moved weights
    np.testing.assert_array_equal(bits(got), bits(want))


def net_desc(rule, sp, seed=5):
    return descs.random_voltage_net(n=300, n_in=200, plastic=True, stdp=sp, stdp_rule=rule, seed=seed)


@gpu
@pytest.mark.parametrize("rule,sp", RULES)
def test_rule_matches_oracle(rule, sp):
    d = net_desc(rule, sp)
    net = Net.from_desc(d.desc)
    o = OracleNet(d.desc)
    for plastic, t in ((True, 0.03), (False, 0.01), (True, 0.03)):
        net.run(t, plastic)
        o.run(t, plastic)
    assert net.synchronize() == 0
    assert_same(net, o, 300, 200, 1, weights=True, tag=f"rule {rule}")
    w = net.weights(o.n_synapses)
    assert (w != d.arrays["weight"]).sum() > 100  # the rule moved weights
    assert len(o.spikes()[0]) > 50


@gpu
@pytest.mark.parametrize("rule,sp", RULES)
def test_rule_in_a_batch_beside_the_event_driven_rule(rule, sp):
    wd = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0)
    da = net_desc(rule, sp, seed=9)
    db = descs.random_voltage_net(n=250, n_in=150, plastic=True, stdp=wd, seed=10)
    sched = schedule(8, 32, 0, 0)  # a batch's networks share warps per CTA
    batched = [Net.from_desc(da.desc, sched), Net.from_desc(db.desc, sched)]
    b = Batch(batched)  # a network with a per-synapse-trace rule puts the batch in bulk mode
    with pytest.raises(N.SpikeError):
        b.set_mode(N.SPK_BATCH_WAVES)
    b.run_steps(500, True)
    assert b.synchronize() == 0
    for x, d, n, n_in in ((batched[0], da, 300, 200), (batched[1], db, 250, 150)):
        o = OracleNet(d.desc)
        o.run_steps(500, True)
        assert_same(x, o, n, n_in, 1, weights=True, tag="batched")
    b.close()


@gpu
def test_snapshot_carries_the_rule_state():
    d = net_desc(N.SPK_STDP_INHIBITORY, VOGELS)
    a = Net.from_desc(d.desc)
    a.run(0.02)
    snap = a.snapshot()
    a.run(0.02)
    assert a.synchronize() == 0
    b = Net.from_desc(d.desc)
    b.restore(snap)
    b.run(0.02)
    assert b.synchronize() == 0
    S = len(d.arrays["weight"])
    np.testing.assert_array_equal(bits(a.weights(S)), bits(b.weights(S)))
    np.testing.assert_array_equal(bits(a.state(N.SPK_FIELD_V, 300)), bits(b.state(N.SPK_FIELD_V, 300)))


def brunel_with_rule(rule, sp):
    """The reference-built Brunel case with the rule on its excitatory
    recurrent synapses, through the C++ front end."""
    import cases
    from spike_gb300 import Model
    from spike_gb300.model import SynapseParams
    m = Model(N.SPK_SYN_VOLTAGE, N.SPK_INPUT_POISSON, synapse_seed=42, timestep=float(cases.DT))
    rid = m.add_stdp_rule(sp, rule)
    args = (0.0, 0.0, 20.0e-3, 2.0e-3, 0.0)
    gin = m.add_input_group(150, 20.0)
    ge = m.add_neuron_group(cases._lif(160, *args))
    gi = m.add_neuron_group(cases._lif(40, *args))
    J = float(cases.F(0.1) * cases.F(10.0 ** -3))
    dl = (cases.steps(1), cases.steps(20))
    m.connect_with_sparsity(gin, ge, 0.1, SynapseParams(weight_range=(0.0, float(cases.F(2.0) * cases.F(J))),
                                                         delay_range=dl))
    m.connect_with_sparsity(ge, ge, 0.1, SynapseParams(weight_range=(J, J), delay_range=dl, plasticity_rule=rid))
    m.connect_with_sparsity(gi, ge, 0.1, SynapseParams(weight_range=(-5 * J, -5 * J), delay_range=dl))
    m.connect_with_sparsity(ge, gi, 0.1, SynapseParams(weight_range=(J, J), delay_range=dl))
    return m


@pytest.mark.parametrize("rule,sp", RULES)
def test_front_end_maps_the_rule_into_the_descriptor(rule, sp):
    """EvansSTDPPlasticity / InhibitorySTDPPlasticity / CustomSTDPPlasticity
    flatten into the descriptor's rule and field mapping and back (CPU)."""
    m = brunel_with_rule(rule, sp)
    d = m.desc()  # points into the model's arrays: keep m alive
    assert d.stdp_rule == rule and d.has_stdp == 1
    st = d.stdp
    if rule == N.SPK_STDP_EVANS:
        got = (st.tau_minus, st.tau_plus, st.a_minus, st.a_plus, st.w_max)
        want = (sp.tau_minus, sp.tau_plus, sp.a_minus, sp.a_plus, 1.0)
    elif rule == N.SPK_STDP_INHIBITORY:
        got = (st.tau_plus, st.tau_minus, st.lambda_, st.alpha, st.w_max)
        want = (sp.tau_plus, sp.tau_plus, sp.lambda_, sp.alpha, 1.0)
    else:
        got = (st.a_minus, st.a_plus, st.tau_minus, st.tau_plus, st.w_max, st.lambda_, st.alpha, st.clip_upper)
        want = (sp.a_minus, sp.a_plus, sp.tau_minus, sp.tau_plus, sp.w_max, sp.lambda_, sp.alpha, int(sp.clip_upper))
    np.testing.assert_array_equal(np.float32(got), np.float32(want))


@gpu
@pytest.mark.parametrize("rule,sp", RULES)
def test_rule_through_the_model_api(rule, sp):
    """The reference-built Brunel case with the rule on its excitatory
    recurrent synapses: the front end's network matches the oracle."""
    m = brunel_with_rule(rule, sp)
    d = m.desc()  # points into the model's arrays: keep m alive
    o = OracleNet(d)
    net = Net.from_desc(d)
    net.run(0.1)
    o.run(0.1)
    assert net.synchronize() == 0
    assert_same(net, o, 200, 150, 1, weights=True, tag=f"model rule {rule}")
