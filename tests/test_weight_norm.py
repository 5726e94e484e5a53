"""Weight normalisation (WeightNormSTDPPlasticity, Spike/Plasticity/
WeightNormSTDPPlasticity.cpp and Spike/Backend/CUDA/Plasticity/
WeightNormSTDPPlasticity.cu): every timestep, each post's plastic weights are
divided by sqrt(S + change) / sqrt(S), the change of their sum of squares
against the initial weights.  It runs before or after the STDP rule, in the
order the rules were added.

CPU: the oracle against a restatement written from the reference kernels,
driven by the oracle's rasters, and the C++ front end's descriptor mapping,
including settarget.  GPU: the engine against the oracle bit for bit with the
event-driven rule (normalised after it: a first propagation pass that only
updates weights, then the normalisation, then a pass that delivers; or before
it) and with the per-synapse-trace rules, in a batch beside networks without
it, and through the model API."""
import numpy as np
import pytest

import descs
from engine_checks import assert_same, bits
from oracle import OracleNet
from restated_rules import Normaliser, host_powf, rasters_of, restated_rule
from spike_gb300 import Batch, Net, schedule
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams

gpu = pytest.mark.gpu

WD = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0)
EVANS = STDPParams(a_plus=0.5, a_minus=0.5, tau_plus=0.004, tau_minus=0.005, lambda_=0.0, alpha=0.0, w_max=1.0)
CUSTOM = STDPParams(a_plus=1.0, a_minus=0.8, tau_plus=0.02, tau_minus=0.03, lambda_=1.0e-5, alpha=0.1, w_max=2.0e-3)
VOGELS = STDPParams(a_plus=0.0, a_minus=0.0, tau_plus=0.02, tau_minus=0.02, lambda_=0.0004, alpha=10.0, w_max=1.0)
AFTER, BEFORE = N.SPK_NORM_AFTER_RULE, N.SPK_NORM_BEFORE_RULE

CASES = [
    (N.SPK_STDP_WEIGHT_DEPENDENT, WD, AFTER),
    (N.SPK_STDP_WEIGHT_DEPENDENT, WD, BEFORE),
    (N.SPK_STDP_EVANS, EVANS, AFTER),
    (N.SPK_STDP_CUSTOM, CUSTOM, BEFORE),
    (N.SPK_STDP_INHIBITORY, VOGELS, AFTER),
]


def net_desc(rule, sp, norm, seed=5, n=300, n_in=200, **kw):
    return descs.random_voltage_net(n=n, n_in=n_in, plastic=True, stdp=sp, stdp_rule=rule, weight_norm=norm,
                                    seed=seed, **kw)


CUSTOM_NEAREST = STDPParams(a_plus=1.0, a_minus=0.8, tau_plus=0.02, tau_minus=0.03, lambda_=2.0e-5, alpha=0.1,
                            w_max=2.0e-3, clip_upper=True)
ORACLE_CASES = [c for c in CASES if c[0] != N.SPK_STDP_WEIGHT_DEPENDENT] + [
    (N.SPK_STDP_INHIBITORY, VOGELS, BEFORE),
    (N.SPK_STDP_CUSTOM, CUSTOM_NEAREST, AFTER),
    (N.SPK_STDP_EVANS, EVANS, BEFORE),
]


@pytest.mark.parametrize("rule,sp,norm", ORACLE_CASES)
def test_oracle_normalisation_follows_the_reference_kernels(rule, sp, norm):
    """The oracle's trace rule with the normalisation before or after it,
    against the restatement driven by the oracle's rasters (CPU)."""
    n, n_in, steps = 300, 200, 500
    d = net_desc(rule, sp, norm, seed=21)
    o = OracleNet(d.desc)
    o.run_steps(steps, True)
    rasters = rasters_of(o, d, steps, n, n_in)
    assert rasters[0].sum() > 20
    want = restated_rule(rule, sp, d, rasters, rasters[0], steps, int(0.8 * n), norm=norm)
    np.testing.assert_array_equal(bits(o.weights()), bits(want))
    # the normalisation changed the outcome
    plain = restated_rule(rule, sp, d, rasters, rasters[0], steps, int(0.8 * n))
    assert (bits(plain) != bits(want)).sum() > 50


def test_normaliser_restores_the_l2_norm():
    """One normalisation step brings each post's plastic weights back to the
    norm sqrt(S) (to float rounding), and leaves unmoved weights alone."""
    rng = np.random.default_rng(3)
    post = rng.integers(0, 20, 400)
    w0 = rng.uniform(0.1, 1.0, 400).astype(np.float32)
    norm = Normaliser(post, w0, 20)
    np.testing.assert_array_equal(norm(w0.copy()), w0)
    w = (w0 * rng.uniform(0.5, 1.5, 400)).astype(np.float32)
    out = norm(w)
    for q in range(20):
        m = post == q
        np.testing.assert_allclose(np.sqrt((out[m].astype(np.float64) ** 2).sum()),
                                   np.sqrt((w0[m].astype(np.float64) ** 2).sum()), rtol=1e-5)


def brunel_model(rule, sp, order, settarget=False, target=0.0):
    """The reference-built Brunel case with the STDP rule and the
    normalisation on its excitatory recurrent synapses; `order` is the order
    the two rules are added in."""
    import cases
    from spike_gb300 import Model
    from spike_gb300.model import SynapseParams
    m = Model(N.SPK_SYN_VOLTAGE, N.SPK_INPUT_POISSON, synapse_seed=42, timestep=float(cases.DT))
    if order == AFTER:
        rid = m.add_stdp_rule(sp, rule)
        nid = m.add_weight_norm_rule(settarget, target)
    else:
        nid = m.add_weight_norm_rule(settarget, target)
        rid = m.add_stdp_rule(sp, rule)
    args = (0.0, 0.0, 20.0e-3, 2.0e-3, 0.0)
    gin = m.add_input_group(150, 20.0)
    ge = m.add_neuron_group(cases._lif(160, *args))
    gi = m.add_neuron_group(cases._lif(40, *args))
    J = float(cases.F(0.1) * cases.F(10.0 ** -3))
    dl = (cases.steps(1), cases.steps(20))
    m.connect_with_sparsity(gin, ge, 0.1, SynapseParams(weight_range=(0.0, float(cases.F(2.0) * cases.F(J))),
                                                         delay_range=dl))
    m.connect_with_sparsity(ge, ge, 0.1, SynapseParams(weight_range=(0.5 * J, 1.5 * J), delay_range=dl,
                                                         plasticity_rule=rid, plasticity_rule_2=nid))
    m.connect_with_sparsity(gi, ge, 0.1, SynapseParams(weight_range=(-5 * J, -5 * J), delay_range=dl))
    m.connect_with_sparsity(ge, gi, 0.1, SynapseParams(weight_range=(J, J), delay_range=dl))
    return m


@pytest.mark.parametrize("order", [AFTER, BEFORE])
def test_front_end_maps_the_normalisation(order):
    """The rule's place among the model's rules, and without a target the
    initial weights and sums left to the engine (CPU)."""
    m = brunel_model(N.SPK_STDP_WEIGHT_DEPENDENT, WD, order)
    d = m.desc()  # points into the model's arrays: keep m alive
    assert d.weight_norm == order and d.has_stdp == 1 and d.stdp_rule == N.SPK_STDP_WEIGHT_DEPENDENT
    assert not d.norm_initial and not d.norm_sum


def test_front_end_settarget_follows_the_reference_host_code():
    """settarget: the descriptor keeps the unscaled weights (the synapses'
    backend copied them before the rule rescaled the host array), the initial
    weights are the rescaled ones w / sqrt(S) * target, and S := target
    (WeightNormSTDPPlasticity.cpp:31-70, CPU)."""
    target = 2.0e-3
    m = brunel_model(N.SPK_STDP_WEIGHT_DEPENDENT, WD, AFTER, settarget=True, target=target)
    d = m.desc()
    S = d.n_synapses
    w = np.ctypeslib.as_array(d.weight, (S,)).copy()
    post = np.ctypeslib.as_array(d.post, (S,))
    plastic = np.ctypeslib.as_array(d.plastic, (S,)).astype(bool)
    w0 = np.ctypeslib.as_array(d.norm_initial, (S,))
    sums = np.ctypeslib.as_array(d.norm_sum, (d.n_neurons,))
    assert plastic.sum() > 100
    ssq = np.zeros(d.n_neurons, np.float32)
    for s in np.nonzero(plastic)[0]:
        ssq[post[s]] = np.float32(ssq[post[s]] + host_powf(w[s], 2.0))
    want = w.copy()
    idx = np.nonzero(plastic)[0]
    want[idx] = (w[idx] / np.sqrt(ssq[post[idx]])) * np.float32(target)
    np.testing.assert_array_equal(bits(w0), bits(want.astype(np.float32)))
    np.testing.assert_array_equal(sums, np.full(d.n_neurons, target, np.float32))


def test_front_end_rejects_unsupported_normalisations():
    """Normalisation on synapses other than the STDP rule's, or without an
    STDP rule: refused when the model is flattened (CPU)."""
    import cases
    from spike_gb300 import Model
    from spike_gb300.model import SynapseParams
    m = Model(N.SPK_SYN_VOLTAGE, N.SPK_INPUT_POISSON, synapse_seed=42, timestep=float(cases.DT))
    rid = m.add_stdp_rule(WD)
    nid = m.add_weight_norm_rule()
    gin = m.add_input_group(50, 20.0)
    ge = m.add_neuron_group(cases._lif(60, 0.0, 0.0, 20.0e-3, 2.0e-3, 0.0))
    dl = (cases.steps(1), cases.steps(5))
    m.connect_with_sparsity(gin, ge, 0.2, SynapseParams(weight_range=(1e-4, 1e-4), delay_range=dl,
                                                         plasticity_rule=rid))
    m.connect_with_sparsity(ge, ge, 0.2, SynapseParams(weight_range=(1e-4, 1e-4), delay_range=dl,
                                                         plasticity_rule=rid, plasticity_rule_2=nid))
    with pytest.raises(N.SpikeError):
        m.desc()
    # the engine refuses a descriptor asking for it without an STDP rule
    d = descs.random_voltage_net(n=50, n_in=20, weight_norm=AFTER)
    import ctypes
    h = ctypes.c_void_p()
    assert N.lib().spk_net_create(ctypes.byref(d.desc), None, ctypes.byref(h)) == N.SPK_ERR_INVALID


@gpu
@pytest.mark.parametrize("rule,sp,norm", CASES)
def test_normalisation_matches_oracle(rule, sp, norm):
    d = net_desc(rule, sp, norm)
    net = Net.from_desc(d.desc)
    o = OracleNet(d.desc)
    for plastic, t in ((True, 0.03), (False, 0.01), (True, 0.03)):
        net.run(t, plastic)
        o.run(t, plastic)
    assert net.synchronize() == 0
    assert_same(net, o, 300, 200, 1, weights=True, tag=f"rule {rule} norm {norm}")
    # the normalisation acted: the same network without it ends elsewhere
    dp = net_desc(rule, sp, N.SPK_NORM_OFF)  # keep the arrays alive while the oracle uses them
    plain = OracleNet(dp.desc)
    for plastic, t in ((True, 0.03), (False, 0.01), (True, 0.03)):
        plain.run(t, plastic)
    S = len(d.arrays["weight"])
    assert (bits(net.weights(S)) != bits(plain.weights())).sum() > 50


@gpu
def test_normalised_networks_in_a_batch():
    """A network normalised after the event-driven rule (two propagation
    passes) beside one normalised after a trace rule, one with the plain
    event-driven rule and a static one, in one bulk batch."""
    sched = schedule(8, 32, 0, 0)
    ds = [net_desc(N.SPK_STDP_WEIGHT_DEPENDENT, WD, AFTER, seed=31, n=260, n_in=150),
          net_desc(N.SPK_STDP_CUSTOM, CUSTOM, AFTER, seed=32, n=200, n_in=120),
          descs.random_voltage_net(n=240, n_in=160, plastic=True, stdp=WD, seed=33),
          descs.random_voltage_net(n=220, n_in=100, seed=34)]
    sizes = [(260, 150), (200, 120), (240, 160), (220, 100)]
    nets = [Net.from_desc(d.desc, sched) for d in ds]
    b = Batch(nets)
    with pytest.raises(N.SpikeError):
        b.set_mode(N.SPK_BATCH_WAVES)
    b.run_steps(400, True)
    b.run_steps(100, False)
    assert b.synchronize() == 0
    for net, d, (n, n_in) in zip(nets, ds, sizes):
        o = OracleNet(d.desc)
        o.run_steps(400, True)
        o.run_steps(100, False)
        assert_same(net, o, n, n_in, 1, weights=True, tag="batched")
    b.close()


@gpu
@pytest.mark.parametrize("order,settarget", [(AFTER, False), (BEFORE, False), (AFTER, True)])
def test_normalisation_through_the_model_api(order, settarget):
    m = brunel_model(N.SPK_STDP_WEIGHT_DEPENDENT, WD, order, settarget=settarget, target=2.0e-3)
    d = m.desc()
    o = OracleNet(d)
    net = Net.from_desc(d)
    net.run(0.1)
    o.run(0.1)
    assert net.synchronize() == 0
    assert_same(net, o, 200, 150, 1, weights=True, tag=f"model norm {order} {settarget}")
