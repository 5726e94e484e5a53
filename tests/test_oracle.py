"""Pins of the oracle: published known answers, hand-computable cases, and
self-consistency (threads, FP64 twin).  CPU only."""
import numpy as np
import pytest

import cases
import descs
from oracle import OracleNet
from oracle.binding import oracle_lib, philox4x32_10
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams

F = np.float32


def test_philox_known_answers():
    """Philox4x32-10 test vectors published with the algorithm (Salmon et al., SC'11)."""
    assert philox4x32_10([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_log_accuracy_over_all_uniforms():
    """The shared logarithm is within 1 ulp of log over every Poisson uniform
    (k * 2^-24, k = 1..2^24), the bound CUDA documents for logf."""
    assert oracle_lib().oracle_log_max_ulp() <= 1.0
    for x in (1.0, 0.5, 0.75, 5.9604644775390625e-08, 0.999999940395):
        assert abs(oracle_lib().oracle_logf(F(x)) - np.log(np.float64(F(x)))) <= 1e-6 * max(1, abs(np.log(x)))


def _single_neuron(i_bg, refractory=0.005, steps=400):
    d = descs.Desc(kind=N.SPK_SYN_VOLTAGE, groups=[dict(count=1, tau_m=0.02, R=1e8, v0=-0.06, vreset=-0.06,
                                                          theta=-0.05)],
                   refractory=refractory, i_bg=i_bg)
    o = OracleNet(d.desc)
    vs = []
    for _ in range(steps):
        o.run_steps(1)
        vs.append(o.state(N.SPK_FIELD_V, 1)[0])
    ids, times = o.spikes()
    return np.array(vs, np.float32), times


def test_single_neuron_matches_float32_recurrence_and_refractory():
    """V_{n+1} = k V0 + (1-k) V_n + k I_bg (LIFSpikingNeurons.cu:169) in float32,
    reset at threshold, frozen for 50 steps after a spike with t_ref = 5 ms and
    updated again at step n + 51 (LIFSpikingNeurons.cu:168)."""
    i_bg = 2.0e-2
    vs, times = _single_neuron(i_bg)
    dt = F(0.0001)
    k = F(dt / F(0.02))
    v, last, spikes = F(-0.06), F(-1000.0), []
    ref = []
    for s in range(len(vs)):
        t = F(F(s) * dt)
        if F(F(F(t + F(0.0) * dt) - last) - F(0.005)) > F(F(0.5) * dt):
            v = F(F(F(k * F(-0.06)) + F(F(F(1) - k) * v)) + F(k * F(i_bg))) + F(0.0)
            if v >= F(-0.05):
                spikes.append(s)
                last = t
                v = F(-0.06)
        ref.append(v)
    assert np.array_equal(vs.view(np.uint32), np.array(ref, np.float32).view(np.uint32))
    steps = np.round(times / 0.0001).astype(int)
    assert list(steps) == spikes and len(spikes) >= 2
    isi = np.diff(steps)
    # every step of the 50 after a spike is frozen at reset, the 51st moves
    for s in spikes[:-1]:
        assert np.all(vs[s + 1:s + 51] == F(-0.06)) and vs[s + 51] != F(-0.06)
    assert np.all(isi > 50)


def test_delay_slot_walk():
    """An input spike at step n reaches a post through a delay-d voltage synapse
    exactly at step n + d: slot (T + d) % B written, read at step T + d
    (SpikingSynapses.cu:127,196 and InlineDeviceFunctions.hpp:86-111)."""
    for d_ in (1, 2, 7, 20):
        w = F(1e-3)
        d = descs.Desc(kind=N.SPK_SYN_VOLTAGE, groups=[dict(count=2, tau_m=1e9, R=1.0, v0=0.0, vreset=0.0,
                                                              theta=1.0)],
                       refractory=0.0, n_inputs=1, rates=[300.0], pre=[-1, -1], post=[0, 1], weight=[w, w],
                       delay=[1, d_], record_inputs=True)
        o = OracleNet(d.desc)
        v = []
        for _ in range(400):
            o.run_steps(1)
            v.append(o.state(N.SPK_FIELD_V, 2).copy())
        v = np.array(v)
        _, tin = o.spikes(N.SPK_POP_INPUTS)
        sin = np.round(tin / 0.0001).astype(int)
        assert len(sin) > 3
        jumps0 = np.flatnonzero(np.diff(np.concatenate([[0.0], v[:, 0]])) > 0)
        jumps1 = np.flatnonzero(np.diff(np.concatenate([[0.0], v[:, 1]])) > 0)
        assert list(jumps0) == [s + 1 for s in sin if s + 1 < 400]
        assert list(jumps1) == [s + d_ for s in sin if s + d_ < 400]


def test_poisson_first_draw_emits_no_spike_and_rate():
    """The first Poisson update after reset only draws (active := true,
    PoissonInputSpikingNeurons.cu:110-125); long-run rate matches."""
    n_in = 400
    d = descs.Desc(kind=N.SPK_SYN_VOLTAGE, groups=[dict(count=1)], n_inputs=n_in, rates=np.full(n_in, 50.0),
                   record_inputs=True)
    o = OracleNet(d.desc)
    o.run_steps(1)
    assert len(o.spikes(N.SPK_POP_INPUTS)[0]) == 0
    o.run(2.0)
    ids, _ = o.spikes(N.SPK_POP_INPUTS)
    rate = len(ids) / (n_in * 2.0001)
    assert abs(rate - 50.0) < 2.0


WD_PARAMS = STDPParams(a_plus=0.005, a_minus=0.00525, lambda_=1.0, alpha=1.0, w_max=1.0)
EVANS_PARAMS = STDPParams(a_plus=0.5, a_minus=0.5, tau_plus=0.004, tau_minus=0.005, lambda_=0.0, alpha=0.0, w_max=1.0)


@pytest.mark.parametrize("rule,sp,norm", [
    (N.SPK_STDP_WEIGHT_DEPENDENT, WD_PARAMS, N.SPK_NORM_OFF),
    (N.SPK_STDP_WEIGHT_DEPENDENT, WD_PARAMS, N.SPK_NORM_AFTER_RULE),
    (N.SPK_STDP_EVANS, EVANS_PARAMS, N.SPK_NORM_BEFORE_RULE),
])
def test_threaded_oracle_is_bit_identical(rule, sp, norm):
    """Post-range threads (with the barriers around the normalisation) give
    the single thread's bits, for the event-driven rule, the normalisation
    after it, and a trace rule with the normalisation before it."""
    d = descs.random_voltage_net(n=240, n_in=160, plastic=True, stdp=sp, stdp_rule=rule, weight_norm=norm)
    a = OracleNet(d.desc)
    b = OracleNet(d.desc, threads=4)
    a.run(0.05)
    b.run(0.05)
    for x, y in zip(a.spikes(), b.spikes()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.state(N.SPK_FIELD_V, 240), b.state(N.SPK_FIELD_V, 240))
    assert np.array_equal(a.weights(), b.weights())
    assert a.events() == b.events()


def test_fp64_twin_agrees_over_short_horizon():
    m = cases.ref_va(True)
    a = OracleNet(m.desc(), 32)
    b = OracleNet(m.desc(), 64)
    a.run(0.005)
    b.run(0.005)
    va = a.state(N.SPK_FIELD_V, 400)
    vb = b.state(N.SPK_FIELD_V, 400)
    assert np.max(np.abs(va - vb)) < 1e-5


def test_weight_dependent_stdp_single_pair():
    """One plastic synapse, pre fires then post fires: LTD on the pre spike is
    -lambda*alpha*w*post_trace/E, LTP on the post spike +lambda*(w_max-w)*pre_trace/E
    (WeightDependentSTDPPlasticity.cu:125-151), evaluated in float32 here."""
    sp = STDPParams(a_plus=0.1, a_minus=0.12, tau_plus=0.02, tau_minus=0.03, lambda_=0.5, alpha=1.5, w_max=1.0)
    # both neurons fire from the background current, at different periods
    d = descs.Desc(kind=N.SPK_SYN_VOLTAGE, groups=[dict(count=1, tau_m=0.02, R=1e8, v0=0.0, vreset=0.0, theta=0.02),
                                                   dict(count=1, tau_m=0.013, R=1e8, v0=0.0, vreset=0.0, theta=0.02)],
                   refractory=0.003, i_bg=0.05, pre=[0], post=[1], weight=[0.5], delay=[1], plastic=[1], stdp=sp)
    o = OracleNet(d.desc)
    dt = F(0.0001)
    Em, Ep = np.exp(F(-(F(1) * dt) / F(0.03)), dtype=F), np.exp(F(-(F(1) * dt) / F(0.02)), dtype=F)
    w = F(0.5)
    pre_tr = post_tr = F(0.0)
    n_pairs = 0
    for s in range(900):
        t = F(o.current_time())  # run_steps(1) starts at the accumulated float time
        o.run_steps(1)
        last = o.state(N.SPK_FIELD_LAST_SPIKE, 2)
        pre_ev = last[0] == t
        post_ev = last[1] == t
        post_tr = F(post_tr * Em)
        post_tr = F(post_tr + (F(F(0.12) * Em) if post_ev else F(0)))
        pre_tr = F(pre_tr * Ep)
        pre_tr = F(pre_tr + (F(F(0.1) * Ep) if pre_ev else F(0)))
        syn = F(0)
        if pre_ev:
            syn = F(syn - F(F(F(F(0.5) * F(1.5)) * w) * F(post_tr * F(F(1) / Em))))
        if post_ev:
            syn = F(syn + F(F(F(0.5) * F(F(1.0) - w)) * F(pre_tr * F(F(1) / Ep))))
        w = F(w + syn)
        if w < 0:
            w = F(0)
        n_pairs += int(pre_ev or post_ev)
        # numpy's exp and the C library's expf may differ in the last place
        assert o.weights()[0] == pytest.approx(float(w), rel=1e-6)
    assert n_pairs >= 8


def test_generator_restatement_order_draws_and_statistics():
    """The oracle's restatement of the device generator: creation order is
    ascending (presynaptic key, post); each pair connects exactly when its
    Philox uniform is <= p; counts, delays and weights follow the projection."""
    from oracle.binding import generate_synapses
    from spike_gb300 import GenNetwork, Projection
    n_in, n = 200, 500
    projs = [Projection(N.SPK_POP_INPUTS, 0, n_in, 0, n, 0.1, weight=(0.0, 1.0), scale=2e-3, delay=(1, 4)),
             Projection(N.SPK_POP_NEURONS, 0, 400, 400, 100, 0.05, weight=(0.5, 1.0), scale=1e-3, delay=(2, 9)),
             Projection(N.SPK_POP_NEURONS, 0, 400, 0, 400, 0.2, weight=(0.5, 1.0), scale=1e-3, delay=(1, 9)),
             Projection(N.SPK_POP_NEURONS, 400, 100, 0, n, 0.3, weight=(-1.0, -0.5), scale=1e-3, delay=(1, 1))]
    gen = GenNetwork(groups=[dict(count=400), dict(count=100)], projections=projs, n_inputs=n_in,
                     rates=np.full(n_in, 10.0, np.float32), connectivity_seed=0x1234567890)
    a = generate_synapses(gen.desc)
    b = generate_synapses(gen.desc)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    pre, post = a["pre"].astype(np.int64), a["post"].astype(np.int64)
    key = np.where(pre < 0, n_in - 1 - (-pre - 1), n_in + pre)
    order = key * n + post
    assert (np.diff(order) > 0).all()
    mu = gen.expected_synapses()
    assert abs(len(pre) - mu) < 6 * np.sqrt(mu)
    seed = 0x1234567890
    for s in range(0, len(pre), max(1, len(pre) // 50)):
        code = (0x80000000 | (-pre[s] - 1)) if pre[s] < 0 else pre[s]
        w = philox4x32_10([post[s] >> 2, code, 0, 0x434f4e4e], [seed & 0xffffffff, seed >> 32])
        u = F(((w[post[s] & 3] >> 8) + 1) * 2.0 ** -24)
        proj = projs[0] if pre[s] < 0 else projs[3] if pre[s] >= 400 else projs[1] if post[s] >= 400 else projs[2]
        assert u <= F(proj.probability)
        assert proj.delay[0] <= a["delay"][s] <= proj.delay[1]
        assert proj.weight[0] <= a["weight"][s] <= proj.weight[1]
    # a pair is in the list exactly when its draw succeeds
    in_list = set(zip(pre[pre >= 400].tolist(), post[pre >= 400].tolist()))
    for p in range(400, 410):
        for q in range(0, 40):
            w = philox4x32_10([q >> 2, p, 0, 0x434f4e4e], [seed & 0xffffffff, seed >> 32])
            u = F(((w[q & 3] >> 8) + 1) * 2.0 ** -24)
            assert (u <= F(0.3)) == ((p, q) in in_list)
