"""Networks shared by the tests.  The ``ref_*`` builders reproduce, through
this repository's model API, exactly the construction calls that
oracle/ref_dump.cpp makes through the reference front end."""
from __future__ import annotations

import numpy as np

from spike_gb300 import _native as N
from spike_gb300.model import LIFParams, Model, STDPParams, SynapseParams

DT = np.float32(0.0001)
F = np.float32


def steps(k):
    """k*dt evaluated in float, as the reference examples write it."""
    return float(F(k) * DT)


def _lif(n, v0, vreset, theta, tref, ibg):
    return LIFParams(n, resting_potential_v0=v0, after_spike_reset_potential_vreset=vreset,
                     threshold_for_action_potential_spike=theta, absolute_refractory_period=tref,
                     somatic_capacitance_Cm=200.0e-12, somatic_leakage_conductance_g0=10.0e-9,
                     background_current=ibg)


def ref_va(mixed: bool, d_lo: int = 1, d_hi: int = 1) -> Model:
    """oracle/ref_cases.inc build_va: the unmixed net takes delays of d_lo..d_hi steps."""
    m = Model(N.SPK_SYN_CONDUCTANCE, N.SPK_INPUT_NONE, synapse_seed=-1, timestep=float(DT))
    nE, nI = (320, 80) if mixed else (3200, 800)
    args = (-60.0e-3, -60.0e-3, -50.0e-3, 5.0e-3, 2.0e-2)
    ge = m.add_neuron_group(_lif(nE, *args))
    gi = m.add_neuron_group(_lif(nI, *args))
    p = 0.1 if mixed else 0.02
    es = SynapseParams(connectivity_type=N.SPK_CONN_RANDOM,
                       delay_range=(steps(1 if mixed else d_lo), steps(4 if mixed else d_hi)),
                       weight_range=(0.2, 0.6) if mixed else (0.4, 0.4), weight_scaling_constant=10.0e-9,
                       random_connectivity_probability=p, reversal_potential_Vhat=0.0, decay_term_tau_g=5.0e-3)
    is_ = SynapseParams(connectivity_type=N.SPK_CONN_RANDOM,
                        delay_range=(steps(1 if mixed else d_lo), steps(6 if mixed else d_hi)),
                        weight_range=(5.1, 6.1) if mixed else (5.1, 5.1), weight_scaling_constant=10.0e-9,
                        random_connectivity_probability=p, reversal_potential_Vhat=-80.0e-3,
                        decay_term_tau_g=10.0e-3)
    m.add_synapse_group(ge, ge, es)
    m.add_synapse_group(ge, gi, es)
    m.add_synapse_group(gi, ge, is_)
    m.add_synapse_group(gi, gi, is_)
    return m


def ref_det(current: bool) -> Model:
    """oracle/ref_cases.inc build_det: the deterministic voltage (vdet) or
    current (cdet) synapse network."""
    kind = N.SPK_SYN_CURRENT if current else N.SPK_SYN_VOLTAGE
    m = Model(kind, N.SPK_INPUT_NONE, synapse_seed=11, timestep=float(DT))
    args = (0.0, 0.0, 20.0e-3, 2.0e-3, 25.0e-3)
    ge = m.add_neuron_group(_lif(800, *args))
    gi = m.add_neuron_group(_lif(200, *args))
    J = 2.0 ** (-29 if current else -8)
    for pre, post in ((ge, ge), (ge, gi), (gi, ge), (gi, gi)):
        exc = pre == ge
        w = 1.0 if exc else -4.0
        sp = SynapseParams(connectivity_type=N.SPK_CONN_RANDOM, weight_range=(w, w), weight_scaling_constant=J,
                           delay_range=(steps(1), steps(30)), random_connectivity_probability=0.05,
                           decay_term_tau=(5.0e-3 if exc else 10.0e-3) if current else 0.001)
        m.add_synapse_group(pre, post, sp)
    return m


def ref_brunel() -> Model:
    m = Model(N.SPK_SYN_VOLTAGE, N.SPK_INPUT_POISSON, synapse_seed=42, timestep=float(DT))
    rule = m.add_stdp_rule(STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02,
                                      lambda_=1.0, alpha=1.0, w_max=1.0))
    args = (0.0, 0.0, 20.0e-3, 2.0e-3, 0.0)
    gin = m.add_input_group(150, 20.0)
    ge = m.add_neuron_group(_lif(160, *args))
    gi = m.add_neuron_group(_lif(40, *args))
    J = float(F(0.1) * F(10.0 ** -3))
    d = (steps(1), steps(20))
    es = SynapseParams(weight_range=(J, J), delay_range=d)
    is_ = SynapseParams(weight_range=(float(F(-5.0) * F(J)), float(F(-5.0) * F(J))), delay_range=d)
    inp = SynapseParams(weight_range=(0.0, float(F(2.0) * F(J))), delay_range=d)
    m.connect_with_sparsity(gin, ge, 0.1, inp)
    m.connect_with_sparsity(gin, gi, 0.1, inp)
    m.connect_with_sparsity(ge, gi, 0.1, es)
    m.connect_with_sparsity(ge, ge, 0.1, SynapseParams(weight_range=(J, J), delay_range=d, plasticity_rule=rule))
    m.connect_with_sparsity(gi, ge, 0.1, is_)
    m.connect_with_sparsity(gi, gi, 0.1, is_)
    return m


def ref_shapes() -> Model:
    m = Model(N.SPK_SYN_VOLTAGE, N.SPK_INPUT_POISSON, synapse_seed=7, timestep=float(DT))
    gin = m.add_input_group(20, 35.0, shape0=4)
    ga = m.add_neuron_group(_lif(12, -0.07, -0.075, -0.05, 0.003, 0.001))
    gb = m.add_neuron_group(_lif(20, -0.065, -0.07, -0.052, 0.002, 0.0015))
    m.add_synapse_group(gin, ga, SynapseParams(connectivity_type=N.SPK_CONN_ALL_TO_ALL, delay_range=(steps(1), steps(3)),
                                               weight_range=(0.0001, 0.0003), weight_scaling_constant=2.0))
    m.add_synapse_group(gin, gb, SynapseParams(connectivity_type=N.SPK_CONN_ONE_TO_ONE, delay_range=(steps(2), steps(2)),
                                               weight_range=(0.0005, 0.0005)))
    m.add_synapse_group(ga, gb, SynapseParams(
        connectivity_type=N.SPK_CONN_PAIRWISE, delay_range=(steps(1), steps(1)),
        pairwise_pre=[0, 3, 3, 11, 5, 0], pairwise_post=[2, 19, 19, 0, 7, 2],
        pairwise_weight=[0.001, -0.002, 0.0015, 0.003, -0.0005, 0.0007],
        pairwise_delay=[steps(k) for k in (1, 5, 5, 2, 9, 3)]))
    m.add_synapse_group(gb, ga, SynapseParams(connectivity_type=N.SPK_CONN_RANDOM, random_connectivity_probability=0.3,
                                              delay_range=(steps(1), steps(7)), weight_range=(-0.0002, 0.0004)))
    return m
