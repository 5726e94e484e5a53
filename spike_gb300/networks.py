"""The benchmark networks, built through the model API exactly as the
reference examples build them.

* ``vogels_abbott`` - Examples/VogelsAbbottNet.cpp (conductance LIF, E/I 4:1,
  random 2 % connectivity, delay 1 step), plus the initial-V extension.
* ``brunel`` - Examples/Brunel10K.cpp structure (voltage-jump LIF, Poisson
  drive, fixed in-degree via connect_with_sparsity, Examples/UtilityFunctions.hpp:51-82),
  with integer delays U{1..d_max} steps and optional weight-dependent STDP on
  E->E.
* ``plastic_ff`` - a large feed-forward + recurrent plastic network: patterned
  Poisson inputs with log-normal rates, fixed in-degree, weights U[0,1].

All sizes are parameters so the same builders give the parity-test networks.
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from .model import GenNetwork, LIFParams, Model, Projection, STDPParams, SynapseParams

DT = 0.0001


def vogels_abbott(n_exc: int = 3200, n_inh: int = 800, p: float = 0.02, delay_steps: int = 1,
                  v_init: bool = True, philox_seed: int = 42, synapse_seed: int = -1) -> Model:
    m = Model(N.SPK_SYN_CONDUCTANCE, N.SPK_INPUT_NONE, synapse_seed=synapse_seed, timestep=DT,
              philox_seed=philox_seed)
    common = dict(somatic_capacitance_Cm=200.0e-12, somatic_leakage_conductance_g0=10.0e-9,
                  resting_potential_v0=-60.0e-3, after_spike_reset_potential_vreset=-60.0e-3,
                  absolute_refractory_period=5.0e-3, threshold_for_action_potential_spike=-50.0e-3,
                  background_current=2.0e-2)
    if v_init:
        common.update(v_init_lo=-60.0e-3, v_init_hi=-50.0e-3)
    e = m.add_neuron_group(LIFParams(n_exc, **common))
    i = m.add_neuron_group(LIFParams(n_inh, **common))
    exc = SynapseParams(connectivity_type=N.SPK_CONN_RANDOM, weight_range=(0.4, 0.4),
                        weight_scaling_constant=10.0e-9, random_connectivity_probability=p,
                        delay_range=(delay_steps * DT, delay_steps * DT), reversal_potential_Vhat=0.0,
                        decay_term_tau_g=5.0e-3)
    inh = SynapseParams(connectivity_type=N.SPK_CONN_RANDOM, weight_range=(5.1, 5.1),
                        weight_scaling_constant=10.0e-9, random_connectivity_probability=p,
                        delay_range=(delay_steps * DT, delay_steps * DT), reversal_potential_Vhat=-80.0e-3,
                        decay_term_tau_g=10.0e-3)
    m.add_synapse_group(e, e, exc)
    m.add_synapse_group(e, i, exc)
    m.add_synapse_group(i, e, inh)
    m.add_synapse_group(i, i, inh)
    return m


def brunel(n_exc: int = 10000, n_inh: int = 2500, n_in: int = 10000, rate: float = 20.0,
           sparseness: float = 0.1, g: float = 5.0, J: float = 0.1e-3, d_max: int = 20,
           plastic: bool = False, stdp: STDPParams | None = None, philox_seed: int = 42,
           synapse_seed: int = 42, norm: int = N.SPK_NORM_OFF) -> Model:
    """Examples/Brunel10K.cpp through the model API; with `plastic` the E->E
    synapses follow the weight-dependent rule, and with `norm` also the
    weight normalisation, added after (SPK_NORM_AFTER_RULE) or before it."""
    m = Model(N.SPK_SYN_VOLTAGE, N.SPK_INPUT_POISSON, synapse_seed=synapse_seed, timestep=DT,
              philox_seed=philox_seed)
    rule = nrule = -1
    plastic = plastic or norm != N.SPK_NORM_OFF
    if norm == N.SPK_NORM_BEFORE_RULE:
        nrule = m.add_weight_norm_rule()
    if plastic:
        rule = m.add_stdp_rule(stdp or STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02,
                                                  tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0))
    if norm == N.SPK_NORM_AFTER_RULE:
        nrule = m.add_weight_norm_rule()
    common = dict(somatic_capacitance_Cm=200.0e-12, somatic_leakage_conductance_g0=10.0e-9,
                  resting_potential_v0=0.0, after_spike_reset_potential_vreset=0.0,
                  absolute_refractory_period=2.0e-3, threshold_for_action_potential_spike=20.0e-3,
                  background_current=0.0)
    inp = m.add_input_group(n_in, rate)
    e = m.add_neuron_group(LIFParams(n_exc, **common))
    i = m.add_neuron_group(LIFParams(n_inh, **common))
    delays = (1 * DT, d_max * DT)
    exc = SynapseParams(weight_range=(J, J), weight_scaling_constant=1.0, delay_range=delays)
    inh = SynapseParams(weight_range=(-g * J, -g * J), weight_scaling_constant=1.0, delay_range=delays)
    ext = SynapseParams(weight_range=(J, J), weight_scaling_constant=1.0, delay_range=delays)
    m.connect_with_sparsity(inp, e, sparseness, ext)
    m.connect_with_sparsity(inp, i, sparseness, ext)
    m.connect_with_sparsity(e, i, sparseness, exc)
    exc_plastic = SynapseParams(weight_range=(J, J), weight_scaling_constant=1.0, delay_range=delays,
                                plasticity_rule=rule, plasticity_rule_2=nrule)
    m.connect_with_sparsity(e, e, sparseness, exc_plastic)
    m.connect_with_sparsity(i, e, sparseness, inh)
    m.connect_with_sparsity(i, i, sparseness, inh)
    return m


def lognormal_rates(n: int, median: float = 5.0, sigma: float = 1.0, hi: float = 100.0,
                    seed: int = 42) -> np.ndarray:
    """Per-input rates exp(ln median + sigma z), clipped to [0, hi] Hz."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal(n)
    return np.clip(np.exp(np.log(median) + sigma * z), 0.0, hi).astype(np.float32)


def plastic_ff(n_in: int = 50000, n_neurons: int = 200000, ff: int = 900, rec: int = 100,
               d_max: int = 10, w_scale: float = 2.0e-4, sigma: float = 1.0, plastic: bool = True,
               philox_seed: int = 42, synapse_seed: int = 42) -> Model:
    m = Model(N.SPK_SYN_VOLTAGE, N.SPK_INPUT_PATTERNED, synapse_seed=synapse_seed, timestep=DT,
              philox_seed=philox_seed)
    rule = -1
    if plastic:
        rule = m.add_stdp_rule(STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02,
                                          lambda_=1.0, alpha=1.0, w_max=1.0, clip_upper=True))
    inp = m.add_input_group(n_in, 0.0)
    m.add_stimulus(lognormal_rates(n_in, sigma=sigma, seed=philox_seed))
    common = dict(somatic_capacitance_Cm=200.0e-12, somatic_leakage_conductance_g0=10.0e-9,
                  resting_potential_v0=0.0, after_spike_reset_potential_vreset=0.0,
                  absolute_refractory_period=2.0e-3, threshold_for_action_potential_spike=20.0e-3)
    pop = m.add_neuron_group(LIFParams(n_neurons, **common))
    delays = (1 * DT, d_max * DT)
    ffp = SynapseParams(weight_range=(0.0, 1.0), weight_scaling_constant=w_scale, delay_range=delays,
                        plasticity_rule=rule)
    recp = SynapseParams(weight_range=(-1.0, 0.0), weight_scaling_constant=w_scale, delay_range=delays)
    m.connect_with_sparsity(inp, pop, ff / n_in, ffp)
    m.connect_with_sparsity(pop, pop, rec / n_neurons, recp)
    return m


BRUNEL_LIF = dict(tau_m=0.02, R=1.0e8, v0=0.0, vreset=0.0, theta=0.02)  # C_m 200 pF, g_0 10 nS


# Evans rule constants for the plastic workloads: alpha_C = a_plus, alpha_D =
# a_minus, tau_C = tau_plus, tau_D = tau_minus (EvansSTDPPlasticity.hpp defaults)
EVANS_STDP = STDPParams(a_plus=0.5, a_minus=0.5, tau_plus=0.004, tau_minus=0.005, lambda_=0.0, alpha=0.0, w_max=1.0)


def plastic_ff_generated(n_in: int = 50000, n_neurons: int = 200000, ff: int = 900, rec: int = 100,
                         d_max: int = 10, w_scale: float = 2.0e-4, sigma: float = 1.0, plastic: bool = True,
                         seed: int = 42, rule: int = N.SPK_STDP_WEIGHT_DEPENDENT) -> GenNetwork:
    """The large plastic feed-forward + recurrent network drawn on the GPU:
    each (input, neuron) pair connects with p = ff / n_in and each (neuron,
    neuron) pair with p = rec / n_neurons (binomial in-degree, mean ff + rec),
    weights U(0, 1] (inputs, plastic) and U(-1, 0] (recurrent) times w_scale
    volts, delays U{1..d_max}, log-normal input rates.  `rule` is the STDP rule
    of the input synapses: weight-dependent (a+ 0.005, a- 0.00525, tau 20 ms,
    weights clipped to [0, 1]) or Evans (EVANS_STDP)."""
    if rule == N.SPK_STDP_EVANS:
        stdp = EVANS_STDP if plastic else None
    elif rule == N.SPK_STDP_WEIGHT_DEPENDENT:
        stdp = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0,
                          w_max=1.0, clip_upper=True) if plastic else None
    else:
        raise ValueError(f"plastic_ff_generated: rule {rule} has no parameter set here")
    projs = [Projection(N.SPK_POP_INPUTS, 0, n_in, 0, n_neurons, ff / n_in, weight=(0.0, 1.0), scale=w_scale,
                        delay=(1, d_max), plastic=plastic),
             Projection(N.SPK_POP_NEURONS, 0, n_neurons, 0, n_neurons, rec / n_neurons, weight=(-1.0, 0.0),
                        scale=w_scale, delay=(1, d_max))]
    return GenNetwork(groups=[dict(count=n_neurons, **BRUNEL_LIF)], projections=projs, refractory=2.0e-3,
                      n_inputs=n_in, rates=lognormal_rates(n_in, sigma=sigma, seed=seed), stdp=stdp, seed=seed,
                      connectivity_seed=seed + 1, stdp_rule=rule)


def sweep_instance(n: int, p: float, g: float, plastic: bool, seed: int, d_max: int = 10,
                   rate: float = 20.0, rule: int = N.SPK_STDP_WEIGHT_DEPENDENT, d_min: int = 1) -> GenNetwork:
    """One instance of the batched sweep: a Brunel-style voltage-jump LIF
    network of n neurons (80 % excitatory), Bernoulli(p) recurrent
    connectivity, J = 0.1 V / C_E with C_E = 0.8 n p (J C_E as in
    Examples/Brunel10K.cpp), inhibitory weight -g J, delays U{d_min..d_max}
    (d_min > 1 groups timesteps), and an external drive of n / 5 Poisson
    inputs at `rate` Hz connected with probability 4p (C_E inputs per neuron,
    nu_ext = 2 nu_thr).  With plasticity the input synapses are plastic, weights U(0, 1] at scale 2J,
    under the weight-dependent rule or (`rule`) the Evans rule."""
    n_e = int(round(0.8 * n))
    n_i = n - n_e
    n_in = max(1, n // 5)
    c_e = max(1.0, 0.8 * n * p)
    J = 0.1 / c_e
    p_in = min(1.0, 4.0 * p)
    stdp = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0,
                      w_max=1.0, clip_upper=True) if plastic else None
    if plastic and rule == N.SPK_STDP_EVANS:
        stdp = EVANS_STDP
    projs = [Projection(N.SPK_POP_INPUTS, 0, n_in, 0, n, p_in,
                        weight=(0.0, 1.0) if plastic else (1.0, 1.0), scale=2.0 * J if plastic else J,
                        delay=(d_min, d_max), plastic=plastic),
             Projection(N.SPK_POP_NEURONS, 0, n_e, 0, n, p, weight=(1.0, 1.0), scale=J, delay=(d_min, d_max)),
             Projection(N.SPK_POP_NEURONS, n_e, n_i, 0, n, p, weight=(-g, -g), scale=J, delay=(d_min, d_max))]
    return GenNetwork(groups=[dict(count=n_e, **BRUNEL_LIF), dict(count=n_i, **BRUNEL_LIF)], projections=projs,
                      refractory=2.0e-3, n_inputs=n_in, rates=np.full(n_in, rate, np.float32), stdp=stdp,
                      seed=seed, connectivity_seed=seed ^ 0x5eed,
                      stdp_rule=rule if plastic else N.SPK_STDP_WEIGHT_DEPENDENT)


def batched_sweep(n_instances: int = 256, n_lo: int = 1000, n_hi: int = 50000, seed: int = 42,
                  plastic_fraction: float = 0.5) -> list:
    """The batched sweep: n_instances independent instances with N
    log-uniform in [n_lo, n_hi], p ~ U[0.01, 0.05], g ~ U[3, 7], delays
    U{1..10}, distinct seeds, the first plastic_fraction of them with STDP."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), n_instances)).astype(int)
    ps = rng.uniform(0.01, 0.05, n_instances)
    gs = rng.uniform(3.0, 7.0, n_instances)
    n_plastic = int(round(plastic_fraction * n_instances))
    return [sweep_instance(int(sizes[k]), float(ps[k]), float(gs[k]), k < n_plastic, seed=1000 + 7 * k)
            for k in range(n_instances)]
