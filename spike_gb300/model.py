"""Python mirror of the reference's model-building API over the C front end.

``Model`` follows ``SpikingModel`` (Spike/Models/SpikingModel.hpp:24-67): add
neuron / input / synapse groups with the reference's parameter fields, add a
weight-dependent STDP rule, ``finalise()``, ``run(seconds, plasticity_on)``,
``reset_state()`` / ``reset_time()``.  Connectivity is built by the C++ front
end with the reference's rand() sequence.  ``Net`` wraps a network created
directly from a flat descriptor; ``Batch`` advances many networks in one
persistent launch.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from ._native import check, lib


@dataclass
class LIFParams:
    """lif_spiking_neuron_parameters_struct (Spike/Neurons/LIFSpikingNeurons.hpp:7-14)."""
    n: int
    resting_potential_v0: float = -0.074
    after_spike_reset_potential_vreset: float = -0.074
    threshold_for_action_potential_spike: float = 0.03
    absolute_refractory_period: float = 0.002
    somatic_capacitance_Cm: float = 0.0
    somatic_leakage_conductance_g0: float = 0.0
    background_current: float = 0.0
    v_init_lo: float = 0.0
    v_init_hi: float = 0.0


@dataclass
class SynapseParams:
    """synapse_parameters_struct and its spiking/conductance/current extensions."""
    connectivity_type: int = N.SPK_CONN_ALL_TO_ALL
    weight_range: tuple = (0.0, 0.0)
    weight_scaling_constant: float = 1.0
    random_connectivity_probability: float = 0.0
    delay_range: tuple = (0.0, 0.0)
    reversal_potential_Vhat: float = 0.0
    decay_term_tau_g: float = 0.001
    decay_term_tau: float = 0.001
    max_number_of_connections_per_pair: int = 1
    gaussian_synapses_per_postsynaptic_neuron: int = 10
    gaussian_synapses_standard_deviation: float = 10.0
    pairwise_pre: list | None = None
    pairwise_post: list | None = None
    pairwise_weight: list | None = None
    pairwise_delay: list | None = None
    plasticity_rule: int = -1
    plasticity_rule_2: int = -1  # a second rule on the same synapses (the weight normalisation)
    _keep: list = field(default_factory=list, repr=False)

    def to_c(self) -> N.SynapseParams:
        s = N.SynapseParams()
        s.connectivity_type = self.connectivity_type
        s.weight_range[0], s.weight_range[1] = self.weight_range
        s.weight_scaling_constant = self.weight_scaling_constant
        s.random_connectivity_probability = self.random_connectivity_probability
        s.delay_range[0], s.delay_range[1] = self.delay_range
        s.reversal_potential_Vhat = self.reversal_potential_Vhat
        s.decay_term_tau_g = self.decay_term_tau_g
        s.decay_term_tau = self.decay_term_tau
        s.max_number_of_connections_per_pair = self.max_number_of_connections_per_pair
        s.gaussian_synapses_per_postsynaptic_neuron = self.gaussian_synapses_per_postsynaptic_neuron
        s.gaussian_synapses_standard_deviation = self.gaussian_synapses_standard_deviation
        s.plasticity_rule = self.plasticity_rule
        s.plasticity_rule_2 = self.plasticity_rule_2
        s.n_pairwise = 0
        self._keep.clear()
        if self.pairwise_pre is not None:
            pre = np.ascontiguousarray(self.pairwise_pre, dtype=np.int32)
            post = np.ascontiguousarray(self.pairwise_post, dtype=np.int32)
            self._keep += [pre, post]
            s.n_pairwise = len(pre)
            s.pairwise_connect_presynaptic = pre.ctypes.data_as(C.POINTER(C.c_int32))
            s.pairwise_connect_postsynaptic = post.ctypes.data_as(C.POINTER(C.c_int32))
            if self.pairwise_weight is not None:
                w = np.ascontiguousarray(self.pairwise_weight, dtype=np.float32)
                self._keep.append(w)
                s.pairwise_connect_weight = w.ctypes.data_as(C.POINTER(C.c_float))
            if self.pairwise_delay is not None:
                d = np.ascontiguousarray(self.pairwise_delay, dtype=np.float32)
                self._keep.append(d)
                s.pairwise_connect_delay = d.ctypes.data_as(C.POINTER(C.c_float))
        return s


@dataclass
class STDPParams:
    """weightdependent_stdp_plasticity_parameters_struct
    (Spike/Plasticity/WeightDependentSTDPPlasticity.hpp:28-40)."""
    a_minus: float = 1.0
    a_plus: float = 1.0
    tau_minus: float = 0.02
    tau_plus: float = 0.02
    lambda_: float = 1.0
    alpha: float = 1.0
    w_max: float = 1.0
    clip_upper: bool = False

    def to_c(self) -> N.StdpParams:
        return N.StdpParams(self.a_minus, self.a_plus, self.tau_minus, self.tau_plus, self.lambda_,
                            self.alpha, self.w_max, 1 if self.clip_upper else 0)


def schedule(warps_per_cta=0, tile_posts=0, ctas=0, steps_per_launch=0) -> N.Schedule:
    return N.Schedule(warps_per_cta, tile_posts, ctas, steps_per_launch)


def _i32(x):
    return C.c_int32(x)


class Net:
    """A network handle of the engine (spk_net_*).  ``owned=False`` borrows a
    handle that belongs to a Model."""

    def __init__(self, handle: C.c_void_p, owned: bool = True):
        self.h = handle
        self.owned = owned

    @classmethod
    def from_desc(cls, desc: N.NetDesc, sched: N.Schedule | None = None) -> "Net":
        h = C.c_void_p()
        check(lib().spk_net_create(C.byref(desc), C.byref(sched) if sched else None, C.byref(h)),
              "spk_net_create")
        return cls(h)

    @classmethod
    def generate(cls, gen: "GenNetwork | N.GenDesc", sched: N.Schedule | None = None) -> "Net":
        """A network whose connectivity the GPU draws (spk_net_generate)."""
        d = gen.desc if isinstance(gen, GenNetwork) else gen
        h = C.c_void_p()
        check(lib().spk_net_generate(C.byref(d), C.byref(sched) if sched else None, C.byref(h)),
              "spk_net_generate")
        return cls(h)

    def set_step_cost(self, cost: float):
        """Cost of one step (e.g. microseconds alone) for batch wave packing."""
        check(lib().spk_net_set_step_cost(self.h, C.c_float(cost)), "spk_net_set_step_cost")

    def synapse_count(self) -> int:
        n = C.c_int64()
        check(lib().spk_net_synapse_count(self.h, C.byref(n)), "spk_net_synapse_count")
        return n.value

    def plastic_synapse_count(self) -> int:
        n = C.c_int64()
        check(lib().spk_net_plastic_synapse_count(self.h, C.byref(n)), "spk_net_plastic_synapse_count")
        return n.value

    def close(self):
        if self.h and self.owned:
            lib().spk_net_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- run control
    def run(self, seconds: float, plasticity_on: bool = True) -> None:
        check(lib().spk_net_run(self.h, C.c_float(seconds), 1 if plasticity_on else 0), "spk_net_run")

    def run_steps(self, steps: int, plasticity_on: bool = True) -> None:
        check(lib().spk_net_run_steps(self.h, steps, 1 if plasticity_on else 0), "spk_net_run_steps")

    def synchronize(self) -> int:
        return lib().spk_net_synchronize(self.h)

    def reset_state(self):
        check(lib().spk_net_reset_state(self.h), "spk_net_reset_state")

    def reset_time(self):
        check(lib().spk_net_reset_time(self.h), "spk_net_reset_time")

    def select_stimulus(self, s: int):
        check(lib().spk_net_select_stimulus(self.h, s), "spk_net_select_stimulus")

    def write_rates(self, stimulus: int, rates_ptr: int, n: int):
        """Asynchronous upload of one stimulus' rates from host address rates_ptr."""
        check(lib().spk_net_write_rates(self.h, stimulus, C.c_void_p(rates_ptr), n), "spk_net_write_rates")

    def current_time(self) -> float:
        t = C.c_float()
        check(lib().spk_net_current_time(self.h, C.byref(t)), "spk_net_current_time")
        return t.value

    def timestep_grouping(self) -> int:
        """The network's minimum delay in steps: runs advance whole groups of it."""
        g = C.c_int32()
        check(lib().spk_net_timestep_grouping(self.h, C.byref(g)), "spk_net_timestep_grouping")
        return g.value

    # ---- readback
    def spikes(self, population: int = N.SPK_POP_NEURONS):
        n = C.c_int64()
        check(lib().spk_net_spike_count(self.h, population, C.byref(n)), "spk_net_spike_count")
        ids = np.empty(n.value, dtype=np.int32)
        times = np.empty(n.value, dtype=np.float32)
        got = C.c_int64()
        check(lib().spk_net_read_spikes(self.h, population, ids.ctypes.data_as(C.POINTER(C.c_int32)),
                                        times.ctypes.data_as(C.POINTER(C.c_float)), n.value, C.byref(got)),
              "spk_net_read_spikes")
        return ids[:got.value], times[:got.value]

    def clear_spikes(self):
        check(lib().spk_net_clear_spikes(self.h), "spk_net_clear_spikes")

    def rate_counts(self, n: int, population: int = N.SPK_POP_NEURONS) -> np.ndarray:
        """Spikes per neuron (or input) since the last clear or reset (the
        rate monitor); n is the population's size."""
        out = np.zeros(n, np.int32)
        check(lib().spk_net_rate_counts(self.h, population, out.ctypes.data_as(C.POINTER(C.c_int32)), n),
              "spk_net_rate_counts")
        return out

    def clear_rate_counts(self):
        check(lib().spk_net_clear_rate_counts(self.h), "spk_net_clear_rate_counts")

    def state(self, field: int, count: int) -> np.ndarray:
        out = np.empty(count, dtype=np.float32)
        check(lib().spk_net_read_state(self.h, field, out.ctypes.data_as(C.c_void_p), count), "spk_net_read_state")
        return out

    def weights(self, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.float32)
        check(lib().spk_net_read_weights(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), n),
              "spk_net_read_weights")
        return out

    def write_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, dtype=np.float32)
        check(lib().spk_net_write_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float)), len(w)),
              "spk_net_write_weights")

    def events(self) -> int:
        e = C.c_uint64()
        check(lib().spk_net_synaptic_events(self.h, C.byref(e)), "spk_net_synaptic_events")
        return e.value

    def snapshot(self) -> bytes:
        """The dynamic state (spk_net_snapshot) as bytes."""
        n = C.c_int64()
        check(lib().spk_net_snapshot_bytes(self.h, C.byref(n)), "spk_net_snapshot_bytes")
        buf = C.create_string_buffer(n.value)
        check(lib().spk_net_snapshot(self.h, buf, n.value), "spk_net_snapshot")
        return buf.raw

    def restore(self, snap: bytes):
        buf = C.create_string_buffer(snap, len(snap))
        check(lib().spk_net_restore(self.h, buf, len(snap)), "spk_net_restore")

    def set_wait_limit(self, seconds: float):
        check(lib().spk_net_set_wait_limit(self.h, C.c_double(seconds)), "spk_net_set_wait_limit")

    def inject_withheld_cta(self, rank: int):
        check(lib().spk_net_inject_withheld_cta(self.h, rank), "spk_net_inject_withheld_cta")

    def stdp_counts(self) -> tuple:
        """(plastic weights updated on presynaptic events, plastic afferents
        updated on postsynaptic spikes) so far."""
        a, b = C.c_uint64(), C.c_uint64()
        check(lib().spk_net_stdp_counts(self.h, C.byref(a), C.byref(b)), "spk_net_stdp_counts")
        return a.value, b.value

    def schedule(self) -> dict:
        s = N.Schedule()
        check(lib().spk_net_get_schedule(self.h, C.byref(s)), "spk_net_get_schedule")
        return dict(warps_per_cta=s.warps_per_cta, tile_posts=s.tile_posts, ctas=s.ctas,
                    steps_per_launch=s.steps_per_launch)

    def device_bytes(self) -> int:
        b = C.c_int64()
        check(lib().spk_net_device_bytes(self.h, C.byref(b)), "spk_net_device_bytes")
        return b.value

    def launches(self) -> int:
        b = C.c_int64()
        check(lib().spk_net_launch_count(self.h, C.byref(b)), "spk_net_launch_count")
        return b.value

    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().spk_net_stream(self.h, C.byref(s)), "spk_net_stream")
        return s.value or 0


@dataclass
class Projection:
    """One spk_projection: Bernoulli(p) connectivity over a (pre, post)
    rectangle, weights ~ U(lo, hi], integer delays ~ U{lo..hi} steps."""
    pre_population: int
    pre_start: int
    pre_count: int
    post_start: int
    post_count: int
    probability: float
    weight: tuple = (1.0, 1.0)
    scale: float = 1.0
    delay: tuple = (1, 1)
    label: int = 0
    plastic: bool = False

    def to_c(self) -> N.Projection:
        return N.Projection(self.pre_population, self.pre_start, self.pre_count, self.post_start, self.post_count,
                            self.probability, self.weight[0], self.weight[1], self.scale, int(self.delay[0]),
                            int(self.delay[1]), self.label, 1 if self.plastic else 0)


class GenNetwork:
    """Descriptor of a network whose connectivity is drawn on the GPU
    (spk_net_generate).  ``groups`` are dicts with count, tau_m, R, v0,
    vreset, theta and optionally v_init_lo / v_init_hi."""

    def __init__(self, *, groups, projections, kind=N.SPK_SYN_VOLTAGE, dt=0.0001, refractory=0.002, i_bg=0.0,
                 rates=None, n_inputs=0, label_tau=None, label_vhat=None, n_labels=1, stdp=None, seed=1,
                 connectivity_seed=1, spike_capacity=0, record_inputs=False, stdp_rule=N.SPK_STDP_WEIGHT_DEPENDENT):
        self.keep = []
        d = N.GenDesc()
        d.stdp_rule = stdp_rule
        d.abi_version = N.SPK_ABI_VERSION
        d.dt = dt
        d.synapse_kind = kind
        gs = (N.NeuronGroup * len(groups))()
        start = 0
        for i, g in enumerate(groups):
            gs[i].start = start
            gs[i].count = g["count"]
            gs[i].tau_m = g.get("tau_m", 0.02)
            gs[i].R = g.get("R", 1.0e8)
            gs[i].v0 = g.get("v0", 0.0)
            gs[i].vreset = g.get("vreset", 0.0)
            gs[i].theta = g.get("theta", 0.02)
            gs[i].v_init_lo = g.get("v_init_lo", 0.0)
            gs[i].v_init_hi = g.get("v_init_hi", 0.0)
            start += g["count"]
        self.keep.append(gs)
        d.n_neurons = start
        d.n_groups = len(groups)
        d.groups = C.cast(gs, C.POINTER(N.NeuronGroup))
        d.refractory_period = refractory
        d.background_current = i_bg
        d.n_inputs = n_inputs
        if n_inputs:
            r = np.ascontiguousarray(rates, dtype=np.float32).reshape(-1)
            self.keep.append(r)
            d.n_stimuli = len(r) // n_inputs
            d.input_rates = r.ctypes.data_as(C.POINTER(C.c_float))
            d.stimulus = 0
        d.n_labels = n_labels
        tau = np.ascontiguousarray(label_tau if label_tau is not None else [0.005] * n_labels, np.float32)
        vh = np.ascontiguousarray(label_vhat if label_vhat is not None else [0.0] * n_labels, np.float32)
        self.keep += [tau, vh]
        d.label_tau = tau.ctypes.data_as(C.POINTER(C.c_float))
        d.label_vhat = vh.ctypes.data_as(C.POINTER(C.c_float))
        ps = (N.Projection * max(len(projections), 1))()
        for i, pr in enumerate(projections):
            ps[i] = pr.to_c()
        self.keep.append(ps)
        self.projections = list(projections)
        d.n_projections = len(projections)
        d.projections = C.cast(ps, C.POINTER(N.Projection))
        if stdp is not None:
            d.has_stdp = 1
            d.stdp = stdp.to_c()
        d.seed = seed
        d.connectivity_seed = connectivity_seed
        d.spike_capacity = spike_capacity
        d.record_inputs = 1 if record_inputs else 0
        # the descriptor keeps its owner (and the arrays it points into) alive, so
        # that a descriptor taken from a temporary stays valid
        d._owner = self
        self.desc = d

    def expected_synapses(self) -> float:
        return sum(p.pre_count * p.post_count * p.probability for p in self.projections)


class Batch:
    """Many networks advanced together by one persistent launch per step block."""

    def __init__(self, nets: list[Net], sched: N.Schedule | None = None):
        arr = (C.c_void_p * len(nets))(*[n.h for n in nets])
        self.nets = nets
        self.h = C.c_void_p()
        check(lib().spk_batch_create(arr, len(nets), C.byref(sched) if sched else None, C.byref(self.h)),
              "spk_batch_create")

    def set_mode(self, mode: int):
        """SPK_BATCH_WAVES (persistent kernel) or SPK_BATCH_BULK (four
        kernels per timestep over all networks)."""
        check(lib().spk_batch_set_mode(self.h, mode), "spk_batch_set_mode")

    @staticmethod
    def autotune(gens: list, trial_steps: int = 200, costs: bool = False, with_mode: bool = False):
        """Measured schedule search (spk_batch_autotune) for generated
        networks: returns (schedules, trial milliseconds of the best policy),
        plus each network's microseconds per step alone when costs=True, plus
        the best execution mode when with_mode=True."""
        descs = (N.GenDesc * len(gens))(*[g.desc for g in gens])
        out = (N.Schedule * len(gens))()
        ms = C.c_float()
        mode = C.c_int32()
        us = (C.c_float * len(gens))() if costs else None
        check(lib().spk_batch_autotune(descs, len(gens), trial_steps, out, C.byref(ms), us, C.byref(mode)),
              "spk_batch_autotune")
        res = [[N.Schedule(o.warps_per_cta, o.tile_posts, o.ctas, o.steps_per_launch) for o in out], ms.value]
        if costs:
            res.append([float(x) for x in us])
        if with_mode:
            res.append(mode.value)
        return tuple(res)

    def run_steps(self, steps: int, plasticity_on: bool = True):
        check(lib().spk_batch_run_steps(self.h, steps, 1 if plasticity_on else 0), "spk_batch_run_steps")

    def run_steps_each(self, steps: list[int], plasticity_on: list[bool] | None = None):
        """Each network its own step count (whole groups of its timestep
        grouping) and plasticity switch."""
        n = len(self.nets)
        st = (C.c_int64 * n)(*steps)
        pl = (C.c_int32 * n)(*[1 if p else 0 for p in plasticity_on]) if plasticity_on is not None else None
        check(lib().spk_batch_run_steps_each(self.h, st, pl), "spk_batch_run_steps_each")

    def synchronize(self) -> int:
        return lib().spk_batch_synchronize(self.h)

    def time_kernels(self, steps: int, plasticity_on: bool = True) -> dict:
        """Advance `steps` timesteps in bulk mode with every kernel timed on
        its own (spk_batch_time_kernels): milliseconds per kernel kind."""
        ms = (C.c_double * N.SPK_KERNEL_KINDS)()
        check(lib().spk_batch_time_kernels(self.h, steps, 1 if plasticity_on else 0, ms), "spk_batch_time_kernels")
        return {name: ms[i] for i, name in enumerate(N.KERNEL_NAMES)}

    def launches(self) -> int:
        b = C.c_int64()
        check(lib().spk_batch_launch_count(self.h, C.byref(b)), "spk_batch_launch_count")
        return b.value

    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().spk_batch_stream(self.h, C.byref(s)), "spk_batch_stream")
        return s.value or 0

    def read_spikes_into(self, ids_ptr: int, times_ptr: int, capacity: int,
                         population: int = N.SPK_POP_NEURONS, clear: bool = False):
        """spk_batch_read_spikes into caller buffers (addresses of int32 ids and
        float32 times, page-locked for a direct copy).  Returns each network's
        count, or None when their sum exceeds capacity (nothing copied)."""
        counts = np.zeros(len(self.nets), np.int64)
        rc = lib().spk_batch_read_spikes(self.h, population, C.cast(C.c_void_p(ids_ptr), C.POINTER(C.c_int32)),
                                         C.cast(C.c_void_p(times_ptr), C.POINTER(C.c_float)), capacity,
                                         counts.ctypes.data_as(C.POINTER(C.c_int64)), 1 if clear else 0)
        if rc == N.SPK_ERR_OVERFLOW:
            return None
        check(rc, "spk_batch_read_spikes")
        return counts

    def spikes(self, population: int = N.SPK_POP_NEURONS, clear: bool = False):
        """Every network's spikes in one call: a list of (ids, times), one per
        network, each as Net.spikes gives it."""
        cap = 1 << 16
        while True:
            ids = np.empty(cap, np.int32)
            times = np.empty(cap, np.float32)
            counts = self.read_spikes_into(ids.ctypes.data, times.ctypes.data, cap, population, clear)
            if counts is not None:
                break
            cap *= 4
        ends = np.cumsum(counts)
        starts = ends - counts
        return [(ids[a:e], times[a:e]) for a, e in zip(starts, ends)]

    def close(self):
        if self.h:
            lib().spk_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Model:
    """SpikingModel over the C front end (spike_gb300_model.h)."""

    def __init__(self, synapse_kind: int = N.SPK_SYN_CONDUCTANCE, input_kind: int = N.SPK_INPUT_NONE,
                 synapse_seed: int = -1, timestep: float = 0.0001, philox_seed: int = 1):
        self.h = C.c_void_p()
        check(lib().spk_model_create(synapse_kind, input_kind, synapse_seed, C.byref(self.h)), "spk_model_create")
        check(lib().spk_model_set_timestep(self.h, C.c_float(timestep)), "spk_model_set_timestep")
        check(lib().spk_model_set_seed(self.h, philox_seed), "spk_model_set_seed")
        self.synapse_kind = synapse_kind
        self.timestep = timestep
        self._net = None

    def close(self):
        if self.h:
            lib().spk_model_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_neuron_group(self, p: LIFParams) -> int:
        c = N.LifParams()
        c.group_shape[0], c.group_shape[1] = 1, p.n
        for f in ("resting_potential_v0", "after_spike_reset_potential_vreset",
                  "threshold_for_action_potential_spike", "absolute_refractory_period",
                  "somatic_capacitance_Cm", "somatic_leakage_conductance_g0", "background_current",
                  "v_init_lo", "v_init_hi"):
            setattr(c, f, getattr(p, f))
        gid = C.c_int32()
        check(lib().spk_model_add_neuron_group(self.h, C.byref(c), C.byref(gid)), "spk_model_add_neuron_group")
        return gid.value

    def add_input_group(self, n: int, rate: float, shape0: int = 1) -> int:
        gid = C.c_int32()
        check(lib().spk_model_add_input_group(self.h, shape0, n // shape0, C.c_float(rate), C.byref(gid)),
              "spk_model_add_input_group")
        return gid.value

    def add_stimulus(self, rates) -> int:
        r = np.ascontiguousarray(rates, dtype=np.float32)
        sid = C.c_int32()
        check(lib().spk_model_add_stimulus(self.h, r.ctypes.data_as(C.POINTER(C.c_float)), len(r), C.byref(sid)),
              "spk_model_add_stimulus")
        return sid.value

    def add_stdp_rule(self, p: STDPParams, rule: int = N.SPK_STDP_WEIGHT_DEPENDENT) -> int:
        """A plasticity rule (SPK_STDP_*; parameters in the descriptor's field
        mapping for the Evans, inhibitory and custom rules)."""
        c = p.to_c()
        rid = C.c_int32()
        check(lib().spk_model_add_plasticity_rule(self.h, rule, C.byref(c), C.byref(rid)),
              "spk_model_add_plasticity_rule")
        return rid.value

    def add_weight_norm_rule(self, settarget: bool = False, target: float = 0.0) -> int:
        """WeightNormSTDPPlasticity: per-post L2 normalisation of the STDP
        rule's synapses (attach it to the same synapse groups as a second
        rule)."""
        rid = C.c_int32()
        check(lib().spk_model_add_weight_norm_rule(self.h, 1 if settarget else 0, C.c_float(target), C.byref(rid)),
              "spk_model_add_weight_norm_rule")
        return rid.value

    def add_synapse_group(self, pre: int, post: int, p: SynapseParams) -> int:
        c = p.to_c()
        gid = C.c_int32()
        check(lib().spk_model_add_synapse_group(self.h, pre, post, C.byref(c), C.byref(gid)),
              "spk_model_add_synapse_group")
        return gid.value

    def connect_with_sparsity(self, pre: int, post: int, sparseness: float, p: SynapseParams) -> int:
        c = p.to_c()
        gid = C.c_int32()
        check(lib().spk_model_connect_with_sparsity(self.h, pre, post, C.c_float(sparseness), C.byref(c),
                                                    C.byref(gid)), "spk_model_connect_with_sparsity")
        return gid.value

    def set_recording(self, record_inputs: bool = False, spike_capacity: int = 0):
        check(lib().spk_model_set_recording(self.h, 1 if record_inputs else 0, spike_capacity),
              "spk_model_set_recording")

    def counts(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int64()
        check(lib().spk_model_counts(self.h, C.byref(a), C.byref(b), C.byref(c)), "spk_model_counts")
        return a.value, b.value, c.value

    def desc(self) -> N.NetDesc:
        d = N.NetDesc()
        check(lib().spk_model_desc(self.h, C.byref(d)), "spk_model_desc")
        d._owner = self  # the descriptor points into the model's arrays
        return d

    def finalise(self, sched: N.Schedule | None = None) -> Net:
        check(lib().spk_model_finalise(self.h, C.byref(sched) if sched else None), "spk_model_finalise")
        h = C.c_void_p()
        check(lib().spk_model_net(self.h, C.byref(h)), "spk_model_net")
        self._net = Net(h, owned=False)
        return self._net

    @property
    def net(self) -> Net:
        if self._net is None:
            self.finalise()
        return self._net

    def run(self, seconds: float, plasticity_on: bool = True) -> int:
        return check(lib().spk_model_run(self.h, C.c_float(seconds), 1 if plasticity_on else 0), "spk_model_run")

    def reset_state(self):
        check(lib().spk_model_reset_state(self.h), "spk_model_reset_state")

    def reset_time(self):
        check(lib().spk_model_reset_time(self.h), "spk_model_reset_time")

    def select_stimulus(self, s: int):
        check(lib().spk_model_select_stimulus(self.h, s), "spk_model_select_stimulus")

    def spikes(self, population: int = N.SPK_POP_NEURONS):
        ids = C.POINTER(C.c_int32)()
        times = C.POINTER(C.c_float)()
        n = C.c_int64()
        check(lib().spk_model_spikes(self.h, population, C.byref(ids), C.byref(times), C.byref(n)),
              "spk_model_spikes")
        if n.value == 0:
            return np.zeros(0, np.int32), np.zeros(0, np.float32)
        return (np.ctypeslib.as_array(ids, (n.value,)).copy(), np.ctypeslib.as_array(times, (n.value,)).copy())

    def clear_spikes(self):
        check(lib().spk_model_clear_spikes(self.h), "spk_model_clear_spikes")

    def add_rate_monitor(self, population: int = N.SPK_POP_NEURONS):
        """A RateActivityMonitor on the neurons or the inputs (before run)."""
        check(lib().spk_model_add_rate_monitor(self.h, population), "spk_model_add_rate_monitor")

    def rate_counts(self, population: int = N.SPK_POP_NEURONS) -> np.ndarray:
        """The rate monitor's spikes per neuron (input) after the last run."""
        p = C.POINTER(C.c_int32)()
        n = C.c_int64()
        check(lib().spk_model_rate_counts(self.h, population, C.byref(p), C.byref(n)), "spk_model_rate_counts")
        if n.value == 0:
            return np.zeros(0, np.int32)
        return np.ctypeslib.as_array(p, (n.value,)).copy()


def desc_arrays(d: N.NetDesc) -> dict:
    """Copy the synapse arrays of a descriptor into numpy (creation order)."""
    S = d.n_synapses

    def arr(ptr, dt):
        if not ptr or S == 0:
            return np.zeros(S, dt)
        return np.ctypeslib.as_array(ptr, (S,)).astype(dt, copy=True)

    return dict(pre=arr(d.pre, np.int32), post=arr(d.post, np.int32), weight=arr(d.weight, np.float32),
                scale=arr(d.scale, np.float32), delay=arr(d.delay, np.int32), label=arr(d.label, np.int32),
                plastic=arr(d.plastic, np.uint8))


class Server:
    """Continuous-batching simulation server (spk_server_*): submit generated
    networks with a step count; the server admits them by free device memory,
    runs them together in step blocks and keeps each job's results."""

    def __init__(self, warps_per_cta=0, tile_posts=0, steps_per_block=0, max_running=0, reserve_bytes=0,
                 record_spikes=True, mode=N.SPK_BATCH_WAVES):
        o = N.ServerOpts(warps_per_cta, tile_posts, steps_per_block, max_running, reserve_bytes,
                         1 if record_spikes else 0, mode)
        self.h = C.c_void_p()
        check(lib().spk_server_start(C.byref(o), C.byref(self.h)), "spk_server_start")
        self._keep = {}

    def submit(self, gen: "GenNetwork", steps: int, plasticity_on: bool = True) -> int:
        j = C.c_int64()
        check(lib().spk_server_submit(self.h, C.byref(gen.desc), steps, 1 if plasticity_on else 0, C.byref(j)),
              "spk_server_submit")
        return j.value

    def poll(self, job: int) -> N.JobInfo:
        info = N.JobInfo()
        check(lib().spk_server_poll(self.h, job, C.byref(info)), "spk_server_poll")
        return info

    def wait(self, job: int, timeout_s: float = 600.0) -> N.JobInfo:
        rc = lib().spk_server_wait(self.h, job, C.c_double(timeout_s))
        if rc != N.SPK_OK:
            raise N.SpikeError(rc, "spk_server_wait", "job did not finish in time" if rc == N.SPK_ERR_BUSY else "")
        return self.poll(job)

    def spikes(self, job: int):
        info = self.poll(job)
        n = int(info.spikes)
        ids = np.empty(n, np.int32)
        times = np.empty(n, np.float32)
        got = C.c_int64()
        check(lib().spk_server_read_spikes(self.h, job, ids.ctypes.data_as(C.POINTER(C.c_int32)),
                                           times.ctypes.data_as(C.POINTER(C.c_float)), n, C.byref(got)),
              "spk_server_read_spikes")
        return ids[:got.value], times[:got.value]

    def cancel(self, job: int):
        check(lib().spk_server_cancel(self.h, job), "spk_server_cancel")

    def release(self, job: int):
        check(lib().spk_server_release(self.h, job), "spk_server_release")

    def stats(self) -> N.ServerStats:
        st = N.ServerStats()
        check(lib().spk_server_stats_get(self.h, C.byref(st)), "spk_server_stats_get")
        return st

    def stop(self):
        if self.h:
            lib().spk_server_stop(self.h)
        self.h = None

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass
