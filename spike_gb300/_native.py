"""ctypes binding of the C ABI (include/spike_gb300.h, include/spike_gb300_model.h).

The structures below mirror the C declarations field for field.  Loading fails
loudly when the native library is missing: there is no Python fallback for the
step engine.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspike_gb300.so")

SPK_ABI_VERSION = 4
SPK_OK = 0
SPK_ERR_INVALID = -1
SPK_ERR_CUDA = -2
SPK_ERR_OOM = -3
SPK_ERR_UNSUPPORTED = -4
SPK_ERR_TIMEOUT = -5
SPK_ERR_OVERFLOW = -6
SPK_STDP_WEIGHT_DEPENDENT = 0
SPK_STDP_EVANS = 1
SPK_STDP_INHIBITORY = 2
SPK_STDP_CUSTOM = 3
SPK_NORM_OFF = 0
SPK_NORM_AFTER_RULE = 1
SPK_NORM_BEFORE_RULE = 2
SPK_ERR_STATE = -7
SPK_ERR_BUSY = -8
ERROR_NAMES = {
    SPK_ERR_INVALID: "SPK_ERR_INVALID", SPK_ERR_CUDA: "SPK_ERR_CUDA", SPK_ERR_OOM: "SPK_ERR_OOM",
    SPK_ERR_UNSUPPORTED: "SPK_ERR_UNSUPPORTED", SPK_ERR_TIMEOUT: "SPK_ERR_TIMEOUT",
    SPK_ERR_OVERFLOW: "SPK_ERR_OVERFLOW", SPK_ERR_STATE: "SPK_ERR_STATE", SPK_ERR_BUSY: "SPK_ERR_BUSY",
}

SPK_SYN_CONDUCTANCE = 1
SPK_SYN_CURRENT = 2
SPK_SYN_VOLTAGE = 3
SPK_POP_NEURONS = 0
SPK_POP_INPUTS = 1
SPK_FIELD_V = 0
SPK_FIELD_LAST_SPIKE = 1
SPK_FIELD_SYN_TRACE = 2
SPK_FIELD_INPUT_NEXT = 3
SPK_FIELD_RING = 4
SPK_FIELD_PRE_TRACE = 5
SPK_FIELD_POST_TRACE = 6

SPK_CONN_ALL_TO_ALL = 0
SPK_CONN_ONE_TO_ONE = 1
SPK_CONN_RANDOM = 2
SPK_CONN_GAUSSIAN_SAMPLE = 3
SPK_CONN_PAIRWISE = 4
SPK_INPUT_NONE = 0
SPK_INPUT_POISSON = 1
SPK_INPUT_PATTERNED = 2

i32, i64, u64, f32 = C.c_int32, C.c_int64, C.c_uint64, C.c_float
P = C.POINTER


class NeuronGroup(C.Structure):
    _fields_ = [("start", i32), ("count", i32), ("tau_m", f32), ("R", f32), ("v0", f32),
                ("vreset", f32), ("theta", f32), ("v_init_lo", f32), ("v_init_hi", f32)]


class StdpParams(C.Structure):
    _fields_ = [("a_minus", f32), ("a_plus", f32), ("tau_minus", f32), ("tau_plus", f32),
                ("lambda_", f32), ("alpha", f32), ("w_max", f32), ("clip_upper", i32)]


class NetDesc(C.Structure):
    _fields_ = [
        ("abi_version", i32), ("dt", f32), ("synapse_kind", i32),
        ("n_neurons", i32), ("n_groups", i32), ("groups", P(NeuronGroup)),
        ("refractory_period", f32), ("background_current", f32),
        ("n_inputs", i32), ("n_stimuli", i32), ("input_rates", P(f32)), ("stimulus", i32),
        ("n_labels", i32), ("label_tau", P(f32)), ("label_vhat", P(f32)),
        ("n_synapses", i64), ("pre", P(i32)), ("post", P(i32)), ("weight", P(f32)),
        ("scale", P(f32)), ("delay", P(i32)), ("label", P(i32)), ("plastic", P(C.c_uint8)),
        ("has_stdp", i32), ("stdp", StdpParams),
        ("seed", u64), ("spike_capacity", i64), ("record_inputs", i32), ("stdp_rule", i32),
        ("weight_norm", i32), ("norm_initial", P(f32)), ("norm_sum", P(f32)),
    ]


class Projection(C.Structure):
    _fields_ = [("pre_population", i32), ("pre_start", i32), ("pre_count", i32), ("post_start", i32),
                ("post_count", i32), ("probability", f32), ("weight_lo", f32), ("weight_hi", f32), ("scale", f32),
                ("delay_lo", i32), ("delay_hi", i32), ("label", i32), ("plastic", i32)]


class GenDesc(C.Structure):
    _fields_ = [
        ("abi_version", i32), ("dt", f32), ("synapse_kind", i32),
        ("n_neurons", i32), ("n_groups", i32), ("groups", P(NeuronGroup)),
        ("refractory_period", f32), ("background_current", f32),
        ("n_inputs", i32), ("n_stimuli", i32), ("input_rates", P(f32)), ("stimulus", i32),
        ("n_labels", i32), ("label_tau", P(f32)), ("label_vhat", P(f32)),
        ("n_projections", i32), ("projections", P(Projection)),
        ("has_stdp", i32), ("stdp", StdpParams),
        ("seed", u64), ("connectivity_seed", u64), ("spike_capacity", i64), ("record_inputs", i32),
        ("stdp_rule", i32),
    ]


class ServerOpts(C.Structure):
    _fields_ = [("warps_per_cta", i32), ("tile_posts", i32), ("steps_per_block", i32), ("max_running", i32),
                ("reserve_bytes", u64), ("record_spikes", i32), ("mode", i32)]


class JobInfo(C.Structure):
    _fields_ = [("state", i32), ("error", i32), ("steps_done", i64), ("steps_total", i64), ("events", u64),
                ("spikes", i64), ("synapses", i64), ("submit_s", C.c_double), ("start_s", C.c_double),
                ("finish_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", i64), ("running", i64), ("queued", i64), ("done", i64), ("failed", i64),
                ("events", u64), ("blocks", i64), ("busy_s", C.c_double), ("uptime_s", C.c_double),
                ("rebuilds", i64)]


SPK_BATCH_WAVES, SPK_BATCH_BULK = 0, 1
(SPK_KERNEL_NEURONS, SPK_KERNEL_LIST, SPK_KERNEL_RULES, SPK_KERNEL_POST, SPK_KERNEL_PROPAGATION,
 SPK_KERNEL_FINISH, SPK_KERNEL_KINDS) = range(7)
KERNEL_NAMES = ("neurons", "list", "rules", "post", "propagation", "finish")
SPK_JOB_QUEUED, SPK_JOB_RUNNING, SPK_JOB_DONE, SPK_JOB_FAILED, SPK_JOB_CANCELLED = 0, 1, 2, 3, 4


class Schedule(C.Structure):
    _fields_ = [("warps_per_cta", i32), ("tile_posts", i32), ("ctas", i32), ("steps_per_launch", i32)]


class LifParams(C.Structure):
    _fields_ = [("group_shape", i32 * 2), ("resting_potential_v0", f32),
                ("after_spike_reset_potential_vreset", f32),
                ("threshold_for_action_potential_spike", f32), ("absolute_refractory_period", f32),
                ("somatic_capacitance_Cm", f32), ("somatic_leakage_conductance_g0", f32),
                ("background_current", f32), ("v_init_lo", f32), ("v_init_hi", f32)]


class SynapseParams(C.Structure):
    _fields_ = [("connectivity_type", i32), ("weight_range", f32 * 2), ("weight_scaling_constant", f32),
                ("random_connectivity_probability", f32), ("delay_range", f32 * 2),
                ("reversal_potential_Vhat", f32), ("decay_term_tau_g", f32), ("decay_term_tau", f32),
                ("max_number_of_connections_per_pair", i32),
                ("gaussian_synapses_per_postsynaptic_neuron", i32),
                ("gaussian_synapses_standard_deviation", f32), ("n_pairwise", i32),
                ("pairwise_connect_presynaptic", P(i32)), ("pairwise_connect_postsynaptic", P(i32)),
                ("pairwise_connect_weight", P(f32)), ("pairwise_connect_delay", P(f32)),
                ("plasticity_rule", i32), ("plasticity_rule_2", i32)]


class DeviceNet(C.Structure):
    """spk_device_net: a network over caller-owned device buffers."""
    _fields_ = [
        ("n_neurons", i32), ("n_inputs", i32), ("n_labels", i32), ("synapse_kind", i32), ("max_delay", i32),
        ("warps_per_cta", i32), ("tile_posts", i32), ("ctas", i32),
        ("dt", f32), ("refractory_period", f32), ("background_current", f32),
        ("n_groups", i32), ("groups", P(NeuronGroup)), ("label_tau", P(f32)), ("label_vhat", P(f32)),
        ("has_stdp", i32), ("stdp", StdpParams), ("n_plastic_scales", i32), ("plastic_scales", P(f32)),
        ("seed", u64), ("record_inputs", i32),
        ("rowptr", C.c_void_p), ("entries", C.c_void_p), ("csc_ptr", C.c_void_p), ("csc", C.c_void_p),
        ("V", C.c_void_p), ("last_spike", C.c_void_p), ("syn_trace", C.c_void_p), ("ring", C.c_void_p),
        ("input_next", C.c_void_p), ("rates", C.c_void_p), ("post_trace", C.c_void_p),
        ("pre_trace", C.c_void_p), ("spikes", C.c_void_p), ("spike_capacity", i64), ("run_state", C.c_void_p),
        ("timestep_grouping", i32), ("group_bits", C.c_void_p),
    ]


SPK_NOALLOC_SCRATCH_BYTES = 4 << 20
SPK_RUN_STATE_BYTES = 128

_VP = C.c_void_p
_SIGS = {
    # spike_gb300.h
    "spk_net_create": (i32, [P(NetDesc), P(Schedule), P(_VP)]),
    "spk_net_generate": (i32, [P(GenDesc), P(Schedule), P(_VP)]),
    "spk_net_synapse_count": (i32, [_VP, P(i64)]),
    "spk_net_plastic_synapse_count": (i32, [_VP, P(i64)]),
    "spk_net_destroy": (i32, [_VP]),
    "spk_net_reset_state": (i32, [_VP]),
    "spk_net_reset_time": (i32, [_VP]),
    "spk_net_select_stimulus": (i32, [_VP, i32]),
    "spk_net_write_rates": (i32, [_VP, i32, _VP, i64]),
    "spk_net_run": (i32, [_VP, f32, i32]),
    "spk_net_run_steps": (i32, [_VP, i64, i32]),
    "spk_net_synchronize": (i32, [_VP]),
    "spk_net_current_time": (i32, [_VP, P(f32)]),
    "spk_net_timestep_grouping": (i32, [_VP, P(i32)]),
    "spk_net_spike_count": (i32, [_VP, i32, P(i64)]),
    "spk_net_read_spikes": (i32, [_VP, i32, P(i32), P(f32), i64, P(i64)]),
    "spk_net_clear_spikes": (i32, [_VP]),
    "spk_net_rate_counts": (i32, [_VP, i32, P(i32), i64]),
    "spk_net_clear_rate_counts": (i32, [_VP]),
    "spk_net_read_state": (i32, [_VP, i32, _VP, i64]),
    "spk_net_read_weights": (i32, [_VP, P(f32), i64]),
    "spk_net_write_weights": (i32, [_VP, P(f32), i64]),
    "spk_net_synaptic_events": (i32, [_VP, P(u64)]),
    "spk_net_stdp_counts": (i32, [_VP, P(u64), P(u64)]),
    "spk_net_get_schedule": (i32, [_VP, P(Schedule)]),
    "spk_net_set_wait_limit": (i32, [_VP, C.c_double]),
    "spk_net_snapshot_bytes": (i32, [_VP, P(i64)]),
    "spk_net_snapshot": (i32, [_VP, _VP, i64]),
    "spk_net_restore": (i32, [_VP, _VP, i64]),
    "spk_net_inject_withheld_cta": (i32, [_VP, i32]),
    "spk_net_device_bytes": (i32, [_VP, P(i64)]),
    "spk_net_launch_count": (i32, [_VP, P(i64)]),
    "spk_net_stream": (i32, [_VP, P(_VP)]),
    "spk_batch_create": (i32, [P(_VP), i32, P(Schedule), P(_VP)]),
    "spk_batch_run_steps": (i32, [_VP, i64, i32]),
    "spk_batch_run_steps_each": (i32, [_VP, P(i64), P(i32)]),
    "spk_batch_step_block": (i32, [_VP]),
    "spk_batch_set_mode": (i32, [_VP, i32]),
    "spk_net_begin_run": (i32, [_VP, i64, i32]),
    "spk_batch_synchronize": (i32, [_VP]),
    "spk_batch_launch_count": (i32, [_VP, P(i64)]),
    "spk_batch_time_kernels": (i32, [_VP, i64, i32, P(C.c_double)]),
    "spk_batch_stream": (i32, [_VP, P(_VP)]),
    "spk_batch_read_spikes": (i32, [_VP, i32, P(i32), P(f32), i64, P(i64), i32]),
    "spk_batch_destroy": (i32, [_VP]),
    "spk_batch_autotune": (i32, [P(GenDesc), i32, i32, P(Schedule), P(f32), P(f32), P(i32)]),
    "spk_net_set_step_cost": (i32, [_VP, f32]),
    "spk_step_noalloc": (i32, [P(DeviceNet), i64, i32, f32, _VP]),
    "spk_server_start": (i32, [P(ServerOpts), P(_VP)]),
    "spk_server_submit": (i32, [_VP, P(GenDesc), i64, i32, P(i64)]),
    "spk_server_poll": (i32, [_VP, i64, P(JobInfo)]),
    "spk_server_wait": (i32, [_VP, i64, C.c_double]),
    "spk_server_read_spikes": (i32, [_VP, i64, P(i32), P(f32), i64, P(i64)]),
    "spk_server_cancel": (i32, [_VP, i64]),
    "spk_server_release": (i32, [_VP, i64]),
    "spk_server_stats_get": (i32, [_VP, P(ServerStats)]),
    "spk_server_stop": (i32, [_VP]),
    "spk_net_generate_estimate": (i32, [P(GenDesc), P(Schedule), P(i64), P(i64)]),
    "spk_memory_info": (i32, [P(u64), P(u64)]),
    "spk_abi_version": (i32, []),
    "spk_last_error": (C.c_char_p, []),
    # spike_gb300_model.h
    "spk_model_create": (i32, [i32, i32, i32, P(_VP)]),
    "spk_model_destroy": (i32, [_VP]),
    "spk_model_set_timestep": (i32, [_VP, f32]),
    "spk_model_set_seed": (i32, [_VP, u64]),
    "spk_model_add_neuron_group": (i32, [_VP, P(LifParams), P(i32)]),
    "spk_model_add_input_group": (i32, [_VP, i32, i32, f32, P(i32)]),
    "spk_model_add_stimulus": (i32, [_VP, P(f32), i32, P(i32)]),
    "spk_model_add_stdp_rule": (i32, [_VP, P(StdpParams), P(i32)]),
    "spk_model_add_plasticity_rule": (i32, [_VP, i32, P(StdpParams), P(i32)]),
    "spk_model_add_weight_norm_rule": (i32, [_VP, i32, f32, P(i32)]),
    "spk_model_add_synapse_group": (i32, [_VP, i32, i32, P(SynapseParams), P(i32)]),
    "spk_model_connect_with_sparsity": (i32, [_VP, i32, i32, f32, P(SynapseParams), P(i32)]),
    "spk_model_set_recording": (i32, [_VP, i32, i64]),
    "spk_model_finalise": (i32, [_VP, P(Schedule)]),
    "spk_model_run": (i32, [_VP, f32, i32]),
    "spk_model_reset_state": (i32, [_VP]),
    "spk_model_reset_time": (i32, [_VP]),
    "spk_model_select_stimulus": (i32, [_VP, i32]),
    "spk_model_net": (i32, [_VP, P(_VP)]),
    "spk_model_desc": (i32, [_VP, P(NetDesc)]),
    "spk_model_counts": (i32, [_VP, P(i32), P(i32), P(i64)]),
    "spk_model_spikes": (i32, [_VP, i32, P(P(i32)), P(P(f32)), P(i64)]),
    "spk_model_clear_spikes": (i32, [_VP]),
    "spk_model_add_rate_monitor": (i32, [_VP, i32]),
    "spk_model_rate_counts": (i32, [_VP, i32, P(P(i32)), P(i64)]),
}

_lib = None


def exported_symbols() -> list[str]:
    return list(_SIGS)


class SpikeError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        self.code = code
        super().__init__(f"{where}: {ERROR_NAMES.get(code, code)}: {message}")


def lib() -> C.CDLL:
    """The loaded engine library (built in-tree by spike_gb300._build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(the CUDA engine has no fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.spk_abi_version() != SPK_ABI_VERSION:
            raise RuntimeError("libspike_gb300.so ABI version mismatch")
        _lib = L
    return _lib


def check(code: int, where: str) -> int:
    if code != SPK_OK:
        msg = lib().spk_last_error()
        raise SpikeError(code, where, msg.decode() if msg else "")
    return code
