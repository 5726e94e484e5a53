"""The C ABI library loads and exports every function include/*.h declares
(CPU: no compute calls)."""
import ctypes
import os
import re

from spike_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("spike_gb300.h", "spike_gb300_model.h"):
        with open(os.path.join(ROOT, "include", h)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(spk_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declarations_are_exported_and_bound():
    lib = ctypes.CDLL(_native.LIB_PATH)
    decl = declared_functions()
    assert len(decl) > 40
    for name in decl:
        assert hasattr(lib, name), f"{name} declared but not exported"
    assert set(decl) == set(_native.exported_symbols())


def test_abi_version_and_error_without_gpu_work():
    lib = _native.lib()
    assert lib.spk_abi_version() == _native.SPK_ABI_VERSION
    # argument validation fails before any device call
    assert lib.spk_net_create(None, None, None) == _native.SPK_ERR_INVALID
    assert lib.spk_net_run(None, ctypes.c_float(1.0), 1) == _native.SPK_ERR_INVALID
    assert isinstance(lib.spk_last_error(), bytes)
    # batch entry points: no handle, no counts, an unknown mode or population
    counts = (ctypes.c_int64 * 4)()
    assert lib.spk_batch_read_spikes(None, 0, None, None, 0, counts, 0) == _native.SPK_ERR_INVALID
    assert lib.spk_batch_set_mode(None, _native.SPK_BATCH_BULK) == _native.SPK_ERR_INVALID
    assert lib.spk_batch_run_steps_each(None, None, None) == _native.SPK_ERR_INVALID
    assert lib.spk_batch_step_block(None) == _native.SPK_ERR_INVALID
    assert lib.spk_batch_destroy(None) == _native.SPK_ERR_INVALID


def test_noalloc_rejects_networks_beyond_its_scratch():
    """spk_step_noalloc checks its fixed scratch limit before any device call
    (zero steps: nothing would run even if the check let it through)."""
    lib = _native.lib()
    g = (_native.NeuronGroup * 1)()
    g[0].start, g[0].count, g[0].tau_m, g[0].R, g[0].theta = 0, 250000, 0.02, 1e8, 0.02
    dummy = ctypes.create_string_buffer(64)
    addr = ctypes.addressof(dummy)
    dn = _native.DeviceNet()
    dn.n_neurons, dn.n_inputs, dn.n_labels, dn.synapse_kind, dn.max_delay = 250000, 0, 1, _native.SPK_SYN_VOLTAGE, 1
    dn.warps_per_cta, dn.tile_posts, dn.ctas = 8, 256, 128  # 4.2 MB of exchange keys
    dn.dt, dn.refractory_period = 1e-4, 2e-3
    dn.n_groups, dn.groups = 1, g
    for f in ("rowptr", "entries", "V", "last_spike", "ring", "spikes", "run_state"):
        setattr(dn, f, addr)
    dn.spike_capacity = 1
    rc = lib.spk_step_noalloc(ctypes.byref(dn), 0, 0, ctypes.c_float(0.0), None)
    assert rc == _native.SPK_ERR_INVALID
    assert b"bytes of step scratch" in lib.spk_last_error()
    dn.tile_posts = 48  # not a multiple of 32
    assert lib.spk_step_noalloc(ctypes.byref(dn), 0, 0, ctypes.c_float(0.0), None) == _native.SPK_ERR_INVALID
    assert lib.spk_step_noalloc(None, 1, 0, ctypes.c_float(0.0), None) == _native.SPK_ERR_INVALID


def test_time_constants_are_validated_before_any_device_call():
    """A zero membrane or synaptic time constant, a non-positive STDP tau or a
    negative refractory period would give inf/NaN decay constants:
    spk_net_create and spk_step_noalloc refuse them before any device call."""
    import descs
    from spike_gb300.model import STDPParams
    lib = _native.lib()
    good = dict(count=10, tau_m=0.02)
    cases = [dict(groups=[dict(count=10, tau_m=0.0)]),
             dict(groups=[good], kind=_native.SPK_SYN_CURRENT, label_tau=[-0.005]),
             dict(groups=[good], refractory=-0.001),
             dict(groups=[good], pre=[0], post=[1], weight=[1e-4], delay=[1], plastic=[1],
                  stdp=STDPParams(tau_plus=0.0, tau_minus=0.02))]
    for kw in cases:
        d = descs.Desc(**kw)
        h = ctypes.c_void_p()
        assert lib.spk_net_create(ctypes.byref(d.desc), None, ctypes.byref(h)) == _native.SPK_ERR_INVALID, kw
        assert b"must be" in lib.spk_last_error(), lib.spk_last_error()
    g = (_native.NeuronGroup * 1)()
    g[0].start, g[0].count, g[0].tau_m, g[0].R, g[0].theta = 0, 64, 0.0, 1e8, 0.02
    dummy = ctypes.create_string_buffer(64)
    addr = ctypes.addressof(dummy)
    dn = _native.DeviceNet()
    dn.n_neurons, dn.n_inputs, dn.n_labels, dn.synapse_kind, dn.max_delay = 64, 0, 1, _native.SPK_SYN_VOLTAGE, 1
    dn.warps_per_cta, dn.tile_posts, dn.ctas = 2, 32, 1
    dn.dt, dn.refractory_period = 1e-4, 2e-3
    dn.n_groups, dn.groups = 1, g
    for f in ("rowptr", "entries", "V", "last_spike", "ring", "spikes", "run_state"):
        setattr(dn, f, addr)
    dn.spike_capacity = 1
    assert lib.spk_step_noalloc(ctypes.byref(dn), 0, 0, ctypes.c_float(0.0), None) == _native.SPK_ERR_INVALID
    assert b"tau_m" in lib.spk_last_error()


def test_malformed_generated_networks_are_rejected_before_any_device_call():
    from spike_gb300 import GenNetwork, Projection
    lib = _native.lib()
    bad = [
        [Projection(_native.SPK_POP_NEURONS, 0, 10, 0, 2000, 0.1)],                 # post range past N
        [Projection(_native.SPK_POP_INPUTS, 0, 10, 0, 100, 0.1)],                   # no inputs exist
        [Projection(_native.SPK_POP_NEURONS, 0, 10, 0, 100, 1.5)],                  # probability > 1
        [Projection(_native.SPK_POP_NEURONS, 0, 10, 0, 100, 0.1, delay=(0, 3))],    # delay 0
        [Projection(_native.SPK_POP_NEURONS, 0, 10, 0, 100, 0.1, plastic=True)],    # plastic without a rule
        [Projection(_native.SPK_POP_NEURONS, 0, 50, 0, 100, 0.1),
         Projection(_native.SPK_POP_NEURONS, 40, 20, 50, 10, 0.1)],                 # overlapping pairs
    ]
    for projs in bad:
        gen = GenNetwork(groups=[dict(count=100)], projections=projs)
        h = ctypes.c_void_p()
        assert lib.spk_net_generate(ctypes.byref(gen.desc), None, ctypes.byref(h)) == _native.SPK_ERR_INVALID
        assert lib.spk_last_error()
    assert lib.spk_net_generate(None, None, None) == _native.SPK_ERR_INVALID


def test_rule_fields_are_validated_before_any_device_call():
    """An unknown STDP rule or normalisation mode, or a normalisation without
    an STDP rule, is refused by spk_net_create before it touches a device."""
    import descs
    from spike_gb300.model import STDPParams
    lib = _native.lib()
    sp = STDPParams()
    cases = [dict(plastic=True, stdp=sp, stdp_rule=9), dict(plastic=True, stdp=sp, weight_norm=7),
             dict(plastic=True, stdp=sp, stdp_rule=-1), dict(weight_norm=_native.SPK_NORM_BEFORE_RULE)]
    for kw in cases:
        d = descs.random_voltage_net(n=40, n_in=10, **kw)
        h = ctypes.c_void_p()
        assert lib.spk_net_create(ctypes.byref(d.desc), None, ctypes.byref(h)) == _native.SPK_ERR_INVALID, kw
        assert lib.spk_last_error()
    # the weight-norm entry point of the model API needs a model
    assert lib.spk_model_add_weight_norm_rule(None, 0, ctypes.c_float(0.0), None) == _native.SPK_ERR_INVALID
    assert lib.spk_net_plastic_synapse_count(None, None) == _native.SPK_ERR_INVALID
