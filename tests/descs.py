"""Flat network descriptors built directly from arrays, for hand-computable
cases (the C ABI's spk_net_desc, include/spike_gb300.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from spike_gb300 import _native as N


class Desc:
    """Owns the numpy arrays a NetDesc points into."""

    def __init__(self, *, kind=N.SPK_SYN_VOLTAGE, groups, dt=0.0001, refractory=0.002, i_bg=0.0,
                 n_inputs=0, rates=None, label_tau=None, label_vhat=None, n_labels=1,
                 pre=(), post=(), weight=(), scale=None, delay=(), label=None, plastic=None,
                 stdp=None, seed=1, spike_capacity=0, record_inputs=False, stdp_rule=0, weight_norm=0,
                 norm_initial=None, norm_sum=None):
        self.keep = []
        d = N.NetDesc()
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
        S = len(pre)
        arrs = dict(pre=np.asarray(pre, np.int32), post=np.asarray(post, np.int32),
                    weight=np.asarray(weight, np.float32),
                    scale=np.asarray(scale if scale is not None else np.ones(S), np.float32),
                    delay=np.asarray(delay, np.int32),
                    label=np.asarray(label if label is not None else np.zeros(S), np.int32))
        self.arrays = {k: np.ascontiguousarray(v) for k, v in arrs.items()}
        self.keep += list(self.arrays.values())
        d.n_synapses = S
        d.pre = self.arrays["pre"].ctypes.data_as(C.POINTER(C.c_int32))
        d.post = self.arrays["post"].ctypes.data_as(C.POINTER(C.c_int32))
        d.weight = self.arrays["weight"].ctypes.data_as(C.POINTER(C.c_float))
        d.scale = self.arrays["scale"].ctypes.data_as(C.POINTER(C.c_float))
        d.delay = self.arrays["delay"].ctypes.data_as(C.POINTER(C.c_int32))
        d.label = self.arrays["label"].ctypes.data_as(C.POINTER(C.c_int32))
        if plastic is not None:
            p = np.ascontiguousarray(plastic, np.uint8)
            self.keep.append(p)
            d.plastic = p.ctypes.data_as(C.POINTER(C.c_uint8))
        if stdp is not None:
            d.has_stdp = 1
            d.stdp = stdp.to_c() if hasattr(stdp, "to_c") else stdp
        d.seed = seed
        d.spike_capacity = spike_capacity
        d.record_inputs = 1 if record_inputs else 0
        d.stdp_rule = stdp_rule
        d.weight_norm = weight_norm
        for name, arr in (("norm_initial", norm_initial), ("norm_sum", norm_sum)):
            if arr is not None:
                a = np.ascontiguousarray(arr, np.float32)
                self.keep.append(a)
                setattr(d, name, a.ctypes.data_as(C.POINTER(C.c_float)))
        # the descriptor keeps its owner (and the arrays it points into) alive, so
        # that a descriptor taken from a temporary stays valid
        d._owner = self
        self.desc = d


def random_voltage_net(n=300, n_in=200, rate=40.0, p=0.08, d_max=12, seed=5, plastic=False, stdp=None,
                       j=8.0e-4, g=4.0, record_inputs=True, stdp_rule=0, weight_norm=0, norm_initial=None,
                       norm_sum=None, d_min=1):
    """A small random voltage-synapse network with inputs, E/I weights and
    delays d_min..d_max (multapses included; d_min > 1 groups timesteps), for
    parity tests."""
    rng = np.random.default_rng(seed)
    n_exc = int(0.8 * n)
    pre, post, w, dl = [], [], [], []
    for q in range(n):
        k_rec = rng.binomial(n, p)
        k_in = rng.binomial(n_in, p)
        pr = rng.integers(0, n, k_rec)
        pi = -rng.integers(0, n_in, k_in) - 1
        for s in pr:
            pre.append(s)
            post.append(q)
            w.append(j if s < n_exc else -g * j)
        for s in pi:
            pre.append(s)
            post.append(q)
            w.append(j * 1.5)
    S = len(pre)
    dl = rng.integers(d_min, d_max + 1, S)
    dl[0] = d_min
    plastic_mask = None
    if plastic:
        pre_a = np.asarray(pre)
        plastic_mask = ((pre_a >= 0) & (pre_a < n_exc)) | (pre_a < 0)
    return Desc(kind=N.SPK_SYN_VOLTAGE,
                groups=[dict(count=n_exc, tau_m=0.02, R=1e8, v0=0.0, vreset=0.0, theta=0.02, v_init_lo=0.0,
                             v_init_hi=0.018),
                        dict(count=n - n_exc, tau_m=0.01, R=1e8, v0=0.0, vreset=0.002, theta=0.018)],
                refractory=0.002, n_inputs=n_in, rates=rng.uniform(0.5 * rate, 1.5 * rate, n_in).astype(np.float32),
                pre=pre, post=post, weight=w, delay=dl, plastic=plastic_mask, stdp=stdp, seed=seed + 100,
                record_inputs=record_inputs, stdp_rule=stdp_rule, weight_norm=weight_norm,
                norm_initial=norm_initial, norm_sum=norm_sum)
