"""ctypes binding of oracle/liboracle.so (TEST INFRASTRUCTURE ONLY)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None


def oracle_lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_PATH):
            from spike_gb300 import _build
            _build.build_oracle()
        L = C.CDLL(ORACLE_PATH)
        vp = C.c_void_p
        sigs = {
            "oracle_create": [vp, C.c_int, C.POINTER(vp)],
            "oracle_destroy": [vp],
            "oracle_set_threads": [vp, C.c_int],
            "oracle_reset_state": [vp],
            "oracle_reset_time": [vp],
            "oracle_select_stimulus": [vp, C.c_int],
            "oracle_run": [vp, C.c_float, C.c_int],
            "oracle_run_steps": [vp, C.c_int64, C.c_int],
            "oracle_current_time": [vp, C.POINTER(C.c_float)],
            "oracle_spike_count": [vp, C.c_int, C.POINTER(C.c_int64)],
            "oracle_read_spikes": [vp, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_float), C.c_int64,
                                   C.POINTER(C.c_int64)],
            "oracle_clear_spikes": [vp],
            "oracle_read_state": [vp, C.c_int, C.POINTER(C.c_float), C.c_int64],
            "oracle_read_weights": [vp, C.POINTER(C.c_float), C.c_int64],
            "oracle_synaptic_events": [vp, C.POINTER(C.c_uint64)],
            "oracle_ring_depth": [vp, C.POINTER(C.c_int32)],
            "oracle_timestep_grouping": [vp, C.POINTER(C.c_int32)],
            "oracle_sorted_synapses": [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                       C.c_int64],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.restype = C.c_int
            fn.argtypes = args
        L.oracle_philox4x32_10.restype = None
        L.oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.oracle_logf.restype = C.c_float
        L.oracle_logf.argtypes = [C.c_float]
        L.oracle_log_max_ulp.restype = C.c_double
        L.oracle_log_max_ulp.argtypes = []
        L.oracle_generate.restype = C.c_int64
        L.oracle_generate.argtypes = [vp] + [vp] * 7 + [C.c_int64]
        _lib = L
    return _lib


def _ok(rc: int, where: str):
    if rc != 0:
        raise RuntimeError(f"{where} failed with status {rc}")


class OracleNet:
    """The reference step loop on the CPU, from the same flat descriptor the
    engine takes.  precision 32 is the bit-exact checker, 64 the FP64 twin."""

    def __init__(self, desc, precision: int = 32, threads: int = 1):
        self.h = C.c_void_p()
        _ok(oracle_lib().oracle_create(C.byref(desc), precision, C.byref(self.h)), "oracle_create")
        self.n_synapses = desc.n_synapses
        self.n_neurons = desc.n_neurons
        self.n_inputs = desc.n_inputs
        if threads > 1:
            _ok(oracle_lib().oracle_set_threads(self.h, threads), "oracle_set_threads")

    def close(self):
        if self.h:
            oracle_lib().oracle_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, seconds: float, plasticity_on: bool = True):
        _ok(oracle_lib().oracle_run(self.h, C.c_float(seconds), 1 if plasticity_on else 0), "oracle_run")

    def run_steps(self, steps: int, plasticity_on: bool = True):
        _ok(oracle_lib().oracle_run_steps(self.h, steps, 1 if plasticity_on else 0), "oracle_run_steps")

    def reset_state(self):
        _ok(oracle_lib().oracle_reset_state(self.h), "oracle_reset_state")

    def reset_time(self):
        _ok(oracle_lib().oracle_reset_time(self.h), "oracle_reset_time")

    def select_stimulus(self, s: int):
        _ok(oracle_lib().oracle_select_stimulus(self.h, s), "oracle_select_stimulus")

    def current_time(self) -> float:
        t = C.c_float()
        _ok(oracle_lib().oracle_current_time(self.h, C.byref(t)), "oracle_current_time")
        return t.value

    def spikes(self, population: int = 0):
        n = C.c_int64()
        _ok(oracle_lib().oracle_spike_count(self.h, population, C.byref(n)), "oracle_spike_count")
        ids = np.empty(n.value, np.int32)
        times = np.empty(n.value, np.float32)
        got = C.c_int64()
        _ok(oracle_lib().oracle_read_spikes(self.h, population, ids.ctypes.data_as(C.POINTER(C.c_int32)),
                                            times.ctypes.data_as(C.POINTER(C.c_float)), n.value, C.byref(got)),
            "oracle_read_spikes")
        return ids[:got.value], times[:got.value]

    def clear_spikes(self):
        _ok(oracle_lib().oracle_clear_spikes(self.h), "oracle_clear_spikes")

    def state(self, field: int, count: int) -> np.ndarray:
        out = np.empty(count, np.float32)
        _ok(oracle_lib().oracle_read_state(self.h, field, out.ctypes.data_as(C.POINTER(C.c_float)), count),
            "oracle_read_state")
        return out

    def weights(self) -> np.ndarray:
        out = np.empty(self.n_synapses, np.float32)
        _ok(oracle_lib().oracle_read_weights(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), self.n_synapses),
            "oracle_read_weights")
        return out

    def events(self) -> int:
        e = C.c_uint64()
        _ok(oracle_lib().oracle_synaptic_events(self.h, C.byref(e)), "oracle_synaptic_events")
        return e.value

    def ring_depth(self) -> int:
        b = C.c_int32()
        _ok(oracle_lib().oracle_ring_depth(self.h, C.byref(b)), "oracle_ring_depth")
        return b.value

    def timestep_grouping(self) -> int:
        g = C.c_int32()
        _ok(oracle_lib().oracle_timestep_grouping(self.h, C.byref(g)), "oracle_timestep_grouping")
        return g.value

    def sorted_synapses(self):
        S = self.n_synapses
        pre = np.empty(S, np.int32)
        post = np.empty(S, np.int32)
        delay = np.empty(S, np.int32)
        _ok(oracle_lib().oracle_sorted_synapses(self.h, pre.ctypes.data_as(C.POINTER(C.c_int32)),
                                                post.ctypes.data_as(C.POINTER(C.c_int32)),
                                                delay.ctypes.data_as(C.POINTER(C.c_int32)), S),
            "oracle_sorted_synapses")
        return pre, post, delay


def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    oracle_lib().oracle_philox4x32_10(c, k, o)
    return list(o)


def generate_synapses(gen) -> dict:
    """Synapse arrays (creation order) of a generated network, from the
    oracle's restatement of the device generator.  `gen` is a GenDesc."""
    L = oracle_lib()
    n = L.oracle_generate(C.byref(gen), None, None, None, None, None, None, None, 0)
    if n < 0:
        raise RuntimeError("oracle_generate rejected the descriptor")
    out = dict(pre=np.empty(n, np.int32), post=np.empty(n, np.int32), weight=np.empty(n, np.float32),
               scale=np.empty(n, np.float32), delay=np.empty(n, np.int32), label=np.empty(n, np.int32),
               plastic=np.empty(n, np.uint8))
    got = L.oracle_generate(C.byref(gen), *(out[k].ctypes.data for k in
                                            ("pre", "post", "weight", "scale", "delay", "label", "plastic")), n)
    assert got == n
    return out
