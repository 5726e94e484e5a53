"""Bit-exact comparison of an engine network with the oracle (shared by the
GPU parity tests)."""
import numpy as np

from oracle import OracleNet
from spike_gb300 import Net
from spike_gb300 import _native as N


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def ring_depth(o: OracleNet) -> int:
    """D_max + 2G + 1 (SpikingSynapses.cu:48) as the oracle sized its ring."""
    return o.ring_depth()


def assert_same(net: Net, o: OracleNet, n: int, n_in: int, n_labels: int, weights: bool = False, tag: str = ""):
    for pop in (N.SPK_POP_NEURONS, N.SPK_POP_INPUTS):
        gi, gt = net.spikes(pop)
        oi, ot = o.spikes(pop)
        assert len(gi) == len(oi), f"{tag} pop {pop}: {len(gi)} spikes vs oracle {len(oi)}"
        np.testing.assert_array_equal(gi, oi, err_msg=f"{tag} pop {pop} ids")
        np.testing.assert_array_equal(bits(gt), bits(ot), err_msg=f"{tag} pop {pop} times")
    for field, cnt in ((N.SPK_FIELD_V, n), (N.SPK_FIELD_LAST_SPIKE, n), (N.SPK_FIELD_SYN_TRACE, n * n_labels),
                       (N.SPK_FIELD_INPUT_NEXT, n_in)):
        np.testing.assert_array_equal(bits(net.state(field, cnt)), bits(o.state(field, cnt)),
                                      err_msg=f"{tag} field {field}")
    B = ring_depth(o)
    np.testing.assert_array_equal(bits(net.state(N.SPK_FIELD_RING, B * n * n_labels)),
                                  bits(o.state(N.SPK_FIELD_RING, B * n * n_labels)), err_msg=f"{tag} ring")
    if weights:
        np.testing.assert_array_equal(bits(net.weights(o.n_synapses)), bits(o.weights()), err_msg=f"{tag} weights")
    assert net.events() == o.events(), tag
