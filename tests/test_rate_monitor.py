"""The rate monitor (GPU): per-neuron spike counts kept on the device as the
spikes are decided (RateActivityMonitor, Spike/ActivityMonitor/
RateActivityMonitor.cpp and Spike/Backend/CUDA/ActivityMonitor/
RateActivityMonitor.cu:50-71) equal the histogram of the recorded raster, for
neurons and inputs, across clears and resets, alone, in both batch modes and
through the model API."""
import numpy as np
import pytest

import cases
import descs
from oracle import OracleNet
from spike_gb300 import Batch, Net
from spike_gb300 import _native as N
from spike_gb300.networks import sweep_instance

pytestmark = pytest.mark.gpu


def histogram(net, pop, n):
    ids, _ = net.spikes(pop)
    return np.bincount(ids, minlength=n).astype(np.int32)


def test_counts_equal_the_raster_across_clear_and_reset():
    d = descs.random_voltage_net(n=300, n_in=200, seed=8)
    net = Net.from_desc(d.desc)
    o = OracleNet(d.desc)
    net.run(0.04)
    o.run(0.04)
    assert net.synchronize() == 0
    for pop, n in ((N.SPK_POP_NEURONS, 300), (N.SPK_POP_INPUTS, 200)):
        counts = net.rate_counts(n, pop)
        np.testing.assert_array_equal(counts, histogram(net, pop, n))
        # the oracle's raster gives the same counts
        oi, _ = o.spikes(pop)
        np.testing.assert_array_equal(counts, np.bincount(oi, minlength=n))
        assert counts.sum() > 0
    # a clear restarts the counts; the spike store keeps its spikes
    net.clear_rate_counts()
    net.clear_spikes()
    net.run(0.02)
    assert net.synchronize() == 0
    np.testing.assert_array_equal(net.rate_counts(300), histogram(net, N.SPK_POP_NEURONS, 300))
    # a reset zeroes them
    net.reset_state()
    assert not net.rate_counts(300).any() and not net.rate_counts(200, N.SPK_POP_INPUTS).any()


@pytest.mark.parametrize("mode", [N.SPK_BATCH_WAVES, N.SPK_BATCH_BULK])
def test_counts_in_batches(mode):
    gens = [sweep_instance(n, 0.04, 5.0, plastic, seed=60 + i, d_max=6)
            for i, (n, plastic) in enumerate(((1200, True), (3000, False), (700, False)))]
    nets = [Net.generate(g) for g in gens]
    b = Batch(nets)
    b.set_mode(mode)
    b.run_steps(400, True)
    assert b.synchronize() == 0
    for g, net in zip(gens, nets):
        n = g.desc.n_neurons
        counts = net.rate_counts(n)
        np.testing.assert_array_equal(counts, histogram(net, N.SPK_POP_NEURONS, n))
        assert counts.sum() > 0
    b.close()


def test_model_rate_monitor():
    m = cases.ref_va(True)
    m.add_rate_monitor()
    m.run(0.03)
    counts = m.rate_counts()
    ids, _ = m.spikes()
    assert len(counts) == 400 and counts.sum() == len(ids) > 0
    np.testing.assert_array_equal(counts, np.bincount(ids, minlength=400))
    m.run(0.02)  # counts accumulate over runs until a reset, as the monitor's spikes do
    ids2, _ = m.spikes()
    np.testing.assert_array_equal(m.rate_counts(), np.bincount(ids2, minlength=400))
    m.reset_state()
    m.clear_spikes()
    m.run(0.01)
    ids3, _ = m.spikes()
    np.testing.assert_array_equal(m.rate_counts(), np.bincount(ids3, minlength=400))
