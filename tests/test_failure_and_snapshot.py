"""Failure detection and state snapshots (GPU).

The timeout test makes a bounded device wait run out by a fault made on the
host - one CTA of a multi-CTA network is left out of a launch, so nothing
ever publishes its step - with a 50 ms wait limit.  The run must end with
SPK_ERR_TIMEOUT (not hang), and after spk_net_reset_state the same handle must
run exactly like a fresh network.  Nothing faults on the device.
"""
import time

import numpy as np
import pytest

import descs
from engine_checks import bits
from spike_gb300 import GenNetwork, Net, Server, schedule
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams

pytestmark = pytest.mark.gpu

STDP = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0)


def state(net, n, n_in):
    ids, t = net.spikes()
    return dict(ids=ids, t=bits(t), V=bits(net.state(N.SPK_FIELD_V, n)),
                last=bits(net.state(N.SPK_FIELD_LAST_SPIKE, n)), nxt=bits(net.state(N.SPK_FIELD_INPUT_NEXT, n_in)))


def test_withheld_cta_times_out_and_reset_recovers():
    d = descs.random_voltage_net(n=300, n_in=200)
    sched = schedule(2, 32, 0, 100)  # 5 CTAs, launches of 100 steps
    net = Net.from_desc(d.desc, sched)
    assert net.schedule()["ctas"] == 5
    net.set_wait_limit(0.05)
    net.inject_withheld_cta(2)
    t0 = time.perf_counter()
    net.run_steps(250)
    rc = net.synchronize()
    assert rc == N.SPK_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 5.0
    # the context is still usable and the handle recovers through reset
    net.reset_state()
    net.reset_time()
    net.clear_spikes()
    net.run_steps(400)
    assert net.synchronize() == N.SPK_OK
    fresh = Net.from_desc(d.desc, sched)
    fresh.run_steps(400)
    assert fresh.synchronize() == N.SPK_OK
    a, b = state(net, 300, 200), state(fresh, 300, 200)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert len(a["ids"]) > 50


def test_snapshot_restore_continues_bit_exact():
    d = descs.random_voltage_net(n=300, n_in=200, plastic=True, stdp=STDP)
    S = d.desc.n_synapses
    a = Net.from_desc(d.desc)
    a.run_steps(300, True)
    snap = a.snapshot()
    a.clear_spikes()
    a.run_steps(400, True)
    assert a.synchronize() == 0
    b = Net.from_desc(d.desc)
    b.run_steps(77, True)  # state that the restore must overwrite
    b.restore(snap)
    b.clear_spikes()
    b.run_steps(400, True)
    assert b.synchronize() == 0
    sa, sb = state(a, 300, 200), state(b, 300, 200)
    for k in sa:
        np.testing.assert_array_equal(sa[k], sb[k], err_msg=k)
    np.testing.assert_array_equal(bits(a.weights(S)), bits(b.weights(S)))
    for f, n in ((N.SPK_FIELD_PRE_TRACE, 500), (N.SPK_FIELD_POST_TRACE, 300), (N.SPK_FIELD_RING, 15 * 300)):
        np.testing.assert_array_equal(bits(a.state(f, n)), bits(b.state(f, n)))
    assert abs(a.current_time() - b.current_time()) == 0
    # a network cut into other tiles cannot take the snapshot
    c = Net.from_desc(d.desc, schedule(4, 64, 0, 0))
    with pytest.raises(N.SpikeError):
        c.restore(snap)


def test_server_rejects_jobs_that_cannot_fit():
    gen = GenNetwork(groups=[dict(count=1000)], projections=[], n_inputs=0)
    srv = Server(reserve_bytes=1 << 62)  # no job can ever be admitted
    j = srv.submit(gen, 100)
    info = srv.wait(j, 30.0)
    assert info.state == N.SPK_JOB_FAILED and info.error == N.SPK_ERR_OOM
    srv.stop()
