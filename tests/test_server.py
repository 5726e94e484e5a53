"""The continuous-batching server (GPU): jobs submitted while others run are
admitted, overlap on the device, and each job's result is bit for bit the
result of the same network run alone."""
import time

import numpy as np
import pytest

from engine_checks import bits
from spike_gb300 import Net, Server
from spike_gb300 import _native as N
from spike_gb300.networks import sweep_instance

pytestmark = pytest.mark.gpu


def jobs(k=8, seed=9):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(400), np.log(5000), k)).astype(int)
    out = []
    for i in range(k):
        gen = sweep_instance(int(sizes[i]), float(rng.uniform(0.02, 0.06)), float(rng.uniform(3, 7)), i % 3 == 0,
                             seed=700 + i, d_max=8)
        out.append((gen, int(rng.integers(300, 1500)), bool(i % 2 == 0)))
    return out


@pytest.mark.parametrize("mode", [N.SPK_BATCH_WAVES, N.SPK_BATCH_BULK])
def test_served_jobs_equal_each_job_alone_and_overlap(mode):
    work = jobs()
    srv = Server(steps_per_block=250, reserve_bytes=1 << 30, mode=mode)
    ids = []
    for i, (gen, steps, plastic) in enumerate(work):
        ids.append(srv.submit(gen, steps, plastic))
        if i == 3:
            time.sleep(0.05)  # later jobs arrive while the first ones run
    infos = [srv.wait(j, 300.0) for j in ids]
    assert all(inf.state == N.SPK_JOB_DONE for inf in infos), [inf.state for inf in infos]
    # work of different jobs overlapped on the device
    assert any(b.start_s < a.finish_s and b.start_s > a.start_s for a in infos for b in infos)
    st = srv.stats()
    assert st.done == len(work) and st.blocks > 1
    for (gen, steps, plastic), j, inf in zip(work, ids, infos):
        ref = Net.generate(gen)
        ref.run_steps(steps, plastic)
        assert ref.synchronize() == 0
        ri, rt = ref.spikes()
        si, stt = srv.spikes(j)
        assert inf.steps_done == steps and inf.synapses == ref.synapse_count()
        np.testing.assert_array_equal(si, ri)
        np.testing.assert_array_equal(bits(stt), bits(rt))
        assert inf.events == ref.events()
        ref.close()
    srv.stop()


@pytest.mark.parametrize("mode", [N.SPK_BATCH_WAVES, N.SPK_BATCH_BULK])
def test_served_jobs_without_spike_recording(mode):
    """A server that records no spikes creates its networks without a spike
    store; the jobs still finish and deliver the events of the same job run
    alone."""
    work = jobs(k=4, seed=13)
    srv = Server(steps_per_block=200, reserve_bytes=1 << 30, mode=mode, record_spikes=False)
    ids = [srv.submit(gen, steps, plastic) for gen, steps, plastic in work]
    infos = [srv.wait(j, 300.0) for j in ids]
    assert all(inf.state == N.SPK_JOB_DONE for inf in infos), [inf.state for inf in infos]
    for (gen, steps, plastic), inf in zip(work, infos):
        ref = Net.generate(gen)
        ref.run_steps(steps, plastic)
        assert ref.synchronize() == 0
        assert inf.steps_done == steps and inf.events == ref.events()
        ref.close()
    srv.stop()


def test_served_jobs_with_the_trace_rules_and_the_event_driven_rule():
    """Jobs with the Evans rule (bulk mode only) served beside jobs with the
    event-driven rule and static jobs by a waves-mode server: a block that
    holds a trace-rule job runs in bulk mode, and every job equals the same
    network run alone."""
    rng = np.random.default_rng(21)
    work = []
    for i in range(6):
        n = int(np.exp(rng.uniform(np.log(500), np.log(3000))))
        rule = N.SPK_STDP_EVANS if i % 3 == 0 else N.SPK_STDP_WEIGHT_DEPENDENT
        gen = sweep_instance(n, float(rng.uniform(0.02, 0.05)), 5.0, i % 3 != 2, seed=900 + i, d_max=6, rule=rule)
        work.append((gen, int(rng.integers(300, 900)), True))
    srv = Server(steps_per_block=200, reserve_bytes=1 << 30, mode=N.SPK_BATCH_WAVES)
    ids = [srv.submit(gen, steps, plastic) for gen, steps, plastic in work]
    infos = [srv.wait(j, 300.0) for j in ids]
    assert all(inf.state == N.SPK_JOB_DONE for inf in infos), [inf.state for inf in infos]
    for (gen, steps, plastic), j, inf in zip(work, ids, infos):
        ref = Net.generate(gen)
        ref.run_steps(steps, plastic)
        assert ref.synchronize() == 0
        ri, rt = ref.spikes()
        si, stt = srv.spikes(j)
        np.testing.assert_array_equal(si, ri)
        np.testing.assert_array_equal(bits(stt), bits(rt))
        assert inf.events == ref.events()
        ref.close()
    srv.stop()


def test_cancel_and_stop_with_work_queued():
    work = jobs(k=5, seed=4)
    srv = Server(steps_per_block=200, reserve_bytes=1 << 30)
    ids = [srv.submit(gen, 50000, plastic) for gen, _, plastic in work]
    srv.cancel(ids[-1])
    time.sleep(0.2)
    srv.cancel(ids[0])
    info0 = srv.wait(ids[0], 120.0)
    assert info0.state == N.SPK_JOB_CANCELLED and info0.steps_done < 50000
    srv.stop()  # cancels the rest and frees every network


def test_served_grouped_jobs():
    """Jobs whose minimum delay is 2 steps (timestep grouping 2) run with
    grouped times, equal to the same network run alone; a job whose step
    count is not whole groups fails with SPK_ERR_INVALID and the others go on."""
    srv = Server(steps_per_block=250, reserve_bytes=1 << 30, mode=N.SPK_BATCH_BULK)
    work = [(sweep_instance(1200 + 300 * i, 0.03, 5.0, False, seed=900 + i, d_min=2, d_max=8), 600) for i in range(3)]
    ids = [srv.submit(gen, steps, False) for gen, steps in work]
    bad = srv.submit(sweep_instance(800, 0.03, 5.0, False, seed=950, d_min=2, d_max=8), 301, False)
    infos = [srv.wait(j, 300.0) for j in ids]
    assert all(inf.state == N.SPK_JOB_DONE for inf in infos), [inf.state for inf in infos]
    binfo = srv.wait(bad, 300.0)
    assert binfo.state == N.SPK_JOB_FAILED and binfo.error == N.SPK_ERR_INVALID
    for (gen, steps), j in zip(work, ids):
        ref = Net.generate(gen)
        assert ref.timestep_grouping() == 2
        ref.run_steps(steps, False)
        assert ref.synchronize() == 0
        ri, rt = ref.spikes()
        si, stt = srv.spikes(j)
        np.testing.assert_array_equal(si, ri)
        np.testing.assert_array_equal(bits(stt), bits(rt))
        ref.close()
    srv.stop()


@pytest.mark.parametrize("seed", range(3))
def test_served_random_jobs(seed):
    """Seeded random job streams: sizes 300-4,000, timestep grouping 1 or 2,
    the event-driven or the Evans rule or none, random step counts in whole
    groups, arrivals spread over the first blocks, either server mode and
    block length.  Every job equals the same network run alone."""
    rng = np.random.default_rng(500 + seed)
    mode = [N.SPK_BATCH_WAVES, N.SPK_BATCH_BULK][seed % 2]
    srv = Server(steps_per_block=int(rng.choice([100, 250, 400])), reserve_bytes=1 << 30, mode=mode)
    work, ids = [], []
    for i in range(int(rng.integers(5, 10))):
        d_min = int(rng.choice([1, 1, 2]))
        plastic = d_min == 1 and rng.random() < 0.5
        rule = N.SPK_STDP_EVANS if plastic and rng.random() < 0.3 else N.SPK_STDP_WEIGHT_DEPENDENT
        gen = sweep_instance(int(np.exp(rng.uniform(np.log(300), np.log(4000)))), float(rng.uniform(0.02, 0.06)),
                             float(rng.uniform(3, 7)), plastic, seed=1000 * seed + i, d_min=d_min,
                             d_max=int(rng.integers(d_min, 11)), rule=rule)
        steps = d_min * int(rng.integers(50, 600))
        on = bool(rng.integers(0, 4))
        work.append((gen, steps, on))
        ids.append(srv.submit(gen, steps, on))
        time.sleep(float(rng.uniform(0.0, 0.03)))
    infos = [srv.wait(j, 300.0) for j in ids]
    assert all(inf.state == N.SPK_JOB_DONE for inf in infos), [(inf.state, inf.error) for inf in infos]
    for (gen, steps, on), j, inf in zip(work, ids, infos):
        ref = Net.generate(gen)
        ref.run_steps(steps, on)
        assert ref.synchronize() == 0
        ri, rt = ref.spikes()
        si, stt = srv.spikes(j)
        assert inf.steps_done == steps
        np.testing.assert_array_equal(si, ri)
        np.testing.assert_array_equal(bits(stt), bits(rt))
        assert inf.events == ref.events()
        ref.close()
    srv.stop()
