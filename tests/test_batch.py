"""Batched stepping of uneven generated networks (GPU): the autotuned batch
gives every instance exactly the result it has alone (bit for bit)."""
import numpy as np
import pytest

from engine_checks import bits
from spike_gb300 import Batch, Net
from spike_gb300 import _native as N
from spike_gb300.networks import sweep_instance

pytestmark = pytest.mark.gpu


def small_sweep(k=12, seed=3):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(300), np.log(6000), k)).astype(int)
    return [sweep_instance(int(sizes[i]), float(rng.uniform(0.02, 0.08)), float(rng.uniform(3, 7)), i % 2 == 0,
                           seed=100 + i, d_max=8) for i in range(k)]


def snapshot(net: Net, n: int, n_in: int, S: int):
    ids, t = net.spikes()
    ii, it = net.spikes(N.SPK_POP_INPUTS)
    return dict(ids=ids, t=bits(t), iids=ii, it=bits(it), V=bits(net.state(N.SPK_FIELD_V, n)),
                last=bits(net.state(N.SPK_FIELD_LAST_SPIKE, n)), w=bits(net.weights(S)), ev=net.events())


def test_autotune_with_a_trace_rule_instance_picks_bulk_mode():
    """A sweep holding an Evans-rule instance (bulk mode only) is tuned over
    bulk-mode trials alone, and the tuned batch equals each instance alone."""
    gens = [sweep_instance(n, 0.04, 5.0, plastic, seed=80 + i, d_max=6, rule=rule)
            for i, (n, plastic, rule) in enumerate(((900, True, N.SPK_STDP_EVANS), (2000, True, 0), (600, False, 0)))]
    scheds, ms, mode = Batch.autotune(gens, trial_steps=40, with_mode=True)
    assert mode == N.SPK_BATCH_BULK and ms > 0
    nets = [Net.generate(g, s) for g, s in zip(gens, scheds)]
    b = Batch(nets)
    b.run_steps(300, True)
    assert b.synchronize() == 0
    for g, net in zip(gens, nets):
        ref = Net.generate(g)
        ref.run_steps(300, True)
        assert ref.synchronize() == 0
        np.testing.assert_array_equal(net.spikes()[0], ref.spikes()[0])
        assert net.events() == ref.events()
        ref.close()
    b.close()


def test_autotuned_batch_equals_each_instance_alone():
    gens = small_sweep()
    scheds, ms, costs, mode = Batch.autotune(gens, trial_steps=60, costs=True, with_mode=True)
    assert ms > 0 and len(scheds) == len(gens) and mode in (N.SPK_BATCH_WAVES, N.SPK_BATCH_BULK)
    assert all(c > 0 for c in costs) if mode == N.SPK_BATCH_WAVES else all(c == 0 for c in costs)
    batched = [Net.generate(g, s) for g, s in zip(gens, scheds)]
    for n, c in zip(batched, costs):
        if c > 0:
            n.set_step_cost(c)
    alone = [Net.generate(g, s) for g, s in zip(gens, scheds)]
    b = Batch(batched)
    b.set_mode(mode)
    for plastic, steps in ((True, 700), (False, 300)):
        b.run_steps(steps, plastic)
        for n in alone:
            n.run_steps(steps, plastic)
    assert b.synchronize() == 0
    total = 0
    for g, x, y in zip(gens, batched, alone):
        assert y.synchronize() == 0
        n, n_in, S = g.desc.n_neurons, g.desc.n_inputs, x.synapse_count()
        sx, sy = snapshot(x, n, n_in, S), snapshot(y, n, n_in, S)
        for k in sx:
            np.testing.assert_array_equal(sx[k], sy[k], err_msg=f"instance n={n} field {k}")
        total += len(sx["ids"])
        assert abs(x.current_time() - y.current_time()) == 0
    assert total > 1000
    b.close()


def test_batch_waves_cover_more_ctas_than_one_launch_holds():
    """Enough multi-CTA instances that the batch needs several waves."""
    gens = [sweep_instance(6000, 0.05, 5.0, False, seed=500 + i, d_max=6) for i in range(40)]
    sched = N.Schedule(8, 32, 0, 0)  # 24 CTAs each: 960 CTAs, more than one wave
    batched = [Net.generate(g, sched) for g in gens]
    b = Batch(batched)
    b.run_steps(200, False)
    assert b.synchronize() == 0
    assert b.launches() >= 2
    ref = Net.generate(gens[-1], sched)
    ref.run_steps(200, False)
    assert ref.synchronize() == 0
    i0, t0 = ref.spikes()
    i1, t1 = batched[-1].spikes()
    np.testing.assert_array_equal(i0, i1)
    np.testing.assert_array_equal(bits(t0), bits(t1))
    b.close()


@pytest.mark.parametrize("plastic_first", [True, False])
def test_bulk_mode_equals_each_instance_alone(plastic_first):
    """Bulk-synchronous batches (three kernels per timestep over all
    instances, state in HBM) give every instance its persistent-kernel result,
    bit for bit, including STDP weights, over blocks that cut runs."""
    gens = small_sweep(k=10, seed=21)
    sched = N.Schedule(8, 64, 0, 150)  # blocks of 150 timesteps
    batched = [Net.generate(g, sched) for g in gens]
    alone = [Net.generate(g, sched) for g in gens]
    b = Batch(batched, sched)
    b.set_mode(N.SPK_BATCH_BULK)
    for plastic, steps in ((plastic_first, 400), (not plastic_first, 230)):
        b.run_steps(steps, plastic)
        for n in alone:
            n.run_steps(steps, plastic)
    assert b.synchronize() == 0
    for g, x, y in zip(gens, batched, alone):
        assert y.synchronize() == 0
        n, n_in, S = g.desc.n_neurons, g.desc.n_inputs, x.synapse_count()
        sx, sy = snapshot(x, n, n_in, S), snapshot(y, n, n_in, S)
        for k in sx:
            np.testing.assert_array_equal(sx[k], sy[k], err_msg=f"instance n={n} field {k}")
        assert x.stdp_counts() == y.stdp_counts()
    # switching back to waves continues the same runs
    b.set_mode(N.SPK_BATCH_WAVES)
    b.run_steps(120, True)
    for n in alone:
        n.run_steps(120, True)
    assert b.synchronize() == 0
    for g, x, y in zip(gens, batched, alone):
        sx, sy = snapshot(x, g.desc.n_neurons, g.desc.n_inputs, x.synapse_count()), \
            snapshot(y, g.desc.n_neurons, g.desc.n_inputs, y.synapse_count())
        for k in sx:
            np.testing.assert_array_equal(sx[k], sy[k], err_msg=k)
    b.close()


@pytest.mark.parametrize("mode", [N.SPK_BATCH_WAVES, N.SPK_BATCH_BULK])
def test_batch_spike_readback_equals_per_network_reads(mode):
    """spk_batch_read_spikes gives every network's spikes exactly as the
    per-network read does, for both populations (one network records its
    inputs, so its store mixes them), and clears every store."""
    from test_generate import small_gen
    gens = small_sweep(k=6, seed=8) + [small_gen(seed=21)]
    nets = [Net.generate(g) for g in gens]
    b = Batch(nets)
    b.set_mode(mode)
    b.run_steps(300, True)
    assert b.synchronize() == 0

    def same_as_alone(got, pop):
        assert len(got) == len(nets)
        for (gi, gt), n in zip(got, nets):
            ri, rt = n.spikes(pop)
            np.testing.assert_array_equal(gi, ri)
            np.testing.assert_array_equal(bits(gt), bits(rt))
        return sum(len(i) for i, _ in got)

    assert same_as_alone(b.spikes(N.SPK_POP_NEURONS), N.SPK_POP_NEURONS) > 1000
    assert same_as_alone(b.spikes(N.SPK_POP_INPUTS), N.SPK_POP_INPUTS) > 0
    assert b.read_spikes_into(0, 0, 0) is None  # too small: nothing copied
    b.spikes(clear=True)
    assert all(len(n.spikes()[0]) == 0 and len(n.spikes(N.SPK_POP_INPUTS)[0]) == 0 for n in nets)
    b.run_steps(100, True)
    assert b.synchronize() == 0
    assert same_as_alone(b.spikes(), N.SPK_POP_NEURONS) > 0
    b.close()


def test_bulk_mode_key_lists_longer_than_one_staged_chunk():
    """Instances whose timesteps have more active keys than the propagation
    kernel stages at once (1,024): inputs at 2 kHz, so a fifth of the inputs
    fire every timestep.  Bulk mode still gives each instance its result
    alone, bit for bit."""
    gens = [sweep_instance(n, 0.02, g, plastic, seed=900 + i, d_max=6, rate=2000.0)
            for i, (n, g, plastic) in enumerate(((30000, 5.0, True), (26000, 6.0, False), (3000, 4.0, True)))]
    sched = N.Schedule(8, 64, 0, 100)
    batched = [Net.generate(g, sched) for g in gens]
    alone = [Net.generate(g, sched) for g in gens]
    b = Batch(batched, sched)
    b.set_mode(N.SPK_BATCH_BULK)
    b.run_steps(150, True)
    for n in alone:
        n.run_steps(150, True)
    assert b.synchronize() == 0
    for g, x, y in zip(gens, batched, alone):
        assert y.synchronize() == 0
        n, n_in, S = g.desc.n_neurons, g.desc.n_inputs, x.synapse_count()
        sx, sy = snapshot(x, n, n_in, S), snapshot(y, n, n_in, S)
        for k in sx:
            np.testing.assert_array_equal(sx[k], sy[k], err_msg=f"instance n={n} field {k}")
    # the big instances' inputs alone put about 1,200 keys on every timestep's list
    assert gens[0].desc.n_inputs * 2000.0 * 1e-4 > 1024
    assert sum(len(x.spikes()[0]) for x in batched) > 1000
    b.close()


def test_batches_keep_their_shared_memory_limits():
    """A kernel function's shared-memory limit holds in the whole process.  A
    batch set up after another, whose propagation needs less shared memory
    (delay 1 against delays 1-20), must not lower the first batch's limit:
    both batches run, each equal to its oracle."""
    import descs
    from engine_checks import assert_same
    from oracle import OracleNet
    from spike_gb300 import schedule
    deep = descs.random_voltage_net(n=300, n_in=100, d_max=20, seed=21)
    shallow = descs.random_voltage_net(n=200, n_in=50, d_max=1, seed=22)
    a_net, b_net = Net.from_desc(deep.desc, schedule(8, 64, 0, 0)), Net.from_desc(shallow.desc, schedule(8, 64, 0, 0))
    a, b = Batch([a_net]), Batch([b_net])
    a.set_mode(N.SPK_BATCH_BULK)
    b.set_mode(N.SPK_BATCH_BULK)
    a.run_steps(200, True)
    b.run_steps(200, True)
    assert a.synchronize() == 0 and b.synchronize() == 0
    for d, net, n, n_in in ((deep, a_net, 300, 100), (shallow, b_net, 200, 50)):
        o = OracleNet(d.desc)
        o.run_steps(200, True)
        assert_same(net, o, n, n_in, 1, weights=False, tag=f"d_max {d.desc.n_synapses}")
