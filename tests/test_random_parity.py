"""Seeded random networks and run sequences: the engine against the oracle,
bit for bit (GPU).

Each case draws from its seed:
- the synapse kind: voltage, current or conductance, with 1-3 labels;
- 60-900 LIF neurons in one to three groups, 0-300 Poisson inputs;
- delays d_min..d_max, d_min in {1, 2, 3} (the timestep grouping), d_max up to 20;
- with d_min = 1, weight-dependent STDP on the excitatory and input synapses (60 %);
- a schedule: the planner's, or 2-8 warps of 32-128 posts over as many CTAs as cover the
  network with launches of 7-1000 timesteps, or (bulk mode) one warp per 512-post range;
- the rule: weight-dependent STDP, sometimes with the weight normalisation, or the Evans,
  inhibitory or custom rule (bulk mode);
- two stimuli when there are inputs;
- four to seven actions: run(seconds) with seconds/dt fractions below and above one half
  (where the next run starts, the timestep index then repeats or skips one, and the
  reference's active lists deliver the last group again), run_steps of whole groups,
  plasticity switched off for some runs, reset_time or reset_state, a stimulus switch, a
  snapshot restored into a fresh network that carries on.
"""
import numpy as np
import pytest

import descs
from engine_checks import assert_same
from oracle import OracleNet
from spike_gb300 import Net, schedule
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams

pytestmark = pytest.mark.gpu

STDP = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0)


def random_case(seed: int, n_range=(60, 900)):
    rng = np.random.default_rng(seed)
    kind = [N.SPK_SYN_VOLTAGE, N.SPK_SYN_CURRENT, N.SPK_SYN_CONDUCTANCE][seed % 3]
    n = int(rng.integers(*n_range))
    n_in = int(rng.choice([0, int(rng.integers(20, 300))]))
    d_min = int(rng.choice([1, 1, 2, 3]))
    d_max = int(rng.integers(d_min, 21))
    plastic = d_min == 1 and rng.random() < 0.6
    rule, norm = N.SPK_STDP_WEIGHT_DEPENDENT, N.SPK_NORM_OFF
    if plastic:
        r = rng.random()
        if r < 0.3:
            rule = [N.SPK_STDP_EVANS, N.SPK_STDP_INHIBITORY, N.SPK_STDP_CUSTOM][int(rng.integers(0, 3))]
        elif r < 0.45:
            norm = [N.SPK_NORM_AFTER_RULE, N.SPK_NORM_BEFORE_RULE][int(rng.integers(0, 2))]
    L = 1 if kind == N.SPK_SYN_VOLTAGE else int(rng.integers(1, 4))
    n_groups = int(rng.integers(1, 4))
    cuts = np.sort(rng.choice(np.arange(1, n), n_groups - 1, replace=False)) if n_groups > 1 else np.array([], int)
    counts = np.diff(np.concatenate([[0], cuts, [n]])).astype(int)
    n_exc = int(0.8 * n)
    if kind == N.SPK_SYN_CONDUCTANCE:
        lif = dict(v0=-0.06, vreset=-0.06, theta=-0.05)
        i_bg = float(rng.uniform(0.011, 0.016))  # over threshold: every network fires
    else:
        lif = dict(v0=0.0, vreset=0.0, theta=0.02)
        i_bg = float(rng.uniform(0.021, 0.03))
    groups = [dict(count=int(c), tau_m=float(rng.uniform(0.01, 0.03)), R=1e8, v_init_lo=lif["v0"],
                   v_init_hi=lif["theta"], **lif) for c in counts]
    # connectivity: Bernoulli p (about 40-90 afferents for the large cases), multapses
    # allowed, inputs at p_in
    p = float(rng.uniform(0.02, 0.1)) if n < 1000 else float(rng.uniform(40, 90)) / n
    pre, post = [], []
    for q in range(n):
        k_rec, k_in = rng.binomial(n, p), rng.binomial(n_in, 2 * p) if n_in else 0
        pre += list(rng.integers(0, n, k_rec)) + list(-rng.integers(0, n_in, k_in) - 1 if k_in else [])
        post += [q] * (k_rec + k_in)
    pre, post = np.asarray(pre, np.int64), np.asarray(post, np.int64)
    S = len(pre)
    exc = (pre < 0) | (pre < n_exc)
    if kind == N.SPK_SYN_VOLTAGE:
        w = np.where(exc, rng.uniform(2e-4, 1.5e-3, S), -rng.uniform(1e-3, 5e-3, S))
    elif kind == N.SPK_SYN_CURRENT:
        w = np.where(exc, rng.uniform(1e-10, 6e-10, S), -rng.uniform(4e-10, 2e-9, S))
    else:
        w = np.where(exc, rng.uniform(1e-9, 6e-9, S), rng.uniform(1e-8, 5e-8, S))
    label = np.where(exc, 0, L - 1) if L > 1 else np.zeros(S, int)
    label = np.where((pre < 0) & (L == 3), 1, label)
    delay = rng.integers(d_min, d_max + 1, S)
    if S:
        delay[0] = d_min
    tau = list(rng.uniform(0.003, 0.012, L))
    vhat = [0.0 if l != L - 1 or L == 1 else -0.08 for l in range(L)]
    from test_stdp_rules import CUSTOM, EVANS, VOGELS
    sp = {N.SPK_STDP_EVANS: EVANS, N.SPK_STDP_INHIBITORY: VOGELS, N.SPK_STDP_CUSTOM: CUSTOM}.get(rule, STDP)
    d = descs.Desc(kind=kind, groups=groups, refractory=float(rng.uniform(0.001, 0.003)), i_bg=i_bg,
                   n_inputs=n_in, rates=rng.uniform(10, 60, 2 * n_in) if n_in else None, n_labels=L, label_tau=tau,
                   label_vhat=vhat, pre=pre, post=post, weight=w, delay=delay, label=label,
                   plastic=exc.astype(int) if plastic else None, stdp=sp if plastic else None, seed=seed,
                   record_inputs=bool(rng.integers(0, 2)), stdp_rule=rule, weight_norm=norm)
    # schedule
    choice = int(rng.integers(0, 3))
    if choice == 0:
        sched = None
    elif choice == 1:
        W = int(rng.choice([2, 4, 8]))
        TS = int(rng.choice([32, 64, 128]))
        C = -(-n // (W * TS))
        sched = schedule(W, TS, C, int(rng.choice([7, 50, 1000])))
    else:
        sched = schedule(1, 512, 0, 0)  # post ranges, bulk mode
    # actions
    actions = []
    for _ in range(int(rng.integers(4, 8))):
        a = int(rng.integers(0, 12))
        if a == 10 and n_in:
            actions.append(("stimulus", int(rng.integers(0, 2))))
            continue
        if a >= 10:
            actions.append(("snapshot",))
            continue
        if a < 6:
            steps = int(rng.integers(20, 300))
            frac = float(rng.choice([0.2, 0.35, 0.65, 0.8]))
            actions.append(("run", float(np.float32((steps + frac) * 1e-4)), bool(rng.integers(0, 4))))
        elif a < 8:
            actions.append(("steps", d_min * int(rng.integers(10, 150)), bool(rng.integers(0, 4))))
        elif a == 8:
            actions.append(("reset_time",))
        else:
            actions.append(("reset_state",))
    return d, sched, actions, n, n_in, L, plastic


@pytest.mark.parametrize("seed,n_range", [(s, (60, 900)) for s in range(48)] +
                         [(s, (3000, 12000)) for s in range(200, 206)] +
                         # stimulus switches in networks with a per-synapse-trace rule
                         # or the weight normalisation (runs through a bulk batch)
                         [(s, (60, 900)) for s in (1050, 1261, 1308)] +
                         [(1141, (60, 900)), (2009, (3000, 12000))])  # refused schedules
def test_random_network_and_runs(seed, n_range):
    d, sched, actions, n, n_in, L, plastic = random_case(seed, n_range)
    o = OracleNet(d.desc)
    try:
        net = Net.from_desc(d.desc, sched)
    except N.SpikeError as e:
        # a drawn schedule whose tiles do not fit shared memory is refused at
        # creation: run the planner's instead
        assert "does not cover" in str(e), e
        sched = None
        net = Net.from_desc(d.desc, sched)
    # Where t/dt stays within rounding of a half, the timestep index can repeat
    # and skip in turn within a run, and the reference's active list then holds
    # more than one earlier group: the engine and the oracle deliver the last
    # one and report SPK_ERR_UNSUPPORTED (sticky until reset_state).
    unsupported = False

    def oracle(call, *args):
        nonlocal unsupported
        try:
            call(*args)
        except RuntimeError as e:
            assert f"status {N.SPK_ERR_UNSUPPORTED}" in str(e), e
            unsupported = True

    for act in actions:
        if act[0] == "stimulus":
            net.select_stimulus(act[1])
            o.select_stimulus(act[1])
        elif act[0] == "snapshot":
            if unsupported:
                continue  # a restore clears the device status; the oracle's stays
            # the spike store is not part of a snapshot: both stores start afresh
            assert net.synchronize() == 0
            net.clear_spikes()
            o.clear_spikes()
            snap = net.snapshot()
            fresh = Net.from_desc(d.desc, sched)
            fresh.restore(snap)
            net.close()
            net = fresh
        elif act[0] == "run":
            net.run(act[1], act[2])
            oracle(o.run, act[1], act[2])
        elif act[0] == "steps":
            net.run_steps(act[1], act[2])
            oracle(o.run_steps, act[1], act[2])
        elif act[0] == "reset_time":
            net.reset_time()
            o.reset_time()
        else:
            assert net.synchronize() == (N.SPK_ERR_UNSUPPORTED if unsupported else 0)
            net.reset_state()
            o.reset_state()
            unsupported = False
    assert net.synchronize() == (N.SPK_ERR_UNSUPPORTED if unsupported else 0)
    assert net.current_time() == o.current_time()
    assert_same(net, o, n, n_in, L, weights=plastic, tag=f"seed {seed} {net.schedule()} {actions}")


@pytest.mark.parametrize("mode", [N.SPK_BATCH_BULK, N.SPK_BATCH_WAVES])
@pytest.mark.parametrize("seed", range(100, 108))
def test_random_batches(seed, mode):
    """Batches of two to five random networks (planner schedules at four warps
    per CTA, so that waves mode can take them), each run its own whole-group
    step counts and plasticity switch twice, with the second stimulus selected
    between the two runs, every network against its oracle."""
    from spike_gb300 import Batch
    rng = np.random.default_rng(seed)
    cases = [random_case(seed * 10 + i) for i in range(int(rng.integers(2, 6)))]
    nets = [Net.from_desc(c[0].desc, schedule(4, 0, 0, 0)) for c in cases]
    orcs = [OracleNet(c[0].desc) for c in cases]
    b = Batch(nets)
    bulk_only = any(c[0].desc.stdp_rule != N.SPK_STDP_WEIGHT_DEPENDENT or c[0].desc.weight_norm != N.SPK_NORM_OFF
                    for c in cases)
    if mode == N.SPK_BATCH_WAVES and bulk_only:
        # the per-synapse-trace rules and the normalisation run in bulk mode only: refused
        with pytest.raises(N.SpikeError):
            b.set_mode(mode)
        mode = N.SPK_BATCH_BULK
    b.set_mode(mode)
    for it in range(2):
        if it == 1:
            # the batch keeps copies of the networks' descriptors: a stimulus
            # switch between batch runs must reach them
            for c, net, o in zip(cases, nets, orcs):
                if c[4]:
                    net.select_stimulus(1)
                    o.select_stimulus(1)
        steps = [int(o.timestep_grouping()) * int(rng.integers(20, 200)) for o in orcs]
        plastic = [bool(rng.integers(0, 4)) for _ in orcs]
        b.run_steps_each(steps, plastic)
        for o, k, pl in zip(orcs, steps, plastic):
            o.run_steps(k, pl)
    assert b.synchronize() == 0
    for (d, _, _, n, n_in, L, pl), net, o in zip(cases, nets, orcs):
        assert_same(net, o, n, n_in, L, weights=pl, tag=f"batch seed {seed} mode {mode}")


@pytest.mark.parametrize("mode", [N.SPK_BATCH_BULK, N.SPK_BATCH_WAVES])
@pytest.mark.parametrize("seed", list(range(110, 118)) + [4041])  # 4041: a second batch with less shared memory
def test_random_batch_sequences(seed, mode):
    """Batch runs interleaved with calls on single networks of the batch: a
    network run alone (run(seconds) with fractions that repeat or skip the
    timestep index, or whole-group run_steps), reset_time, reset_state, a
    stimulus switch, a snapshot restored into the same network.  Every
    network against its oracle at the end."""
    from spike_gb300 import Batch
    rng = np.random.default_rng(seed)
    cases = [random_case(seed * 10 + i) for i in range(int(rng.integers(2, 5)))]
    nets = [Net.from_desc(c[0].desc, schedule(4, 0, 0, 0)) for c in cases]
    orcs = [OracleNet(c[0].desc) for c in cases]
    b = Batch(nets)
    if mode == N.SPK_BATCH_WAVES and any(c[0].desc.stdp_rule != N.SPK_STDP_WEIGHT_DEPENDENT or
                                         c[0].desc.weight_norm != N.SPK_NORM_OFF for c in cases):
        mode = N.SPK_BATCH_BULK  # the per-synapse-trace rules and the normalisation run in bulk mode only
    b.set_mode(mode)
    unsupported = [False] * len(nets)

    def oracle(i, call, *args):
        try:
            call(*args)
        except RuntimeError as e:
            assert f"status {N.SPK_ERR_UNSUPPORTED}" in str(e), e
            unsupported[i] = True

    actions = []
    for _ in range(int(rng.integers(5, 10))):
        a, i = int(rng.integers(0, 8)), int(rng.integers(0, len(nets)))
        net, o, n_in = nets[i], orcs[i], cases[i][4]
        if a <= 2:
            steps = [int(x.timestep_grouping()) * int(rng.integers(10, 120)) for x in orcs]
            plastic = [bool(rng.integers(0, 4)) for _ in orcs]
            actions.append(("batch", steps, plastic))
            b.run_steps_each(steps, plastic)
            for j, (x, k, pl) in enumerate(zip(orcs, steps, plastic)):
                oracle(j, x.run_steps, k, pl)
        elif a == 3:
            sec = float(np.float32((int(rng.integers(20, 200)) + float(rng.choice([0.2, 0.35, 0.65, 0.8]))) * 1e-4))
            pl = bool(rng.integers(0, 4))
            actions.append(("run", i, sec, pl))
            net.run(sec, pl)
            oracle(i, o.run, sec, pl)
        elif a == 4:
            actions.append(("reset_time", i))
            net.reset_time()
            o.reset_time()
        elif a == 5:
            actions.append(("reset_state", i))
            assert net.synchronize() == (N.SPK_ERR_UNSUPPORTED if unsupported[i] else 0)
            net.reset_state()
            o.reset_state()
            unsupported[i] = False
        elif a == 6 and n_in:
            stim = int(rng.integers(0, 2))
            actions.append(("stimulus", i, stim))
            net.select_stimulus(stim)
            o.select_stimulus(stim)
        elif a == 7 and not unsupported[i]:
            # the spike store is not part of a snapshot: both stores start afresh
            actions.append(("restore", i))
            assert net.synchronize() == 0
            net.clear_spikes()
            o.clear_spikes()
            net.restore(net.snapshot())
    assert b.synchronize() in (0, N.SPK_ERR_UNSUPPORTED)
    for i, ((d, _, _, n, n_in, L, pl), net, o) in enumerate(zip(cases, nets, orcs)):
        assert net.synchronize() == (N.SPK_ERR_UNSUPPORTED if unsupported[i] else 0)
        assert net.current_time() == o.current_time()
        assert_same(net, o, n, n_in, L, weights=pl, tag=f"batch seed {seed} mode {mode} net {i} {actions}")
