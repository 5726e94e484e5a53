"""Timestep grouping: networks whose minimum delay G is above one step.

The reference advances such a network G timesteps per step of its run loop
(Spike/Models/SpikingModel.cpp:98, :221-228): the group's time is
start + s*G*dt in float, substep g's time that + g*dt, and run(seconds)
simulates whole groups only (the integer division of :222).  Every delay is
at least G steps, so a group's deliveries all land past it and the engine may
advance the group substep by substep.

CPU: the oracle against a literal restatement of the reference's grouped loop
(below), the run-length rule, and the refusals.  GPU: the engine against the
oracle, bit for bit, on the persistent path under several schedules (blocks
that cut groups), in batches (bulk and waves mode) and through
spk_step_noalloc (tests/test_zz_no_alloc.py).
"""
import ctypes
import math

import numpy as np
import pytest

import cases
import descs
from engine_checks import assert_same, bits
from oracle import OracleNet
from spike_gb300 import _native as N
from spike_gb300 import desc_arrays
from spike_gb300.model import STDPParams

F = np.float32


def _tiny_net(G: int, d_max: int, seed: int = 11):
    """Forty voltage-synapse LIF neurons driven by a background current over
    threshold (no inputs, so no random draws during the run), random E/I
    weights and delays G..d_max."""
    rng = np.random.default_rng(seed)
    n, S = 40, 420
    pre = rng.integers(0, n, S)
    post = rng.integers(0, n, S)
    w = np.where(pre < 32, rng.uniform(1e-3, 4e-3, S), -rng.uniform(2e-3, 9e-3, S)).astype(np.float32)
    delay = rng.integers(G, d_max + 1, S)
    delay[0] = G
    groups = [dict(count=32, tau_m=0.005, R=1e8, v0=0.0, vreset=0.0, theta=0.02, v_init_lo=0.0, v_init_hi=0.02),
              dict(count=8, tau_m=0.004, R=1e8, v0=0.0, vreset=0.005, theta=0.02, v_init_lo=0.0, v_init_hi=0.02)]
    return descs.Desc(kind=N.SPK_SYN_VOLTAGE, groups=groups, refractory=0.002, i_bg=0.03, n_inputs=0,
                      pre=pre, post=post, weight=w, scale=np.ones(S), delay=delay, record_inputs=False)


class GroupedReference:
    """SpikingModel::run with timestep grouping G, written as the reference's
    kernels are structured: per step, lif_update_membrane_potentials loops
    over the neurons and, inside, over the G substeps
    (Spike/Backend/CUDA/Neurons/LIFSpikingNeurons.cu:105-193, voltage
    injection), appending each spike (neuron, substep) to active list
    (T/G) % 2 (get_active_synapses, Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:151-162);
    then activate_synapses empties the other list and delivers the whole
    current one to (bufferloc + delay + g) % B (:168-202), B = D_max + 2G + 1
    (:48).  Float32 throughout, no contraction; the ring additions in the
    canonical order of the engine and the oracle (by substep, then
    presynaptic key, carried entries merged with the group's own, a key in
    both once; sorted synapse order)."""

    def __init__(self, d, o: OracleNet):
        a = desc_arrays(d)
        pre, post, delay = o.sorted_synapses()
        # the oracle's sorted order (stable by presynaptic key) with each synapse's weight
        order = np.argsort(a["pre"], kind="stable")
        assert np.array_equal(a["pre"][order], pre) and np.array_equal(a["post"][order], post)
        self.post, self.delay = post, delay
        self.c = (a["weight"][order].astype(F) * a["scale"][order].astype(F)).astype(F)
        self.start = np.searchsorted(pre, np.arange(d.n_neurons + 1))
        self.n, self.G = d.n_neurons, int(delay.min())
        self.B = int(delay.max()) + 2 * self.G + 1
        self.dt = F(d.dt)
        self.ring = np.zeros((self.B, self.n), F)
        grp = np.ctypeslib.as_array(d.groups, (d.n_groups,))
        self.k, self.v0, self.vr, self.th = (np.empty(self.n, F) for _ in range(4))
        for g in grp:
            sl = slice(g["start"], g["start"] + g["count"])
            self.k[sl] = F(self.dt / F(g["tau_m"]))
            self.v0[sl], self.vr[sl], self.th[sl] = F(g["v0"]), F(g["vreset"]), F(g["theta"])
        self.ibg, self.tref = F(d.background_current), F(d.refractory_period)
        self.V = o.state(N.SPK_FIELD_V, self.n).copy()  # the initial potentials (Philox-drawn)
        self.last = np.full(self.n, F(-1000.0), F)
        self.time = F(0.0)
        self.ids, self.times = [], []
        self.lists = [[], []]  # the two active lists: (neuron, substep) entries
        self.repeats = 0       # group steps that delivered a carried group

    def run(self, seconds: float):
        G, dt, half = self.G, self.dt, F(F(0.5) * self.dt)
        n_timesteps = int(np.ceil(F(seconds) / dt))
        start = self.time
        for s in range(n_timesteps // G):
            t = F(start + F(s * G) * dt)
            tidx = int(math.floor(float(F(t / dt)) + 0.5))  # (int)roundf(t/dt), t >= 0
            fired = [[] for _ in range(G)]
            cur = self.lists[(tidx // G) % 2]
            self.repeats += bool(cur)
            for idx in range(self.n):
                Vi = self.V[idx]
                for g in range(G):
                    cell = ((tidx + g) % self.B, idx)
                    inp = F(F(0.0) + self.ring[cell])
                    self.ring[cell] = F(0.0)
                    tg = F(t + F(g) * dt)
                    if F(F(tg - self.last[idx]) - self.tref) > half:
                        k = self.k[idx]
                        Vi = F(F(F(F(k * self.v0[idx]) + F(F(F(1.0) - k) * Vi)) + F(k * self.ibg)) + inp)
                        if Vi >= self.th[idx]:
                            self.last[idx] = tg
                            Vi = self.vr[idx]
                            fired[g].append(idx)
                self.V[idx] = Vi
            for g in range(G):
                for idx in fired[g]:
                    self.ids.append(idx)
                    self.times.append(F(t + F(g) * dt))
                    cur.append((idx, g))
            self.lists[(tidx // G + 1) % 2] = []
            for g in range(G):  # canonical order: by substep, then key; an entry listed twice once
                for idx in sorted({i for i, gg in cur if gg == g}):
                    for syn in range(self.start[idx], self.start[idx + 1]):
                        cell = ((tidx + self.delay[syn] + g) % self.B, self.post[syn])
                        self.ring[cell] = F(self.ring[cell] + self.c[syn])
        self.time = F(start + F(seconds))


@pytest.mark.parametrize("G,d_max", [(1, 4), (2, 2), (3, 7)])
def test_oracle_follows_the_reference_group_loop(G, d_max):
    """The oracle (substep by substep) against the reference's grouped loop,
    bit for bit: spike ids and float times, potentials and the end time, over
    runs whose step counts are not whole groups (rounded down) and whose
    first group index repeats or skips one, so that the earlier group is
    delivered again."""
    d = _tiny_net(G, d_max)
    o = OracleNet(d.desc)
    assert o.timestep_grouping() == G
    ref = GroupedReference(d.desc, o)
    for sec in (0.0137, 0.0071, 0.0173, 0.0101, 0.0337, 0.0173, 0.02):
        o.run(sec)
        ref.run(sec)
        assert o.current_time() == ref.time
    assert ref.repeats >= 1
    ids, times = o.spikes()
    assert len(ids) == len(ref.ids) > 200
    np.testing.assert_array_equal(ids, np.asarray(ref.ids))
    np.testing.assert_array_equal(bits(times), bits(np.asarray(ref.times, F)))
    np.testing.assert_array_equal(bits(o.state(N.SPK_FIELD_V, 40)), bits(ref.V))
    np.testing.assert_array_equal(bits(o.state(N.SPK_FIELD_LAST_SPIKE, 40)), bits(ref.last))


def test_oracle_run_length_is_whole_groups():
    """run(seconds) simulates floor(ceil(seconds/dt) / G) groups; the time
    still advances by the seconds asked for, and step counts must be whole
    groups."""
    d = _tiny_net(3, 5)
    o, o9, o12 = OracleNet(d.desc), OracleNet(d.desc), OracleNet(d.desc)
    o.run(0.0011)  # ceil(11) timesteps = 3 groups = 9 timesteps
    o9.run_steps(9)
    o12.run_steps(12)
    assert o.current_time() == F(0.0011)
    assert o9.current_time() == F(F(9) * F(1e-4))
    v, v9, v12 = (x.state(N.SPK_FIELD_V, 40) for x in (o, o9, o12))
    np.testing.assert_array_equal(bits(v), bits(v9))
    assert not np.array_equal(bits(v), bits(v12))
    o.run_steps(6)
    with pytest.raises(RuntimeError):
        o.run_steps(4)


def test_grouped_spike_times_are_group_time_plus_substep():
    """Recorded times are (start + (s*G)*dt) + g*dt in float, the spike
    monitor's current_time + g*timestep, not start + (s*G + g)*dt."""
    d = descs.random_voltage_net(n=200, n_in=100, d_min=3, d_max=9, rate=80.0)
    o = OracleNet(d.desc)
    o.run(0.05)
    o.run(0.0371)
    ids, times = o.spikes()
    dt = F(1e-4)
    start = F(0.05)
    late = times > start
    # in the second run: group s of 3, substep g; the times are exactly those of the formula
    allowed = {F(F(start + F(s * 3) * dt) + F(g) * dt) for s in range(200) for g in range(3)}
    assert late.sum() > 50
    assert set(times[late].tolist()) <= {float(x) for x in allowed}


def test_plasticity_with_grouping_is_refused_before_any_device_call():
    stdp = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0,
                      w_max=1.0)
    d = descs.random_voltage_net(n=60, n_in=30, d_min=2, plastic=True, stdp=stdp)
    h = ctypes.c_void_p()
    assert N.lib().spk_net_create(ctypes.byref(d.desc), None, ctypes.byref(h)) == N.SPK_ERR_UNSUPPORTED
    assert b"timestep grouping" in N.lib().spk_last_error()
    with pytest.raises(RuntimeError):
        OracleNet(d.desc)


def test_noalloc_grouping_checks_before_any_device_call():
    lib = N.lib()
    g = (N.NeuronGroup * 1)()
    g[0].start, g[0].count, g[0].tau_m, g[0].R, g[0].theta = 0, 64, 0.02, 1e8, 0.02
    dummy = ctypes.create_string_buffer(64)
    addr = ctypes.addressof(dummy)
    dn = N.DeviceNet()
    dn.n_neurons, dn.n_inputs, dn.n_labels, dn.synapse_kind, dn.max_delay = 64, 0, 1, N.SPK_SYN_VOLTAGE, 4
    dn.warps_per_cta, dn.tile_posts, dn.ctas = 2, 32, 1
    dn.dt, dn.refractory_period = 1e-4, 2e-3
    dn.n_groups, dn.groups = 1, g
    for f in ("rowptr", "entries", "V", "last_spike", "ring", "spikes", "run_state"):
        setattr(dn, f, addr)
    dn.spike_capacity = 1
    dn.timestep_grouping = 3
    # 0 steps of a grouping of 3 pass the checks (nothing would run); 4 steps are not whole groups
    assert lib.spk_step_noalloc(ctypes.byref(dn), 4, 0, ctypes.c_float(0.0), None) == N.SPK_ERR_INVALID
    assert b"timestep grouping" in lib.spk_last_error()
    dn.timestep_grouping = 5  # above the maximum delay
    assert lib.spk_step_noalloc(ctypes.byref(dn), 0, 0, ctypes.c_float(0.0), None) == N.SPK_ERR_INVALID


# ---- GPU: the engine against the oracle --------------------------------------------------

@pytest.mark.gpu
def test_grouped_vogels_abbott_engine_equals_oracle():
    """The Vogels-Abbott network with delays of 3-5 steps (G = 3)."""
    from spike_gb300 import Net
    m = cases.ref_va(False, 3, 5)
    d = m.desc()
    o = OracleNet(d)
    net = Net.from_desc(d)
    assert net.timestep_grouping() == o.timestep_grouping() == 3
    for sec in (0.05, 0.0333, 0.05):
        net.run(sec)
        o.run(sec)
    net.run_steps(3 * 37)
    o.run_steps(3 * 37)
    assert net.synchronize() == 0
    assert net.current_time() == o.current_time()
    assert_same(net, o, 4000, 0, 2, tag="va_g3")
    assert len(o.spikes()[0]) > 1000
    with pytest.raises(RuntimeError):
        net.run_steps(4)


@pytest.mark.gpu
@pytest.mark.parametrize("sched", [None, (8, 32, 0, 0), (4, 64, 0, 7), (2, 32, 6, 50)])
@pytest.mark.parametrize("G", [2, 3])
def test_grouped_voltage_net_with_inputs_across_schedules(sched, G):
    """Poisson inputs and recurrent synapses with delays G..12; launches of 7
    and 50 timesteps cut groups in two."""
    from spike_gb300 import Net, schedule
    d = descs.random_voltage_net(n=300, n_in=200, d_min=G, d_max=12, seed=G)
    o = OracleNet(d.desc)
    net = Net.from_desc(d.desc, schedule(*sched) if sched else None)
    for sec in (0.0301, 0.0173, 0.04):
        net.run(sec)
        o.run(sec)
    assert net.synchronize() == 0
    assert_same(net, o, 300, 200, 1, tag=f"G={G} {net.schedule()}")
    assert len(o.spikes()[0]) > 200


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [N.SPK_BATCH_BULK, N.SPK_BATCH_WAVES])
def test_batch_of_grouped_networks_equals_each_alone(mode):
    """Networks with groupings 1, 2 and 3 in one batch; each run's step count
    is whole groups of its own network."""
    from spike_gb300 import Batch, Net, schedule
    ds = [descs.random_voltage_net(n=n, n_in=ni, seed=s, d_min=g, d_max=10)
          for n, ni, s, g in ((150, 100, 1, 1), (420, 90, 2, 2), (64, 300, 3, 3), (700, 50, 4, 2))]
    nets = [Net.from_desc(x.desc, schedule(4, 0, 0, 0)) for x in ds]
    orcs = [OracleNet(x.desc) for x in ds]
    b = Batch(nets)
    b.set_mode(mode)
    steps = [330, 330, 330, 330]
    b.run_steps_each(steps)
    assert b.synchronize() == 0
    for x, net, o, k in zip(ds, nets, orcs, steps):
        o.run_steps(k)
        assert_same(net, o, x.desc.n_neurons, x.desc.n_inputs, 1, tag=f"batch mode {mode}")
    with pytest.raises(RuntimeError):
        b.run_steps_each([330, 331, 330, 330])


# ---- GPU: run boundaries where the reference delivers the last group again --------------
# (Spike/Backend/CUDA/Synapses/SpikingSynapses.cu:179-182: active list (T/G) % 2 is emptied
# only by a group step of the other parity.)  The run lengths below make the first group
# index of some runs repeat (0.0173 s is 174 steps at dt 1e-4, the next run starts at
# index 173) or skip one (grouped networks).
BOUNDARY_RUNS = (0.0137, 0.0071, 0.0173, 0.0101, 0.0337, 0.0173, 0.02)
STDP = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0,
                  w_max=1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("sched", [None, (2, 32, 10, 50), (1, 512, 0, 0)])
@pytest.mark.parametrize("G", [1, 3])
def test_run_boundaries_deliver_the_carried_group_again(sched, G):
    """The engine delivers the carried group again exactly as the oracle does:
    persistent schedules (one and several CTAs, launches of 50 timesteps) and
    bulk mode over post ranges (one warp per CTA, 512-post tiles)."""
    from spike_gb300 import Net, schedule
    d = descs.random_voltage_net(n=600, n_in=200, d_min=G, d_max=12, seed=20 + G)
    o = OracleNet(d.desc)
    net = Net.from_desc(d.desc, schedule(*sched) if sched else None)
    for sec in BOUNDARY_RUNS:
        net.run(sec)
        o.run(sec)
    assert net.synchronize() == 0
    assert_same(net, o, 600, 200, 1, tag=f"G={G} {net.schedule()}")


@pytest.mark.gpu
def test_plastic_run_boundaries_and_snapshot():
    """Weight-dependent STDP (the carried group is delivered with the current
    weights), and a snapshot taken between runs keeps the active-list state:
    the restored network repeats the next group start as the original does."""
    from spike_gb300 import Net
    d = descs.random_voltage_net(n=300, n_in=200, plastic=True, stdp=STDP, seed=31)
    o = OracleNet(d.desc)
    a = Net.from_desc(d.desc)
    for sec in (0.0173, 0.0101, 0.0173):
        a.run(sec)
        o.run(sec)
    assert a.synchronize() == 0
    snap = a.snapshot()
    b = Net.from_desc(d.desc)
    b.run(0.005)  # state that the restore must overwrite
    b.restore(snap)
    a.clear_spikes()
    b.clear_spikes()
    o.clear_spikes()
    for sec in (0.0173, 0.0337, 0.0173):
        a.run(sec)
        b.run(sec)
        o.run(sec)
    assert a.synchronize() == 0 and b.synchronize() == 0
    assert_same(a, o, 300, 200, 1, weights=True, tag="plastic")
    assert_same(b, o, 300, 200, 1, weights=True, tag="restored")


def _expf():
    libm = ctypes.CDLL("libm.so.6")
    f = libm.expf
    f.argtypes, f.restype = [ctypes.c_float], ctypes.c_float
    return lambda x: F(f(float(x)))


class PlasticReference:
    """SpikingModel::run of a voltage-synapse network with weight-dependent
    STDP on its excitatory synapses, G = 1, written as the reference's step is:
    lif_update_membrane_potentials (spikes appended to active list T % 2), then
    ltp_and_ltd for every plastic synapse with its own traces and expf terms
    (Spike/Backend/CUDA/Plasticity/WeightDependentSTDPPlasticity.cu:85-161),
    then activate_synapses (the other list emptied, the current one delivered
    with the weights just updated).  A run that starts at the timestep index
    where the last one ended finds the last step's spikes still in its list,
    and their last-spike times give them STDP events again.  The list is
    delivered in key order (carried keys merged with the step's), the
    canonical order of the engine and the oracle."""

    def __init__(self, d, o: OracleNet, sp):
        self.base = GroupedReference(d, o)
        a = desc_arrays(d)
        order = np.argsort(a["pre"], kind="stable")
        self.pl = a["plastic"][order].astype(bool)
        self.w = a["weight"][order].astype(F)
        self.scale = a["scale"][order].astype(F)
        self.pre_tr = np.zeros(len(order), F)
        self.post_tr = np.zeros(len(order), F)
        self.pre = np.sort(a["pre"], kind="stable")
        self.sp = sp
        self.expf = _expf()
        self.order = order

    def stdp(self, t):
        b, sp, expf, dt = self.base, self.sp, self.expf, self.base.dt
        am, ap, tm, tp = F(sp.a_minus), F(sp.a_plus), F(sp.tau_minus), F(sp.tau_plus)
        lam, alpha, wmax = F(sp.lambda_), F(sp.alpha), F(sp.w_max)
        for s in np.flatnonzero(self.pl):
            pre_g = int(math.floor(float(F(F(b.last[self.pre[s]] - t) / dt)) + 0.5))
            post_g = int(math.floor(float(F(F(b.last[b.post[s]] - t) / dt)) + 0.5))
            if pre_g >= 1:
                pre_g *= -1
            pot, prt = self.post_tr[s], self.pre_tr[s]
            pot = F(pot * expf(F(-F(F(1) * dt)) / tm))
            prt = F(prt * expf(F(-F(F(1) * dt)) / tp))
            pot = F(pot + (F(am * expf(F(-F(F(1 - post_g) * dt)) / tm)) if post_g >= 0 else F(0)))
            prt = F(prt + (F(ap * expf(F(-F(F(1 - pre_g) * dt)) / tp)) if pre_g >= 0 else F(0)))
            old = self.w[s]
            syn = F(0)
            if pre_g >= 0:
                tpt = pot
                if post_g > pre_g:
                    tpt = F(tpt + F(-am * expf(F(-F(F(1 - post_g) * dt)) / tm)))
                tpt = F(tpt * F(F(1) / expf(F(F(F(-(1 - pre_g)) * dt) / tm))))
                syn = F(syn - F(F(F(lam * alpha) * old) * tpt))
            if post_g >= 0:
                tpr = prt
                if pre_g > post_g:
                    tpr = F(tpr + F(-ap * expf(F(-F(F(1 - pre_g) * dt)) / tp)))
                tpr = F(tpr * F(F(1) / expf(F(F(F(-(1 - post_g)) * dt) / tp))))
                syn = F(syn + F(F(lam * F(wmax - old)) * tpr))
            nw = F(old + syn)
            self.w[s] = F(0) if nw < 0 else nw
            self.post_tr[s], self.pre_tr[s] = pot, prt

    def run(self, seconds: float):
        b = self.base
        dt, half = b.dt, F(F(0.5) * b.dt)
        start = b.time
        for s in range(int(np.ceil(F(seconds) / dt))):
            t = F(start + F(s) * dt)
            T = int(math.floor(float(F(t / dt)) + 0.5))
            cur = b.lists[T % 2]
            b.repeats += bool(cur)
            for idx in range(b.n):
                cell = (T % b.B, idx)
                inp = F(F(0.0) + b.ring[cell])
                b.ring[cell] = F(0.0)
                if F(F(t - b.last[idx]) - b.tref) > half:
                    k = b.k[idx]
                    Vi = F(F(F(F(k * b.v0[idx]) + F(F(F(1.0) - k) * b.V[idx])) + F(k * b.ibg)) + inp)
                    if Vi >= b.th[idx]:
                        b.last[idx] = t
                        Vi = b.vr[idx]
                        cur.append(idx)
                        b.ids.append(idx)
                        b.times.append(t)
                    b.V[idx] = Vi
            self.stdp(t)
            b.lists[(T + 1) % 2] = []
            for idx in sorted(set(cur)):
                for syn in range(b.start[idx], b.start[idx + 1]):
                    cell = ((T + b.delay[syn]) % b.B, b.post[syn])
                    b.ring[cell] = F(b.ring[cell] + F(self.w[syn] * self.scale[syn]))
        b.time = F(start + F(seconds))

    def weights(self):
        out = np.empty(len(self.order), F)
        out[self.order] = self.w
        return out


def test_oracle_stdp_at_repeating_run_starts_follows_the_reference():
    """Weight-dependent STDP across run starts that repeat the timestep index
    (0.00233 s is 24 steps at dt 1e-4, and start + 0.00233 often rounds to the
    last step's index): the oracle against the reference's step written out
    above, bit for bit (spikes, potentials, every weight)."""
    d0 = _tiny_net(1, 4, seed=13)
    a = desc_arrays(d0.desc)
    sp = STDPParams(a_plus=0.05, a_minus=0.0525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=0.01)
    groups = [dict(count=32, tau_m=0.005, R=1e8, v0=0.0, vreset=0.0, theta=0.02, v_init_lo=0.0, v_init_hi=0.02),
              dict(count=8, tau_m=0.004, R=1e8, v0=0.0, vreset=0.005, theta=0.02, v_init_lo=0.0, v_init_hi=0.02)]
    d = descs.Desc(kind=N.SPK_SYN_VOLTAGE, groups=groups, refractory=0.002, i_bg=0.03, n_inputs=0,
                   pre=a["pre"], post=a["post"], weight=a["weight"], scale=np.ones(len(a["pre"])),
                   delay=a["delay"], plastic=(a["pre"] < 32).astype(int), stdp=sp, record_inputs=False)
    o = OracleNet(d.desc)
    ref = PlasticReference(d.desc, o, sp)
    for sec in [0.0173] + [0.00233] * 24:  # 24 steps each, many starting at the last index
        o.run(sec)
        ref.run(sec)
        assert o.current_time() == ref.base.time
    assert ref.base.repeats >= 3
    ids, times = o.spikes()
    np.testing.assert_array_equal(ids, np.asarray(ref.base.ids))
    np.testing.assert_array_equal(bits(times), bits(np.asarray(ref.base.times, F)))
    np.testing.assert_array_equal(bits(o.state(N.SPK_FIELD_V, 40)), bits(ref.base.V))
    w = ref.weights()
    assert not np.array_equal(w, a["weight"].astype(F))
    np.testing.assert_array_equal(bits(o.weights()), bits(w))


@pytest.mark.gpu
@pytest.mark.parametrize("sched", [None, (1, 512, 0, 0)])
@pytest.mark.parametrize("plastic", [False, True])
def test_index_repeats_within_runs(sched, plastic):
    """Runs of 0.00233 s (24 steps) whose start drifts to a half timestep:
    the index from roundf(t/dt) then repeats and skips within a run, and each
    repeat delivers the step before's spikes again (the engine's step kernels
    against the oracle), with and without STDP, persistent and in bulk mode."""
    from spike_gb300 import Net, schedule
    d = descs.random_voltage_net(n=600, n_in=200, d_max=12, seed=41, plastic=plastic, stdp=STDP if plastic else None)
    o = OracleNet(d.desc)
    net = Net.from_desc(d.desc, schedule(*sched) if sched else None)
    for sec in [0.0173] + [0.00233] * 24:
        net.run(sec)
        o.run(sec)
    assert net.synchronize() == 0
    assert_same(net, o, 600, 200, 1, weights=plastic, tag=f"plastic={plastic} {net.schedule()}")


@pytest.mark.gpu
@pytest.mark.parametrize("rule,norm", [(N.SPK_STDP_EVANS, 0), (N.SPK_STDP_INHIBITORY, 0), (N.SPK_STDP_CUSTOM, 0),
                                       (N.SPK_STDP_WEIGHT_DEPENDENT, N.SPK_NORM_AFTER_RULE)])
def test_bulk_only_rules_at_repeating_boundaries(rule, norm):
    """The per-synapse-trace rules and the weight normalisation (bulk mode)
    across run starts and within-run index repeats: carried keys delivered
    after the rules' updates, the rules' spike lookups unchanged."""
    from spike_gb300 import Net
    from test_stdp_rules import CUSTOM, EVANS, VOGELS
    sp = {N.SPK_STDP_EVANS: EVANS, N.SPK_STDP_INHIBITORY: VOGELS, N.SPK_STDP_CUSTOM: CUSTOM}.get(rule, STDP)
    d = descs.random_voltage_net(n=300, n_in=200, plastic=True, stdp=sp, stdp_rule=rule, weight_norm=norm, seed=43)
    o = OracleNet(d.desc)
    net = Net.from_desc(d.desc)
    for sec in [0.0173] + [0.00233] * 12:
        net.run(sec)
        o.run(sec)
    assert net.synchronize() == 0
    assert_same(net, o, 300, 200, 1, weights=True, tag=f"rule {rule} norm {norm}")
