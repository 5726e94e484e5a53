"""spk_step_noalloc, the allocation-free step entry point, against
spk_net_run_steps on the same network and schedule (GPU, through the C ABI).

The caller-owned buffers are built here in the layout include/spike_gb300.h
documents (with torch as the caller's allocator) from the same descriptor the
reference entry point is created from.  Both entry points run the same step
kernel with the same schedule, so the test's tolerance is zero: spikes, state,
weights and event counts agree bit for bit after each of two calls in a row.

The file is named so that pytest collects it last: it has to pass both alone
in a fresh process and after every other test of a session has used the
library.
"""
import ctypes as C

import numpy as np
import pytest

import cases
import descs
from spike_gb300 import Net, schedule
from spike_gb300 import _native as N
from spike_gb300.model import STDPParams, desc_arrays

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX_ULP = 0  # the two entry points must agree exactly
STDP = STDPParams(a_plus=0.005, a_minus=0.00525, tau_plus=0.02, tau_minus=0.02, lambda_=1.0, alpha=1.0, w_max=1.0)


def f32bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.int64)


def assert_close(got, want, what):
    diff = np.abs(f32bits(got) - f32bits(want))
    assert diff.size == 0 or diff.max() <= MAX_ULP, f"{what}: {int((diff > MAX_ULP).sum())} values differ"


class CallerNet:
    """Device buffers of one network in the spk_step_noalloc layout."""

    def __init__(self, d: N.NetDesc, W: int, TS: int, ctas: int, ref: Net, spike_capacity: int = 1 << 20):
        dev = torch.device("cuda:0")
        a = desc_arrays(d)
        Nn, Nin, L = d.n_neurons, d.n_inputs, d.n_labels
        n_tiles = W * ctas
        its = ((Nin + n_tiles - 1) // n_tiles + 31) // 32 * 32 if Nin else 0
        KL = n_tiles * its
        n_keys = KL + n_tiles * TS
        S = len(a["pre"])
        max_delay = int(a["delay"].max()) if S else 1
        G = int(a["delay"].min()) if S else 1  # timestep grouping: the minimum delay
        B = max_delay + 2 * G + 1
        self.N, self.Nin, self.L, self.KL, self.B, self.TS, self.n_tiles = Nn, Nin, L, KL, B, TS, n_tiles

        # scale classes of plastic synapses, numbered by first appearance
        cls = np.zeros(S, np.uint32)
        scales = []
        plastic = a["plastic"].astype(bool) if d.has_stdp else np.zeros(S, bool)
        for s in np.nonzero(plastic)[0]:
            v = np.float32(a["scale"][s])
            if v not in scales:
                scales.append(v)
            cls[s] = scales.index(v) + 1
        self.scales = np.asarray(scales if scales else [1.0], np.float32)

        pre = a["pre"].astype(np.int64)
        post = a["post"].astype(np.int64)
        key = np.where(pre < 0, Nin + pre, KL + pre)
        cell = key * n_tiles + post // TS
        order = np.argsort(cell, kind="stable")  # entry i holds synapse order[i]
        entry_of = np.empty(S, np.int64)
        entry_of[order] = np.arange(S)
        rowptr = np.zeros(n_keys * n_tiles + 1, np.int32)
        rowptr[1:] = np.cumsum(np.bincount(cell, minlength=n_keys * n_tiles))
        # plastic afferent records per post, creation order: (pre key, weight)
        pl = np.nonzero(cls)[0]
        csc_ptr = np.zeros(Nn + 1, np.int32)
        csc_ptr[1:] = np.cumsum(np.bincount(post[pl], minlength=Nn))
        by_post = pl[np.argsort(post[pl], kind="stable")]
        csc_of = np.full(S, -1, np.int64)
        csc_of[by_post] = np.arange(len(by_post))
        csc = np.stack([key[by_post].astype(np.uint32), a["weight"][by_post].astype(np.float32).view(np.uint32)],
                       axis=1)
        self.csc_of = csc_of
        # entries: w*scale for static synapses, the afferent record for plastic ones
        y = np.where(cls == 0, (a["weight"] * a["scale"]).astype(np.float32).view(np.uint32),
                     csc_of.astype(np.uint32)).astype(np.uint32)
        x = (post % TS).astype(np.uint32) | (a["delay"].astype(np.uint32) << 16) | \
            (a["label"].astype(np.uint32) << 24) | (cls << 28)
        entries = np.stack([x, y], axis=1)[order]
        self.entry_of = entry_of
        self.plastic = cls != 0

        def dbuf(arr, dtype=None):
            t = torch.from_numpy(np.ascontiguousarray(arr if dtype is None else arr.astype(dtype)))
            return t.to(dev) if t.numel() else torch.zeros(1, dtype=t.dtype, device=dev)

        rates = np.ctypeslib.as_array(d.input_rates, (d.n_stimuli * Nin,))[d.stimulus * Nin:(d.stimulus + 1) * Nin] \
            if Nin else np.zeros(1, np.float32)
        self.t = dict(
            rowptr=dbuf(rowptr), entries=dbuf(entries.view(np.int32)), csc_ptr=dbuf(csc_ptr),
            csc=dbuf(csc.view(np.int32).reshape(-1)),
            V=dbuf(ref.state(N.SPK_FIELD_V, Nn)), last=torch.full((Nn,), -1000.0, device=dev),
            syn=torch.zeros(Nn * L, device=dev), ring=torch.zeros(n_tiles * B * TS * L, device=dev),
            innext=torch.full((max(Nin, 1),), -1000.0, device=dev), rates=dbuf(rates, np.float32),
            post_tr=torch.zeros(Nn, device=dev), pre_tr=torch.zeros(n_keys, device=dev),
            spikes=torch.zeros(2 * spike_capacity, dtype=torch.int32, device=dev),
            group_bits=torch.zeros(G * n_keys // 32, dtype=torch.int32, device=dev),
            run_state=torch.zeros(N.SPK_RUN_STATE_BYTES // 4, dtype=torch.int32, device=dev),
        )
        t = self.t
        dn = N.DeviceNet()
        dn.n_neurons, dn.n_inputs, dn.n_labels, dn.synapse_kind, dn.max_delay = Nn, Nin, L, d.synapse_kind, max_delay
        dn.warps_per_cta, dn.tile_posts, dn.ctas = W, TS, ctas
        dn.dt, dn.refractory_period, dn.background_current = d.dt, d.refractory_period, d.background_current
        dn.n_groups, dn.groups = d.n_groups, d.groups
        dn.label_tau, dn.label_vhat = d.label_tau, d.label_vhat
        dn.has_stdp, dn.stdp = d.has_stdp, d.stdp
        dn.n_plastic_scales = len(scales)
        dn.plastic_scales = self.scales.ctypes.data_as(C.POINTER(C.c_float))
        dn.seed, dn.record_inputs = d.seed, d.record_inputs
        dn.rowptr, dn.entries = t["rowptr"].data_ptr(), t["entries"].data_ptr()
        dn.csc_ptr, dn.csc = t["csc_ptr"].data_ptr(), t["csc"].data_ptr()
        dn.V, dn.last_spike, dn.syn_trace, dn.ring = (t[k].data_ptr() for k in ("V", "last", "syn", "ring"))
        dn.input_next, dn.rates = t["innext"].data_ptr(), t["rates"].data_ptr()
        dn.post_trace, dn.pre_trace = t["post_tr"].data_ptr(), t["pre_tr"].data_ptr()
        dn.spikes, dn.spike_capacity = t["spikes"].data_ptr(), spike_capacity
        dn.run_state = t["run_state"].data_ptr()
        dn.timestep_grouping = G
        dn.group_bits = t["group_bits"].data_ptr()
        self.G = G
        self.dn = dn
        self.dt = np.float32(d.dt)
        self.time = np.float32(0.0)
        torch.cuda.synchronize()

    def step(self, n_steps: int, plastic: bool):
        stream = torch.cuda.current_stream().cuda_stream
        N.check(N.lib().spk_step_noalloc(C.byref(self.dn), n_steps, 1 if plastic else 0, C.c_float(self.time),
                                         C.c_void_p(stream)), "spk_step_noalloc")
        # the time bookkeeping of spk_net_run_steps: start + (float)steps * dt
        self.time = np.float32(self.time + np.float32(np.float32(n_steps) * self.dt))

    def run_seconds(self, seconds: float, plastic: bool):
        """spk_net_run's steps and time bookkeeping: ceil(seconds/dt) rounded
        down to whole groups, then start + seconds."""
        start = self.time
        steps = int(np.ceil(np.float32(seconds) / self.dt)) // self.G * self.G
        self.step(steps, plastic)
        self.time = np.float32(start + np.float32(seconds))

    def compare(self, ref: Net, n_synapses: int, tag: str, status: int = 0):
        """Everything the two entry points hold, and their device status
        (0, or SPK_ERR_UNSUPPORTED after an active list of two carried groups)."""
        torch.cuda.synchronize()
        assert ref.synchronize() == status
        rs = self.t["run_state"].cpu().numpy()
        count, events = int(rs[8:10].view(np.uint64)[0]), int(rs[10:12].view(np.uint64)[0])
        assert int(rs[12]) == status, f"{tag}: device status {int(rs[12])}"
        assert events == ref.events(), tag
        store = self.t["spikes"][:2 * count].cpu().numpy().reshape(-1, 2)
        keys, tbits = store[:, 0].astype(np.int64), store[:, 1].copy().view(np.float32)
        neu = keys >= self.KL
        for pop, mask, ids in ((N.SPK_POP_NEURONS, neu, keys - self.KL),
                               (N.SPK_POP_INPUTS, ~neu, self.Nin - 1 - keys)):
            ri, rt = ref.spikes(pop)
            assert mask.sum() == len(ri), f"{tag} pop {pop}: {mask.sum()} spikes vs {len(ri)}"
            np.testing.assert_array_equal(ids[mask], ri, err_msg=f"{tag} pop {pop} ids")
            assert_close(tbits[mask], rt, f"{tag} pop {pop} times")
        Nn, L, B, TS = self.N, self.L, self.B, self.TS
        assert_close(self.t["V"].cpu().numpy(), ref.state(N.SPK_FIELD_V, Nn), f"{tag} V")
        assert_close(self.t["last"].cpu().numpy(), ref.state(N.SPK_FIELD_LAST_SPIKE, Nn), f"{tag} last")
        assert_close(self.t["syn"].cpu().numpy(), ref.state(N.SPK_FIELD_SYN_TRACE, Nn * L), f"{tag} traces")
        if self.Nin:
            assert_close(self.t["innext"].cpu().numpy(), ref.state(N.SPK_FIELD_INPUT_NEXT, self.Nin),
                         f"{tag} input next")
        ring = self.t["ring"].cpu().numpy().reshape(self.n_tiles, B, TS, L).transpose(1, 0, 2, 3)
        ring = ring.reshape(B, self.n_tiles * TS, L)[:, :Nn].reshape(-1)
        assert_close(ring, ref.state(N.SPK_FIELD_RING, B * Nn * L), f"{tag} ring")
        if self.dn.has_stdp:
            csc = self.t["csc"].cpu().numpy().reshape(-1, 2)
            w = ref.weights(n_synapses)
            mine = csc[self.csc_of[self.plastic], 1].copy().view(np.float32)
            assert_close(mine, w[self.plastic], f"{tag} plastic weights")
            assert_close(self.t["post_tr"].cpu().numpy(), ref.state(N.SPK_FIELD_POST_TRACE, Nn), f"{tag} post")
            pre = self.t["pre_tr"].cpu().numpy()
            pre_c = np.concatenate([pre[self.Nin - 1 - np.arange(self.Nin)], pre[self.KL:self.KL + Nn]])
            assert_close(pre_c, ref.state(N.SPK_FIELD_PRE_TRACE, self.Nin + Nn), f"{tag} pre")
        return count


def run_both(d, W, TS, ctas, calls):
    ref = Net.from_desc(d, schedule(W, TS, ctas, 0))
    cn = CallerNet(d, W, TS, ctas, ref)
    spikes = 0
    for i, (n_steps, plastic) in enumerate(calls):
        ref.run_steps(n_steps, plastic)
        assert ref.synchronize() == 0  # one persistent kernel on the GPU at a time
        cn.step(n_steps, plastic)
        spikes = cn.compare(ref, d.n_synapses, f"call {i + 1} W={W} TS={TS} C={ctas}")
    ref.close()
    return spikes


def test_noalloc_matches_run_steps_with_stdp_multi_cta():
    d = descs.random_voltage_net(n=300, n_in=200, plastic=True, stdp=STDP)
    spikes = run_both(d.desc, 4, 32, 3, [(350, True), (250, True)])
    assert spikes > 200


def test_noalloc_matches_run_steps_conductance():
    m = cases.ref_va(True)
    d = m.desc()
    spikes = run_both(d, 8, 32, 2, [(300, False), (300, False)])
    assert spikes > 100


def test_noalloc_matches_run_steps_current_synapses_single_cta():
    """Current synapses with two labels on one CTA (no cooperative launch),
    recording the inputs' spikes too."""
    rng = np.random.default_rng(3)
    n, S = 120, 3000
    pre = rng.integers(-50, n, S)
    post = rng.integers(0, n, S)
    d = descs.Desc(kind=N.SPK_SYN_CURRENT, n_labels=2, label_tau=[0.003, 0.008],
                   groups=[dict(count=n, tau_m=0.02, R=1e8, v0=-0.07, vreset=-0.07, theta=-0.055)],
                   refractory=0.002, i_bg=0.0, n_inputs=50, rates=rng.uniform(5, 60, 50),
                   pre=pre, post=post, weight=rng.uniform(0, 3e-10, S), scale=np.ones(S),
                   delay=np.maximum(1, rng.integers(0, 9, S)), label=(pre < 0).astype(int), record_inputs=True)
    spikes = run_both(d.desc, 4, 32, 1, [(400, False), (300, False)])
    assert spikes > 100


def test_noalloc_matches_run_steps_two_plastic_scale_classes():
    """Plastic synapses in two weight-scale classes (input and recurrent
    excitatory synapses scaled differently)."""
    base = descs.random_voltage_net(n=300, n_in=200, plastic=True, stdp=STDP, seed=9)
    a = base.arrays
    scale = np.where(a["pre"] < 0, 1.0, 0.5).astype(np.float32)
    pl = np.ctypeslib.as_array(base.desc.plastic, (base.desc.n_synapses,)).copy()
    groups = [dict(count=240, tau_m=0.02, R=1e8, v0=0.0, vreset=0.0, theta=0.02, v_init_lo=0.0, v_init_hi=0.018),
              dict(count=60, tau_m=0.01, R=1e8, v0=0.0, vreset=0.002, theta=0.018)]
    rates = np.ctypeslib.as_array(base.desc.input_rates, (200,)).copy()
    d = descs.Desc(kind=N.SPK_SYN_VOLTAGE, groups=groups, refractory=0.002, n_inputs=200, rates=rates,
                   pre=a["pre"], post=a["post"], weight=a["weight"] / scale, scale=scale, delay=a["delay"],
                   plastic=pl, stdp=STDP, seed=base.desc.seed, record_inputs=True)
    cn_scales = run_both(d.desc, 4, 32, 3, [(300, True), (200, True)])
    assert cn_scales > 200


def test_noalloc_spike_store_overflow_sets_status():
    """A spike store too small for the run: the device status in run_state
    becomes SPK_ERR_OVERFLOW and stays there for the next call, while the
    network state goes on exactly as the reference entry point's."""
    d = descs.random_voltage_net(n=300, n_in=200, plastic=False, seed=11)
    ref = Net.from_desc(d.desc, schedule(4, 32, 3, 0))
    cn = CallerNet(d.desc, 4, 32, 3, ref, spike_capacity=50)
    for i, n_steps in enumerate((300, 200)):
        ref.run_steps(n_steps, False)
        assert ref.synchronize() == 0
        cn.step(n_steps, False)
        torch.cuda.synchronize()
        rs = cn.t["run_state"].cpu().numpy()
        assert int(rs[12]) == N.SPK_ERR_OVERFLOW, f"call {i + 1}: status {int(rs[12])}"
        assert int(rs[8:10].view(np.uint64)[0]) == 50
        assert int(rs[10:12].view(np.uint64)[0]) == ref.events()
        assert_close(cn.t["V"].cpu().numpy(), ref.state(N.SPK_FIELD_V, 300), f"call {i + 1} V")
    ref.close()


def test_noalloc_matches_run_steps_grouped():
    """A network whose minimum delay is 3 steps (timestep grouping 3), with
    Poisson inputs, on three CTAs."""
    d = descs.random_voltage_net(n=300, n_in=200, d_min=3, d_max=10, seed=7)
    spikes = run_both(d.desc, 4, 32, 3, [(300, False), (201, False)])
    assert spikes > 200


@pytest.mark.parametrize("d_min", [1, 3])
def test_noalloc_run_boundaries_deliver_the_carried_group_again(d_min):
    """Runs of seconds whose first group index repeats (d_min 1: 0.0173 s is
    174 steps, the next run starts at index 173) or skips one (d_min 3): the
    carried group is delivered again through group_bits, as spk_net_run does."""
    d = descs.random_voltage_net(n=300, n_in=200, d_min=d_min, d_max=10, seed=8)
    ref = Net.from_desc(d.desc, schedule(4, 32, 3, 0))
    cn = CallerNet(d.desc, 4, 32, 3, ref)
    for i, sec in enumerate((0.0173, 0.0173, 0.0337, 0.0101, 0.05)):
        ref.run(sec)
        assert ref.synchronize() == 0
        cn.run_seconds(sec, False)
        cn.compare(ref, d.desc.n_synapses, f"run {i + 1} d_min={d_min}")
    ref.close()


@pytest.mark.parametrize("seed", range(40, 52))
def test_noalloc_random_networks(seed):
    """Seeded networks of the random parity test whose plasticity the
    persistent kernel runs (the weight-dependent rule, or none), under the
    planner's schedule, through that test's random run sequences: run(seconds)
    with fractions that repeat or skip the timestep index, whole-group
    run_steps, plasticity switched off, reset_time.  reset_state, stimulus
    switches and snapshots have no allocation-free form and are skipped."""
    from test_random_parity import random_case
    for s in range(seed * 100, seed * 100 + 100):  # even seeds: a plastic network
        d, _, actions, n, n_in, L, plastic = random_case(s)
        if d.desc.stdp_rule == N.SPK_STDP_WEIGHT_DEPENDENT and d.desc.weight_norm == N.SPK_NORM_OFF and \
                plastic == (seed % 2 == 0):
            break
    probe = Net.from_desc(d.desc, None)
    sc = probe.schedule()
    probe.close()
    W, TS, ctas = sc["warps_per_cta"], sc["tile_posts"], sc["ctas"]
    ref = Net.from_desc(d.desc, schedule(W, TS, ctas, 0))
    cn = CallerNet(d.desc, W, TS, ctas, ref)
    for i, act in enumerate(actions):
        if act[0] == "run":
            ref.run(act[1], act[2])
            assert ref.synchronize() in (0, N.SPK_ERR_UNSUPPORTED)
            cn.run_seconds(act[1], act[2])
        elif act[0] == "steps":
            ref.run_steps(act[1], act[2])
            assert ref.synchronize() in (0, N.SPK_ERR_UNSUPPORTED)
            cn.step(act[1], act[2])
        elif act[0] == "reset_time":
            ref.reset_time()
            cn.time = np.float32(0.0)
        else:
            continue
        cn.compare(ref, d.desc.n_synapses, f"seed {s} {sc} action {i} of {actions}", ref.synchronize())
    ref.close()
