"""Restatements, over whole numpy arrays, of the reference's per-synapse
STDP kernels (EvansSTDPPlasticity.cu, InhibitorySTDPPlasticity.cu,
CustomSTDPPlasticity.cu) and of its weight normalisation
(WeightNormSTDPPlasticity.cpp / .cu), written from the reference kernels
independently of the oracle's C++ code, in float32 without contraction.
Driven by recorded rasters, they pin the oracle's rule arithmetic (CPU)."""
import ctypes
import ctypes.util

import numpy as np

from spike_gb300 import _native as N

_libm = ctypes.CDLL(ctypes.util.find_library("m"))
_libm.expf.restype = ctypes.c_float
_libm.expf.argtypes = [ctypes.c_float]
_libm.powf.restype = ctypes.c_float
_libm.powf.argtypes = [ctypes.c_float, ctypes.c_float]


def host_expf(x):
    """The C library's expf, with which the reference computes the decays on
    the host."""
    return np.float32(_libm.expf(float(x)))


def host_powf(x, y):
    return np.float32(_libm.powf(float(x), float(y)))


def rasters_of(o, d, steps, n, n_in):
    """Boolean [steps, n] rasters of neurons and inputs from an oracle run
    that started at time 0."""
    dt = np.float32(d.desc.dt)
    out = []
    for pop, count in ((N.SPK_POP_NEURONS, n), (N.SPK_POP_INPUTS, n_in)):
        ids, times = o.spikes(pop)
        r = np.zeros((steps, count), bool)
        r[np.rint(times / dt).astype(np.int64), ids] = True
        out.append(r)
    return out


class Normaliser:
    """WeightNormSTDPPlasticity over the plastic synapses `idx` (creation
    order): S per post is the sum of powf(w, 2) over its plastic afferents in
    that order (WeightNormSTDPPlasticity.cpp:52-58); each step the change
    (w - w0)^2 + 2 w0 (w - w0) of the afferents whose weight moved is summed
    per post in the order the engine fixes for the reference's atomicAdd
    (partial sum j over afferents j, j + 32, ... in creation order, then a
    pairwise tree over the 32 partials: j + 16, + 8, + 4, + 2, + 1), the
    divisor is sqrt(S + change) / sqrt(S), and the weights are divided when it
    is not 1 (WeightNormSTDPPlasticity.cu:101-176)."""

    def __init__(self, post_of_plastic, w0, n_posts, sums=None):
        f32 = np.float32
        self.w0 = w0.astype(f32)
        posts = np.asarray(post_of_plastic)
        order = np.argsort(posts, kind="stable")  # creation order within each post
        counts = np.bincount(posts, minlength=n_posts)
        self.posts = np.nonzero(counts)[0]
        width = -(-counts.max() // 32) * 32  # whole rows of 32 partial sums
        self.slot = np.full((len(self.posts), width), -1, np.int64)
        row = np.searchsorted(self.posts, posts[order])
        start = np.concatenate(([0], np.cumsum(counts[self.posts])[:-1]))
        rank = np.arange(len(order)) - start[row]
        self.slot[row, rank] = order
        if sums is None:
            sums = np.zeros(n_posts, f32)
            for j in range(len(posts)):  # creation order
                sums[posts[j]] = f32(sums[posts[j]] + host_powf(self.w0[j], 2.0))
        self.S = np.asarray(sums, f32)[self.posts]
        self.row_of = np.searchsorted(self.posts, posts)

    def __call__(self, wp, w0=None):
        f32 = np.float32
        w0 = self.w0 if w0 is None else w0
        dw = wp - w0
        term = np.where(dw != 0, dw * dw + f32(2) * w0 * dw, f32(0)).astype(f32)
        part = np.zeros((len(self.posts), 32), f32)
        for k in range(self.slot.shape[1] // 32):
            cols = self.slot[:, 32 * k:32 * (k + 1)]
            part = part + np.where(cols >= 0, term[np.maximum(cols, 0)], f32(0))
        o = 16
        while o >= 1:
            part = part[:, :o] + part[:, o:2 * o]
            o //= 2
        upd = part[:, 0]
        div = np.sqrt(self.S + upd) / np.sqrt(self.S)
        dv = div[self.row_of]
        return np.where(dv != f32(1), wp / dv, wp).astype(f32)


def restated_rule(rule, sp, d, pre_spk, post_spk, steps, n_exc, norm=N.SPK_NORM_OFF):
    """The three kernels' per-synapse updates restated over whole arrays of
    plastic synapses (float32 as the kernels compute, no contraction), driven
    by the recorded rasters: at timestep T the postsynaptic bit is T and the
    presynaptic bit is T - delay (EvansSTDPPlasticity.cu:96-131,
    InhibitorySTDPPlasticity.cu:108-143, CustomSTDPPlasticity.cu:99-142)."""
    f32, f64 = np.float32, np.float64
    pre_a, post_a = d.arrays["pre"], d.arrays["post"]
    plastic = pre_a < n_exc  # inputs and excitatory neurons
    pre_key = np.where(pre_a >= 0, pre_a, 0)
    pre_is_input = pre_a < 0
    in_key = np.where(pre_is_input, -pre_a - 1, 0)
    delay = d.arrays["delay"]
    w = d.arrays["weight"].copy()
    idx = np.nonzero(plastic)[0]
    wp = w[idx].astype(f32)
    tp = np.zeros(len(idx), f32)  # presynaptic trace
    tq = np.zeros(len(idx), f32)  # postsynaptic trace
    dt = f32(d.desc.dt)
    one = f32(1)
    normalise = Normaliser(post_a[idx], wp, post_spk.shape[1]) if norm != N.SPK_NORM_OFF else None
    for T in range(steps):
        if norm == N.SPK_NORM_BEFORE_RULE:
            wp = normalise(wp)
        pT = T - delay[idx]
        ok = pT >= 0
        pTc = np.where(ok, pT, 0)
        pre = ok & np.where(pre_is_input[idx], pre_spk[1][pTc, in_key[idx]], pre_spk[0][pTc, pre_key[idx]])
        post = post_spk[T, post_a[idx]]
        if rule == N.SPK_STDP_EVANS:
            tp = (one - (dt / f32(sp.tau_plus))) * tp
            tq = (one - (dt / f32(sp.tau_minus))) * tq
            tp = np.where(pre, tp + dt * f32(sp.a_plus) * (one - tp), tp)
            tq = np.where(post, tq + dt * f32(sp.a_minus) * (one - tq), tq)
            syn = np.zeros_like(wp)
            syn = np.where(pre, syn - (wp * tq), syn)
            syn = np.where(post, syn + ((one - wp) * tp), syn)
            wp = np.clip(wp + syn, f32(0), f32(1))
        elif rule == N.SPK_STDP_INHIBITORY:
            decay = host_expf(-dt / f32(sp.tau_plus))
            tp = tp * decay
            tq = tq * decay
            tp = np.where(pre, tp + one, tp)
            tq = np.where(post, tq + one, tq)
            lr = f32(sp.lambda_)
            syn = np.zeros_like(wp)
            syn = np.where(pre, syn + lr * tq, syn)
            const = f64(-lr) * (2.0 * f64(f32(sp.alpha)) * f64(f32(sp.tau_plus)))
            syn = np.where(pre, (syn.astype(f64) + const).astype(f32), syn)
            syn = np.where(post, syn + lr * tp, syn)
            wp = np.maximum(wp + syn, f32(0))
        else:
            tq = tq * host_expf(-dt / f32(sp.tau_minus))
            tp = tp * host_expf(-dt / f32(sp.tau_plus))
            a_plus, a_minus = f32(sp.a_plus), f32(sp.a_minus)
            tp = np.where(pre, a_plus if sp.clip_upper else tp + a_plus, tp)
            tq = np.where(post, a_minus if sp.clip_upper else tq + a_minus, tq)
            lr, a_star, w_max = f32(sp.lambda_), f32(sp.alpha), f32(sp.w_max)
            syn = np.zeros_like(wp)
            syn = np.where(pre, syn - (lr * (wp / w_max) * tq + lr * a_star), syn)
            syn = np.where(post, syn + lr * tp, syn)
            wp = np.maximum(wp + syn, f32(0))
        if norm == N.SPK_NORM_AFTER_RULE:
            wp = normalise(wp)
    w[idx] = wp
    return w


