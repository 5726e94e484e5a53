"""The model-building front end against the reference front end's own output.

Fixtures in tests/golden/ were produced by the reference's Spike front end
(compiled from the reference sources, tests/golden/make_golden.py).  Each case
is rebuilt here through this repository's front end and every array must be
identical: presynaptic/postsynaptic ids, weights, scales, delays, labels, in
creation order, plus the presynaptic sort and the plastic-synapse set.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import cases
from spike_gb300 import desc_arrays

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(case):
    return dict(np.load(os.path.join(GOLD, f"ref_{case}.npz")))


def _check_created(m, g):
    d = m.desc()
    a = desc_arrays(d)
    assert d.n_synapses == int(g["n_synapses"][0])
    for k in ("pre", "post", "delay", "label"):
        np.testing.assert_array_equal(a[k], g["created_" + k], err_msg=k)
    for k in ("weight", "scale"):
        assert np.array_equal(a[k].view(np.uint32), g["created_" + k].view(np.uint32)), k
    return d, a


@pytest.mark.parametrize("case", ["va_mix", "brunel", "shapes"])
def test_connectivity_matches_reference(case):
    m = {"va_mix": lambda: cases.ref_va(True), "brunel": cases.ref_brunel, "shapes": cases.ref_shapes}[case]()
    g = _load(case)
    d, a = _check_created(m, g)
    # number of labels, group constants derived by the front end
    assert d.n_labels == int(g["num_syn_labels"][0])
    taus = np.array([d.groups[i].tau_m for i in range(d.n_groups)], np.float32)
    assert set(taus.tolist()) == set(g["tau_m"].tolist())
    if "vhat" in g:
        assert np.array_equal(np.ctypeslib.as_array(d.label_vhat, (d.n_labels,)), g["vhat"])


def test_stable_presynaptic_sort_matches_reference():
    """The oracle's sorted order (key N_in + pre, stable) is the reference's
    Synapses::sort_synapses order."""
    from oracle import OracleNet
    m = cases.ref_brunel()
    g = _load("brunel")
    o = OracleNet(m.desc())
    pre, post, delay = o.sorted_synapses()
    np.testing.assert_array_equal(pre, g["sorted_pre"])
    np.testing.assert_array_equal(post, g["sorted_post"])
    np.testing.assert_array_equal(delay, g["sorted_delay"])


def test_plastic_synapses_match_reference():
    m = cases.ref_brunel()
    g = _load("brunel")
    a = desc_arrays(m.desc())
    created_plastic = np.flatnonzero(a["plastic"])
    # reference plastic indices are in sorted order (STDPPlasticity::prepare_backend_early)
    rs = g["reversesort"]
    np.testing.assert_array_equal(np.sort(rs[created_plastic]), np.sort(g["plastic_sorted"]))


def test_vogels_abbott_full_network_digests():
    """Examples/VogelsAbbottNet.cpp defaults: 4,000 neurons and exactly 320,261
    synapses under srand(42), every array bit-identical (SHA-256)."""
    with open(os.path.join(GOLD, "ref_va.json")) as f:
        meta = json.load(f)
    m = cases.ref_va(False)
    nn, ni, ns = m.counts()
    assert (nn, ni, ns) == (4000, 0, 320261) == (meta["n_neurons"], meta["n_inputs"], meta["n_synapses"])
    a = desc_arrays(m.desc())
    for k, h in meta["digests_created"].items():
        assert hashlib.sha256(np.ascontiguousarray(a[k]).tobytes()).hexdigest() == h, k


@pytest.mark.parametrize("case,d_lo,d_hi", [("va_g2", 2, 2), ("va_g3", 3, 5)])
def test_grouped_vogels_abbott_digests(case, d_lo, d_hi):
    """The network with delays of d_lo..d_hi steps: every array bit-identical,
    and its minimum delay is the timestep grouping the reference's
    finalise_model chose (Spike/Models/SpikingModel.cpp:98)."""
    with open(os.path.join(GOLD, "ref_va_grouped.json")) as f:
        meta = json.load(f)[case]
    m = cases.ref_va(False, d_lo, d_hi)
    assert m.counts() == (meta["n_neurons"], meta["n_inputs"], meta["n_synapses"])
    a = desc_arrays(m.desc())
    for k, h in meta["digests_created"].items():
        assert hashlib.sha256(np.ascontiguousarray(a[k]).tobytes()).hexdigest() == h, k
    assert int(a["delay"].min()) == meta["min_delay"] == meta["timestep_grouping"] == d_lo
    assert int(a["delay"].max()) == meta["max_delay"]


@pytest.mark.parametrize("case,current", [("vdet", False), ("cdet", True)])
def test_deterministic_network_digests(case, current):
    """The deterministic voltage and current synapse networks of the
    bit-exact comparison with the reference's kernels: every array
    bit-identical, and the labels the reference front end made."""
    with open(os.path.join(GOLD, "ref_det.json")) as f:
        meta = json.load(f)[case]
    m = cases.ref_det(current)
    assert m.counts() == (meta["n_neurons"], meta["n_inputs"], meta["n_synapses"])
    a = desc_arrays(m.desc())
    for k, h in meta["digests_created"].items():
        assert hashlib.sha256(np.ascontiguousarray(a[k]).tobytes()).hexdigest() == h, k
    assert int(a["label"].max()) + 1 == meta["num_syn_labels"]
