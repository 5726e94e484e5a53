"""The oracle and the engine against spike trains of the REFERENCE's own GPU
kernels, bit for bit.

tests/golden/ref_gpu_exact.npz holds what the reference's CUDA backend,
compiled for this GPU from the reference sources with every float expression
as written (oracle/build_ref_gpu.sh, REF_STRICT_FP=1), did on three
deterministic networks (tests/golden/make_ref_gpu_exact.py): the
Vogels-Abbott network of Examples/VogelsAbbottNet.cpp (one weight per synapse
label, so the atomic order of the reference's ring additions cannot change a
sum; no Poisson inputs) with delays of 1 step, 2 steps (timestep grouping 2)
and 3-5 steps (grouping 3), each run for 0.5 s, then 0.0337 s and 0.2 s.
The second run is not whole groups: the third starts one timestep index on
(grouping 2) or at a group index of the last group's parity (grouping 3),
where the reference's double-buffered active lists deliver the last group's
spikes again.  vdet (voltage synapses) has weights that are integer
multiples of a power of two, whose sums are exact in any order.  Every spike
id and float time must be identical: 48,000-72,000 spikes in 7,335-7,338
timesteps per network.  (The reference's current-synapse backend faults on
the GPU, CurrentSpikingSynapses.cu:27-29, so current synapses have no such
record.)
"""
import os

import numpy as np
import pytest

import cases
from oracle import OracleNet

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_gpu_exact.npz")
CASES = [("va", lambda: cases.ref_va(False)), ("va_g2", lambda: cases.ref_va(False, 2, 2)),
         ("va_g3", lambda: cases.ref_va(False, 3, 5)), ("vdet", lambda: cases.ref_det(False))]


def _gold():
    if not os.path.exists(GOLD):
        pytest.skip("no reference GPU spike trains recorded")
    return np.load(GOLD)


def _sorted(ids, times):
    order = np.lexsort((ids, times))
    return ids[order], times[order]


def _check(ids, times, z, case):
    ri, rt = z[case + "_ids"], z[case + "_times"]
    assert len(ids) == len(ri) > 40000, (case, len(ids), len(ri))
    np.testing.assert_array_equal(ids, ri, err_msg=case)
    np.testing.assert_array_equal(times.view(np.uint32), rt.view(np.uint32), err_msg=case)


@pytest.mark.parametrize("case,build", CASES)
def test_oracle_reproduces_reference_gpu_spike_trains(case, build):
    z = _gold()
    m = build()  # owns the descriptor's arrays
    o = OracleNet(m.desc())
    for sec in z["runs"]:
        o.run(float(sec))
    _check(*_sorted(*o.spikes()), z, case)


@pytest.mark.gpu
@pytest.mark.parametrize("case,build", CASES)
def test_engine_reproduces_reference_gpu_spike_trains(case, build):
    z = _gold()
    m = build()
    net = m.finalise()
    for sec in z["runs"]:
        net.run(float(sec))
    assert net.synchronize() == 0
    _check(*_sorted(*net.spikes()), z, case)
