"""Spike trains of the REFERENCE's own GPU kernels on deterministic networks.

The reference's CUDA backend orders its float ring additions by atomics, so
its runs are not reproducible in general.  They are when every contribution a
ring cell can receive has the same value: n equal summands give the same sum
in any order.  The Vogels-Abbott network (Examples/VogelsAbbottNet.cpp) is
such a network: one weight per synapse label (0.4 and 5.1 times 10 nS), no
Poisson inputs, all neurons starting at V0.  With the kernels compiled as
written (no fused multiply-add, oracle/build_ref_gpu.sh with REF_STRICT_FP=1),
its spike train is a bit pattern that the oracle and the engine must
reproduce exactly.

The same holds for networks whose weights are integer multiples of a power
of two (partial sums are exact in any order): vdet, voltage synapses with E
weight J and I weight -4 J.

Cases (oracle/ref_cases.inc): va (delay 1 step), va_g2 (2 steps: timestep
grouping 2), va_g3 (3-5 steps: grouping 3), vdet; each run(0.5) from the model's
initial state, then run(0.0337) (not whole groups: the next run starts at
start + seconds) and run(0.2).  Per case the neuron spikes, sorted by (time,
id) (the reference's monitor stores a step's spikes in atomic order), go to
tests/golden/ref_gpu_exact.npz.

Usage, on a machine with the GPU and the reference sources:
    REF_STRICT_FP=1 bash oracle/build_ref_gpu.sh REFERENCE_ROOT
    python tests/golden/make_ref_gpu_exact.py OUT.npz
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# cdet (current synapses) is not run: the reference's current-synapse backend
# never sets its device decay-constant pointer (CurrentSpikingSynapses.cu:27-29)
# and its injection kernel faults on it
CASES = ("va", "va_g2", "va_g3", "vdet")
RUNS = (0.5, 0.0337, 0.2)


def main(out: str) -> int:
    binary = os.path.join(ROOT, "oracle", "_ref", "gpu_strict", "ref_gpu_run")
    arrays, meta = {}, {}
    with tempfile.TemporaryDirectory() as td:
        for case in CASES:
            res = subprocess.run([binary, case, ",".join(str(s) for s in RUNS), "1", td], check=True,
                                 capture_output=True, text=True, timeout=1800)
            line = json.loads([x for x in res.stdout.splitlines() if x.startswith("{")][-1])
            ids = np.fromfile(os.path.join(td, f"{case}_neurons_SpikeIDs.bin"), np.int32)
            times = np.fromfile(os.path.join(td, f"{case}_neurons_SpikeTimes.bin"), np.float32)
            order = np.lexsort((ids, times))
            arrays[f"{case}_ids"], arrays[f"{case}_times"] = ids[order], times[order]
            meta[case] = line
            print(case, json.dumps(line), flush=True)
    np.savez_compressed(out, runs=np.asarray(RUNS, np.float32), meta=json.dumps(meta), **arrays)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1]))
