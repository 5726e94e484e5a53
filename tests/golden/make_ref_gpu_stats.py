"""Statistics of the REFERENCE's own GPU kernels on benchmark networks.

Builds the reference's CUDA backend for this GPU (oracle/build_ref_gpu.sh,
from a checkout of the reference sources given on the command line), runs the
networks of oracle/ref_cases.inc on it (oracle/ref_gpu_run.cpp) and reduces
what they did to the numbers the GPU test tests/test_reference_gpu_stats.py
compares this library against:

* ``va``: Examples/VogelsAbbottNet.cpp defaults (4,000 conductance LIF
  neurons, 320,261 synapses, all neurons starting at V0), 1 s;
* ``brunel_cfg2``: benchmark configuration 2 at full size (12,500 LIF,
  10,000 Poisson inputs, 28.1 M synapses), 2 s;
* ``brunel_cfg2_plastic``: the same with weight-dependent STDP on E->E, 1 s.

Per network: population rate (whole run, and its second half), mean ISI CV
over neurons with at least three spikes, spike and synaptic-event counts, the
wall time of run() with and without the spike monitor (the latter gives the
reference's events/s), and for the plastic network a 20-bin histogram of the
final E->E weights on [0, w_max].  The reference is not bit-reproducible (its
float ring additions are ordered by atomics and its Poisson inputs come from
cuRAND), so these are compared statistically.

Usage, on a machine with the GPU and the reference sources:
    python tests/golden/make_ref_gpu_stats.py REFERENCE_ROOT OUT.json
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
CASES = [("va", 1.0, None), ("brunel_cfg2", 2.0, None), ("brunel_cfg2_plastic", 1.0, 2.0e-4)]


def spike_stats(ids: np.ndarray, times: np.ndarray, n: int, seconds: float) -> dict:
    order = np.lexsort((times, ids))
    ids, times = ids[order], times[order]
    late = times >= seconds / 2
    cvs = []
    starts = np.searchsorted(ids, np.arange(n + 1))
    for k in range(n):
        t = times[starts[k]:starts[k + 1]]
        if len(t) >= 3:
            isi = np.diff(t.astype(np.float64))
            if isi.mean() > 0:
                cvs.append(isi.std() / isi.mean())
    return {"rate_hz": len(ids) / (n * seconds), "rate_late_hz": int(late.sum()) / (n * seconds / 2),
            "cv_isi": float(np.mean(cvs)) if cvs else None, "cv_neurons": len(cvs)}


def run(binary: str, case: str, seconds: float, monitor: int, out: str) -> dict:
    res = subprocess.run([binary, case, str(seconds), str(monitor), out], check=True, capture_output=True,
                         text=True, timeout=1800)
    line = [x for x in res.stdout.splitlines() if x.startswith("{")][-1]
    return json.loads(line)


def main(ref_root: str, out_json: str) -> int:
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref_gpu.sh"), ref_root], check=True)
    binary = os.path.join(ROOT, "oracle", "_ref", "gpu", "ref_gpu_run")
    result = {}
    with tempfile.TemporaryDirectory() as td:
        for case, seconds, wmax in CASES:
            mon = run(binary, case, seconds, 1, td)
            fast = run(binary, case, seconds, 0, td)
            ids = np.fromfile(os.path.join(td, f"{case}_neurons_SpikeIDs.bin"), np.int32)
            times = np.fromfile(os.path.join(td, f"{case}_neurons_SpikeTimes.bin"), np.float32)
            r = {k: mon[k] for k in ("synapses", "neurons", "inputs", "seconds", "timesteps", "neuron_spikes",
                                     "input_spikes", "events", "cuda_status")}
            r.update(spike_stats(ids, times, mon["neurons"], seconds))
            r["wall_s_monitor"] = mon["wall_s"]
            r["wall_s"] = fast["wall_s"]
            r["events_per_s"] = mon["events"] / fast["wall_s"] if fast["wall_s"] > 0 else None
            if wmax:
                w = np.fromfile(os.path.join(td, f"{case}_final_SynapticWeights.bin"), np.float32)
                h, _ = np.histogram(np.clip(w, 0.0, wmax), bins=20, range=(0.0, wmax))
                r["weights"] = {"w_max": wmax, "count": int(len(w)), "mean": float(w.mean()),
                                "hist": (h / max(1, len(w))).tolist()}
            result[case] = r
            print(case, json.dumps(r), flush=True)
    with open(out_json, "w") as f:
        json.dump(result, f, indent=1, sort_keys=True)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1], sys.argv[2]))
