"""Generate the connectivity golden fixtures from the REFERENCE front end.

Runs oracle/_ref/ref_dump (the reference's own Spike front end and Dummy
backend compiled from the reference sources by oracle/build_ref.sh) on the
cases defined in oracle/ref_dump.cpp and stores what it produced:

* small cases (va_mix, brunel, shapes): every array, as .npz;
* the full VogelsAbbottNet network (va, 320,261 synapses): counts and SHA-256
  digests of every array, as .json; the same for its grouped variants va_g2
  and va_g3 (delays of 2 and 3-5 steps) with the front end's timestep
  grouping, as ref_va_grouped.json, and of the deterministic voltage and
  current synapse networks vdet and cdet, as ref_det.json;
* the weight and connectivity files the reference's save functions write for
  each case (Spike/Synapses/Synapses.cpp:423-614, SpikingSynapses.cpp:136-189;
  ref_dump's save mode), and the weights read back from the text file and
  written again: size and SHA-256 of every file, as ref_checkpoint.json; for
  the seeded random networks rand1..rand30 of oracle/ref_cases.inc, the file
  names, one SHA-256 over all files and one over the synapse arrays in
  creation order with the label constants, as ref_checkpoint_random.json.

Usage (in a checkout where the reference sources are present):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def read_dump(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    o = 0
    while o < len(data):
        (nl,) = struct.unpack_from("<i", data, o)
        o += 4
        name = data[o:o + nl].decode()
        o += nl
        typ = chr(data[o])
        o += 1
        (cnt,) = struct.unpack_from("<q", data, o)
        o += 8
        dt = np.int32 if typ == "i" else np.float32
        arr = np.frombuffer(data, dtype=dt, count=cnt, offset=o).copy()
        o += 4 * cnt
        out[name] = arr
    return out


def creation_order(d: dict) -> dict:
    """Arrays in creation order: sorted_x[reversesort[i]] (the reference's
    readback mapping, Spike/Synapses/Synapses.cpp:525-584)."""
    rs = d["reversesort"]
    out = {}
    for k in ("pre", "post", "weight", "scale", "delay", "label"):
        out[k] = d["sorted_" + k][rs]
    return out


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(ref_dump: str, case: str) -> dict:
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, case + ".bin")
        subprocess.run([ref_dump, case, out], check=True, capture_output=True)
        return read_dump(out)


def checkpoint_digests(ref_dump: str, case: str) -> dict:
    with tempfile.TemporaryDirectory() as td:
        subprocess.run([ref_dump, "save", case, td], check=True, capture_output=True)
        out = {}
        for name in sorted(os.listdir(td)):
            with open(os.path.join(td, name), "rb") as f:
                data = f.read()
            out[name] = {"bytes": len(data), "sha256": hashlib.sha256(data).hexdigest()}
        return out


def main() -> int:
    sys.path.insert(0, ROOT)
    from spike_gb300 import _build
    ref_dump = _build.build_reference_frontend()
    if not ref_dump:
        print("reference sources not available; fixtures unchanged")
        return 1
    for case in ("va_mix", "brunel", "shapes"):
        d = run_case(ref_dump, case)
        c = creation_order(d)
        arrays = {**{"sorted_" + k: d["sorted_" + k] for k in ("pre", "post", "weight", "scale", "delay", "label")},
                  **{"created_" + k: v for k, v in c.items()},
                  **{k: v for k, v in d.items() if not k.startswith("sorted_")}}
        np.savez_compressed(os.path.join(HERE, f"ref_{case}.npz"), **arrays)
        print(case, int(d["n_synapses"][0]), "synapses")
    def digests(case):
        d = run_case(ref_dump, case)
        c = creation_order(d)
        meta = {k: int(d[k][0]) for k in ("n_synapses", "n_neurons", "n_inputs", "min_delay", "max_delay",
                                          "num_syn_labels", "timestep_grouping")}
        meta["digests_created"] = {k: digest(v) for k, v in c.items()}
        meta["digests_sorted"] = {k: digest(d["sorted_" + k]) for k in ("pre", "post", "weight", "delay", "label")}
        meta["eff_count_digest"] = digest(d["eff_count"])
        meta["tau_m"] = float(d["tau_m"][0])
        meta["R"] = float(d["R"][0])
        for k in ("vhat", "tau_g"):  # conductance synapses only
            if k in d:
                meta[k] = [float(x) for x in d[k]]
        print(case, meta["n_synapses"], "synapses, grouping", meta["timestep_grouping"])
        return meta

    with open(os.path.join(HERE, "ref_va.json"), "w") as f:
        json.dump(digests("va"), f, indent=1, sort_keys=True)
    with open(os.path.join(HERE, "ref_va_grouped.json"), "w") as f:
        json.dump({case: digests(case) for case in ("va_g2", "va_g3")}, f, indent=1, sort_keys=True)
    with open(os.path.join(HERE, "ref_det.json"), "w") as f:
        json.dump({case: digests(case) for case in ("vdet", "cdet")}, f, indent=1, sort_keys=True)
    ck = {case: checkpoint_digests(ref_dump, case) for case in ("va", "va_mix", "brunel", "shapes")}
    with open(os.path.join(HERE, "ref_checkpoint.json"), "w") as f:
        json.dump(ck, f, indent=1, sort_keys=True)
    print("checkpoint files", {k: len(v) for k, v in ck.items()})
    # seeded random networks (oracle/ref_cases.inc, case rand<seed>): the file
    # names and one SHA-256 over every file's name and bytes
    rnd = {}
    for seed in RANDOM_SEEDS:
        files = checkpoint_digests(ref_dump, f"rand{seed}")
        d = run_case(ref_dump, f"rand{seed}")
        rnd[str(seed)] = {"files": sorted(files), "sha256": combined_digest(ref_dump, f"rand{seed}"),
                          "arrays_sha256": arrays_digest(creation_order(d), d)}
    with open(os.path.join(HERE, "ref_checkpoint_random.json"), "w") as f:
        json.dump(rnd, f, indent=1, sort_keys=True)
    print("random checkpoint cases", len(rnd))
    return 0


RANDOM_SEEDS = range(1, 31)


def files_digest(dirname: str) -> str:
    """SHA-256 over every file of a directory, by name: name, size, bytes."""
    h = hashlib.sha256()
    for name in sorted(os.listdir(dirname)):
        with open(os.path.join(dirname, name), "rb") as f:
            data = f.read()
        h.update(name.encode() + b"\0" + str(len(data)).encode() + b"\0" + data)
    return h.hexdigest()


def arrays_digest(created: dict, d: dict) -> str:
    """SHA-256 over a network's synapse arrays in creation order (pre, post,
    weight, scale, delay, label), its label count and delay bounds, and the
    labels' constants (reversal potentials and conductance or current decay
    times) when the synapses have them."""
    h = hashlib.sha256()
    for k in ("pre", "post", "weight", "scale", "delay", "label"):
        h.update(k.encode() + np.ascontiguousarray(created[k]).tobytes())
    for k in ("num_syn_labels", "min_delay", "max_delay", "vhat", "tau_g", "tau_syn"):
        if k in d:
            h.update(k.encode() + np.ascontiguousarray(d[k]).tobytes())
    return h.hexdigest()


def combined_digest(ref_dump: str, case: str) -> str:
    with tempfile.TemporaryDirectory() as td:
        subprocess.run([ref_dump, "save", case, td], check=True, capture_output=True)
        return files_digest(td)


if __name__ == "__main__":
    sys.exit(main())
