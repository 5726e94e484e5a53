"""Weight and connectivity files against the reference's own (CPU).

The reference saves a network's connectivity and weights with
Synapses::save_connectivity_as_{binary,txt} / save_weights_as_{binary,txt}
(Spike/Synapses/Synapses.cpp:423-562; SpikingSynapses.cpp:136-189 adds the
delays) and loads weights with load_weights_from_{txt,binary}
(Synapses.cpp:565-614).  tests/golden/ref_checkpoint.json holds the size and
SHA-256 of every file the reference front end wrote for four networks
(tests/golden/make_golden.py).  Here the same networks are built from the same
C++ source (oracle/ref_cases.inc) through this library's model API and saved
with the same calls (tests/cpp/checkpoint_model.cpp); every file must be the
reference's byte for byte, including the text formatting, the group-relative
ids of a single synapse group, and the weights read back from the text file.
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys

import pytest

from spike_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "ref_checkpoint.json")


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    lib_dir = os.path.dirname(N.LIB_PATH)
    out = str(tmp_path_factory.mktemp("cpp") / "checkpoint_model")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "checkpoint_model.cpp"), "-L" + lib_dir, "-lspike_gb300",
                    "-Wl,-rpath," + lib_dir, "-o", out], check=True, capture_output=True, text=True)
    return out


def _files(dirname):
    out = {}
    for name in sorted(os.listdir(dirname)):
        with open(os.path.join(dirname, name), "rb") as f:
            data = f.read()
        out[name] = (len(data), hashlib.sha256(data).hexdigest(), data)
    return out


@pytest.mark.parametrize("case", ["va", "va_mix", "brunel", "shapes"])
def test_saved_files_match_the_reference(program, tmp_path, case):
    with open(GOLD) as f:
        gold = json.load(f)[case]
    subprocess.run([program, case, str(tmp_path)], check=True, capture_output=True, text=True, timeout=300)
    ours = _files(tmp_path)
    rebin = ours.pop("rebin_SynapticWeights.bin")
    assert sorted(ours) == sorted(gold)
    for name, g in gold.items():
        n, digest, _ = ours[name]
        assert (n, digest) == (g["bytes"], g["sha256"]), f"{case}: {name} differs from the reference's file"
    # the binary weights read back and written again are the same bytes
    assert rebin[2] == ours["w_SynapticWeights.bin"][2]


sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_golden  # noqa: E402  (the fixtures' record reader and digests)

RANDOM_GOLD = os.path.join(ROOT, "tests", "golden", "ref_checkpoint_random.json")
REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")


def _files_digest(dirname):
    """SHA-256 over every file of a directory, by name: name, size, bytes
    (the digest tests/golden/make_golden.py records)."""
    h = hashlib.sha256()
    for name in sorted(os.listdir(dirname)):
        with open(os.path.join(dirname, name), "rb") as f:
            data = f.read()
        h.update(name.encode() + b"\0" + str(len(data)).encode() + b"\0" + data)
    return h.hexdigest()


with open(RANDOM_GOLD) as _f:
    _RANDOM = json.load(_f)


@pytest.mark.parametrize("seed", sorted(_RANDOM, key=int))
def test_random_models_save_the_reference_files(program, tmp_path, seed):
    """Seeded random networks (oracle/ref_cases.inc, case rand<seed>: every
    connectivity type, shapes, weight ranges, scales, fractional delay ranges
    and pairwise weights and delays, over voltage, current and conductance
    synapses) saved through this library's front end: every file equals the
    one the reference front end wrote for the same source."""
    subprocess.run([program, f"rand{seed}", str(tmp_path)], check=True, capture_output=True, text=True, timeout=300)
    os.remove(os.path.join(tmp_path, "rebin_SynapticWeights.bin"))
    assert sorted(os.listdir(tmp_path)) == _RANDOM[seed]["files"]
    assert _files_digest(tmp_path) == _RANDOM[seed]["sha256"], f"rand{seed}: files differ from the reference's"
    # the synapse arrays in creation order (labels and scales included) and the label constants
    out = str(tmp_path / "arrays.bin")
    subprocess.run([program, "dump", f"rand{seed}", out], check=True, capture_output=True, timeout=300)
    d = make_golden.read_dump(out)
    created = {k: d["created_" + k] for k in ("pre", "post", "weight", "scale", "delay", "label")}
    assert make_golden.arrays_digest(created, d) == _RANDOM[seed]["arrays_sha256"], f"rand{seed}: arrays differ"


@pytest.mark.parametrize("seed", range(100, 140))
def test_random_models_against_the_reference_front_end(program, tmp_path, seed):
    """More seeds, against the reference front end itself where its build
    (oracle/build_ref.sh) exists: both front ends save the same network and
    every file must be the same bytes."""
    from spike_gb300 import _build
    ref_dump = _build.build_reference_frontend() if os.path.exists(REF_DUMP) else None
    if not ref_dump:
        pytest.skip("the reference front end is not built here")
    ours, theirs = tmp_path / "ours", tmp_path / "ref"
    ours.mkdir()
    theirs.mkdir()
    subprocess.run([ref_dump, "save", f"rand{seed}", str(theirs)], check=True, capture_output=True, timeout=300)
    subprocess.run([program, f"rand{seed}", str(ours)], check=True, capture_output=True, timeout=300)
    for name in sorted(os.listdir(theirs)):
        with open(theirs / name, "rb") as a, open(ours / name, "rb") as b:
            assert a.read() == b.read(), f"rand{seed}: {name} differs from the reference's file"
    subprocess.run([ref_dump, f"rand{seed}", str(tmp_path / "ref.bin")], check=True, capture_output=True, timeout=300)
    subprocess.run([program, "dump", f"rand{seed}", str(tmp_path / "ours.bin")], check=True, capture_output=True,
                   timeout=300)
    r, o = make_golden.read_dump(str(tmp_path / "ref.bin")), make_golden.read_dump(str(tmp_path / "ours.bin"))
    c = make_golden.creation_order(r)
    for k in ("pre", "post", "weight", "scale", "delay", "label"):
        assert c[k].tobytes() == o["created_" + k].tobytes(), f"rand{seed}: {k}"
    for k in ("num_syn_labels", "min_delay", "max_delay", "vhat", "tau_g", "tau_syn"):
        assert (k in r) == (k in o) and (k not in r or r[k].tobytes() == o[k].tobytes()), f"rand{seed}: {k}"
