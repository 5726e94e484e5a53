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
