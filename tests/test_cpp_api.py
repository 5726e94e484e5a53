"""The C++ model API used from C++ (tests/cpp/plastic_model.cpp): a program
written the way a Spike user writes one builds against include/ and links
libspike_gb300.so.  CPU: the models flatten into descriptors carrying the
plasticity rules (weight-dependent STDP with the weight normalisation after
it; the Evans rule).  GPU: the same program runs both models."""
import os
import re
import shutil
import subprocess

import pytest

from spike_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    lib_dir = os.path.dirname(N.LIB_PATH)
    out = str(tmp_path_factory.mktemp("cpp") / "plastic_model")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "plastic_model.cpp"), "-L" + lib_dir, "-lspike_gb300",
                    "-Wl,-rpath," + lib_dir, "-o", out], check=True, capture_output=True, text=True)
    return out


def test_cpp_models_flatten_with_their_rules(program):
    res = subprocess.run([program, "desc"], check=True, capture_output=True, text=True, timeout=120)
    rows = [dict(re.findall(r"(\w+) (-?\d+)", line)) for line in res.stdout.strip().splitlines()]
    assert len(rows) == 2
    wd, ev = rows
    assert wd["rc"] == "0" and wd["has_stdp"] == "1"
    assert int(wd["stdp_rule"]) == N.SPK_STDP_WEIGHT_DEPENDENT and int(wd["weight_norm"]) == N.SPK_NORM_AFTER_RULE
    assert ev["rc"] == "0" and int(ev["stdp_rule"]) == N.SPK_STDP_EVANS and int(ev["weight_norm"]) == N.SPK_NORM_OFF
    assert int(wd["plastic"]) > 1000 and int(ev["plastic"]) > 1000


@pytest.mark.gpu
def test_cpp_models_run(program):
    res = subprocess.run([program, "run"], check=True, capture_output=True, text=True, timeout=300)
    rows = [dict(re.findall(r"(\w+) (-?\d+)", line)) for line in res.stdout.strip().splitlines()]
    assert len(rows) == 2
    for r in rows:
        assert r["status"] == "0" and int(r["spikes"]) > 0, res.stdout
