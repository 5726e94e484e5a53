"""The C ABI library loads and exports every function include/*.h declares
(CPU: no compute calls)."""
import ctypes
import os
import re

from spike_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("spike_gb300.h", "spike_gb300_model.h"):
        with open(os.path.join(ROOT, "include", h)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(spk_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declarations_are_exported_and_bound():
    lib = ctypes.CDLL(_native.LIB_PATH)
    decl = declared_functions()
    assert len(decl) > 40
    for name in decl:
        assert hasattr(lib, name), f"{name} declared but not exported"
    assert set(decl) == set(_native.exported_symbols())


def test_abi_version_and_error_without_gpu_work():
    lib = _native.lib()
    assert lib.spk_abi_version() == _native.SPK_ABI_VERSION
    # argument validation fails before any device call
    assert lib.spk_net_create(None, None, None) == _native.SPK_ERR_INVALID
    assert lib.spk_net_run(None, ctypes.c_float(1.0), 1) == _native.SPK_ERR_INVALID
    assert isinstance(lib.spk_last_error(), bytes)
