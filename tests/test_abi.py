"""The C-ABI library loads and exports every entry point include/cac.h declares (no GPU calls)."""
import os
import re
import subprocess

from conftest import ROOT


def _declared():
    with open(os.path.join(ROOT, "include", "cac.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cac_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(libcac):
    declared = _declared()
    assert len(declared) >= 19
    out = subprocess.run(["nm", "-D", "--defined-only", libcac.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (cac_[a-z0-9_]+)", out))
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    lib = libcac.lib()
    for s in declared:
        assert getattr(lib, s) is not None


def test_python_mirror_binds_every_symbol(libcac):
    bound = {name for name, _, _ in libcac.EXPORTS}
    assert set(_declared()) == bound


def test_error_strings_without_gpu(libcac):
    lib = libcac.lib()
    assert lib.cac_error_string(0) == b"ok"
    assert lib.cac_error_string(-3) == b"malformed edge-list input"
    assert lib.cac_error_string(-99) == b"unknown status"
