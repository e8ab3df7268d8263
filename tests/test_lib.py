"""CPU: the C-ABI library builds for sm_103a, loads, and exports every
function include/dpgb.h declares (no compute calls without a GPU)."""
import ctypes
import os
import re
import subprocess

from conftest import REPO


def _declared():
    with open(os.path.join(REPO, "include", "dpgb.h")) as f:
        txt = f.read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dpgb_\w+)\s*\(", txt)))


def test_library_exports_header():
    from dpgb import _lib, build

    path = build.build()
    assert os.path.exists(path)
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (dpgb_\w+)", out))
    declared = _declared()
    assert declared, "no declarations parsed"
    missing = [d for d in declared if d not in exported]
    assert not missing, f"declared but not exported: {missing}"
    # the ctypes binding covers the whole header
    assert set(declared) <= set(_lib.EXPORTED)
    h = ctypes.CDLL(path)
    for d in declared:
        getattr(h, d)


def test_build_flags():
    from dpgb import build

    assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
