"""CPU: the plugin's C++ interface matches the reference's.

include/deepmd_backend_abi.h declares deepmd::DeepPotBackend and
deepmd::InputNlist for the GB300 backend plugin.  A host built from the
reference calls the plugin through its own declarations, so tests/plugin/
abi_probe.cc -- the vtable slot of every virtual method and the field
offsets of InputNlist -- must print the same against both headers (the
reference's are read from DPGB_REFERENCE when it names a checkout; the
comparison is skipped otherwise).  Without a GPU the plugin's creation fails
cleanly: NULL and the message through the C symbols, from a host compiled
against the header."""
import os
import subprocess

import pytest

from conftest import GOLDEN, REPO

HERE = os.path.dirname(os.path.abspath(__file__))
PROBE = os.path.join(HERE, "plugin", "abi_probe.cc")


def _probe(tmp_path, flags, name):
    exe = str(tmp_path / name)
    subprocess.run(["g++", "-std=c++17", *flags, PROBE, "-o", exe], check=True, capture_output=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout


def test_vtable_and_nlist_layout_match_the_reference(tmp_path):
    ref = os.environ.get("DPGB_REFERENCE", "")
    api = os.path.join(ref, "source", "api_cc", "include")
    built = os.path.join(REPO, "oracle", "_ref", "abi_probe_reference.txt")  # oracle/build_ref.sh
    if ref and os.path.isdir(api):
        # the reference's common.h includes a header its build generates
        (tmp_path / "version.h").write_text("#pragma once\n")
        theirs = _probe(tmp_path, ["-DPROBE_REFERENCE", "-I", str(tmp_path), "-I", api, "-I",
                                   os.path.join(ref, "source", "lib", "include")], "theirs")
    elif os.path.exists(built):
        with open(built) as f:
            theirs = f.read()
    else:
        pytest.skip("no reference checkout (DPGB_REFERENCE) and no probe output of oracle/build_ref.sh")
    ours = _probe(tmp_path, ["-I", os.path.join(REPO, "include")], "ours")
    assert ours == theirs
    assert "computew nlist double                    13" in ours


def test_plugin_exports_and_fails_cleanly_without_gpu(tmp_path):
    torch = pytest.importorskip("torch")
    from dpgb import _lib, build

    _lib.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", build.PLUGIN], capture_output=True, text=True).stdout
    for sym in ("deepmd_create_deeppot_backend_v1", "deepmd_delete_deeppot_backend_v1",
                "deepmd_free_backend_error_v1"):
        assert f" T {sym}" in out
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: tests/test_gpu_plugin.py covers the plugin")
    import plugin_host as H

    exe = H.build_host(str(tmp_path))
    rc, text, _ = H.run(exe, build.PLUGIN, os.path.join(GOLDEN, "deeppot_sea.pth"), [])
    assert rc == 3 and "no CUDA device" in text
