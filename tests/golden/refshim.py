"""Import shim for the reference's Python package (deepmd.pt) in the build
container only.  Used by make_golden.py to run the reference model and dump
fixtures; never imported by tests on the GPU machine or by the product.

The reference imports a few pip packages that are absent here (pyyaml, h5py,
lmdb, wcmatch, e3nn, array_api_compat) and a generated ``deepmd.lib`` package.
Inert stand-ins are installed for them before ``deepmd`` is imported.
"""
import os
import sys
import tempfile
import types

import torch  # noqa: F401  (must come before deepmd)
import numpy as np

REF = os.environ.get("DPGB_REFERENCE", "")  # the reference checkout (required)
if not os.path.isdir(os.path.join(REF, "deepmd")):
    raise ImportError("refshim: set DPGB_REFERENCE to the deepmd-kit reference checkout")


class _Stub(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Stub(f"{self.__name__}.{name}")

    def __call__(self, *a, **k):
        return None


def _stub(name):
    mod = _Stub(name)
    sys.modules[name] = mod
    return mod


def _array_api_compat():
    m = types.ModuleType("array_api_compat")

    def array_namespace(*xs):
        for x in xs:
            if isinstance(x, torch.Tensor):
                return torch
        return np

    m.array_namespace = array_namespace
    m.device = lambda x: getattr(x, "device", "cpu")
    m.is_numpy_array = lambda x: isinstance(x, np.ndarray)
    m.is_array_api_obj = lambda x: isinstance(x, (np.ndarray, np.generic, torch.Tensor))
    m.is_torch_array = lambda x: isinstance(x, torch.Tensor)
    m.is_jax_array = lambda x: False
    m.is_array_api_strict_namespace = lambda x: False
    m.is_jax_namespace = lambda x: False
    m.size = lambda x: int(np.prod(x.shape))
    m.to_device = lambda x, d, **k: x
    sys.modules["array_api_compat"] = m


def install():
    if "deepmd" in sys.modules:
        return
    for name in ("yaml", "h5py", "lmdb", "e3nn", "e3nn.o3", "wcmatch",
                 "wcmatch.glob", "dargs", "dargs.json_schema"):
        if name not in sys.modules:
            _stub(name)
    sys.modules["wcmatch.glob"].globfilter = lambda *a, **k: []
    _array_api_compat()
    if REF not in sys.path:
        sys.path.insert(0, REF)
    import deepmd  # noqa: E402

    libdir = tempfile.mkdtemp(prefix="dpgb_reflib_")
    with open(os.path.join(REF, "source/config/run_config.ini")) as f:
        txt = f.read()
    import re

    txt = re.sub(r"@[A-Za-z_]+@", "", txt).replace("ENABLE_PYTORCH = ", "ENABLE_PYTORCH = 1")
    txt = txt.replace("PT_VERSIOn = ", "PT_VERSIOn = " + torch.__version__.split("+")[0])
    txt = txt.replace("PT_CXX11_ABI_FLAG = ", "PT_CXX11_ABI_FLAG = 1")
    with open(os.path.join(libdir, "run_config.ini"), "w") as f:
        f.write(txt)
    op = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))),
                      "oracle", "_ref", "libdeepmd_op_pt.so")
    if os.path.exists(op):
        os.symlink(op, os.path.join(libdir, "libdeepmd_op_pt.so"))
    lib = types.ModuleType("deepmd.lib")
    lib.__path__ = [libdir]
    lib.__file__ = os.path.join(libdir, "__init__.py")
    sys.modules["deepmd.lib"] = lib
    deepmd.lib = lib
