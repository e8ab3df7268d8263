"""GPU: dpgb_prod_force_a_f64_noalloc, the force product for callers that
cannot allocate device memory during the call (a host engine that owns the
device memory through its own pool, or an inner loop where cudaMalloc's
device-wide synchronisation is not acceptable).  It keeps its scratch in one
fixed device array of the library, so its result must equal the allocating
dpgb_prod_force_a_f64 on every call, including back-to-back calls that reuse
the array with different inputs, and many calls in a row must leave the
device's free memory unchanged.  Collected last so that a failure here
cannot hide the other tests' results; the last test runs the first one again
alone, in a fresh process.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _forces(name, nd, ed, nl, nloc, nall, nnei, nframes):
    import torch
    from dpgb import _lib

    f = torch.full((nframes, nall, 3), float("nan"), dtype=torch.float64, device=nd.device)
    _lib.call(name, _vp(f), _vp(nd), _vp(ed), _vp(nl), nloc, nall, nnei, nframes, _stream())
    return f


def _random_case(cuda, seed, nloc, nall, nnei, nframes):
    import torch

    rng = np.random.default_rng(seed)
    nl = rng.integers(-1, nall, size=(nframes * nloc, nnei)).astype(np.int32)
    nl[:, nnei // 2:] = -1  # trailing padding as in a formatted list
    nd = rng.normal(size=(nframes * nloc, 4 * nnei))
    ed = rng.normal(size=(nframes * nloc, 4 * nnei, 3))
    t = lambda a, dt=None: torch.tensor(a, device=cuda, dtype=dt)
    return t(nd), t(ed), t(nl, torch.int32)


def test_matches_allocating_entry_point_on_consecutive_calls(cuda):
    import torch

    g = golden("prod_force_a")
    nloc, nall = len(g["atype"]), g["coord_ext"].shape[0]
    nnei = g["nlist"].shape[1]
    nd = torch.tensor(g["net_deriv"], device=cuda)
    ed = torch.tensor(g["em_deriv"], device=cuda)
    nl = torch.tensor(g["nlist"], device=cuda, dtype=torch.int32)
    cases = [(nd, ed, nl, nloc, nall, nnei, 1)]
    nd2, ed2, nl2 = _random_case(cuda, 7, 300, 2000, 40, 2)
    cases.append((nd2, ed2, nl2, 300, 2000, 40, 2))
    for case in cases + cases[::-1]:  # two calls in a row with different inputs, then again
        ref = _forces("dpgb_prod_force_a_f64", *case)
        got = _forces("dpgb_prod_force_a_f64_noalloc", *case)
        torch.testing.assert_close(got, ref, rtol=1e-12, atol=1e-12)
    # the golden values of source/lib/tests/test_prod_force_a.cc
    got = _forces("dpgb_prod_force_a_f64_noalloc", *cases[0])
    np.testing.assert_allclose(got.cpu().numpy().reshape(-1), g["expected_force"], atol=1e-5)


def test_rejects_sizes_beyond_the_fixed_scratch(cuda):
    import torch
    from dpgb import _lib

    nloc, nall, nnei = 3000, 3000, 100  # 300,000 pairs > 262,144
    nd = torch.zeros(nloc, 4 * nnei, dtype=torch.float64, device=cuda)
    ed = torch.zeros(nloc, 4 * nnei, 3, dtype=torch.float64, device=cuda)
    nl = torch.full((nloc, nnei), -1, dtype=torch.int32, device=cuda)
    f = torch.zeros(1, nall, 3, dtype=torch.float64, device=cuda)
    with pytest.raises(_lib.DpgbError, match="must not exceed 262144"):
        _lib.call("dpgb_prod_force_a_f64_noalloc", _vp(f), _vp(nd), _vp(ed), _vp(nl), nloc, nall, nnei, 1, _stream())


def test_no_device_allocation_over_many_calls(cuda):
    """After one warm-up call, back-to-back calls change neither the device's
    free memory (cudaMemGetInfo) nor torch's reserved pool."""
    import torch

    nd, ed, nl = _random_case(cuda, 11, 200, 900, 30, 3)
    f = torch.zeros(3, 900, 3, dtype=torch.float64, device=cuda)
    from dpgb import _lib

    args = (_vp(f), _vp(nd), _vp(ed), _vp(nl), 200, 900, 30, 3, _stream())
    _lib.call("dpgb_prod_force_a_f64_noalloc", *args)
    torch.cuda.synchronize()
    free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
    for _ in range(50):
        _lib.call("dpgb_prod_force_a_f64_noalloc", *args)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_reserved() == reserved0


def test_runs_alone_in_a_fresh_process(cuda):
    here = os.path.dirname(os.path.abspath(__file__))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-m", "gpu", "-p", "no:cacheprovider",
                        os.path.join(here, "test_zz_no_alloc.py") + "::test_matches_allocating_entry_point_on_consecutive_calls"],
                       capture_output=True, text=True, timeout=600, cwd=os.path.dirname(here))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "1 passed" in r.stdout
