"""GPU: environment matrix and force / virial products against the reference
unit-test goldens (source/lib/tests/test_env_mat_a.cc, test_prod_force_a.cc,
test_prod_virial_a.cc), the oracle, and the reference's own library outputs
stored in the fixtures (1e-10)."""
import numpy as np
import pytest

from conftest import golden

import oracle as O

pytestmark = pytest.mark.gpu


def _t(a, cuda, dtype=None):
    import torch

    return torch.tensor(np.ascontiguousarray(a), device=cuda, dtype=dtype)


def _vp(t):
    import ctypes

    return ctypes.c_void_p(t.data_ptr())


def _stream():
    import ctypes
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_prod_env_mat_a_golden(cuda):
    import ctypes
    import torch
    from dpgb import _lib

    g = golden("env_mat_a")
    nloc, nall = len(g["atype"]), g["coord_ext"].shape[0]
    sel = np.array([10, 10], np.int32)
    nnei = 20
    em = torch.empty(nloc, nnei, 4, dtype=torch.float64, device=cuda)
    der = torch.empty(nloc, nnei, 4, 3, dtype=torch.float64, device=cuda)
    rij = torch.empty(nloc, nnei, 3, dtype=torch.float64, device=cuda)
    nl = torch.empty(nloc, nnei, dtype=torch.int32, device=cuda)
    avg = torch.zeros(2, nnei, 4, dtype=torch.float64, device=cuda)
    std = torch.ones(2, nnei, 4, dtype=torch.float64, device=cuda)
    # every device buffer is bound to a name for the duration of the call
    rows = _t(g["rows"], cuda, torch.int32)
    cext = _t(g["coord_ext"], cuda)
    text = _t(g["atype_ext"], cuda, torch.int32)
    counts = _t(g["counts"], cuda, torch.int32)
    _lib.call("dpgb_prod_env_mat_a_f64", _vp(em), _vp(der), _vp(rij), _vp(nl), _vp(cext),
              _vp(text), _vp(rows), _vp(counts),
              rows.shape[1], _vp(avg), _vp(std), nloc, nall, ctypes.c_double(float(g["rc"])),
              ctypes.c_double(float(g["rc_smth"])), sel.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), 2, _stream())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(nl.cpu().numpy(), g["nlist"])
    np.testing.assert_allclose(em.cpu().numpy().reshape(-1), g["expected_env"], atol=1e-5)
    np.testing.assert_allclose(em.cpu().numpy(), g["em"], atol=1e-10, rtol=1e-10)
    np.testing.assert_allclose(der.cpu().numpy(), g["em_deriv"], atol=1e-10, rtol=1e-10)
    np.testing.assert_allclose(rij.cpu().numpy(), g["rij"], atol=1e-12)


def _prod_force(cuda, nd, ed, nl, nloc, nall, nnei, nframes=1):
    import torch
    from dpgb import _lib

    f = torch.empty(nframes, nall, 3, dtype=torch.float64, device=cuda)
    _lib.call("dpgb_prod_force_a_f64", _vp(f), _vp(nd), _vp(ed), _vp(nl), nloc, nall, nnei, nframes, _stream())
    return f


def test_prod_force_virial_golden(cuda):
    import torch
    from dpgb import _lib

    g = golden("prod_force_a")
    nloc, nall = len(g["atype"]), g["coord_ext"].shape[0]
    nnei = g["nlist"].shape[1]
    nd = _t(g["net_deriv"], cuda)
    ed = _t(g["em_deriv"], cuda)
    nl = _t(g["nlist"], cuda, torch.int32)
    f = _prod_force(cuda, nd, ed, nl, nloc, nall, nnei)
    np.testing.assert_allclose(f.cpu().numpy().reshape(-1), g["expected_force"], atol=1e-5)
    ref = O.prod_force_a(g["net_deriv"].reshape(nloc, -1), g["em_deriv"], g["nlist"], nall)
    np.testing.assert_allclose(f.cpu().numpy()[0], ref, atol=1e-12, rtol=1e-12)
    # two frames stacked: frame-major indices, same answer per frame
    f2 = _prod_force(cuda, torch.cat([nd, nd]), torch.cat([ed, ed]), torch.cat([nl, nl]), nloc, nall, nnei, 2)
    np.testing.assert_array_equal(f2.cpu().numpy()[1], f.cpu().numpy()[0])

    g = golden("prod_virial_a")
    v = torch.empty(9, dtype=torch.float64, device=cuda)
    av = torch.empty(nall, 9, dtype=torch.float64, device=cuda)
    vnd, ved, vrij = _t(g["net_deriv"], cuda), _t(g["em_deriv"], cuda), _t(g["rij"], cuda)
    vnl = _t(g["nlist"], cuda, torch.int32)
    _lib.call("dpgb_prod_virial_a_f64", _vp(v), _vp(av), _vp(vnd), _vp(ved), _vp(vrij), _vp(vnl), nloc, nall, nnei,
              _stream())
    np.testing.assert_allclose(v.cpu().numpy(), g["expected_virial"], atol=1e-5)
    np.testing.assert_allclose(av.cpu().numpy().reshape(-1), g["expected_atom_virial"], atol=1e-5)


def test_prod_force_deterministic_and_grads(cuda):
    import torch
    from dpgb import _lib

    g = golden("prod_force_a")
    nloc, nall = len(g["atype"]), g["coord_ext"].shape[0]
    nnei = g["nlist"].shape[1]
    nd, ed, nl = _t(g["net_deriv"], cuda), _t(g["em_deriv"], cuda), _t(g["nlist"], cuda, torch.int32)
    a = _prod_force(cuda, nd, ed, nl, nloc, nall, nnei)
    b = _prod_force(cuda, nd, ed, nl, nloc, nall, nnei)
    assert torch.equal(a, b)
    rng = np.random.default_rng(2)
    grad = rng.normal(size=(nloc, 3))
    out = torch.empty(nloc, 4 * nnei, dtype=torch.float64, device=cuda)
    grad_d = _t(grad, cuda)
    _lib.call("dpgb_prod_force_grad_a_f64", _vp(out), _vp(grad_d), _vp(ed), _vp(nl), nloc, nnei, 1, _stream())
    np.testing.assert_allclose(out.cpu().numpy(), O.prod_force_grad_a(grad, g["em_deriv"], g["nlist"]), atol=1e-12)
    gv = rng.normal(size=9)
    out2 = torch.empty(nloc, 4 * nnei, dtype=torch.float64, device=cuda)
    gv_d, rij_d = _t(gv, cuda), _t(g["rij"], cuda)
    _lib.call("dpgb_prod_virial_grad_a_f64", _vp(out2), _vp(gv_d), _vp(ed), _vp(rij_d), _vp(nl),
              nloc, nnei, _stream())
    np.testing.assert_allclose(out2.cpu().numpy(), O.prod_virial_grad_a(gv, g["em_deriv"], g["rij"], g["nlist"]),
                               atol=1e-12)


def test_env_mat_pt_matches_reference_model(cuda):
    """PyTorch env-mat semantics on the water box vs the reference model's
    prod_env_mat output of the first atoms (fixture)."""
    import torch
    from dpgb import _lib

    g = golden("water192")
    nall = g["coord_ext"].shape[0]
    nnei = 138
    em = torch.empty(192, nnei, 4, dtype=torch.float64, device=cuda)
    diff = torch.empty(192, nnei, 3, dtype=torch.float64, device=cuda)
    sw = torch.empty(192, nnei, dtype=torch.float64, device=cuda)
    avg = torch.zeros(2, nnei, 4, dtype=torch.float64, device=cuda)
    std = torch.ones(2, nnei, 4, dtype=torch.float64, device=cuda)
    at = np.tile(g["atype"], nall // 192).astype(np.int32)
    import ctypes

    cext, at_d, nl_d = _t(g["coord_ext"], cuda), _t(at, cuda, torch.int32), _t(g["nlist"], cuda, torch.int32)
    _lib.call("dpgb_env_mat_pt_f64", _vp(em), _vp(diff), _vp(sw), _vp(cext), _vp(at_d), _vp(nl_d), _vp(avg), _vp(std), 1, 192,
              nall, nnei, ctypes.c_double(6.0), ctypes.c_double(0.5), _stream())
    np.testing.assert_allclose(em.cpu().numpy()[:8], g["env_mat"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(sw.cpu().numpy()[:8], g["sw"], rtol=1e-12, atol=1e-14)
