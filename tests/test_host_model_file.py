"""CPU: the frozen-model reader (dpgb_model_file_*) on .pth files written
the way the reference freezes models (tests/golden/deeppot_sea.pth, made by
tests/golden/make_golden.py make_pth through the reference's own get_model
and torch.jit.save): every weight equals torch.jit.load's state dict bit for
bit, the architecture comes out as the reference model's, and files that
are not se_e2_a energy models are refused with a message."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN, deeppot_sea_params

FIXTURE = os.path.join(GOLDEN, "deeppot_sea.pth")


@pytest.fixture(scope="module")
def lib():
    from dpgb import _lib

    return _lib.lib()


def _open(lib, path=None, content=None):
    if content is not None:
        return lib.dpgb_model_file_open(None, content, len(content))
    return lib.dpgb_model_file_open(path.encode(), None, 0)


def _tensor(lib, mf, name):
    n = lib.dpgb_model_file_tensor(mf, name.encode(), None, 0, None, None)
    assert n >= 0, name
    out = np.zeros(n)
    shape = (C.c_longlong * 8)()
    nd = C.c_int(8)
    lib.dpgb_model_file_tensor(mf, name.encode(), out.ctypes.data_as(C.POINTER(C.c_double)), n, shape, C.byref(nd))
    return out.reshape([shape[i] for i in range(nd.value)])


def test_weights_equal_torch_jit_load(lib):
    torch = pytest.importorskip("torch")
    from dpgb import ops

    ops.register()  # the scripted model calls torch.ops.deepmd.tabulate_fusion_se_a
    sd = torch.jit.load(FIXTURE, map_location="cpu").state_dict()
    mf = _open(lib, FIXTURE)
    assert mf, lib.dpgb_last_error()
    try:
        for k, v in sd.items():
            np.testing.assert_array_equal(_tensor(lib, mf, k), v.double().numpy(), err_msg=k)
    finally:
        lib.dpgb_model_file_close(mf)


def test_architecture_and_type_map(lib):
    from dpgb import _lib

    p = deeppot_sea_params()
    with open(FIXTURE, "rb") as f:
        content = f.read()
    mf = _open(lib, content=content)  # from the file's content, as file_content passes it
    assert mf, lib.dpgb_last_error()
    try:
        d = C.cast(lib.dpgb_model_file_desc(mf), C.POINTER(_lib.SeADesc)).contents
        c = p.config
        assert d.ntypes == 2 and list(d.sel[:2]) == c.sel
        assert d.rcut == c.rcut and d.rcut_smth == c.rcut_smth
        assert d.type_one_side == 1 and d.n_emb == 3 and list(d.emb_neuron[:3]) == c.neuron
        assert d.axis_neuron == c.axis_neuron and d.dim_descrpt == c.dim_descrpt
        assert d.n_fit == 3 and list(d.fit_neuron[:3]) == c.fit_neuron
        assert d.compressed == 0
        assert lib.dpgb_model_file_type_map(mf).decode() == "O H"
        # the energy bias the handle gets: bias_atom_e + out_bias
        bias = np.ctypeslib.as_array(d.atom_ener_bias, shape=(2,))
        np.testing.assert_array_equal(bias, p.atom_ener_bias())
        np.testing.assert_array_equal(np.ctypeslib.as_array(d.davg, shape=(2 * 138 * 4,)), p.mean.reshape(-1))
        np.testing.assert_array_equal(np.ctypeslib.as_array(d.fit_w[1][2], shape=(100,)),
                                      p.fit[1][2][0].reshape(-1))
    finally:
        lib.dpgb_model_file_close(mf)


def test_refuses_what_it_cannot_read(lib, tmp_path):
    bad = tmp_path / "not_a_model.pth"
    bad.write_bytes(b"this is not a zip archive" * 4)
    assert not _open(lib, str(bad))
    assert "zip" in lib.dpgb_last_error().decode()
    with open(FIXTURE, "rb") as f:
        content = f.read()
    assert not _open(lib, content=content[: len(content) // 2])  # truncated
    assert lib.dpgb_last_error().decode()
    ref = os.environ.get("DPGB_REFERENCE", "")
    fparam = os.path.join(ref, "source", "tests", "infer", "fparam_aparam_default.pth")
    if ref and os.path.exists(fparam):
        assert not _open(lib, fparam)
        assert "frame / atomic parameters" in lib.dpgb_last_error().decode()
