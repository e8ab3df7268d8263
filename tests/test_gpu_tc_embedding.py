"""GPU: the tensor-core (tcgen05) embedding of the mixed-precision DeepPot
against the FP64 plain form and the FP32 SIMT form, plus run-to-run bitwise
reproducibility.  Tolerances: force RMSE <= 1e-3 eV/A (the benchmark bound)
and, relative to the RMS force, <= 2e-2; energy per atom <= 1e-4 relative."""
import os

import numpy as np
import pytest

from conftest import deeppot_sea_params, golden, water_params

pytestmark = pytest.mark.gpu


def _errors(a, b, natom):
    (ea, fa, va), (eb, fb, vb) = a, b
    rmse = float(np.sqrt(np.mean((fa - fb) ** 2)))
    rms = float(np.sqrt(np.mean(fb ** 2)))
    return dict(e=abs(ea[0] - eb[0]) / natom, e_rel=abs(ea[0] - eb[0]) / abs(eb[0]), f_rmse=rmse, f_rel=rmse / rms,
                v_rel=float(np.abs(va - vb).max() / np.abs(vb).max()))


def test_tc_mixed_vs_fp64_water(cuda):
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    coord, atype, box = synth.water_box(8, seed=4)
    p = water_params()
    ref = DeepPot(p, "fp64").eval(coord.reshape(1, -1), box, atype)
    mixed = DeepPot(p, "mixed")
    got = mixed.eval(coord.reshape(1, -1), box, atype)
    err = _errors(got, ref, atype.size)
    print("tc mixed vs fp64", err)
    assert err["f_rmse"] <= 1e-3
    assert err["f_rel"] <= 2e-2
    assert err["e_rel"] <= 1e-4
    assert err["v_rel"] <= 2e-2
    again = mixed.eval(coord.reshape(1, -1), box, atype)
    for x, y in zip(got, again):
        np.testing.assert_array_equal(x, y)


def test_tc_matches_simt_fp32(cuda, monkeypatch):
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    coord, atype, box = synth.water_box(6, seed=9)
    p = water_params()
    tc = DeepPot(p, "mixed").eval(coord.reshape(1, -1), box, atype)
    monkeypatch.setenv("DPGB_NO_TENSOR_CORES", "1")
    simt = DeepPot(p, "mixed").eval(coord.reshape(1, -1), box, atype)
    err = _errors(tc, simt, atype.size)
    print("tc vs simt fp32", err)
    assert err["f_rel"] <= 2e-2 and err["e_rel"] <= 1e-4


def test_tc_mixed_deeppot_testcase(cuda):
    from dpgb.deeppot import DeepPot

    c = golden("deeppot_sea_case")
    p = deeppot_sea_params()
    dp64, dp32 = DeepPot(p, "fp64"), DeepPot(p, "mixed")
    for b in range(int(c["nblock"])):
        box = c[f"b{b}_box"]
        box = None if box.size == 0 else box
        a = dp32.eval(c[f"b{b}_coord"], box, c[f"b{b}_atype"])
        r = dp64.eval(c[f"b{b}_coord"], box, c[f"b{b}_atype"])
        err = _errors(a, r, 6)
        print("deeppot_sea mixed", b, err)
        assert err["f_rmse"] <= 1e-3 and err["e_rel"] <= 1e-4


def test_tc_mixed_vs_fp64_resnet_dt(cuda):
    """Embedding layers with idt (resnet_dt): the tensor-core kernels'
    idt form against the FP64 form."""
    from dpgb import params as P
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    cfg = P.water_config()
    cfg.resnet_dt = True
    p = P.init_params(cfg, seed=3)
    coord, atype, box = synth.water_box(6, seed=5)
    ref = DeepPot(p, "fp64").eval(coord.reshape(1, -1), box, atype)
    got = DeepPot(p, "mixed").eval(coord.reshape(1, -1), box, atype)
    err = _errors(got, ref, atype.size)
    print("tc mixed vs fp64, resnet_dt", err)
    assert err["f_rmse"] <= 1e-3
    assert err["f_rel"] <= 2e-2
    assert err["e_rel"] <= 1e-4
