"""CPU: the oracle against the reference's golden vectors and, where the
reference tree is present, against the reference's own compiled library."""
import numpy as np
import pytest

from conftest import assert_table_close, deeppot_sea_params, golden, water_params

import oracle as O


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("dtype,tol", [(np.float64, 1e-10), (np.float32, 1e-5)])
def test_tabulate_golden(dtype, tol):
    g = golden("tabulate_se_a_op")
    nl = int(g["last_layer_size"])
    em = g["em"].astype(dtype)
    em_x = g["em_x"].astype(dtype)
    out = O.tabulate_fusion_se_a(g["table"].astype(dtype), g["table_info"].astype(dtype), em_x, em, nl)
    np.testing.assert_allclose(out, g["descriptor"], atol=tol, rtol=tol)
    dx, dem = O.tabulate_fusion_se_a_grad(g["table"].astype(dtype), g["table_info"].astype(dtype), em_x, em,
                                          np.ones_like(out))
    np.testing.assert_allclose(dx, g["dy_dem_x"], atol=tol, rtol=tol)
    np.testing.assert_allclose(dem, g["dy_dem"], atol=tol, rtol=tol)


def test_tabulate_vs_reference_lib():
    if O.ref_lib() is None:
        pytest.skip("reference library unavailable")
    rng = np.random.default_rng(3)
    g = golden("tabulate_se_a_op")
    table, info = g["table"], g["table_info"]
    nloc, nnei, nl = 7, 9, 8
    em_x = rng.uniform(-0.1, 0.6, size=(nloc * nnei, 1))
    em = rng.normal(size=(nloc, nnei, 4))
    em[:, -3:, :] = 0.0  # trailing padding exercises the sorted fold
    em_x.reshape(nloc, nnei)[:, -3:] = em_x.reshape(nloc, nnei)[:, -1:]
    for srt in (True, False):
        a = O.tabulate_fusion_se_a(table, info, em_x, em, nl, srt)
        b = O.tabulate_fusion_se_a(table, info, em_x, em, nl, srt, use_ref=True)
        np.testing.assert_array_equal(a, b)
        dy = rng.normal(size=a.shape)
        for x, y in zip(O.tabulate_fusion_se_a_grad(table, info, em_x, em, dy, srt),
                        O.tabulate_fusion_se_a_grad(table, info, em_x, em, dy, srt, use_ref=True)):
            np.testing.assert_array_equal(x, y)
        dzx, dzm = rng.normal(size=em_x.shape), rng.normal(size=em.shape)
        np.testing.assert_array_equal(
            O.tabulate_fusion_se_a_grad_grad(table, info, em_x, em, dzx, dzm, nl, srt),
            O.tabulate_fusion_se_a_grad_grad(table, info, em_x, em, dzx, dzm, nl, srt, use_ref=True))


def test_env_mat_golden():
    g = golden("env_mat_a")
    sel = g["sel"]
    nloc = len(g["atype"])
    nl = O.format_nlist_cpp(g["coord_ext"], g["atype_ext"], g["rows"], g["counts"], nloc, float(g["rc"]), sel)
    np.testing.assert_array_equal(nl, g["nlist"])
    nnei = int(sel.sum())
    em, der, rij = O.env_mat_a(g["coord_ext"], g["atype_ext"], nl, np.zeros((2, nnei, 4)), np.ones((2, nnei, 4)),
                               float(g["rc"]), float(g["rc_smth"]))
    np.testing.assert_allclose(em.reshape(-1), g["expected_env"], atol=1e-5)
    np.testing.assert_allclose(em, g["em"], atol=1e-12)
    np.testing.assert_allclose(der, g["em_deriv"], atol=1e-12)
    np.testing.assert_allclose(rij, g["rij"], atol=1e-12)


def test_fmt_nlist_golden():
    g = golden("fmt_nlist")
    nloc = len(g["atype"])
    nl = O.format_nlist_cpp(g["coord_ext"], g["atype_ext"], g["rows"], g["counts"], nloc, float(g["rc"]), g["sel"])
    np.testing.assert_array_equal(nl.reshape(-1), g["expect_nlist_cpy"])


def test_prod_force_virial_golden():
    g = golden("prod_force_a")
    nall = g["coord_ext"].shape[0]
    nd = g["net_deriv"].reshape(len(g["atype"]), -1)
    f = O.prod_force_a(nd, g["em_deriv"], g["nlist"], nall)
    np.testing.assert_allclose(f.reshape(-1), g["expected_force"], atol=1e-5)
    g = golden("prod_virial_a")
    nd = g["net_deriv"].reshape(len(g["atype"]), -1)
    v, av = O.prod_virial_a(nd, g["em_deriv"], g["rij"], g["nlist"], nall)
    np.testing.assert_allclose(v, g["expected_virial"], atol=1e-5)
    np.testing.assert_allclose(av.reshape(-1), g["expected_atom_virial"], atol=1e-5)


def test_prod_grads_vs_reference_lib():
    if O.ref_lib() is None:
        pytest.skip("reference library unavailable")
    g = golden("prod_force_a")
    rng = np.random.default_rng(0)
    nloc = len(g["atype"])
    gr = rng.normal(size=(nloc, 3))
    a = O.prod_force_grad_a(gr, g["em_deriv"], g["nlist"])
    b = O.prod_force_grad_a(gr, g["em_deriv"], g["nlist"], use_ref=True)
    np.testing.assert_allclose(a, b, atol=1e-13)
    gv = rng.normal(size=9)
    a = O.prod_virial_grad_a(gv, g["em_deriv"], g["rij"], g["nlist"])
    b = O.prod_virial_grad_a(gv, g["em_deriv"], g["rij"], g["nlist"], use_ref=True)
    np.testing.assert_allclose(a, b, atol=1e-13)


def test_deeppot_testcase_golden():
    c = golden("deeppot_sea_case")
    om = O.OracleModel(deeppot_sea_params())
    for b in range(int(c["nblock"])):
        box = c[f"b{b}_box"]
        r = om.evaluate(c[f"b{b}_coord"], c[f"b{b}_atype"].astype(np.int32), None if box.size == 0 else box)
        np.testing.assert_allclose(r["atom_energy"], c[f"b{b}_atomic_energy"], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(r["force"].reshape(-1), c[f"b{b}_force"], rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(r["atom_virial"].reshape(-1), c[f"b{b}_atomic_virial"], rtol=1e-10, atol=1e-12)


def test_water192_golden():
    g = golden("water192")
    om = O.OracleModel(water_params())
    r = om.evaluate(g["coord"], g["atype"], g["box"], order=g["shift_order"])
    np.testing.assert_array_equal(r["nlist"], g["nlist"])  # bit-exact
    assert rel(r["energy"], g["energy"][0]) < 1e-12
    assert rel(r["force"], g["force"]) < 1e-10
    assert rel(r["virial"], g["virial"]) < 1e-10
    assert rel(r["atom_virial"], g["atom_virial"]) < 1e-10
    assert rel(r["descriptor"][:8], g["descriptor"]) < 1e-12


def test_water192_compressed_golden():
    g = golden("water192_compressed")
    w = golden("water192")
    om = O.OracleModel(water_params(compressed=True))
    r = om.evaluate(w["coord"], w["atype"], w["box"], order=w["shift_order"])
    assert rel(r["energy"], g["energy"][0]) < 1e-12
    assert rel(r["force"], g["force"]) < 1e-10
    assert rel(r["virial"], g["virial"]) < 1e-10


def test_table_build_matches_reference_tables():
    """The table-build restatement against the reference's own compression
    tables of the water model (enable_compression, strides 0.1 / 1.0)."""
    g = golden("water192_compressed")
    p = water_params()
    lower, upper = O.table_env_range(p.mean, p.stddev, float(g["min_nbor_dist"]), p.config.rcut_smth,
                                     p.config.rcut)
    nt = len(p.config.sel)
    for e in range(nt * nt):
        ti = e % nt
        layers = [(W, b) for W, b, _ in p.emb[e]]
        t = O.table_build(layers, lower[ti], upper[ti], float(g["extrapolate"]), float(g["stride0"]),
                          float(g["stride1"]))
        np.testing.assert_allclose(g[f"info_{e}"][:2], [lower[ti], upper[ti]])
        assert t.shape == g[f"table_{e}"].shape
        assert_table_close(t, g[f"table_{e}"], lower[ti], upper[ti], float(g["stride0"]), float(g["stride1"]))

