"""GPU: the DeepPot backend plugin (deepmd-kit_gb300/dpgb/
libdeepmd_backend_pt.so) driven the way a reference host drives a backend
plugin -- dlopen, deepmd_create_deeppot_backend_v1 with a frozen .pth model,
then deepmd::DeepPotBackend's virtual methods (tests/plugin/host.cc, built
against include/deepmd_backend_abi.h, whose layout test_plugin_abi.py pins
to the reference's headers):

* computew (FP64, no list) reproduces the reference C/C++ API golden case
  (source/tests/infer/deeppot-testcase.yaml with deeppot_sea: periodic, open
  boundary, elongated box) to 1e-10;
* the FP32 overload agrees to single precision;
* computew with a LAMMPS-style InputNlist and ghosts, ago 0 then ago 1,
  gives the periodic result once ghost forces are folded back;
* computew_mixed_type equals frame-by-frame results;
* DP_GB300_PRECISION=mixed selects the mixed form."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden
import plugin_host as H

pytestmark = pytest.mark.gpu

MODEL = os.path.join(GOLDEN, "deeppot_sea.pth")


@pytest.fixture(scope="module")
def host(tmp_path_factory, cuda):
    from dpgb import _lib, build

    _lib.lib()
    return H.build_host(str(tmp_path_factory.mktemp("plugin"))), build.PLUGIN


def _case_jobs(c, kind=0):
    jobs = []
    for b in range(int(c["nblock"])):
        box = c[f"b{b}_box"]
        jobs.append(H.job_frames(c[f"b{b}_coord"], c[f"b{b}_atype"], None if box.size == 0 else box, kind))
    return jobs


def test_plugin_reproduces_deeppot_testcase(host):
    exe, plugin = host
    c = golden("deeppot_sea_case")
    rc, out, res = H.run(exe, plugin, MODEL, _case_jobs(c))
    assert rc == 0, out
    assert "cutoff 6 ntypes 2 type_map O H fparam 0 aparam 0" in out
    for b, (e, f, v, ae, av) in enumerate(res):
        np.testing.assert_allclose(ae, c[f"b{b}_atomic_energy"], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(f, c[f"b{b}_force"], rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(av, c[f"b{b}_atomic_virial"], rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(e[0], c[f"b{b}_atomic_energy"].sum(), rtol=1e-12)
        np.testing.assert_allclose(v, c[f"b{b}_atomic_virial"].reshape(-1, 9).sum(0), rtol=1e-10, atol=1e-12)


def test_plugin_float_overload(host):
    exe, plugin = host
    c = golden("deeppot_sea_case")
    rc, out, res = H.run(exe, plugin, MODEL, _case_jobs(c, kind=1))
    assert rc == 0, out
    for b, (e, f, v, ae, av) in enumerate(res):
        ref = c[f"b{b}_force"]
        assert np.abs(f - ref).max() <= 1e-5 * max(np.abs(ref).max(), 1.0)


def test_plugin_neighbour_list_and_ago(host):
    from test_gpu_deeppot import _fold, _lammps_like_input

    exe, plugin = host
    rng = np.random.default_rng(17)
    g, ext, ext_t, mapping, rows, ilist = _lammps_like_input(rng)
    nloc = g["atype"].shape[0]
    nghost = ext.shape[0] - nloc
    moved = ext + rng.normal(0, 0.01, size=(nloc, 3))[mapping]
    jobs = [H.job_frames(g["coord"], g["atype"], g["box"]),
            H.job_nlist(ext, ext_t, nghost, ilist, rows, ago=0),
            H.job_nlist(moved, ext_t, nghost, [], [], ago=1),
            H.job_nlist(moved, ext_t, nghost, ilist, rows, ago=0)]
    rc, out, res = H.run(exe, plugin, MODEL, jobs)
    assert rc == 0, out
    (e0, f0, v0, ae0, av0), (e1, f1, v1, ae1, av1), r2, r3 = res
    assert abs(e1[0] - e0[0]) <= 1e-12 * abs(e0[0])
    np.testing.assert_allclose(_fold(f1.reshape(-1, 3), mapping, nloc).reshape(-1), f0, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(v1, v0, rtol=1e-10, atol=1e-12)
    for a, b in zip(r2, r3):  # the kept list on moved coordinates == a fresh one
        np.testing.assert_array_equal(a, b)


def test_plugin_mixed_type_frames(host):
    exe, plugin = host
    c = golden("deeppot_sea_case")
    coord, atype, box = c["b0_coord"].reshape(-1), c["b0_atype"].reshape(-1), c["b0_box"].reshape(-1)
    rng = np.random.default_rng(3)
    c2 = coord + rng.normal(0, 0.02, size=coord.shape)
    t2 = atype[::-1].copy()
    jobs = [H.job_frames(np.concatenate([coord, c2]), np.stack([atype, t2]), np.stack([box, box]), kind=3),
            H.job_frames(coord, atype, box), H.job_frames(c2, t2, box)]
    rc, out, res = H.run(exe, plugin, MODEL, jobs)
    assert rc == 0, out
    (e, f, v, ae, av), r0, r1 = res
    n = atype.size
    np.testing.assert_array_equal(e, [r0[0][0], r1[0][0]])
    np.testing.assert_array_equal(f, np.concatenate([r0[1], r1[1]]))
    np.testing.assert_array_equal(av[: 9 * n], r0[4])


def test_plugin_mixed_precision_and_errors(host):
    exe, plugin = host
    c = golden("deeppot_sea_case")
    rc, out, res = H.run(exe, plugin, MODEL, _case_jobs(c)[:1], env={"DP_GB300_PRECISION": "mixed"})
    assert rc == 0, out
    ref = c["b0_force"]
    rmse = float(np.sqrt(np.mean((res[0][1] - ref) ** 2)))
    assert 0 < rmse <= 2e-2 * float(np.sqrt(np.mean(ref ** 2)))
    rc, out, _ = H.run(exe, plugin, os.path.join(GOLDEN, "water192.npz"), [])
    assert rc == 3 and "GB300 backend" in out  # not a model file: NULL and a message
