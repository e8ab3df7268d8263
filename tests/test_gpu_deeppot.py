"""GPU: the whole energy / force / virial path (DeepPot) against the
reference's own outputs:

* the reference PyTorch model on the 64-molecule water box (FP64 plain form,
  1e-10 relative) and its compressed form (FP64 table);
* the reference C/C++ API golden case (source/tests/infer/
  deeppot-testcase.yaml with deeppot_sea.pth: periodic, open boundary and an
  elongated box);
* the mixed-precision form against FP64 (force RMSE <= 1e-3 eV/A, the bound
  the benchmark metric is quoted at);
* bitwise reproducibility and multi-frame batching.
"""
import numpy as np
import pytest

from conftest import deeppot_sea_params, golden, water_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def water_fp64(cuda):
    from dpgb.deeppot import DeepPot

    return DeepPot(water_params(), "fp64")


def test_water192_fp64_matches_reference(water_fp64):
    g = golden("water192")
    e, f, v, ae, av = water_fp64.eval(g["coord"].reshape(1, -1), g["box"].reshape(1, 9), g["atype"], atomic=True)
    assert rel(e, g["energy"]) < 1e-10
    assert rel(f[0], g["force"]) < 1e-10
    assert rel(v[0], g["virial"]) < 1e-10
    assert rel(ae[0], g["atom_energy"]) < 1e-10
    assert rel(av[0], g["atom_virial"]) < 1e-10


def test_deeppot_testcase(cuda):
    from dpgb.deeppot import DeepPot

    c = golden("deeppot_sea_case")
    dp = DeepPot(deeppot_sea_params(), "fp64")
    for b in range(int(c["nblock"])):
        box = c[f"b{b}_box"]
        e, f, v, ae, av = dp.eval(c[f"b{b}_coord"], None if box.size == 0 else box, c[f"b{b}_atype"], atomic=True)
        np.testing.assert_allclose(ae[0], c[f"b{b}_atomic_energy"], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(f[0].reshape(-1), c[f"b{b}_force"], rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(av[0].reshape(-1), c[f"b{b}_atomic_virial"], rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(e[0], c[f"b{b}_atomic_energy"].sum(), rtol=1e-12)


def test_deeppot_testcase_from_model_file(cuda):
    """The same golden case through a frozen .pth model file read by the
    library (DP_NewDeepPot's input), FP64 and the mixed form."""
    import os

    from conftest import GOLDEN
    from dpgb.deeppot import DeepPot

    c = golden("deeppot_sea_case")
    for prec, tol in (("fp64", 1e-10), ("mixed", None)):
        dp = DeepPot.from_file(os.path.join(GOLDEN, "deeppot_sea.pth"), prec)
        assert dp.type_map == ["O", "H"] and dp.rcut == 6.0 and dp.ntypes == 2
        for b in range(int(c["nblock"])):
            box = c[f"b{b}_box"]
            e, f, v, ae, av = dp.eval(c[f"b{b}_coord"], None if box.size == 0 else box, c[f"b{b}_atype"],
                                      atomic=True)
            if tol:
                np.testing.assert_allclose(ae[0], c[f"b{b}_atomic_energy"], rtol=tol, atol=tol)
                np.testing.assert_allclose(f[0].reshape(-1), c[f"b{b}_force"], rtol=tol, atol=1e-12)
                np.testing.assert_allclose(av[0].reshape(-1), c[f"b{b}_atomic_virial"], rtol=tol, atol=1e-12)
            else:
                ref = c[f"b{b}_force"]
                rmse = float(np.sqrt(np.mean((f[0].reshape(-1) - ref) ** 2)))
                assert rmse <= 2e-2 * float(np.sqrt(np.mean(ref ** 2)))


def test_water192_compressed_matches_reference(cuda):
    from dpgb.deeppot import DeepPot

    g = golden("water192_compressed")
    w = golden("water192")
    dp = DeepPot(water_params(compressed=True), "fp64")
    e, f, v = dp.eval(w["coord"].reshape(1, -1), w["box"].reshape(1, 9), w["atype"])
    assert rel(e, g["energy"]) < 1e-10
    assert rel(f[0], g["force"]) < 1e-10
    assert rel(v[0], g["virial"]) < 1e-10


def test_mixed_vs_fp64(cuda, water_fp64):
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    coord, atype, box = synth.water_box(8, seed=4)
    e64, f64, v64 = water_fp64.eval(coord.reshape(1, -1), box, atype)
    mixed = DeepPot(water_params(), "mixed")
    e32, f32, v32 = mixed.eval(coord.reshape(1, -1), box, atype)
    n = atype.shape[0]
    rmse = float(np.sqrt(np.mean((f32 - f64) ** 2)))
    assert rmse <= 1e-3
    assert rmse <= 2e-2 * float(np.sqrt(np.mean(f64 ** 2)))  # also within 2 % of the RMS force
    assert abs(e32[0] - e64[0]) / n < 2e-4  # eV/atom: BF16 descriptor into the fitting GEMMs
    assert rel(v32[0], v64[0]) < 2e-2


def test_bitwise_reproducible(water_fp64):
    g = golden("water192")
    a = water_fp64.eval(g["coord"].reshape(1, -1), g["box"].reshape(1, 9), g["atype"])
    b = water_fp64.eval(g["coord"].reshape(1, -1), g["box"].reshape(1, 9), g["atype"])
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("compressed", [False, True])
def test_mixed_forces_bitwise_reproducible(cuda, compressed):
    """The mixed form's forces are summed with integer atomics (2^-32 fixed
    point): whatever order the adds land in, repeated evaluations agree
    bitwise."""
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    coord, atype, box = synth.water_box(8, seed=11)
    dp = DeepPot(water_params(compressed=compressed), "mixed")
    runs = [dp.eval(coord.reshape(1, -1), box, atype) for _ in range(3)]
    for other in runs[1:]:
        for x, y in zip(runs[0], other):
            np.testing.assert_array_equal(x, y)
    # the forces sum to zero over the box (every pair adds g to one row and
    # -g to another; what is left is the rows' own FP32 sums' rounding, far
    # below a dropped pair's share)
    f = runs[0][1][0]
    assert np.abs(f.sum(axis=0)).max() < 1e-3


def test_multi_frame_batch(water_fp64):
    from dpgb import synth

    c1, atype, box = synth.water_box(4, seed=1)
    c2, _, _ = synth.water_box(4, seed=2)
    e, f, v = water_fp64.eval(np.stack([c1.reshape(-1), c2.reshape(-1)]), np.stack([box, box]), atype)
    e1, f1, v1 = water_fp64.eval(c1.reshape(1, -1), box, atype)
    e2, f2, v2 = water_fp64.eval(c2.reshape(1, -1), box, atype)
    np.testing.assert_allclose(e, [e1[0], e2[0]], rtol=1e-13)
    np.testing.assert_allclose(f, np.concatenate([f1, f2]), rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(v, np.concatenate([v1, v2]), rtol=1e-12, atol=1e-15)


def test_device_api_matches_host_api(water_fp64):
    import torch

    g = golden("water192")
    e, f, v = water_fp64.eval(g["coord"].reshape(1, -1), g["box"].reshape(1, 9), g["atype"])
    out = water_fp64.eval_device(torch.tensor(g["coord"].reshape(1, -1), device="cuda"), g["box"].reshape(1, 9),
                                 g["atype"])
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out["energy"].cpu().numpy(), e)
    np.testing.assert_array_equal(out["force"].cpu().numpy(), f)
    np.testing.assert_array_equal(out["virial"].cpu().numpy(), v)


def test_mixed_compressed_vs_fp64_compressed(cuda):
    """The fused FP32 table kernels (mixed form of a compressed model)
    against the FP64 table form on a 1,536-atom box."""
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    coord, atype, box = synth.water_box(8, seed=5)
    p = water_params(compressed=True)
    e64, f64, v64 = DeepPot(p, "fp64").eval(coord.reshape(1, -1), box, atype)
    e32, f32, v32 = DeepPot(p, "mixed").eval(coord.reshape(1, -1), box, atype)
    n = atype.shape[0]
    rmse = float(np.sqrt(np.mean((f32 - f64) ** 2)))
    assert rmse <= 1e-3
    assert rmse <= 2e-2 * float(np.sqrt(np.mean(f64 ** 2)))
    assert abs(e32[0] - e64[0]) / n < 2e-4
    assert rel(v32[0], v64[0]) < 2e-2


def _lammps_like_input(rng, skin=2.0, rcut=6.0):
    """water192 as an MD engine hands it over: local atoms, all periodic
    images as ghosts, and a full neighbour list at rcut + skin in random
    order."""
    import oracle as O

    g = golden("water192")
    cn = O.normalize_coord(g["coord"], g["box"])
    ext, ext_t, mapping = O.extend_coord_with_ghosts(cn, g["atype"], g["box"], rcut, None)
    nloc = cn.shape[0]
    d = np.linalg.norm(ext[None, :, :] - cn[:, None, :], axis=-1)
    rows = []
    for i in range(nloc):
        js = np.nonzero((d[i] <= rcut + skin) & (np.arange(ext.shape[0]) != i))[0]
        rows.append(rng.permutation(js).astype(np.int32))
    ilist = rng.permutation(nloc).astype(np.int32)
    return g, ext, ext_t.astype(np.int32), mapping, [rows[i] for i in ilist], ilist


def _fold(x, mapping, nloc):
    out = np.zeros((nloc,) + x.shape[1:])
    np.add.at(out, mapping, x)
    return out


@pytest.mark.parametrize("skin", [2.0, 0.0])
def test_external_neighbour_list_matches_periodic(cuda, water_fp64, skin):
    """dpgb_deeppot_compute_nlist (LAMMPS InputNlist with ghosts): a skin
    list wider than sum(sel) (sorted, cut to the nearest) and an rcut list in
    the caller's order both give the periodic E / F / V once the ghost forces
    are folded back."""
    rng = np.random.default_rng(7)
    g, ext, ext_t, mapping, rows, ilist = _lammps_like_input(rng, skin=skin)
    nloc = g["atype"].shape[0]
    nghost = ext.shape[0] - nloc
    e, f, v, ae, av = water_fp64.eval_nlist(ext, ext_t, nghost, ilist, [len(r) for r in rows], rows, ago=0,
                                            atomic=True)
    e0, f0, v0, ae0, av0 = water_fp64.eval(g["coord"].reshape(1, -1), g["box"].reshape(1, 9), g["atype"], atomic=True)
    assert rel(e, e0[0]) < 1e-12
    assert rel(_fold(f, mapping, nloc), f0[0]) < 1e-10
    assert rel(v, v0[0]) < 1e-10
    assert rel(ae[:nloc], ae0[0]) < 1e-10 and np.all(ae[nloc:] == 0)
    assert rel(_fold(av, mapping, nloc), av0[0]) < 1e-10


def test_external_neighbour_list_reuse(cuda, water_fp64):
    """ago > 0 keeps the list and takes the new coordinates: equal to a fresh
    call on the same coordinates; the mixed form within the stated tolerance."""
    from dpgb.deeppot import DeepPot

    rng = np.random.default_rng(8)
    g, ext, ext_t, mapping, rows, ilist = _lammps_like_input(rng)
    nloc = g["atype"].shape[0]
    nghost = ext.shape[0] - nloc
    nn = [len(r) for r in rows]
    water_fp64.eval_nlist(ext, ext_t, nghost, ilist, nn, rows, ago=0)
    moved = ext + rng.normal(0, 0.01, size=(nloc, 3))[mapping]  # ghosts move with their owners
    e1, f1, v1 = water_fp64.eval_nlist(moved, ext_t, nghost, None, None, [], ago=1)
    e2, f2, v2 = water_fp64.eval_nlist(moved, ext_t, nghost, ilist, nn, rows, ago=0)
    assert e1 == e2 and np.array_equal(f1, f2) and np.array_equal(v1, v2)
    mixed = DeepPot(water_params(), "mixed")
    em, fm, vm = mixed.eval_nlist(moved, ext_t, nghost, ilist, nn, rows, ago=0)
    fl, fml = _fold(f2, mapping, nloc), _fold(fm, mapping, nloc)
    assert float(np.sqrt(np.mean((fml - fl) ** 2))) <= 1e-3
    assert abs(em - e2) / nloc < 2e-4


def test_list_read_waits_for_the_callers_stream(cuda):
    """The device form runs on the caller's stream; reading the list back
    (and the status words) afterwards waits for that evaluation even while
    it is still queued behind other work on that stream."""
    import torch

    from dpgb import synth
    from dpgb.deeppot import DeepPot

    coord, atype, box = synth.water_box(8, seed=5)
    dp = DeepPot(water_params(), "fp64")
    x = torch.tensor(coord.reshape(1, -1), dtype=torch.float64, device="cuda")
    dp.eval_device(x, box.reshape(1, 9), atype)
    torch.cuda.synchronize()
    first = dp.last_nlist()[0]
    x2 = x + torch.randn(x.shape, dtype=x.dtype, device="cuda", generator=torch.Generator("cuda").manual_seed(3)) * 0.05
    torch.cuda.synchronize()
    torch.cuda._sleep(200_000_000)  # ~0.1 s of work queued ahead of the evaluation
    dp.eval_device(x2, box.reshape(1, 9), atype)
    early = dp.last_nlist()[0]
    dp.check_status()
    torch.cuda.synchronize()
    late = dp.last_nlist()[0]
    assert not np.array_equal(first, late)  # the walk changed the list
    np.testing.assert_array_equal(early, late)


def test_host_api_with_pinned_buffers(cuda):
    """Page-locked caller buffers (copied without staging) give the same
    results as pageable ones."""
    from dpgb import synth
    from dpgb.deeppot import DeepPot, pinned_empty

    coord, atype, box = synth.water_box(6, seed=9)
    dp = DeepPot(water_params(), "mixed")
    e0, f0, v0 = dp.eval(coord.reshape(1, -1), box.reshape(1, 9), atype)
    cp = pinned_empty((1, coord.size))
    cp[:] = coord.reshape(1, -1)
    outs = (pinned_empty((1,)), pinned_empty((1, atype.size, 3)), pinned_empty((1, 9)))
    e1, f1, v1 = dp.eval(cp, box.reshape(1, 9), atype, out=outs)
    assert e1 is outs[0] and f1 is outs[1]
    np.testing.assert_array_equal(e1, e0)
    np.testing.assert_array_equal(f1, f0)
    np.testing.assert_array_equal(v1, v0)
