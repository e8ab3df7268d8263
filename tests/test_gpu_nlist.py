"""GPU: neighbour lists, bit-exact.

* the cell-list build against the reference PyTorch model's own list on the
  64-molecule water box (golden, same image order);
* against the oracle on larger / skewed / small boxes and open boundaries;
* the C++ formatter against the reference unit-test golden list
  (source/lib/tests/test_fmt_nlist.cc) and the oracle.
"""
import numpy as np
import pytest

from conftest import golden

import oracle as O

pytestmark = pytest.mark.gpu


def _t(a, cuda, dtype=None):
    import torch

    return torch.tensor(np.ascontiguousarray(a), device=cuda, dtype=dtype)


def test_water192_matches_reference_nlist(cuda):
    import torch
    from dpgb import nlist as N

    g = golden("water192")
    shifts = O.ghost_shifts(g["box"], 6.0, g["shift_order"]).astype(np.int32)
    ext, ext_t, mp, nl = N.extend_input_and_build_neighbor_list(
        _t(g["coord"].reshape(1, -1, 3), cuda), _t(g["atype"], cuda, torch.int32), 6.0, [46, 92],
        box=g["box"].reshape(1, 9), shifts=shifts)
    np.testing.assert_array_equal(nl[0].cpu().numpy(), g["nlist"])
    np.testing.assert_array_equal(ext[0].cpu().numpy(), g["coord_ext"])  # wrap + images bitwise
    np.testing.assert_array_equal(mp[0].cpu().numpy(), g["mapping"])


@pytest.mark.parametrize("nmol,sel,rcut", [(8, [46, 92], 6.0), (3, [46, 92], 6.0), (2, [20, 40], 4.0)])
def test_water_vs_oracle(cuda, nmol, sel, rcut):
    import torch
    from dpgb import nlist as N, synth

    coord, atype, box = synth.water_box(nmol, seed=nmol + 11)
    cn = O.normalize_coord(coord, box)
    shifts = O.ghost_shifts(box, rcut).astype(np.int32)
    ext, ext_t, _ = O.extend_coord_with_ghosts(cn, atype, box, rcut, None)
    ref = O.build_nlist_pt(ext, ext_t, coord.shape[0], rcut, sel)
    nl = N.build_neighbor_list_local(_t(cn, cuda), _t(atype, cuda, torch.int32), box, rcut, sel, shifts)
    np.testing.assert_array_equal(nl.cpu().numpy(), ref)


def test_triclinic_and_open_boundary(cuda):
    import torch
    from dpgb import nlist as N

    rng = np.random.default_rng(5)
    n = 300
    box = np.array([14.0, 0, 0, 2.5, 13.0, 0, -1.5, 1.0, 15.0])
    frac = rng.uniform(size=(n, 3))
    coord = frac @ box.reshape(3, 3)
    atype = rng.integers(0, 3, size=n).astype(np.int32)
    sel = [40, 40, 40]
    shifts = O.ghost_shifts(box, 5.0).astype(np.int32)
    ext, ext_t, _ = O.extend_coord_with_ghosts(coord, atype, box, 5.0, None)
    ref = O.build_nlist_pt(ext, ext_t, n, 5.0, sel)
    nl = N.build_neighbor_list_local(_t(coord, cuda), _t(atype, cuda, torch.int32), box, 5.0, sel, shifts)
    np.testing.assert_array_equal(nl.cpu().numpy(), ref)
    # open boundary: the list is over the local atoms only
    ref_open = O.build_nlist_pt(coord, atype, n, 5.0, sel)
    nl_open = N.build_neighbor_list_local(_t(coord, cuda), _t(atype, cuda, torch.int32), None, 5.0, sel)
    np.testing.assert_array_equal(nl_open.cpu().numpy(), ref_open)


def test_sel_truncation_is_global_topk(cuda):
    """More neighbours than sum(sel): the nearest sum(sel) overall are kept
    before the type split (nlist.py:134-199)."""
    import torch
    from dpgb import nlist as N, synth

    coord, atype, box = synth.water_box(4, seed=3)
    sel = [10, 25]
    shifts = O.ghost_shifts(box, 6.0).astype(np.int32)
    ext, ext_t, _ = O.extend_coord_with_ghosts(O.normalize_coord(coord, box), atype, box, 6.0, None)
    ref = O.build_nlist_pt(ext, ext_t, coord.shape[0], 6.0, sel)
    nl = N.build_neighbor_list_local(_t(O.normalize_coord(coord, box), cuda), _t(atype, cuda, torch.int32), box, 6.0,
                                     sel, shifts)
    np.testing.assert_array_equal(nl.cpu().numpy(), ref)


def test_format_nlist_cpp_golden(cuda):
    import torch
    from dpgb import nlist as N

    g = golden("fmt_nlist")
    nloc = len(g["atype"])
    nl, dropped = N.format_nlist_a(_t(g["coord_ext"], cuda), _t(g["atype_ext"], cuda, torch.int32),
                                   _t(g["rows"], cuda, torch.int32), _t(g["counts"], cuda, torch.int32), nloc,
                                   float(g["rc"]), [10, 10])
    np.testing.assert_array_equal(nl.cpu().numpy().reshape(-1), g["expect_nlist_cpy"])
    assert dropped == 0
    # short sel: rows drop neighbours and say so
    nl2, dropped2 = N.format_nlist_a(_t(g["coord_ext"], cuda), _t(g["atype_ext"], cuda, torch.int32),
                                     _t(g["rows"], cuda, torch.int32), _t(g["counts"], cuda, torch.int32), nloc,
                                     float(g["rc"]), [1, 1])
    ref2 = O.format_nlist_cpp(g["coord_ext"], g["atype_ext"], g["rows"], g["counts"], nloc, float(g["rc"]), [1, 1])
    np.testing.assert_array_equal(nl2.cpu().numpy(), ref2)
    assert dropped2 > 0


def test_overflow_is_an_error(cuda):
    """A dense cluster (more than 1024 atoms within rcut) is reported, not
    truncated silently."""
    import torch
    from dpgb import _lib, nlist as N

    rng = np.random.default_rng(0)
    coord = rng.uniform(0, 4.0, size=(1100, 3))
    atype = np.zeros(1100, np.int32)
    with pytest.raises(_lib.DpgbError, match="within rcut"):
        N.build_neighbor_list_local(_t(coord, cuda), _t(atype, cuda, torch.int32), None, 6.0, [100])


def test_dense_cell_takes_the_per_atom_path(cuda):
    """A box one cell wide whose 27-cell stencil holds more atoms than the
    staged kernel keeps in shared memory: the cell is handled by the per-atom
    search, with the same list as the oracle."""
    import torch
    from dpgb import nlist as N

    rng = np.random.default_rng(11)
    n = 120
    box = np.diag([7.5, 7.5, 7.5]).reshape(-1)
    coord = rng.uniform(size=(n, 3)) * 7.5
    atype = rng.integers(0, 2, size=n).astype(np.int32)
    sel = [100, 100]
    shifts = O.ghost_shifts(box, 6.0).astype(np.int32)
    ext, ext_t, _ = O.extend_coord_with_ghosts(coord, atype, box, 6.0, None)
    ref = O.build_nlist_pt(ext, ext_t, n, 6.0, sel)
    nl = N.build_neighbor_list_local(_t(coord, cuda), _t(atype, cuda, torch.int32), box, 6.0, sel, shifts)
    np.testing.assert_array_equal(nl.cpu().numpy(), ref)


@pytest.mark.parametrize("spacing", [2.0, 1.5])
def test_perfect_lattice_ties_and_cutoff(cuda, spacing):
    """A simple cubic lattice: whole shells of exactly equal distances (ties
    broken by extended index) and a shell exactly at rcut (6 = 3 x 2.0 = 4 x
    1.5).  The FP32 distances cannot order such atoms, so their lists come
    from the exact FP64 ranking: bitwise the oracle's."""
    import torch
    from dpgb import nlist as N

    n = int(round(21.0 / spacing))
    L = n * spacing
    g = np.arange(n, dtype=np.float64) * spacing
    coord = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    atype = (np.arange(coord.shape[0]) % 3 == 0).astype(np.int32)
    box = np.diag([L, L, L]).reshape(-1)
    sel = [140, 280]
    shifts = O.ghost_shifts(box, 6.0).astype(np.int32)
    ext, ext_t, _ = O.extend_coord_with_ghosts(coord, atype, box, 6.0, None)
    ref = O.build_nlist_pt(ext, ext_t, coord.shape[0], 6.0, sel)
    nl = N.build_neighbor_list_local(_t(coord, cuda), _t(atype, cuda, torch.int32), box, 6.0, sel, shifts)
    np.testing.assert_array_equal(nl.cpu().numpy(), ref)


def test_frames_in_one_call_equal_frame_by_frame(cuda):
    """dpgb_extend_input_and_build_nlist over several frames (one call) gives
    each frame's wrap, images, mapping and list bit for bit as the one-frame
    functions do."""
    import torch

    from dpgb import nlist as N, synth

    frames = [synth.water_box(4, seed=60 + k) for k in range(5)]
    coord = torch.tensor(np.stack([f[0] for f in frames]), dtype=torch.float64, device=cuda)
    coord = coord + 7.5  # some atoms outside the cell: the wrap matters
    atype = torch.tensor(np.stack([f[1] for f in frames]), device=cuda)
    box = np.stack([f[2].reshape(9) for f in frames])
    ext, ext_t, mp, nl = N.extend_input_and_build_neighbor_list(coord, atype, 6.0, [46, 92], box)
    for f in range(len(frames)):
        e1, t1, m1, n1 = N.extend_input_and_build_neighbor_list(coord[f:f + 1], atype[f:f + 1], 6.0, [46, 92],
                                                                box[f:f + 1])
        assert torch.equal(ext[f], e1[0]) and torch.equal(ext_t[f], t1[0].to(ext_t.dtype))
        assert torch.equal(mp[f], m1[0].to(mp.dtype)) and torch.equal(nl[f], n1[0].to(nl.dtype))
