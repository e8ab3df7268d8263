"""Neighbour lists on the GPU, mirroring deepmd/pt/utils/nlist.py and
deepmd/pt/utils/region.py (same argument meaning and output layout).

* :func:`extend_input_and_build_neighbor_list` — wrap, periodic images in the
  reference's image order, typed neighbour list (O(N) cell list in libdpgb).
* :func:`build_neighbor_list` — typed list from already extended coordinates
  laid out image-major (the layout of :func:`extend_coord_with_ghosts`).
* :func:`format_nlist_a` — the C++ formatter (type, fp32 r^2, index order).
"""
from __future__ import annotations

import ctypes as C
import functools
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _lib


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return C.cast(None, C.POINTER(C.c_double))
    return a.ctypes.data_as(C.POINTER(C.c_double))


def to_face_distance(box: np.ndarray) -> np.ndarray:
    """deepmd/pt/utils/region.py:50-83 (numpy)."""
    cell = np.asarray(box, np.float64).reshape(3, 3)
    vol = np.linalg.det(cell)
    return np.array([vol / np.linalg.norm(np.cross(cell[1], cell[2])),
                     vol / np.linalg.norm(np.cross(cell[2], cell[0])),
                     vol / np.linalg.norm(np.cross(cell[0], cell[1]))])


def image_shifts(box: np.ndarray, rcut: float) -> np.ndarray:
    """Integer image shifts [(2nbuff+1)^3, 3] in the order the reference sorts
    them (deepmd/pt/utils/nlist.py:470-498): the same ``torch.argsort`` of the
    shift norms on the CPU, so extended indices match the reference's.
    Cached per buffer count (frames of one box size share it)."""
    nbuff = np.ceil(rcut / np.abs(to_face_distance(box))).astype(np.int64)
    return _image_shifts(tuple(int(n) for n in nbuff)).copy()


@functools.lru_cache(maxsize=64)
def _image_shifts(nbuff) -> np.ndarray:
    xi = [torch.arange(-int(n), int(n) + 1, dtype=torch.int64) for n in nbuff]
    eye = torch.eye(3, dtype=torch.float64)
    xyz = (xi[0].view(-1, 1, 1, 1) * eye[0] + xi[1].view(1, -1, 1, 1) * eye[1]
           + xi[2].view(1, 1, -1, 1) * eye[2]).view(-1, 3)
    order = torch.argsort(torch.linalg.norm(xyz, dim=-1))
    return xyz[order].numpy().astype(np.int32)


def normalize_coord(coord: torch.Tensor, box: np.ndarray) -> torch.Tensor:
    """deepmd/pt/utils/region.py:86-105 on the GPU ([natom, 3] float64)."""
    coord = coord.reshape(-1, 3).contiguous()
    out = torch.empty_like(coord)
    b = np.ascontiguousarray(box, np.float64).reshape(9)
    _lib.call("dpgb_normalize_coord", _vp(out), _vp(coord), coord.shape[0], _dp(b), _stream())
    return out


def extend_coord_with_ghosts(coord: torch.Tensor, atype: torch.Tensor, box: np.ndarray, rcut: float,
                             shifts: Optional[np.ndarray] = None):
    """All periodic images, image-major (nlist.py:424-513).  Returns
    (extended_coord [nall,3], extended_atype [nall], mapping [nall])."""
    coord = coord.reshape(-1, 3).contiguous()
    nloc = coord.shape[0]
    shifts = image_shifts(box, rcut) if shifts is None else np.ascontiguousarray(shifts, np.int32)
    ns = shifts.shape[0]
    dev = coord.device
    ext = torch.empty(ns * nloc, 3, dtype=torch.float64, device=dev)
    ext_t = torch.empty(ns * nloc, dtype=torch.int32, device=dev)
    mapping = torch.empty(ns * nloc, dtype=torch.int32, device=dev)
    b = np.ascontiguousarray(box, np.float64).reshape(9)
    at = atype.to(device=dev, dtype=torch.int32).contiguous()
    _lib.call("dpgb_extend_coord", _vp(ext), _vp(ext_t), _vp(mapping), _vp(coord), _vp(at), nloc, _dp(b),
              _ip(shifts), ns, _stream())
    return ext, ext_t, mapping


def build_neighbor_list_local(coord: torch.Tensor, atype: torch.Tensor, box: Optional[np.ndarray], rcut: float,
                              sel: Sequence[int], shifts: Optional[np.ndarray] = None) -> torch.Tensor:
    """Typed neighbour list of the local atoms of one frame (already wrapped)
    holding extended indices in the image-major layout."""
    coord = coord.reshape(-1, 3).contiguous()
    nloc = coord.shape[0]
    sel_a = np.ascontiguousarray(sel, np.int32)
    out = torch.empty(nloc, int(sel_a.sum()), dtype=torch.int32, device=coord.device)
    at = atype.to(device=coord.device, dtype=torch.int32).contiguous()
    if box is not None:
        shifts = image_shifts(box, rcut) if shifts is None else np.ascontiguousarray(shifts, np.int32)
        b = np.ascontiguousarray(box, np.float64).reshape(9)
        _lib.call("dpgb_build_nlist_pt", _vp(out), _vp(coord), _vp(at), nloc, _dp(b), _ip(shifts), shifts.shape[0],
                  C.c_double(rcut), _ip(sel_a), len(sel_a), _stream())
    else:
        z = np.zeros(3, np.int32)
        _lib.call("dpgb_build_nlist_pt", _vp(out), _vp(coord), _vp(at), nloc, _dp(None), _ip(z), 1,
                  C.c_double(rcut), _ip(sel_a), len(sel_a), _stream())
    return out


def extend_input_and_build_neighbor_list(coord: torch.Tensor, atype: torch.Tensor, rcut: float,
                                         sel: List[int], box: Optional[np.ndarray] = None,
                                         shifts: Optional[np.ndarray] = None):
    """deepmd/pt/utils/nlist.py:14-46 for one or more frames with the same
    atom count: returns (extended_coord [nf, nall, 3], extended_atype
    [nf, nall], mapping [nf, nall], nlist [nf, nloc, sum(sel)]) with the
    types already distinguished."""
    atype = atype.reshape(-1) if atype.dim() == 1 else atype
    nf = coord.shape[0] if coord.dim() == 3 or (coord.dim() == 2 and atype.dim() == 2) else 1
    coord = coord.reshape(nf, -1, 3)
    atype2 = atype.reshape(nf, -1) if atype.dim() == 2 else atype.reshape(1, -1).expand(nf, -1)
    if box is not None and nf > 1:
        return _extend_and_build_frames(coord, atype2, rcut, sel, np.asarray(box, np.float64).reshape(nf, 9), shifts)
    exts, ext_ts, maps, nls = [], [], [], []
    for f in range(nf):
        bf = None if box is None else np.asarray(box, np.float64).reshape(nf, 9)[f]
        c = coord[f]
        if bf is not None:
            c = normalize_coord(c, bf)
            ext, ext_t, mp = extend_coord_with_ghosts(c, atype2[f], bf, rcut, shifts)
        else:
            ext, ext_t, mp = c.clone(), atype2[f].to(torch.int32), torch.arange(c.shape[0], dtype=torch.int32,
                                                                                  device=c.device)
        nls.append(build_neighbor_list_local(c, atype2[f], bf, rcut, sel, shifts))
        exts.append(ext)
        ext_ts.append(ext_t)
        maps.append(mp)
    return torch.stack(exts), torch.stack(ext_ts), torch.stack(maps), torch.stack(nls)


def _extend_and_build_frames(coord: torch.Tensor, atype: torch.Tensor, rcut: float, sel: Sequence[int],
                             box: np.ndarray, shifts: Optional[np.ndarray] = None):
    """Periodic frames in one library call (dpgb_extend_input_and_build_nlist):
    the image table from the largest buffer count over the frames, as the
    reference builds one extended layout for a batch (nlist.py:470-498)."""
    nf, nloc = coord.shape[0], coord.shape[1]
    if shifts is None:
        nbuff = np.max(np.stack([np.ceil(rcut / np.abs(to_face_distance(b))) for b in box]), axis=0)
        shifts = _image_shifts(tuple(int(n) for n in nbuff)).copy()
    shifts = np.ascontiguousarray(shifts, np.int32)
    ns = shifts.shape[0]
    sel_a = np.ascontiguousarray(sel, np.int32)
    dev = coord.device
    c = coord.to(torch.float64).contiguous()
    at = atype.to(device=dev, dtype=torch.int32).contiguous()
    ext = torch.empty(nf, ns * nloc, 3, dtype=torch.float64, device=dev)
    ext_t = torch.empty(nf, ns * nloc, dtype=torch.int32, device=dev)
    mapping = torch.empty(nf, ns * nloc, dtype=torch.int32, device=dev)
    nl = torch.empty(nf, nloc, int(sel_a.sum()), dtype=torch.int32, device=dev)
    b = np.ascontiguousarray(box, np.float64).reshape(nf * 9)
    _lib.call("dpgb_extend_input_and_build_nlist", _vp(ext), _vp(ext_t), _vp(mapping), _vp(nl), _vp(c), _vp(at),
              nf, nloc, _dp(b), _ip(shifts), ns, C.c_double(rcut), _ip(sel_a), len(sel_a), _stream())
    return ext, ext_t, mapping, nl


def format_nlist_a(coord_ext: torch.Tensor, atype_ext: torch.Tensor, rows: torch.Tensor, counts: torch.Tensor,
                   nloc: int, rcut: float, sel: Sequence[int]):
    """C++ formatter (source/lib/src/fmt_nlist.cc:98-150) on the GPU.
    Returns (nlist [nloc, sum(sel)], number of rows that dropped neighbours)."""
    sel_a = np.ascontiguousarray(sel, np.int32)
    out = torch.empty(nloc, int(sel_a.sum()), dtype=torch.int32, device=coord_ext.device)
    ov = np.zeros(1, np.int32)
    # converted copies must stay referenced until the call returns
    c = coord_ext.contiguous()
    t = atype_ext.to(torch.int32).contiguous()
    r = rows.to(torch.int32).contiguous()
    n = counts.to(torch.int32).contiguous()
    _lib.call("dpgb_format_nlist_a", _vp(out), _vp(c), _vp(t), _vp(r), _vp(n), r.shape[1], nloc,
              c.reshape(-1, 3).shape[0], C.c_double(rcut), _ip(sel_a), len(sel_a), _ip(ov), _stream())
    return out, int(ov[0])
