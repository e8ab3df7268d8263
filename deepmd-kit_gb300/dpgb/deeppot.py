"""DeepPot: energy / force / virial of se_e2_a models through libdpgb.

Mirrors the reference inference API (deepmd/infer/deep_pot.py ``DeepPot.eval``
and the C API ``DP_DeepPotCompute``, source/api_c/include/c_api.h:244-254):

    dp = DeepPot(params, precision="fp64")          # or "mixed"
    e, f, v = dp.eval(coord, box, atype)            # host numpy in/out
    e, f, v, ae, av = dp.eval(coord, box, atype, atomic=True)

``coord`` is [nframes, natom*3] (or [natom, 3] for one frame), ``box``
[nframes, 9] or None (open boundary), ``atype`` [natom].  Energies, virials
and forces come back in FP64.  :meth:`eval_device` keeps coordinates and
outputs on the GPU (torch tensors) for MD loops.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from .params import SeAParams

PRECISIONS = {"fp64": 0, "float64": 0, "mixed": 1}


def pack_desc(params: SeAParams):
    """Fill a dpgb_se_a_desc from SeAParams; returns (struct, keepalive)."""
    c = params.config
    c.validate()
    keep = []

    def ptr(a, ctype=C.c_double):
        if a is None:
            return C.cast(None, C.POINTER(ctype))
        a = np.ascontiguousarray(a, dtype=np.float64 if ctype is C.c_double else np.int32)
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(ctype))

    d = _lib.SeADesc()
    d.ntypes = c.ntypes
    for i, s in enumerate(c.sel):
        d.sel[i] = s
    d.rcut, d.rcut_smth = c.rcut, c.rcut_smth
    d.type_one_side = int(c.type_one_side)
    d.n_emb = len(c.neuron)
    for i, w in enumerate(c.neuron):
        d.emb_neuron[i] = w
    d.axis_neuron = c.axis_neuron
    d.n_fit = len(c.fit_neuron)
    for i, w in enumerate(c.fit_neuron):
        d.fit_neuron[i] = w
    d.dim_descrpt = c.dim_descrpt
    d.davg = ptr(params.mean)
    d.dstd = ptr(params.stddev)
    for e, layers in enumerate(params.emb):
        for l, (w, b, idt) in enumerate(layers):
            d.emb_w[e][l] = ptr(w)
            d.emb_b[e][l] = ptr(b)
            d.emb_idt[e][l] = ptr(idt)
    for t, layers in enumerate(params.fit):
        for l, (w, b, idt) in enumerate(layers):
            d.fit_w[t][l] = ptr(w)
            d.fit_b[t][l] = ptr(b)
            d.fit_idt[t][l] = ptr(idt)
    d.atom_ener_bias = ptr(params.atom_ener_bias())
    pm = c.pair_mask()
    d.pair_mask = ptr(pm, C.c_int) if pm is not None else C.cast(None, C.POINTER(C.c_int))
    if params.compressed:
        d.compressed = 1
        for e, (tab, info) in enumerate(zip(params.tables, params.table_info)):
            d.table[e] = ptr(tab)
            for k in range(6):
                d.table_info[e][k] = float(info[k])
    return d, keep


def pinned_empty(shape, dtype=np.float64) -> np.ndarray:
    """A numpy array in page-locked host memory (kept alive by the array);
    the host API copies such buffers without staging."""
    import torch

    t = torch.empty(int(np.prod(shape)) * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
    return t.numpy().view(dtype).reshape(shape)  # the array's base holds the tensor


def _shape_key(d, precision: str) -> str:
    """What a launch configuration depends on: the model's sizes (not its
    weights) and the precision."""
    nt = int(d.ntypes)
    return (f"se_e2_a nt{nt} sel{[int(d.sel[i]) for i in range(nt)]} rc{float(d.rcut):g} "
            f"emb{[int(d.emb_neuron[i]) for i in range(int(d.n_emb))]} ax{int(d.axis_neuron)} "
            f"fit{[int(d.fit_neuron[i]) for i in range(int(d.n_fit))]} compressed{int(d.compressed)} "
            f"one_side{int(d.type_one_side)} {precision}")


class DeepPot:
    def __init__(self, params: SeAParams, precision: str = "fp64", device: int = 0):
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("dpgb DeepPot needs a CUDA device")
        torch.cuda.set_device(device)
        self.params = params
        self.precision = precision
        self.device = device
        lib = _lib.lib()
        desc, keep = pack_desc(params)
        self.shape_key = _shape_key(desc, precision)
        self._h = lib.dpgb_deeppot_new(C.byref(desc), PRECISIONS[precision])
        del keep
        if not self._h:
            raise _lib.DpgbError(-1, lib.dpgb_last_error().decode())

    @classmethod
    def from_file(cls, path: str, precision: str = "fp64", device: int = 0) -> "DeepPot":
        """A DeepPot from a frozen DeePMD-kit PyTorch model file (.pth, the
        file DP_NewDeepPot takes), read without libtorch
        (dpgb_model_file_open)."""
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("dpgb DeepPot needs a CUDA device")
        torch.cuda.set_device(device)
        lib = _lib.lib()
        mf = lib.dpgb_model_file_open(str(path).encode(), None, 0)
        if not mf:
            raise _lib.DpgbError(-1, lib.dpgb_last_error().decode())
        try:
            self = cls.__new__(cls)
            self.params = None
            self.precision = precision
            self.device = device
            self.type_map = lib.dpgb_model_file_type_map(mf).decode().split()
            desc = C.cast(lib.dpgb_model_file_desc(mf), C.POINTER(_lib.SeADesc)).contents
            self._rcut, self._ntypes = float(desc.rcut), int(desc.ntypes)
            self.shape_key = _shape_key(desc, precision)
            self._h = lib.dpgb_deeppot_new(C.byref(desc), PRECISIONS[precision])
        finally:
            lib.dpgb_model_file_close(mf)
        if not self._h:
            raise _lib.DpgbError(-1, lib.dpgb_last_error().decode())
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.lib().dpgb_deeppot_delete(h)
            self._h = None

    @property
    def rcut(self) -> float:
        return self.params.config.rcut if self.params is not None else self._rcut

    @property
    def ntypes(self) -> int:
        return self.params.config.ntypes if self.params is not None else self._ntypes

    def last_launches(self) -> int:
        return int(_lib.lib().dpgb_deeppot_last_launches(self._h))

    def last_nlist(self):
        """(nlist [nframes*natom, nnei] int32, coord [nframes*natom, 3],
        shift [nframes, nshift, 3]) of the list the last evaluation built:
        extended index e = s*natom + j is image s of atom j at coord[j] +
        shift[frame, s]; None when that evaluation had no list of its own."""
        lib = _lib.lib()
        info = np.zeros(4, dtype=np.int32)
        ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
        _lib.check(lib.dpgb_deeppot_last_nlist(self._h, info.ctypes.data_as(ip), C.cast(None, ip),
                                               C.cast(None, dp), C.cast(None, dp)))
        nf, natom, nnei, nshift = (int(v) for v in info)
        if nf <= 0:
            return None
        nl = np.empty((nf * natom, nnei), dtype=np.int32)
        coord = np.empty((nf * natom, 3))
        shift = np.empty((nf, nshift, 3))
        _lib.check(lib.dpgb_deeppot_last_nlist(self._h, info.ctypes.data_as(ip), nl.ctypes.data_as(ip),
                                               coord.ctypes.data_as(dp), shift.ctypes.data_as(dp)))
        return nl, coord, shift

    def set_skin(self, skin: float, every: int = 1) -> None:
        """Reuse neighbour lists over calls on periodic frames: candidates
        within rcut + skin, rebuilt every ``every`` calls or when an atom has
        moved more than skin / 2 (``skin=0``: a fresh list each call)."""
        _lib.check(_lib.lib().dpgb_deeppot_set_skin(self._h, float(skin), int(every)))

    def set_graph(self, on: bool = True) -> None:
        """Replay the evaluation of a periodic system from a CUDA graph while
        its shape, box, buffers and the handle's state stay the same."""
        _lib.check(_lib.lib().dpgb_deeppot_set_graph(self._h, int(on)))

    def check_status(self, stream=None) -> None:
        """Synchronise and raise the device-side errors of the last
        evaluation (the device form does not synchronise)."""
        _lib.check(_lib.lib().dpgb_deeppot_check_status(self._h, None if stream is None else C.c_void_p(stream)))

    def set_profiling(self, on: bool) -> None:
        _lib.check(_lib.lib().dpgb_deeppot_set_profiling(self._h, int(on)))

    def collect_stages(self) -> None:
        _lib.check(_lib.lib().dpgb_deeppot_collect_stages(self._h))

    def stage_times(self):
        """{stage: total ms}, number of collected calls."""
        ms = (C.c_double * len(_lib.STAGES))()
        n = C.c_int(0)
        _lib.check(_lib.lib().dpgb_deeppot_stage_times(self._h, ms, C.byref(n)))
        return dict(zip(_lib.STAGES, list(ms))), int(n.value)

    def eval(self, coord, box, atype, atomic: bool = False, out=None):
        """Host arrays in and out (DP_DeepPotCompute).  ``out``: optional
        (energy [nf], force [nf, natom, 3], virial [nf, 9]) arrays to fill,
        e.g. views of page-locked memory (``pinned_empty``), which the call
        copies into directly."""
        atype = np.ascontiguousarray(atype, dtype=np.int32).reshape(-1)
        natom = atype.shape[0]
        coord = np.ascontiguousarray(coord, dtype=np.float64).reshape(-1, natom * 3)
        nf = coord.shape[0]
        boxa = None if box is None else np.ascontiguousarray(box, dtype=np.float64).reshape(nf, 9)
        if out is not None:
            e, f, v = out
            if not (e.flags.c_contiguous and f.flags.c_contiguous and v.flags.c_contiguous) or \
                    e.size != nf or f.size != nf * natom * 3 or v.size != nf * 9:
                raise ValueError("out arrays must be C-contiguous float64 of the output sizes")
        else:
            e = np.empty(nf)  # every output element is written by the call
            f = np.empty((nf, natom, 3))
            v = np.empty((nf, 9))
        ae = np.empty((nf, natom)) if atomic else None
        av = np.empty((nf, natom, 9)) if atomic else None
        dp = C.POINTER(C.c_double)

        def P(a):
            return C.cast(None, dp) if a is None else a.ctypes.data_as(dp)

        rc = _lib.lib().dpgb_deeppot_compute(self._h, nf, natom, P(coord), atype.ctypes.data_as(C.POINTER(C.c_int)),
                                             P(boxa), P(e), P(f), P(v), P(ae), P(av))
        _lib.check(rc)
        if atomic:
            return e, f, v, ae, av
        return e, f, v

    def eval_nlist(self, coord, atype, nghost, ilist, numneigh, firstneigh, ago=0, atomic=False):
        """One frame with explicit ghosts and the caller's neighbour list
        (DP_DeepPotComputeNList): coord [nall, 3] (local atoms first), atype
        [nall], the InputNlist arrays (firstneigh: one integer array per
        entry of ilist).  Returns energy, force [nall, 3] and virial (and the
        atomic energy [nall] / virial [nall, 9]) — forces on the ghosts
        included."""
        atype = np.ascontiguousarray(atype, dtype=np.int32).reshape(-1)
        nall = atype.shape[0]
        coord = np.ascontiguousarray(coord, dtype=np.float64).reshape(nall * 3)
        ip = C.POINTER(C.c_int)
        rows = [np.ascontiguousarray(r, dtype=np.int32) for r in (firstneigh or [])]
        fn = (ip * max(len(rows), 1))(*[r.ctypes.data_as(ip) for r in rows])
        ilist_p = numneigh_p = C.cast(None, ip)
        if ilist is not None:  # ago > 0 may pass no list
            ilist = np.ascontiguousarray(ilist, dtype=np.int32)
            numneigh = np.ascontiguousarray(numneigh, dtype=np.int32)
            ilist_p, numneigh_p = ilist.ctypes.data_as(ip), numneigh.ctypes.data_as(ip)
        e = np.zeros(1)
        f = np.zeros((nall, 3))
        v = np.zeros(9)
        ae = np.zeros(nall) if atomic else None
        av = np.zeros((nall, 9)) if atomic else None
        dp = C.POINTER(C.c_double)

        def P(a):
            return C.cast(None, dp) if a is None else a.ctypes.data_as(dp)

        rc = _lib.lib().dpgb_deeppot_compute_nlist(self._h, nall, int(nghost), P(coord), atype.ctypes.data_as(ip),
                                                   C.cast(None, dp), len(rows), ilist_p, numneigh_p, fn, int(ago),
                                                   P(e), P(f), P(v), P(ae), P(av))
        _lib.check(rc)
        if atomic:
            return e[0], f, v, ae, av
        return e[0], f, v

    def batch(self, frames):
        """A :class:`DeepPotBatch` over frames = [(coord [n_f, 3], atype [n_f],
        box [9]), ...] of different sizes."""
        return DeepPotBatch(self, frames)

    def eval_device(self, coord, box, atype, atomic: bool = False, out=None):
        """Device form: ``coord`` a CUDA float64 tensor [nframes, natom*3]
        (or [natom, 3]); ``box`` host array or None; ``atype`` host array.
        Returns CUDA tensors; nothing is synchronised."""
        import torch

        atype = np.ascontiguousarray(atype, dtype=np.int32).reshape(-1)
        natom = atype.shape[0]
        coord = coord.reshape(-1, natom * 3)
        if coord.dtype != torch.float64 or not coord.is_cuda:
            raise TypeError("coord must be a CUDA float64 tensor")
        coord = coord.contiguous()
        nf = coord.shape[0]
        boxa = None if box is None else np.ascontiguousarray(box, dtype=np.float64).reshape(nf, 9)
        if out is None:
            dev = coord.device
            out = dict(energy=torch.empty(nf, dtype=torch.float64, device=dev),
                       force=torch.empty(nf, natom, 3, dtype=torch.float64, device=dev),
                       virial=torch.empty(nf, 9, dtype=torch.float64, device=dev))
            if atomic:
                out["atom_energy"] = torch.empty(nf, natom, dtype=torch.float64, device=dev)
                out["atom_virial"] = torch.empty(nf, natom, 9, dtype=torch.float64, device=dev)
        vp = C.c_void_p
        ae = out.get("atom_energy") if atomic else None
        av = out.get("atom_virial") if atomic else None
        rc = _lib.lib().dpgb_deeppot_compute_device(
            self._h, nf, natom, vp(coord.data_ptr()), atype.ctypes.data_as(C.POINTER(C.c_int)),
            C.cast(None, C.POINTER(C.c_double)) if boxa is None else boxa.ctypes.data_as(C.POINTER(C.c_double)),
            vp(out["energy"].data_ptr()), vp(out["force"].data_ptr()), vp(out["virial"].data_ptr()),
            vp(ae.data_ptr()) if ae is not None else None, vp(av.data_ptr()) if av is not None else None,
            vp(torch.cuda.current_stream().cuda_stream))
        _lib.check(rc)
        return out


class DeepPotBatch:
    """Many periodic frames of different sizes evaluated together
    (``dpgb_batch_*``): one set of launches for all frames, optionally
    captured in a CUDA graph and replayed."""

    def __init__(self, dp: "DeepPot", frames):
        self.dp = dp
        self.natoms = np.array([len(f[1]) for f in frames], dtype=np.int32)
        self.nframes = len(frames)
        atype = np.ascontiguousarray(np.concatenate([np.asarray(f[1]) for f in frames]), dtype=np.int32)
        box = np.ascontiguousarray(np.stack([np.asarray(f[2], dtype=np.float64).reshape(9) for f in frames]))
        ip = C.POINTER(C.c_int)
        self._h = _lib.lib().dpgb_batch_new(dp._h, self.nframes, self.natoms.ctypes.data_as(ip),
                                            atype.ctypes.data_as(ip), box.ctypes.data_as(C.POINTER(C.c_double)))
        if not self._h:
            raise _lib.DpgbError(-1, _lib.lib().dpgb_last_error().decode())
        self.offsets = np.concatenate([[0], np.cumsum(self.natoms)])

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.lib().dpgb_batch_delete(self._h)
            self._h = None

    def eval(self, coords, use_graph: bool = False):
        """Host coordinates (list of [n_f, 3] arrays or the concatenation) ->
        (energy [nframes], list of forces [n_f, 3], virial [nframes, 9])."""
        if isinstance(coords, (list, tuple)):
            coords = np.concatenate([np.asarray(c, dtype=np.float64).reshape(-1, 3) for c in coords])
        c = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1)
        e = np.zeros(self.nframes)
        f = np.zeros((int(self.offsets[-1]), 3))
        v = np.zeros((self.nframes, 9))
        dp = C.POINTER(C.c_double)
        _lib.check(_lib.lib().dpgb_batch_compute(self._h, c.ctypes.data_as(dp), e.ctypes.data_as(dp),
                                                 f.ctypes.data_as(dp), v.ctypes.data_as(dp), int(use_graph)))
        return e, [f[self.offsets[k]:self.offsets[k + 1]] for k in range(self.nframes)], v

    def buckets(self):
        """(frames [4], atoms [4]) of the size buckets <= 128, <= 512,
        <= 2048 and > 2048 atoms (dpgb_batch_buckets)."""
        fr, at = (C.c_int * 4)(), (C.c_int * 4)()
        _lib.check(_lib.lib().dpgb_batch_buckets(self._h, fr, at))
        return list(fr), list(at)

    def set_tiles(self, rows_per_item):
        """Rows per work item of each size bucket (0 = the default split);
        see dpgb_batch_set_tiles."""
        t = (C.c_int * 4)(*[int(x) for x in rows_per_item])
        _lib.check(_lib.lib().dpgb_batch_set_tiles(self._h, t))

    def tiles(self):
        t = (C.c_int * 4)()
        _lib.check(_lib.lib().dpgb_batch_get_tiles(self._h, t))
        return list(t)

    def eval_device(self, coord, out=None, use_graph: bool = False, stream=None):
        """CUDA float64 coordinates [natoms, 3] -> dict of CUDA tensors on the
        current torch stream; nothing is synchronised."""
        import torch

        n = int(self.offsets[-1])
        if out is None:
            out = {"energy": torch.empty(self.nframes, dtype=torch.float64, device=coord.device),
                   "force": torch.empty((n, 3), dtype=torch.float64, device=coord.device),
                   "virial": torch.empty((self.nframes, 9), dtype=torch.float64, device=coord.device)}
        st = torch.cuda.current_stream().cuda_stream if stream is None else stream
        _lib.check(_lib.lib().dpgb_batch_compute_device(
            self._h, C.c_void_p(coord.data_ptr()), C.c_void_p(out["energy"].data_ptr()),
            C.c_void_p(out["force"].data_ptr()), C.c_void_p(out["virial"].data_ptr()), C.c_void_p(st),
            int(use_graph)))
        return out
