"""Compression tables of se_e2_a embedding nets, built on the GPU.

Mirrors ``DPTabulate(...).build(min_nbor_dist, extrapolate, stride0,
stride1)`` for se_e2_a (deepmd/utils/tabulate.py:67-148, 275-370,
468-498; deepmd/pt/utils/tabulate.py): the per-type range comes from the
descriptor's davg/dstd and the nearest neighbour distance, and each net's
table (quintic coefficients per interval and neuron) is computed by
``dpgb_se_a_table_build_f64`` (csrc/table_build.cu).  Tables are named
``filter_{ti}_net_{ii}`` (``filter_-1_net_{ii}`` with type_one_side), as the
reference names them.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib


def _switch(x, rmin, rmax):
    if x < rmin:
        return 1.0
    if x < rmax:
        uu = (x - rmin) / (rmax - rmin)
        return uu * uu * uu * (-6 * uu * uu + 15 * uu - 10) + 1
    return 0.0


def env_mat_range(davg, dstd, min_nbor_dist, rcut_smth, rcut):
    """Per-type [lower, upper] of the tabulated input (tabulate.py:468-498 and
    the per-type reduction of build(), 91-96)."""
    sw = _switch(float(min_nbor_dist), rcut_smth, rcut)
    davg = np.asarray(davg, dtype=np.float64)
    dstd = np.asarray(dstd, dtype=np.float64)
    lower = np.floor(-davg[:, 0] / dstd[:, 0])
    upper = np.ceil(((1 / min_nbor_dist) * sw - davg[:, 0]) / dstd[:, 0])
    if lower.ndim > 1:
        lower = np.min(lower, axis=tuple(range(1, lower.ndim)))
        upper = np.max(upper, axis=tuple(range(1, upper.ndim)))
    return lower, upper


def compress_params(params, min_nbor_dist, extrapolate=5, stride0=0.01, stride1=0.1, device="cuda"):
    """A copy of a SeAParams model with GPU-built tables installed (the
    DeepPot compressed form): tables[e] / table_info[e] per embedding net."""
    import copy

    from .descriptor import DescrptSeA

    c = params.config
    d = DescrptSeA(c.rcut, c.rcut_smth, c.sel, neuron=c.neuron, axis_neuron=c.axis_neuron,
                   type_one_side=c.type_one_side, resnet_dt=c.resnet_dt, exclude_types=c.exclude_types,
                   device=device)
    sd = {k[len("atomic_model.descriptor."):]: torch.as_tensor(v) for k, v in params.to_state_dict().items()
          if k.startswith("atomic_model.descriptor.")}
    d.load_state_dict(sd, strict=False)
    data, lo, up = build_tables(d, min_nbor_dist, extrapolate, stride0, stride1)
    nt = len(c.sel)
    out = copy.copy(params)
    out.tables, out.table_info = [], []
    for e in range(len(params.emb)):
        name = f"filter_-1_net_{e}" if c.type_one_side else f"filter_{e % nt}_net_{e // nt}"
        out.tables.append(data[name].double().cpu().numpy())
        out.table_info.append(np.array([lo[name], up[name], up[name] * extrapolate, stride0, stride1, -1.0]))
    return out


def build_tables(descrpt, min_nbor_dist, extrapolate=5, stride0=0.01, stride1=0.1):
    """(data {name: table [nspline, 6*ng] on the descriptor's device}, lower
    {name: int}, upper {name: int}) for a dpgb DescrptSeA / DescrptBlockSeA."""
    sea = getattr(descrpt, "sea", descrpt)
    nt = sea.ntypes
    lower, upper = env_mat_range(sea.mean.detach().cpu().numpy(), sea.stddev.detach().cpu().numpy(), min_nbor_dist,
                                 sea.rcut_smth, sea.rcut)
    params = sea.flat_params().detach().to(torch.float64).contiguous()
    if params.device.type != "cuda":
        raise NotImplementedError("dpgb builds compression tables on CUDA only")
    blk = sea._block_desc()
    excl = {tuple(t) for t in sea.exclude_types}
    data, lo, up = {}, {}, {}
    ng = sea.neuron[-1]
    lib = _lib.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    nnets = nt if sea.type_one_side else nt * nt
    for e in range(nnets):
        if sea.type_one_side:
            name = f"filter_-1_net_{e}"
            idx = [(ti, e) not in excl and sea.sel[ti] > 0 for ti in range(nt)]
            if not any(idx):
                continue
            ll, uu = float(np.min(lower[idx])), float(np.max(upper[idx]))
        else:
            ii, ti = e // nt, e % nt
            name = f"filter_{ti}_net_{ii}"
            if (ti, ii) in excl:
                continue
            ll, uu = float(lower[ti]), float(upper[ti])
        nrow = lib.dpgb_se_a_table_rows(ll, uu, float(extrapolate), float(stride0), float(stride1))
        if nrow < 1:
            raise ValueError(f"empty tabulation range for {name}: [{ll}, {uu}]")
        table = torch.empty((nrow, 6 * ng), dtype=torch.float64, device=params.device)
        _lib.call("dpgb_se_a_table_build_f64", C.c_void_p(table.data_ptr()), C.byref(blk),
                  C.c_void_p(params.data_ptr()), e, ll, uu, float(extrapolate), float(stride0), float(stride1),
                  stream)
        data[name] = table.to(sea.prec)
        lo[name] = int(ll)
        up[name] = int(uu)
    return data, lo, up
