"""``torch.ops.deepmd.tabulate_fusion_se_a`` backed by libdpgb.

Same schema, argument meaning, autograd structure and errors as the
reference op (source/op/pt/tabulate_multi_device.cc:33-55, 731-962,
1630-1684): ``table_info`` must be a CPU tensor, every other tensor on the
table's device, dims 2/2/3, the basis dimension of ``em`` 4; first-order
backward gives d/d(em_x) and d/d(em); its own backward (the double backward)
gives d/d(dy) through the grad-grad kernel, as in the reference.

The kernels run on CUDA only: a CPU tensor raises, there is no fallback.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib

_registered = False


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


def _info_ptr(info: torch.Tensor, dtype):
    info = info.detach().to(dtype).contiguous()
    ct = C.c_double if dtype == torch.float64 else C.c_float
    arr = (ct * 6)(*[float(x) for x in info.tolist()[:6]])
    return arr


def _check(table, table_info, tensors):
    if not table_info.device.type == "cpu":
        raise RuntimeError("table_info must be on the CPU")
    for name, t in tensors:
        if t is not None and t.device != table.device:
            raise RuntimeError(f"{name} must be on the same device as table; table is on "
                               f"{table.device} but {name} is on {t.device}")
    if table.device.type != "cuda":
        raise NotImplementedError("dpgb runs tabulate_fusion_se_a on CUDA only")
    if table.dtype not in (torch.float64, torch.float32):
        raise TypeError("table must be float64 or float32")


def _sfx(t):
    return "f64" if t.dtype == torch.float64 else "f32"


def tab_forward(table, info, em_x, em, nl, is_sorted=True):
    _check(table, info, [("em_x", em_x), ("em", em)])
    if table.dim() != 2:
        raise ValueError("Dim of table should be 2")
    if em_x.dim() != 2:
        raise ValueError("Dim of input should be 2")
    if em.dim() != 3:
        raise ValueError("Dim of input should be 3")
    if em.shape[2] != 4:
        raise RuntimeError(f"The environment basis dimension must be 4, got {em.shape[2]}")
    table, em_x, em = table.contiguous(), em_x.contiguous(), em.contiguous()
    nloc, nnei = em.shape[0], em.shape[1]
    out = torch.empty((nloc, 4, nl), dtype=table.dtype, device=table.device)
    _lib.call(f"dpgb_tabulate_fusion_se_a_{_sfx(table)}", _ptr(out), _ptr(table), _info_ptr(info, table.dtype),
              _ptr(em_x), _ptr(em), nloc, nnei, int(nl), int(is_sorted), _stream())
    return out


def tab_grad(table, info, em_x, em, dy, is_sorted=True):
    _check(table, info, [("em_x", em_x), ("em", em), ("dy", dy)])
    if dy.dim() != 3:
        raise ValueError("Dim of dy_tensor should be 3")
    table, em_x, em, dy = table.contiguous(), em_x.contiguous(), em.contiguous(), dy.contiguous()
    nloc, nnei = em.shape[0], em.shape[1]
    dx = torch.zeros_like(em_x)
    dem = torch.zeros_like(em)
    _lib.call(f"dpgb_tabulate_fusion_se_a_grad_{_sfx(table)}", _ptr(dx), _ptr(dem), _ptr(table),
              _info_ptr(info, table.dtype), _ptr(em_x), _ptr(em), _ptr(dy), nloc, nnei, dy.shape[2],
              int(is_sorted), _stream())
    return dx, dem


def tab_grad_grad(table, info, em_x, em, dz_dx, dz_dem, nl, is_sorted=True):
    _check(table, info, [("em_x", em_x), ("em", em), ("dz_dy_dem_x", dz_dx), ("dz_dy_dem", dz_dem)])
    if dz_dx.dim() != 2:
        raise ValueError("Dim of dz_dy_dem_x should be 2")
    if dz_dem.dim() != 3:
        raise ValueError("Dim of dz_dy_dem should be 3")
    if nl > 1024:
        raise RuntimeError("In the process of model compression, the size of the last layer of "
                           "embedding net must be less than 1024!")
    table, em_x, em = table.contiguous(), em_x.contiguous(), em.contiguous()
    dz_dx, dz_dem = dz_dx.contiguous(), dz_dem.contiguous()
    nloc, nnei = em.shape[0], em.shape[1]
    out = torch.empty((nloc, 4, nl), dtype=table.dtype, device=table.device)
    _lib.call(f"dpgb_tabulate_fusion_se_a_grad_grad_{_sfx(table)}", _ptr(out), _ptr(table),
              _info_ptr(info, table.dtype), _ptr(em_x), _ptr(em), _ptr(dz_dx), _ptr(dz_dem), nloc, nnei,
              int(nl), int(is_sorted), _stream())
    return out


class _TabGradFn(torch.autograd.Function):
    """TabulateFusionSeAGradOp: forward = first derivative, backward = grad-grad
    with respect to dy only (tabulate_multi_device.cc:731-831)."""

    @staticmethod
    def forward(ctx, table, info, em_x, em, dy, nl):
        ctx.save_for_backward(table, info, em_x, em)
        ctx.nl = nl
        return tab_grad(table, info, em_x, em, dy)

    @staticmethod
    def backward(ctx, dz_dx, dz_dem):
        table, info, em_x, em = ctx.saved_tensors
        dz_dx = dz_dx if dz_dx is not None else torch.zeros_like(em_x)
        dz_dem = dz_dem if dz_dem is not None else torch.zeros_like(em)
        dz_dy = tab_grad_grad(table, info, em_x, em, dz_dx, dz_dem, ctx.nl)
        return None, None, None, None, dz_dy, None


class _TabFn(torch.autograd.Function):
    """TabulateFusionSeAOp (tabulate_multi_device.cc:881-962)."""

    @staticmethod
    def forward(ctx, table, info, em_x, em, nl):
        out = tab_forward(table, info, em_x, em, nl)
        ctx.save_for_backward(table, info, em_x, em)
        ctx.nl = nl
        return out

    @staticmethod
    def backward(ctx, dy):
        table, info, em_x, em = ctx.saved_tensors
        dx, dem = _TabGradFn.apply(table, info, em_x, em, dy.contiguous(), ctx.nl)
        return None, None, dx, dem, None


def tabulate_fusion_se_a(table, table_info, em_x, em, last_layer_size):
    """The op body: returns ``[descriptor]`` like the reference."""
    return [_TabFn.apply(table, table_info, em_x, em, int(last_layer_size))]


def register() -> None:
    """Registers ``torch.ops.deepmd.tabulate_fusion_se_a`` (idempotent)."""
    global _registered
    if _registered:
        return
    if hasattr(torch.ops, "deepmd") and hasattr(torch.ops.deepmd, "tabulate_fusion_se_a"):
        _registered = True
        return
    _lib.lib()  # fail loudly now if the CUDA library is missing
    lib = torch.library.Library("deepmd", "FRAGMENT")
    lib.define("tabulate_fusion_se_a(Tensor table, Tensor table_info, Tensor em_x, Tensor em, "
               "int last_layer_size) -> Tensor[]")
    lib.impl("tabulate_fusion_se_a", tabulate_fusion_se_a, "CompositeImplicitAutograd")
    globals()["_library"] = lib  # keep the registration alive
    _registered = True
