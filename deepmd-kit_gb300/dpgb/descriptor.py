"""``DescrptSeA`` / ``prod_env_mat`` with the deepmd.pt API, on libdpgb kernels.

Drop-in for ``deepmd.pt.model.descriptor.se_a.DescrptSeA`` /
``DescrptBlockSeA`` (deepmd/pt/model/descriptor/se_a.py:92-858) and
``deepmd.pt.model.descriptor.env_mat.prod_env_mat`` (env_mat.py:58-119):
same constructor arguments, forward signature and outputs, state-dict keys
(``sea.mean``, ``sea.stddev``, ``sea.filter_layers.networks.{e}.layers.{l}.
{matrix,bias,idt}``, ``sea.compress_data.{e}``, ``sea.compress_info.{e}``),
so a reference state dict loads unchanged.

Every derivative is written by hand in CUDA behind ``torch.autograd.Function``:
the environment matrix (first and second derivative with respect to the
coordinates, ``csrc/env_mat_pt.cu``) and the embedding block (first and
second derivative with respect to the environment matrix and the embedding
parameters, activations recomputed, ``csrc/se_a_block.cu``).  Forces through
``torch.autograd.grad`` and force-loss training (grad of grad) therefore run
on these kernels.  The compressed form calls ``torch.ops.deepmd.
tabulate_fusion_se_a`` (``dpgb.ops``), as the reference does.

``precision="mixed"`` (a dpgb option beside the reference's float64 /
float32) runs the block on the mixed form's kernels instead: the tcgen05
embedding GEMMs (split BF16, FP32 accumulation) fused with the environment
matrix and the contraction to D — or, compressed, the fused FP32 table
kernels — through ``dpgb_deeppot_descrpt_fwd`` / ``_bwd``.  Its autograd
gives dE/d coordinates (forces) but no weight gradients and no second
derivative: an inference option (the parameters stay FP64).

CUDA tensors only: there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch
from torch.autograd.function import once_differentiable

from . import _lib

PRECISION = {"float64": torch.float64, "float32": torch.float32, "double": torch.float64,
             "single": torch.float32, "default": torch.float64,
             "mixed": torch.float64}  # mixed: FP64 parameters, mixed-form kernels


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _sfx(dtype):
    if dtype == torch.float64:
        return "f64"
    if dtype == torch.float32:
        return "f32"
    raise TypeError(f"dpgb descriptor kernels take float64 or float32, not {dtype}")


def _cuda_only(*ts):
    for t in ts:
        if t is not None and t.device.type != "cuda":
            raise NotImplementedError("dpgb descriptor kernels run on CUDA tensors only (no CPU path)")


def _c(t, dtype=None):
    if t is None:
        return None
    if dtype is not None:
        t = t.to(dtype)
    return t.contiguous()


# ---------------------------------------------------------------------------
# environment matrix


class _EnvMatFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coord, nlist, atype, mean, stddev, rcut, rcut_smth, protection):
        nf, nloc, nnei = nlist.shape
        nall = coord.shape[1] // 3
        dt = coord.dtype
        em = torch.empty((nf, nloc, nnei, 4), dtype=dt, device=coord.device)
        diff = torch.empty((nf, nloc, nnei, 3), dtype=dt, device=coord.device)
        sw = torch.empty((nf, nloc, nnei, 1), dtype=dt, device=coord.device)
        _lib.call(f"dpgb_env_mat_pt2_{_sfx(dt)}", _p(em), _p(diff), _p(sw), _p(coord), _p(atype), _p(nlist),
                  _p(mean), _p(stddev), nf, nloc, nall, nnei, float(rcut), float(rcut_smth), float(protection),
                  _stream())
        ctx.save_for_backward(coord, nlist, atype, stddev)
        ctx.cfg = (float(rcut), float(rcut_smth), float(protection))
        return em, diff, sw

    @staticmethod
    def backward(ctx, g_em, g_diff, g_sw):
        coord, nlist, atype, stddev = ctx.saved_tensors
        g_coord = None
        if ctx.needs_input_grad[0]:
            g_coord = _EnvMatBwdFn.apply(_c(g_em), _c(g_diff), _c(g_sw), coord, nlist, atype, stddev, ctx.cfg)
        return g_coord, None, None, None, None, None, None, None


class _EnvMatBwdFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, g_em, g_diff, g_sw, coord, nlist, atype, stddev, cfg):
        nf, nloc, nnei = nlist.shape
        nall = coord.shape[1] // 3
        g_coord = torch.empty_like(coord)
        _lib.call(f"dpgb_env_mat_pt_bwd_{_sfx(coord.dtype)}", _p(g_coord), _p(g_em), _p(g_diff), _p(g_sw),
                  _p(coord), _p(atype), _p(nlist), _p(stddev), nf, nloc, nall, nnei, cfg[0], cfg[1], cfg[2], _stream())
        ctx.save_for_backward(g_em, g_diff, g_sw, coord, nlist, atype, stddev)
        ctx.cfg = cfg
        ctx.has = (g_em is not None, g_diff is not None, g_sw is not None)
        return g_coord

    @staticmethod
    @once_differentiable
    def backward(ctx, u):
        g_em, g_diff, g_sw, coord, nlist, atype, stddev = ctx.saved_tensors
        nf, nloc, nnei = nlist.shape
        nall = coord.shape[1] // 3
        u = u.contiguous()
        dt = coord.dtype
        gg_em = torch.empty((nf, nloc, nnei, 4), dtype=dt, device=coord.device)
        gg_diff = torch.empty((nf, nloc, nnei, 3), dtype=dt, device=coord.device) if ctx.has[1] else None
        gg_sw = torch.empty((nf, nloc, nnei, 1), dtype=dt, device=coord.device) if ctx.has[2] else None
        gg_coord = torch.empty_like(coord) if ctx.needs_input_grad[3] else None
        cfg = ctx.cfg
        _lib.call(f"dpgb_env_mat_pt_bwd_bwd_{_sfx(dt)}", _p(gg_em), _p(gg_diff), _p(gg_sw), _p(gg_coord), _p(u),
                  _p(g_em), _p(g_diff), _p(g_sw), _p(coord), _p(atype), _p(nlist), _p(stddev), nf, nloc, nall, nnei,
                  cfg[0], cfg[1], cfg[2], _stream())
        return (gg_em if ctx.has[0] else None, gg_diff, gg_sw, gg_coord, None, None, None, None)


def prod_env_mat(extended_coord, nlist, atype, mean, stddev, rcut: float, rcut_smth: float,
                 radial_only: bool = False, protection: float = 0.0, use_exp_switch: bool = False):
    """Smooth environment matrix (deepmd/pt/model/descriptor/env_mat.py:58-119).

    extended_coord [nf, nall*3], nlist [nf, nloc, nnei], atype [nf, nloc],
    mean / stddev [ntypes, nnei, 4] -> (env_mat [nf, nloc, nnei, 4],
    diff [nf, nloc, nnei, 3], sw [nf, nloc, nnei, 1]), differentiable twice
    with respect to extended_coord.
    """
    if radial_only or use_exp_switch:
        raise NotImplementedError("se_e2_a uses the full 4-vector and the polynomial switch only")
    _cuda_only(extended_coord, nlist, atype, mean, stddev)
    dt = extended_coord.dtype
    nf = nlist.shape[0]
    coord = extended_coord.reshape(nf, -1)
    return _EnvMatFn.apply(coord.contiguous(), nlist.to(torch.int32).contiguous(),
                           atype.to(torch.int32).contiguous(), _c(mean, dt), _c(stddev, dt), rcut, rcut_smth,
                           protection)


# ---------------------------------------------------------------------------
# the block on the mixed form's kernels


class _MixedBlockFn(torch.autograd.Function):
    """D (and xyz) of the block from extended coordinates through a mixed
    DeepPot handle's descriptor stage; backward: dE/dD -> dE/d coordinates."""

    @staticmethod
    def forward(ctx, coord, handle, nlist, atype_ext, atype_loc, nf, nloc, nall, ng, dim):
        D = torch.empty((nf, nloc, dim), dtype=torch.float32, device=coord.device)
        X = torch.empty((nf, nloc, 4, ng), dtype=torch.float32, device=coord.device)
        ticket = C.c_ulonglong(0)
        _lib.call("dpgb_deeppot_descrpt_fwd", handle._h, nf, nloc, nall, _p(coord), _p(atype_ext),
                  atype_loc.ctypes.data_as(C.POINTER(C.c_int)), _p(nlist), _p(D), _p(X), C.byref(ticket), _stream())
        ctx.handle, ctx.shape, ctx.ticket = handle, (nf, nall), ticket.value
        ctx.mark_non_differentiable(X)
        return D, X

    @staticmethod
    @once_differentiable
    def backward(ctx, gD, gX):
        nf, nall = ctx.shape
        g = torch.empty((nf, nall * 3), dtype=torch.float64, device=gD.device)
        _lib.call("dpgb_deeppot_descrpt_bwd", ctx.handle._h, ctx.ticket, _p(gD.to(torch.float32).contiguous()), _p(g),
                  _stream())
        return g, None, None, None, None, None, None, None, None, None


# ---------------------------------------------------------------------------
# embedding block


class _BlockFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rr, params, nlist, atype_ext, blk, nf, nloc, nall):
        dt = rr.dtype
        nnei = rr.shape[1]
        ng, M = blk.neuron[blk.n_layer - 1], blk.axis_neuron
        D = torch.empty((nf * nloc, ng * M), dtype=dt, device=rr.device)
        X = torch.empty((nf * nloc, 4, ng), dtype=dt, device=rr.device)
        _lib.call(f"dpgb_se_a_block_fwd_{_sfx(dt)}", C.byref(blk), _p(params), _p(rr), _p(nlist), _p(atype_ext),
                  nf, nloc, nall, _p(D), _p(X), _stream())
        ctx.save_for_backward(rr, params, nlist, atype_ext, X)
        ctx.cfg = (blk, nf, nloc, nall, nnei)
        return D, X

    @staticmethod
    def backward(ctx, gD, gX):
        rr, params, nlist, atype_ext, X = ctx.saved_tensors
        if gD is None:
            gD = torch.zeros((rr.shape[0], X.shape[2] * ctx.cfg[0].axis_neuron), dtype=rr.dtype, device=rr.device)
        g_rr, g_par = _BlockBwdFn.apply(gD.contiguous(), _c(gX), rr, params, nlist, atype_ext, X,
                                        ctx.needs_input_grad[1], ctx.cfg)
        return (g_rr if ctx.needs_input_grad[0] else None, g_par if ctx.needs_input_grad[1] else None,
                None, None, None, None, None, None)


def _workspace(blk, nf, nloc, dtype, device):
    nbytes = _lib.lib().dpgb_se_a_block_workspace_bytes(C.byref(blk), nf, nloc, 8 if dtype == torch.float64 else 4)
    return torch.empty((max(int(nbytes), 1),), dtype=torch.uint8, device=device), int(nbytes)


class _BlockBwdFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, gD, gX, rr, params, nlist, atype_ext, X, want_par, cfg):
        blk, nf, nloc, nall, nnei = cfg
        dt = rr.dtype
        g_rr = torch.empty_like(rr)
        g_par = torch.zeros_like(params)
        ws, nbytes = (None, 0)
        if want_par:
            ws, nbytes = _workspace(blk, nf, nloc, dt, rr.device)
        _lib.call(f"dpgb_se_a_block_bwd_{_sfx(dt)}", C.byref(blk), _p(params), _p(rr), _p(nlist), _p(atype_ext),
                  nf, nloc, nall, _p(X), _p(gD), _p(gX), _p(g_rr), _p(g_par) if want_par else C.c_void_p(0),
                  _p(ws), C.c_size_t(nbytes), _stream())
        ctx.save_for_backward(gD, gX, rr, params, nlist, atype_ext)
        ctx.cfg = cfg
        ctx.has_gX = gX is not None
        return g_rr, g_par

    @staticmethod
    @once_differentiable
    def backward(ctx, u_rr, u_par):
        gD, gX, rr, params, nlist, atype_ext = ctx.saved_tensors
        blk, nf, nloc, nall, nnei = ctx.cfg
        if u_par is not None and bool((u_par != 0).any()):
            raise NotImplementedError("the derivative of the embedding-parameter gradient is not provided")
        dt = rr.dtype
        ng = gD.shape[1] // blk.axis_neuron
        if u_rr is None:
            u_rr = torch.zeros_like(rr)
        u_rr = u_rr.contiguous()
        gg_D = torch.empty_like(gD)
        gg_X = torch.empty((rr.shape[0], 4, ng), dtype=dt, device=rr.device) if ctx.has_gX else None
        gg_rr = torch.empty_like(rr)
        want_par = ctx.needs_input_grad[3]
        gg_par = torch.zeros_like(params)
        ws, nbytes = (None, 0)
        if want_par:
            ws, nbytes = _workspace(blk, nf, nloc, dt, rr.device)
        _lib.call(f"dpgb_se_a_block_bwd_bwd_{_sfx(dt)}", C.byref(blk), _p(params), _p(rr), _p(nlist),
                  _p(atype_ext), nf, nloc, nall, _p(gD), _p(gX), _p(u_rr), _p(gg_D), _p(gg_X), _p(gg_rr),
                  _p(gg_par) if want_par else C.c_void_p(0), _p(ws), C.c_size_t(nbytes), _stream())
        return (gg_D, gg_X, gg_rr, gg_par if want_par else None, None, None, None, None, None)


# ---------------------------------------------------------------------------
# modules with the reference's structure and state-dict names


class MLPLayer(torch.nn.Module):
    """One embedding layer: y = tanh(x W + b) [* idt] (+ x, + [x, x]) — the
    parameter names of deepmd/pt/model/network/mlp.py:81-219.  As there, the
    timestep idt exists only where a skip connection does (nout == nin or
    2 nin, mlp.py:89-92): never on the first layer (1 -> neuron[0])."""

    def __init__(self, nin, nout, resnet_dt, dtype, device, gen):
        super().__init__()
        std = 1.0 / np.sqrt(nin + nout)
        self.matrix = torch.nn.Parameter(
            torch.tensor(gen.normal(0.0, std, size=(nin, nout)), dtype=dtype, device=device))
        self.bias = torch.nn.Parameter(torch.tensor(gen.normal(0.0, 1.0, size=(nout,)), dtype=dtype, device=device))
        self.idt = (torch.nn.Parameter(torch.tensor(gen.normal(0.1, 0.001, size=(nout,)), dtype=dtype, device=device))
                    if resnet_dt and (nout == nin or nout == 2 * nin) else None)


class EmbeddingNet(torch.nn.Module):
    def __init__(self, neuron, resnet_dt, dtype, device, gen):
        super().__init__()
        widths = [1, *neuron]
        self.layers = torch.nn.ModuleList(
            [MLPLayer(widths[i], widths[i + 1], resnet_dt, dtype, device, gen) for i in range(len(neuron))])


class NetworkCollection(torch.nn.Module):
    def __init__(self, nets):
        super().__init__()
        self.networks = torch.nn.ModuleList(nets)


class DescrptBlockSeA(torch.nn.Module):
    """se_e2_a block (deepmd/pt/model/descriptor/se_a.py:480-858)."""

    def __init__(self, rcut, rcut_smth, sel, neuron=(25, 50, 100), axis_neuron=16, set_davg_zero=False,
                 activation_function="tanh", precision="float64", resnet_dt=False, exclude_types=(),
                 env_protection=0.0, type_one_side=True, trainable=True, seed=None, device="cuda", **kwargs):
        super().__init__()
        if activation_function != "tanh":
            raise NotImplementedError("the dpgb kernels implement the tanh embedding only")
        if isinstance(sel, int):
            sel = [sel]
        self.rcut = float(rcut)
        self.rcut_smth = float(rcut_smth)
        self.neuron = list(neuron)
        self.filter_neuron = self.neuron
        self.axis_neuron = int(axis_neuron)
        self.set_davg_zero = set_davg_zero
        self.activation_function = activation_function
        self.precision = precision
        self.prec = PRECISION[precision]
        self.resnet_dt = bool(resnet_dt)
        self.env_protection = float(env_protection)
        self.ntypes = len(sel)
        self.type_one_side = bool(type_one_side)
        self.seed = seed
        self.sel = list(sel)
        self.sec = [0, *np.cumsum(self.sel).tolist()]
        self.split_sel = self.sel
        self.nnei = sum(self.sel)
        self.ndescrpt = self.nnei * 4
        if self.ntypes > _lib.MAX_TYPES or len(self.neuron) > _lib.MAX_LAYERS:
            raise ValueError("too many types or embedding layers for the dpgb kernels")
        self.reinit_exclude(list(exclude_types))
        shape = (self.ntypes, self.nnei, 4)
        self.register_buffer("mean", torch.zeros(shape, dtype=self.prec, device=device))
        self.register_buffer("stddev", torch.ones(shape, dtype=self.prec, device=device))
        gen = np.random.default_rng(seed if isinstance(seed, int) else 0)
        nnets = self.ntypes if self.type_one_side else self.ntypes ** 2
        self.filter_layers = NetworkCollection(
            [EmbeddingNet(self.neuron, self.resnet_dt, self.prec, device, gen) for _ in range(nnets)])
        self.trainable = trainable
        for p in self.parameters():
            p.requires_grad = trainable
        self.compress = False
        self.compress_info = torch.nn.ParameterList(
            [torch.nn.Parameter(torch.zeros(0, dtype=self.prec, device="cpu")) for _ in range(nnets)])
        self.compress_data = torch.nn.ParameterList(
            [torch.nn.Parameter(torch.zeros(0, dtype=self.prec, device=device)) for _ in range(nnets)])
        self.stats = None

    # ---- reference accessors
    def get_rcut(self):
        return self.rcut

    def get_rcut_smth(self):
        return self.rcut_smth

    def get_nsel(self):
        return sum(self.sel)

    def get_sel(self):
        return self.sel

    def get_ntypes(self):
        return self.ntypes

    def get_dim_out(self):
        return self.dim_out

    def get_dim_rot_mat_1(self):
        return self.filter_neuron[-1]

    def get_dim_emb(self):
        return self.neuron[-1]

    def get_dim_in(self):
        return 0

    def mixed_types(self):
        return False

    def get_env_protection(self):
        return self.env_protection

    @property
    def dim_out(self):
        return self.filter_neuron[-1] * self.axis_neuron

    @property
    def dim_in(self):
        return 0

    def has_message_passing(self):
        return False

    def need_sorted_nlist_for_lower(self):
        return self.compress

    def __setitem__(self, key, value):
        if key in ("avg", "data_avg", "davg"):
            self.mean = value
        elif key in ("std", "data_std", "dstd"):
            self.stddev = value
        else:
            raise KeyError(key)

    def __getitem__(self, key):
        if key in ("avg", "data_avg", "davg"):
            return self.mean
        if key in ("std", "data_std", "dstd"):
            return self.stddev
        raise KeyError(key)

    def reinit_exclude(self, exclude_types=()):
        self.exclude_types = [tuple(t) for t in exclude_types]
        keep = np.ones((self.ntypes + 1, self.ntypes + 1), dtype=np.int32)
        for a, b in self.exclude_types:
            keep[a, b] = 0
            keep[b, a] = 0
        self._keep = keep

    def _block_desc(self):
        b = _lib.SeABlock()
        b.ntypes = self.ntypes
        for t, s in enumerate(self.sel):
            b.sel[t] = s
        b.type_one_side = int(self.type_one_side)
        b.n_layer = len(self.neuron)
        for i, w in enumerate(self.neuron):
            b.neuron[i] = w
        b.axis_neuron = self.axis_neuron
        b.resnet_dt = int(self.resnet_dt)
        stride = _lib.MAX_TYPES + 1
        for a in range(self.ntypes + 1):
            for c in range(self.ntypes + 1):
                b.pair_keep[a * stride + c] = int(self._keep[a, c])
        return b

    def flat_params(self):
        """All embedding parameters as one vector in the kernels' layout
        (with resnet_dt every layer has an idt slot; a layer without a
        timestep gets ones there, an exact no-op)."""
        parts = []
        for net in self.filter_layers.networks:
            for layer in net.layers:
                parts += [layer.matrix.reshape(-1), layer.bias.reshape(-1)]
                if self.resnet_dt:
                    parts.append(layer.idt.reshape(-1) if layer.idt is not None
                                 else torch.ones_like(layer.bias).reshape(-1))
        return torch.cat(parts)

    def enable_compression(self, table_data, table_config, lower, upper):
        """Install tables (se_a.py:692-724): per net name "filter_{ti}_net_{ii}"
        ("filter_-1_net_{ii}" for type_one_side)."""
        for e in range(len(self.filter_layers.networks)):
            if self.type_one_side:
                ii, ti = e, -1
            else:
                ii, ti = e // self.ntypes, e % self.ntypes
            net = f"filter_{ti}_net_{ii}"
            info = torch.as_tensor([lower[net], upper[net], upper[net] * table_config[0], table_config[1],
                                    table_config[2], table_config[3]], dtype=self.prec, device="cpu")
            self.compress_data[e] = torch.nn.Parameter(
                torch.as_tensor(table_data[net]).to(device=self.mean.device, dtype=self.prec), requires_grad=False)
            self.compress_info[e] = torch.nn.Parameter(info, requires_grad=False)
        self.compress = True

    def forward(self, nlist, extended_coord, extended_atype, extended_atype_embd=None, mapping=None,
                type_embedding=None):
        del extended_atype_embd, mapping, type_embedding
        nf, nloc, nnei = nlist.shape
        if nnei != self.nnei:
            raise ValueError(f"nlist has {nnei} slots, the descriptor expects sum(sel) = {self.nnei}")
        _cuda_only(extended_coord, nlist, extended_atype)
        coord = extended_coord.reshape(nf, -1).to(self.prec)
        nall = coord.shape[1] // 3
        atype = extended_atype[:, :nloc]
        nl32 = nlist.to(torch.int32).contiguous()
        if self.precision == "mixed":
            return self._mixed_forward(coord, nl32, extended_atype, atype, nf, nloc, nall)
        dmatrix, diff, sw = prod_env_mat(coord, nl32, atype, self.mean, self.stddev, self.rcut, self.rcut_smth,
                                         protection=self.env_protection)
        rr = dmatrix.view(nf * nloc, self.nnei, 4)
        if self.compress:
            X = self._compressed_xyz(rr, nl32, extended_atype, atype, nf, nloc)
            xs1 = X.permute(0, 2, 1)
            D = torch.matmul(xs1, X[:, :, : self.axis_neuron]).view(nf * nloc, -1)
        else:
            D, X = _BlockFn.apply(rr, self.flat_params(), nl32, extended_atype.to(torch.int32).contiguous(),
                                  self._block_desc(), nf, nloc, nall)
        rot_mat = X.permute(0, 2, 1)[:, :, 1:4]
        ng = self.filter_neuron[-1]
        return (D.view(nf, nloc, ng * self.axis_neuron), rot_mat.reshape(nf, nloc, ng, 3), None, None, sw)

    def _mixed_params(self):
        """The block as an SeAParams (with a zero 16-wide fitting the
        descriptor stage never runs), for a mixed DeepPot handle."""
        from .params import SeAConfig, SeAParams

        cfg = SeAConfig(sel=list(self.sel), rcut=self.rcut, rcut_smth=self.rcut_smth, neuron=list(self.neuron),
                        axis_neuron=self.axis_neuron, type_one_side=self.type_one_side, resnet_dt=self.resnet_dt,
                        fit_neuron=[16], fit_resnet_dt=False, exclude_types=[list(t) for t in self.exclude_types])
        npf = lambda t: t.detach().to(torch.float64).cpu().numpy()  # noqa: E731
        emb = [[(npf(l.matrix), npf(l.bias), npf(l.idt) if l.idt is not None else None) for l in net.layers]
               for net in self.filter_layers.networks]
        dim = cfg.dim_descrpt
        fit = [[(np.zeros((dim, 16)), np.zeros(16), None), (np.zeros((16, 1)), np.zeros(1), None)]
               for _ in range(self.ntypes)]
        tables = infos = None
        if self.compress:
            tables = [npf(t) for t in self.compress_data]
            infos = [npf(t) for t in self.compress_info]
        return SeAParams(config=cfg, mean=npf(self.mean), stddev=npf(self.stddev), emb=emb, fit=fit,
                         bias_atom_e=np.zeros(self.ntypes), out_bias=np.zeros(self.ntypes), tables=tables,
                         table_info=infos)

    def _mixed_handle(self):
        """A mixed DeepPot handle holding the block's current weights (rebuilt
        when a parameter, the statistics or the tables change)."""
        from .deeppot import DeepPot

        key = (self.compress, tuple(t._version for t in self.parameters()), self.mean._version,
               self.stddev._version, self.mean.data_ptr(), self.stddev.data_ptr())
        cached = getattr(self, "_mixed", None)
        if cached is None or cached[0] != key:
            dev = self.mean.device.index if self.mean.device.index is not None else torch.cuda.current_device()
            self._mixed = (key, DeepPot(self._mixed_params(), "mixed", device=dev))
        return self._mixed[1]

    def _mixed_forward(self, coord, nl32, extended_atype, atype, nf, nloc, nall):
        at = atype.to(torch.int32).cpu().numpy()
        if nf > 1 and not (at == at[:1]).all():
            raise NotImplementedError("the mixed descriptor needs the same local atom types in every frame")
        ng = self.filter_neuron[-1]
        dim = ng * self.axis_neuron
        D, X = _MixedBlockFn.apply(coord.contiguous(), self._mixed_handle(), nl32,
                                   extended_atype.to(torch.int32).contiguous(), np.ascontiguousarray(at[0]), nf,
                                   nloc, nall, ng, dim)
        with torch.no_grad():  # the switch function output (not differentiated here)
            _, _, sw = prod_env_mat(coord.detach(), nl32, atype, self.mean, self.stddev, self.rcut, self.rcut_smth,
                                    protection=self.env_protection)
        rot_mat = X[:, :, 1:4, :].transpose(2, 3).to(torch.float64)
        return D.to(torch.float64), rot_mat, None, None, sw

    def _compressed_xyz(self, rr, nl32, extended_atype, atype, nf, nloc):
        """xyz_scatter of the compressed form: the reference's per-net loop
        around torch.ops.deepmd.tabulate_fusion_se_a (se_a.py:787-836)."""
        from . import ops

        ops.register()
        nfnl = nf * nloc
        ng = self.filter_neuron[-1]
        xyz = torch.zeros((nfnl, 4, ng), dtype=self.prec, device=rr.device)
        if self._keep.min() == 0:
            nall = extended_atype.shape[1]
            ae = torch.cat([extended_atype, torch.full((nf, 1), self.ntypes, dtype=extended_atype.dtype,
                                                       device=extended_atype.device)], dim=1)
            idx = torch.where(nl32 < 0, torch.full_like(nl32, nall), nl32).view(nf, -1).long()
            tj = torch.gather(ae, 1, idx).view(nfnl, self.nnei)
            ti = atype.reshape(nfnl, 1)
            keep = torch.as_tensor(self._keep, device=rr.device)
            mask = keep[ti.long(), tj.long()].to(self.prec)
        else:
            mask = None
        flat_t = atype.reshape(-1)
        for e in range(len(self.filter_layers.networks)):
            if self.type_one_side:
                ii, sel_rows = e, None
            else:
                ii, ti = e // self.ntypes, e % self.ntypes
                sel_rows = flat_t.eq(ti)
            sl = slice(self.sec[ii], self.sec[ii + 1])
            r = rr[:, sl, :] if sel_rows is None else rr[sel_rows, sl, :]
            if mask is not None:
                m = mask[:, sl] if sel_rows is None else mask[sel_rows, sl]
                r = r * m[:, :, None]
            ss = r[:, :, :1].reshape(-1, 1)
            gr = torch.ops.deepmd.tabulate_fusion_se_a(self.compress_data[e].contiguous(),
                                                       self.compress_info[e].cpu().contiguous(), ss.contiguous(),
                                                       r.contiguous(), ng)[0]
            if sel_rows is None:
                xyz = xyz + gr
            else:
                xyz = xyz.index_put((sel_rows.nonzero().squeeze(1),), gr, accumulate=True)
        return xyz / self.nnei


class DescrptSeA(torch.nn.Module):
    """deepmd.pt DescrptSeA (se_a.py:92-480) on dpgb kernels."""

    def __init__(self, rcut, rcut_smth, sel, neuron=(25, 50, 100), axis_neuron=16, set_davg_zero=False,
                 activation_function="tanh", precision="float64", resnet_dt=False, exclude_types=(),
                 env_protection=0.0, type_one_side=True, trainable=True, seed=None, ntypes=None, type_map=None,
                 spin=None, device="cuda"):
        del ntypes
        if spin is not None:
            raise NotImplementedError("old implementation of spin is not supported.")
        super().__init__()
        self.type_map = type_map
        self.compress = False
        self.prec = PRECISION[precision]
        self.sea = DescrptBlockSeA(rcut, rcut_smth, sel, neuron=neuron, axis_neuron=axis_neuron,
                                   set_davg_zero=set_davg_zero, activation_function=activation_function,
                                   precision=precision, resnet_dt=resnet_dt, exclude_types=exclude_types,
                                   env_protection=env_protection, type_one_side=type_one_side,
                                   trainable=trainable, seed=seed, device=device)

    def get_rcut(self):
        return self.sea.get_rcut()

    def get_rcut_smth(self):
        return self.sea.get_rcut_smth()

    def get_nsel(self):
        return self.sea.get_nsel()

    def get_sel(self):
        return self.sea.get_sel()

    def get_ntypes(self):
        return self.sea.get_ntypes()

    def get_type_map(self):
        return self.type_map

    def get_dim_out(self):
        return self.sea.get_dim_out()

    def get_dim_emb(self):
        return self.sea.get_dim_emb()

    def mixed_types(self):
        return self.sea.mixed_types()

    def has_message_passing(self):
        return self.sea.has_message_passing()

    def need_sorted_nlist_for_lower(self):
        return self.sea.need_sorted_nlist_for_lower()

    def get_env_protection(self):
        return self.sea.get_env_protection()

    @property
    def dim_out(self):
        return self.sea.dim_out

    def set_stat_mean_and_stddev(self, mean, stddev):
        self.sea.mean = mean
        self.sea.stddev = stddev

    def get_stat_mean_and_stddev(self):
        return self.sea.mean, self.sea.stddev

    def enable_compression(self, min_nbor_dist, table_extrapolate=5, table_stride_1=0.01, table_stride_2=0.1,
                           check_frequency=-1):
        """Tabulate the embedding nets (se_a.py:269-314) with dpgb's table
        builder and switch the forward to tabulate_fusion_se_a."""
        if self.compress:
            raise ValueError("Compression is already enabled.")
        from . import tabulate

        data, lower, upper = tabulate.build_tables(self, min_nbor_dist, table_extrapolate, table_stride_1,
                                                   table_stride_2)
        self.sea.enable_compression(data, [table_extrapolate, table_stride_1, table_stride_2, check_frequency],
                                    lower, upper)
        self.compress = True

    def forward(self, coord_ext, atype_ext, nlist, mapping=None, comm_dict=None, fparam=None, charge_spin=None):
        """(descriptor [nf, nloc, ng*M], rot_mat [nf, nloc, ng, 3], None, None,
        sw [nf, nloc, nnei, 1]) — se_a.py:316-377."""
        coord_ext = coord_ext.to(dtype=self.prec)
        g1, rot_mat, g2, h2, sw = self.sea.forward(nlist, coord_ext, atype_ext, None, mapping)
        out = torch.float64  # the reference casts to GLOBAL_PT_FLOAT_PRECISION
        return g1.to(out), rot_mat.to(out), None, None, sw.to(out)

    def serialize(self) -> dict:
        """The reference's serialised dict (se_a.py:392-423)."""
        obj = self.sea
        nets = []
        for net in obj.filter_layers.networks:
            layers = []
            for layer in net.layers:  # NativeLayer.serialize (dpmodel/utils/network.py:153-177)
                var = {"w": layer.matrix.detach().cpu().numpy(), "b": layer.bias.detach().cpu().numpy(),
                       "idt": None if layer.idt is None else layer.idt.detach().cpu().numpy()}
                layers.append({"@class": "Layer", "@version": 2, "bias": True, "use_timestep": layer.idt is not None,
                               "activation_function": obj.activation_function, "resnet": True,
                               "precision": obj.precision, "trainable": True, "@variables": var})
            # EmbeddingNet.serialize (network.py:782-801)
            nets.append({"@class": "EmbeddingNetwork", "@version": 2, "in_dim": 1, "neuron": list(obj.neuron),
                         "activation_function": obj.activation_function, "resnet_dt": obj.resnet_dt,
                         "bias": True, "precision": obj.precision, "layers": layers})
        ndim = 1 if obj.type_one_side else 2
        return {
            "@class": "Descriptor", "type": "se_e2_a", "@version": 2, "rcut": obj.rcut, "rcut_smth": obj.rcut_smth,
            "sel": obj.sel, "neuron": obj.neuron, "axis_neuron": obj.axis_neuron, "resnet_dt": obj.resnet_dt,
            "set_davg_zero": obj.set_davg_zero, "activation_function": obj.activation_function,
            "precision": obj.precision,
            "embeddings": {"@class": "NetworkCollection", "@version": 1, "ndim": ndim, "ntypes": obj.ntypes,
                           "network_type": "embedding_network",
                           "networks": nets},  # NetworkCollection.serialize (network.py:1247-1266)
            "env_mat": {"@class": "EnvMat", "@version": 1, "rcut": obj.rcut, "rcut_smth": obj.rcut_smth,
                        "protection": obj.env_protection},
            "exclude_types": obj.exclude_types, "env_protection": obj.env_protection,
            "@variables": {"davg": obj.mean.detach().cpu().numpy(), "dstd": obj.stddev.detach().cpu().numpy()},
            "type_map": self.type_map, "trainable": True, "type_one_side": obj.type_one_side, "spin": None,
        }

    @classmethod
    def deserialize(cls, data: dict, device="cuda") -> "DescrptSeA":
        data = dict(data)
        data.pop("@version", None)
        data.pop("@class", None)
        data.pop("type", None)
        variables = data.pop("@variables")
        embeddings = data.pop("embeddings")
        data.pop("env_mat", None)
        data.pop("compress", None)
        obj = cls(**data, device=device)
        sea = obj.sea
        sea.mean = torch.as_tensor(np.asarray(variables["davg"]), dtype=sea.prec, device=device)
        sea.stddev = torch.as_tensor(np.asarray(variables["dstd"]), dtype=sea.prec, device=device)
        nets = embeddings["networks"]
        if isinstance(nets, dict):
            nets = [nets[k] for k in sorted(nets, key=lambda s: int(s))]
        with torch.no_grad():
            for net, nd in zip(sea.filter_layers.networks, nets):
                for layer, ld in zip(net.layers, nd["layers"]):
                    v = ld["@variables"]
                    layer.matrix.copy_(torch.as_tensor(np.asarray(v["w"]), dtype=sea.prec))
                    layer.bias.copy_(torch.as_tensor(np.asarray(v["b"]), dtype=sea.prec))
                    if layer.idt is not None and v.get("idt") is not None:
                        layer.idt.copy_(torch.as_tensor(np.asarray(v["idt"]), dtype=sea.prec))
        return obj
