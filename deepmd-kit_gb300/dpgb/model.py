"""se_e2_a energy model and the energy/force loss, for inference through
autograd and for force-loss training, on the dpgb descriptor kernels.

Mirrors ``deepmd.pt`` ``EnergyModel`` (deepmd/pt/model/model/make_model.py:
136-220; the energy fitting of deepmd/pt/model/task/fitting.py:734-899; the
outputs of deepmd/pt/model/model/transform_output.py:68-209) and
``EnergyStdLoss`` (deepmd/pt/loss/ener.py:216-330, the mean-squared energy /
force / virial terms with prefactors interpolated by the learning rate).

The descriptor is :class:`dpgb.descriptor.DescrptSeA`, whose environment
matrix and embedding block carry hand-written CUDA first and second
derivatives; the fitting net is a plain per-type MLP in torch (its GEMMs are
library GEMMs).  Forces are -dE/dr through autograd on the extended
coordinates and reduced to the local atoms through the ghost mapping;
``create_graph=True`` keeps them differentiable for force-loss training.
State-dict keys are the reference's (``atomic_model.descriptor.*``,
``atomic_model.fitting_net.*``, ``atomic_model.out_bias``,
``atomic_model.out_std``), so a reference checkpoint's state dict loads
unchanged.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np
import torch

from . import nlist as N
from .descriptor import PRECISION, DescrptSeA


class _Layer(torch.nn.Module):
    def __init__(self, nin, nout, bias, idt, dtype, device, gen):
        super().__init__()
        std = 1.0 / np.sqrt(nin + nout)
        self.matrix = torch.nn.Parameter(torch.tensor(gen.normal(0, std, (nin, nout)), dtype=dtype, device=device))
        self.bias = (torch.nn.Parameter(torch.tensor(gen.normal(0, 1, (nout,)), dtype=dtype, device=device))
                     if bias else None)
        self.idt = (torch.nn.Parameter(torch.tensor(gen.normal(0.1, 0.001, (nout,)), dtype=dtype, device=device))
                    if idt else None)


class _FitNet(torch.nn.Module):
    def __init__(self, dim, neuron, resnet_dt, dtype, device, gen):
        super().__init__()
        widths = [dim, *neuron]
        layers = []
        for l in range(len(neuron)):
            nin, nout = widths[l], widths[l + 1]
            # the timestep exists only where a skip connection does (mlp.py:90-92)
            layers.append(_Layer(nin, nout, True, resnet_dt and (nout == nin or nout == 2 * nin), dtype, device, gen))
        layers.append(_Layer(widths[-1], 1, True, False, dtype, device, gen))
        self.layers = torch.nn.ModuleList(layers)

    def forward(self, x):
        for layer in self.layers[:-1]:
            y = torch.tanh(x @ layer.matrix + layer.bias)
            if layer.idt is not None:
                y = y * layer.idt
            nin, nout = layer.matrix.shape
            if nout == nin:
                y = y + x
            elif nout == 2 * nin:
                y = y + torch.cat([x, x], dim=-1)
            x = y
        out = self.layers[-1]
        return x @ out.matrix + out.bias


class _Networks(torch.nn.Module):
    def __init__(self, nets):
        super().__init__()
        self.networks = torch.nn.ModuleList(nets)


class EnergyFittingNet(torch.nn.Module):
    """Per-type energy fitting (fitting.py:734-899): atom energy =
    MLP_t(D) + bias_atom_e[t]."""

    def __init__(self, ntypes, dim_descrpt, neuron=(240, 240, 240), resnet_dt=True, precision="float64",
                 seed=None, device="cuda"):
        super().__init__()
        self.ntypes = ntypes
        self.prec = PRECISION[precision]
        gen = np.random.default_rng(seed if isinstance(seed, int) else 1)
        self.filter_layers = _Networks([_FitNet(dim_descrpt, list(neuron), resnet_dt, self.prec, device, gen)
                                        for _ in range(ntypes)])
        self.register_buffer("bias_atom_e", torch.zeros((ntypes, 1), dtype=self.prec, device=device))

    def forward(self, descriptor, atype):
        """descriptor [nf, nloc, dim], atype [nf, nloc] -> atom energy [nf, nloc, 1]."""
        x = descriptor.to(self.prec)
        out = torch.zeros(x.shape[:2] + (1,), dtype=self.prec, device=x.device)
        for t, net in enumerate(self.filter_layers.networks):
            mask = (atype == t).unsqueeze(-1)
            out = out + torch.where(mask, net(x) + self.bias_atom_e[t], torch.zeros_like(out))
        return out


class _AtomicModel(torch.nn.Module):
    def __init__(self, descriptor, fitting_net, ntypes, prec, device):
        super().__init__()
        self.descriptor = descriptor
        self.fitting_net = fitting_net
        self.register_buffer("out_bias", torch.zeros((1, ntypes, 1), dtype=prec, device=device))
        # kept for the state dict (base_atomic_model.py:134-145); the energy
        # output adds out_bias only
        self.register_buffer("out_std", torch.ones((1, ntypes, 1), dtype=prec, device=device))


class EnergyModelSeA(torch.nn.Module):
    """se_e2_a energy model: forward(coord [nf, nloc*3], atype [nf, nloc],
    box [nf, 9] or None) -> {energy [nf, 1], atom_energy [nf, nloc, 1],
    force [nf, nloc, 3], virial [nf, 9], atom_virial [nf, nloc, 9] when
    asked} (make_model.py:136-220, transform_output.py:68-209)."""

    def __init__(self, descriptor: DescrptSeA, fitting_net: EnergyFittingNet, type_map=None):
        super().__init__()
        sea = descriptor.sea
        self.type_map = type_map
        self.atomic_model = _AtomicModel(descriptor, fitting_net, sea.ntypes, sea.prec, sea.mean.device)

    @classmethod
    def from_params(cls, params, device="cuda", precision="float64"):
        """A model with the weights of a dpgb.params.SeAParams (the reference
        state-dict layout)."""
        c = params.config
        d = DescrptSeA(c.rcut, c.rcut_smth, c.sel, neuron=c.neuron, axis_neuron=c.axis_neuron,
                       type_one_side=c.type_one_side, resnet_dt=c.resnet_dt, exclude_types=c.exclude_types,
                       precision=precision, device=device)
        f = EnergyFittingNet(c.ntypes, c.dim_descrpt, c.fit_neuron, c.fit_resnet_dt, precision=precision,
                             device=device)
        m = cls(d, f)
        sd = m.state_dict()
        for k, v in params.to_state_dict().items():
            if k in sd:
                sd[k] = torch.as_tensor(np.asarray(v), dtype=sd[k].dtype).reshape(sd[k].shape)
        m.load_state_dict(sd)
        return m

    def get_rcut(self):
        return self.atomic_model.descriptor.get_rcut()

    def get_sel(self):
        return self.atomic_model.descriptor.get_sel()

    def get_ntypes(self):
        return self.atomic_model.descriptor.get_ntypes()

    def forward(self, coord, atype, box=None, fparam=None, aparam=None, do_atomic_virial=False,
                create_graph=None) -> Dict[str, torch.Tensor]:
        desc = self.atomic_model.descriptor
        prec = desc.prec
        if create_graph is None:
            create_graph = torch.is_grad_enabled() and any(p.requires_grad for p in self.parameters())
        coord = coord.to(prec)
        nf = coord.shape[0]
        coord = coord.reshape(nf, -1, 3)
        nloc = coord.shape[1]
        atype = atype.reshape(nf, nloc)
        box_h = None if box is None else box.detach().to(torch.float64).cpu().numpy().reshape(nf, 9)
        with torch.no_grad():  # wrap, images and typed list: integer metadata
            ext0, ext_t, mapping, nl = N.extend_input_and_build_neighbor_list(
                coord.detach().to(torch.float64), atype, desc.get_rcut(), desc.get_sel(), box_h)
        # the extended coordinates as a differentiable function of coord: the
        # wrap and the image shifts are constant offsets
        mapping = mapping.long()
        offset = ext0.to(prec) - torch.gather(coord.detach(), 1, mapping.unsqueeze(-1).expand(-1, -1, 3))
        with torch.enable_grad():
            coord_g = coord if coord.requires_grad else coord.detach().requires_grad_(True)
            ext = torch.gather(coord_g, 1, mapping.unsqueeze(-1).expand(-1, -1, 3)) + offset
            d, _, _, _, _ = desc(ext.reshape(nf, -1), ext_t.long(), nl.long())
            atom_e = self.atomic_model.fitting_net(d, atype)
            atom_e = atom_e + torch.where(atype.unsqueeze(-1) >= 0,
                                          self.atomic_model.out_bias[0, atype.clamp(min=0)],
                                          torch.zeros_like(atom_e))
            energy = atom_e.sum(dim=1)
            (g_ext,) = torch.autograd.grad(energy.sum(), ext, create_graph=create_graph)
        force_ext = -g_ext
        force = torch.zeros_like(coord_g).index_add(1, mapping[0], force_ext) if nf == 1 else torch.stack(
            [torch.zeros_like(coord_g[f]).index_add(0, mapping[f], force_ext[f]) for f in range(nf)])
        # virial = -sum over extended atoms of dE/dr (x) r (transform_output.py:68-209)
        atom_vir_ext = torch.einsum("fai,faj->faij", force_ext, ext).reshape(nf, -1, 9)
        out = {"energy": energy, "atom_energy": atom_e, "force": force, "virial": atom_vir_ext.sum(dim=1)}
        if do_atomic_virial:
            out["atom_virial"] = torch.stack([torch.zeros((nloc, 9), dtype=prec, device=coord.device).index_add(
                0, mapping[f], atom_vir_ext[f]) for f in range(nf)])
        return out


class EnergyStdLoss(torch.nn.Module):
    """Energy / force / virial mean-squared loss of deepmd/pt/loss/ener.py:
    216-330, 636-680: pref = limit + (start - limit) * lr / starter_lr;
    loss = pref_e * find_e * mean(dE^2) / natoms^k + pref_f * find_f * mean(dF^2)
         + pref_v * find_v * mean(dV^2) / natoms^k, k = 2 with
    ``intensive_ener_virial`` else 1.  A term is on when both its start and
    limit prefactors are nonzero (ener.py:160-162); ``find_<label>`` is 0
    unless the label dict sets it, and a figure whose label is not found
    displays as NaN (deepmd/pt/loss/loss.py:74-84)."""

    def __init__(self, starter_learning_rate=1.0, start_pref_e=0.02, limit_pref_e=1.0, start_pref_f=1000.0,
                 limit_pref_f=1.0, start_pref_v=0.0, limit_pref_v=0.0, intensive_ener_virial=False, **kwargs):
        super().__init__()
        self.starter_learning_rate = starter_learning_rate
        self.start_pref_e, self.limit_pref_e = start_pref_e, limit_pref_e
        self.start_pref_f, self.limit_pref_f = start_pref_f, limit_pref_f
        self.start_pref_v, self.limit_pref_v = start_pref_v, limit_pref_v
        self.has_e = start_pref_e != 0.0 and limit_pref_e != 0.0
        self.has_f = start_pref_f != 0.0 and limit_pref_f != 0.0
        self.has_v = start_pref_v != 0.0 and limit_pref_v != 0.0
        self.norm_exp = 2 if intensive_ener_virial else 1

    def forward(self, input_dict, model, label, natoms, learning_rate, mae=False):
        pred = model(**input_dict)
        coef = learning_rate / self.starter_learning_rate
        pref_e = self.limit_pref_e + (self.start_pref_e - self.limit_pref_e) * coef
        pref_f = self.limit_pref_f + (self.start_pref_f - self.limit_pref_f) * coef
        pref_v = self.limit_pref_v + (self.start_pref_v - self.limit_pref_v) * coef
        # the reference weights the energy and virial terms by 1 / (number of
        # real atoms) taken from an integer atom mask, which torch divides in
        # single precision (ener.py:262-266): the same float32 value here
        atom_norm = float(np.float32(1.0) / np.float32(natoms))
        loss = torch.zeros((), dtype=torch.float64, device=pred["energy"].device)
        more = {}
        norm = atom_norm ** self.norm_exp

        def shown(v, find):
            return v if bool(find) else torch.nan

        if self.has_e and "energy" in label:
            find = float(label.get("find_energy", 0.0))
            l2 = torch.mean(torch.square(pred["energy"] - label["energy"].reshape(pred["energy"].shape)))
            loss = loss + norm * (pref_e * find * l2)
            more["rmse_e"] = shown(l2.detach().sqrt() * atom_norm, find)
        if self.has_f and "force" in label:
            find = float(label.get("find_force", 0.0))
            l2 = torch.mean(torch.square(pred["force"] - label["force"].reshape(pred["force"].shape)))
            loss = loss + pref_f * find * l2
            more["rmse_f"] = shown(l2.detach().sqrt(), find)
        if self.has_v and "virial" in label:
            find = float(label.get("find_virial", 0.0))
            l2 = torch.mean(torch.square(pred["virial"] - label["virial"].reshape(pred["virial"].shape)))
            loss = loss + norm * (pref_v * find * l2)
            more["rmse_v"] = shown(l2.detach().sqrt() * atom_norm, find)
        more["rmse"] = loss.detach().sqrt()
        return pred, loss, more
