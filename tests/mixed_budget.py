"""Per-stage error budget of the mixed-precision se_e2_a path (test
infrastructure): the model written with torch in FP64 (forces by autograd)
with the roundings of the GPU's mixed form injected one stage at a time, so
each stage's share of the force / energy error against FP64 can be read off.

Stages (the CUDA kernels they emulate):
  env       FP32 environment matrix (emb_tc.cu pair_env, tab_fused.cu slot_env)
  emb_op    operands of the embedding layers 2 and 3 (A: activations, W:
            weights): "bf16" one BF16 rounding, "split" hi + lo BF16
  emb_grad  the gradient operands dP3, dP2 of the embedding backward MMAs
  emb_tanh  tanh.approx.f32 in the embedding (relative error within 2^-11)
  D         the descriptor D as the first fitting GEMM reads it
  fit1_op   first fitting layer operands (D and W1)
  fit1_grad its backward operand dP1 (fit_dxyz)
  fit_op    fitting layers 2.. operands
  fit_grad  their backward operands
  fit_tanh  tanh.approx.f32 in the fitting
An operand mode is "act:weight" or one mode for both; the gradient modes
round the gradient arriving at the GEMM output, which is what the GPU's
backward GEMMs read.
"""
import numpy as np
import torch


def _bf16(x):
    return x.to(torch.bfloat16).to(torch.float64)


def _split(x):
    hi = _bf16(x)
    return hi + _bf16(x - hi)


ROUND = {"bf16": _bf16, "split": _split, "fp32": lambda x: x.float().double(), "none": lambda x: x}


class _Fwd(torch.autograd.Function):  # rounds the value, passes the gradient
    @staticmethod
    def forward(ctx, x, mode):
        return ROUND[mode](x)

    @staticmethod
    def backward(ctx, g):
        return g, None


class _Bwd(torch.autograd.Function):  # passes the value, rounds the gradient
    @staticmethod
    def forward(ctx, x, mode):
        ctx.mode = mode
        return x.clone()

    @staticmethod
    def backward(ctx, g):
        return ROUND[ctx.mode](g), None


def _qf(x, mode):
    return x if mode == "none" else _Fwd.apply(x, mode)


def _qb(x, mode):
    return x if mode == "none" else _Bwd.apply(x, mode)


def _tanh(z, approx, key):
    t = torch.tanh(z)
    if not approx:
        return t
    g = torch.Generator().manual_seed(key)
    return t * (1 + (torch.rand(z.shape, generator=g, dtype=torch.float64) * 2 - 1) * 2.0 ** -11)


def _gemm(a, w, op, grad):
    ma, mw = op.split(":") if ":" in op else (op, op)
    wr = ROUND[mw](w)
    return _qb(_qf(a, ma) @ wr, grad)


def energy(coord_ext, nlist, atype_ext, params, S):
    c = params.config
    nloc = nlist.shape[0]
    mask = torch.tensor(nlist >= 0)
    nl = torch.tensor(np.where(nlist >= 0, nlist, 0))
    diff = coord_ext[nl] - coord_ext[:nloc][:, None, :]
    r = torch.linalg.norm(torch.where(mask[..., None], diff, torch.ones_like(diff)), dim=-1)
    rr = torch.clamp(r, c.rcut_smth, c.rcut)
    uu = (rr - c.rcut_smth) / (c.rcut - c.rcut_smth)
    sw = uu ** 3 * (-6 * uu ** 2 + 15 * uu - 10) + 1
    em = torch.cat([(1 / r)[..., None], diff / (r ** 2)[..., None]], -1) * (sw * mask)[..., None]
    em = _qf(em, S.get("env", "none"))
    sec = np.concatenate([[0], np.cumsum(c.sel)])
    at = torch.tensor(atype_ext[:nloc])
    xyz = torch.zeros(nloc, 4, c.ng, dtype=torch.float64)
    et = S.get("emb_tanh") == "approx"
    for e, layers in enumerate(params.emb):
        ii, ti = (e, None) if c.type_one_side else (e // c.ntypes, e % c.ntypes)
        rows = torch.arange(nloc) if ti is None else (at == ti).nonzero().squeeze(1)
        R = em[rows][:, sec[ii]:sec[ii + 1], :]
        x = R[..., :1]
        h = x
        for l, (w, b, _) in enumerate(layers):
            w, b = torch.tensor(w), torch.tensor(b)
            z = (h @ w if l == 0 else _gemm(h, w, S.get("emb_op", "none"), S.get("emb_grad", "none"))) + b
            y = _tanh(z, et, 1000 * e + l)
            if w.shape[1] == w.shape[0]:
                y = y + h
            elif w.shape[1] == 2 * w.shape[0]:
                y = y + torch.cat([h, h], -1)
            h = y
        xyz = xyz.index_add(0, rows, R.transpose(1, 2) @ h)
    xyz = xyz / c.nnei
    D = (xyz.transpose(1, 2) @ xyz[:, :, :c.axis_neuron]).reshape(nloc, -1)
    D = _qf(D, S.get("D", "none"))
    E = torch.zeros((), dtype=torch.float64)
    ft = S.get("fit_tanh") == "approx"
    for t, layers in enumerate(params.fit):
        rows = (at == t).nonzero().squeeze(1)
        x = D[rows]
        for l, (w, b, idt) in enumerate(layers[:-1]):
            w = torch.tensor(w)
            op = S.get("fit1_op" if l == 0 else "fit_op", "none")
            gr = S.get("fit1_grad" if l == 0 else "fit_grad", "none")
            y = _tanh(_gemm(x, w, op, gr) + torch.tensor(b), ft, 10 * t + l)
            if idt is not None:
                y = y * torch.tensor(idt)
            if w.shape[0] == w.shape[1]:
                y = y + x
            x = y
        w, b, _ = layers[-1]
        out = x @ torch.tensor(w)
        E = E + (out + torch.tensor(b)).sum() if b is not None else E + out.sum()
    return E + float(np.sum(params.atom_ener_bias()[atype_ext[:nloc]]))


def forces(coord, atype, box, params, S):
    """(energy, forces [natoms, 3]) of one periodic frame under stage settings S."""
    import oracle as O

    c = params.config
    cn = O.normalize_coord(coord, box)
    ext, ext_t, mapping = O.extend_coord_with_ghosts(cn, atype, box, c.rcut)
    nl = O.build_nlist_pt(ext, ext_t, coord.shape[0], c.rcut, c.sel)
    x = torch.tensor(ext, requires_grad=True)
    E = energy(x, nl, ext_t, params, S)
    (g,) = torch.autograd.grad(E, x)
    F = np.zeros((coord.shape[0], 3))
    np.add.at(F, mapping, -g.numpy().reshape(-1, 3))
    return float(E.detach()), F


# the mixed form as built: FP32 environment; the embedding with split-BF16
# activations and (forward) weights, BF16 gradient operands, tanh.approx;
# the fitting with D in BF16, split weights, split activations of the hidden
# layers, the first layer's gradient split, the others BF16, accurate tanh
AS_BUILT = {"env": "fp32", "emb_op": "split:split", "emb_grad": "bf16", "emb_tanh": "approx", "D": "bf16",
            "fit1_op": "bf16:split", "fit1_grad": "split", "fit_op": "split:split", "fit_grad": "bf16"}
# everything in single BF16 roundings with tanh.approx (the form before the splits)
ALL_BF16 = {"env": "fp32", "emb_op": "bf16", "emb_grad": "bf16", "emb_tanh": "approx", "D": "bf16",
            "fit1_op": "bf16", "fit1_grad": "bf16", "fit_op": "bf16", "fit_grad": "bf16", "fit_tanh": "approx"}


def budget(params, coord, atype, box, cases):
    """{name: (force RMSE, relative to the RMS force, |dE| per atom)}."""
    e0, f0 = forces(coord, atype, box, params, {})
    rms = float(np.sqrt(np.mean(f0 ** 2)))
    out = {}
    for name, S in cases.items():
        e, f = forces(coord, atype, box, params, S)
        rmse = float(np.sqrt(np.mean((f - f0) ** 2)))
        out[name] = (rmse, rmse / rms, abs(e - e0) / coord.shape[0])
    return rms, out
