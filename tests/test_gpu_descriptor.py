"""DescrptSeA / prod_env_mat drop-in (dpgb.descriptor) on the GPU: forward
against the reference model's own outputs, first and second derivatives
against torch autograd of the plain-PyTorch restatement (torch_sea_ref), and
central finite differences (FP64, h = 1e-5) for forces and for the gradient
of a force loss with respect to embedding weights."""
import numpy as np
import pytest

from conftest import golden, water_params

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _strip(sd, prefix="atomic_model.descriptor."):
    return {k[len(prefix):]: torch.as_tensor(v) for k, v in sd.items() if k.startswith(prefix)}


def _water_desc(cuda, precision="float64", **kw):
    from dpgb.descriptor import DescrptSeA

    p = water_params()
    c = p.config
    args = dict(rcut=c.rcut, rcut_smth=c.rcut_smth, sel=c.sel, neuron=c.neuron, axis_neuron=c.axis_neuron,
                type_one_side=c.type_one_side, resnet_dt=c.resnet_dt, precision=precision, device=cuda)
    args.update(kw)
    d = DescrptSeA(**args)
    if not kw:
        d.load_state_dict(_strip(p.to_state_dict()), strict=False)
    return d


def _water_inputs(cuda, dtype=torch.float64):
    g = golden("water192")
    coord_ext = torch.tensor(g["coord_ext"], dtype=dtype, device=cuda).reshape(1, -1)
    atype_ext = torch.tensor(g["atype"][g["mapping"]], dtype=torch.int64, device=cuda).reshape(1, -1)
    nlist = torch.tensor(g["nlist"], dtype=torch.int64, device=cuda).reshape(1, 192, -1)
    return g, coord_ext, atype_ext, nlist


def test_descriptor_forward_matches_reference_model(cuda):
    d = _water_desc(cuda)
    g, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    desc, rot, g2, h2, sw = d(coord_ext, atype_ext, nlist)
    assert g2 is None and h2 is None
    assert desc.shape == (1, 192, 1600) and rot.shape == (1, 192, 100, 3) and sw.shape == (1, 192, 138, 1)
    ref_d, ref_r, ref_sw = g["descriptor"], g["rot_mat"], g["sw"]
    np.testing.assert_allclose(desc[0, :8].detach().cpu().numpy(), ref_d, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(rot[0, :8].detach().cpu().numpy(), ref_r, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(sw[0, :8, :, 0].detach().cpu().numpy(), ref_sw, rtol=1e-12, atol=1e-14)


def test_prod_env_mat_matches_reference_model(cuda):
    from dpgb.descriptor import prod_env_mat

    p = water_params()
    g, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    mean = torch.tensor(p.mean, device=cuda)
    std = torch.tensor(p.stddev, device=cuda)
    em, diff, sw = prod_env_mat(coord_ext, nlist, atype_ext[:, :192], mean, std, 6.0, 0.5)
    np.testing.assert_allclose(em[0, :8].detach().cpu().numpy(), g["env_mat"], rtol=1e-12, atol=1e-14)


def _rand_like(t, seed):
    gen = torch.Generator(device=t.device).manual_seed(seed)
    return torch.randn(t.shape, dtype=t.dtype, device=t.device, generator=gen)


@pytest.mark.parametrize("protection", [0.0, 0.05])
def test_env_mat_first_and_second_derivative(cuda, protection):
    import torch_sea_ref as R
    from dpgb.descriptor import prod_env_mat

    g, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    gen = torch.Generator(device=cuda).manual_seed(3)
    mean = 0.1 * torch.randn((2, 138, 4), dtype=torch.float64, device=cuda, generator=gen)
    std = 1.0 + 0.2 * torch.rand((2, 138, 4), dtype=torch.float64, device=cuda, generator=gen)
    atype = atype_ext[:, :192]
    outs = []
    for fn in (prod_env_mat, R.env_mat):
        x = coord_ext.clone().requires_grad_(True)
        em, diff, sw = fn(x, nlist, atype, mean, std, 6.0, 0.5, protection=protection)
        ge, gd, gs = _rand_like(em, 1), _rand_like(diff, 2), _rand_like(sw, 4)
        ge.requires_grad_(True)
        (gx,) = torch.autograd.grad((em, diff, sw), x, (ge, gd, gs), create_graph=True)
        u = _rand_like(gx, 5)
        phi = (gx * u).sum()
        gg_x, gg_e = torch.autograd.grad(phi, (x, ge))
        outs.append([t.detach() for t in (em, diff, sw, gx, gg_x, gg_e)])
    names = ["em", "diff", "sw", "grad", "hvp", "jvp"]
    for n, a, b in zip(names, outs[0], outs[1]):
        scale = b.abs().max().item()
        err = (a - b).abs().max().item()
        assert err <= 1e-11 * max(scale, 1.0), f"{n}: max err {err} (scale {scale})"


@pytest.mark.parametrize("variant", ["two_side", "one_side_resnet", "exclude"])
def test_block_first_and_second_derivative(cuda, variant):
    import torch_sea_ref as R
    from dpgb.descriptor import prod_env_mat

    kw = {}
    if variant == "one_side_resnet":
        kw = dict(type_one_side=True, resnet_dt=True, seed=7)
    elif variant == "exclude":
        kw = dict(exclude_types=[[0, 1]], seed=9)
    d = _water_desc(cuda, **kw) if kw else _water_desc(cuda)
    sea = d.sea
    g, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    em, _, _ = prod_env_mat(coord_ext, nlist, atype_ext[:, :192], sea.mean, sea.stddev, 6.0, 0.5)
    rr0 = em.view(192, 138, 4).detach()
    flat0 = sea.flat_params().detach()
    keep = torch.as_tensor(sea._keep) if variant == "exclude" else None
    outs = []
    for impl in ("dpgb", "torch"):
        rr = rr0.clone().requires_grad_(True)
        flat = flat0.clone().requires_grad_(True)
        if impl == "dpgb":
            from dpgb.descriptor import _BlockFn

            D, X = _BlockFn.apply(rr, flat, nlist.to(torch.int32).contiguous(),
                                  atype_ext.to(torch.int32).contiguous(), sea._block_desc(), 1, 192, 5184)
        else:
            nets = R.nets_from_flat(flat, 2, sea.neuron, sea.type_one_side, sea.resnet_dt)
            D, X = R.block(rr, nlist, atype_ext, nets, sea.sel, sea.type_one_side, sea.resnet_dt, 16, keep)
        gD, gX = _rand_like(D, 11), _rand_like(X, 12)
        gD.requires_grad_(True)
        g_rr, g_par = torch.autograd.grad((D, X), (rr, flat), (gD, gX), create_graph=True)
        u = _rand_like(g_rr, 13)
        phi = (g_rr * u).sum()
        gg_rr, gg_par, gg_D = torch.autograd.grad(phi, (rr, flat, gD))
        outs.append([t.detach() for t in (D, X, g_rr, g_par, gg_rr, gg_par, gg_D)])
    names = ["D", "xyz", "grad_rr", "grad_params", "gg_rr", "gg_params", "gg_descriptor"]
    for n, a, b in zip(names, outs[0], outs[1]):
        scale = b.abs().max().item()
        err = (a - b).abs().max().item()
        assert err <= 1e-10 * max(scale, 1e-3), f"{n}: max err {err} (scale {scale})"


def test_block_float32_forward(cuda):
    d64 = _water_desc(cuda)
    d32 = _water_desc(cuda, precision="float32")
    d32.load_state_dict({k: v.float() if v.is_floating_point() else v for k, v in d64.state_dict().items()})
    g, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    a = d64(coord_ext, atype_ext, nlist)[0]
    b = d32(coord_ext, atype_ext, nlist)[0]
    assert b.dtype == torch.float64  # cast to the global precision like the reference
    err = (a - b).abs().max().item()
    assert err <= 2e-5 * a.abs().max().item()


def _energy(d, coord_ext, atype_ext, nlist, c):
    desc = d(coord_ext, atype_ext, nlist)[0]
    return torch.tanh(desc @ c).sum()


def test_descriptor_forces_finite_difference(cuda):
    d = _water_desc(cuda)
    g, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    c = _rand_like(torch.empty((1600,), dtype=torch.float64, device=cuda), 21) * 0.05
    x = coord_ext.clone().requires_grad_(True)
    (gx,) = torch.autograd.grad(_energy(d, x, atype_ext, nlist, c), x)
    gen = np.random.default_rng(5)
    h = 1e-5
    for k in gen.choice(192 * 3, size=12, replace=False):
        xp = coord_ext.clone()
        xm = coord_ext.clone()
        xp[0, k] += h
        xm[0, k] -= h
        with torch.no_grad():
            fd = (_energy(d, xp, atype_ext, nlist, c) - _energy(d, xm, atype_ext, nlist, c)).item() / (2 * h)
        an = gx[0, k].item()
        assert abs(an - fd) <= 1e-6 * max(abs(fd), 1e-3 * gx.abs().max().item()), (k, an, fd)


def test_force_loss_weight_gradient_finite_difference(cuda):
    """d/dW of a force loss through the hand-written double backward vs
    central differences in FP64 (h = 1e-5)."""
    d = _water_desc(cuda)
    g, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    c = _rand_like(torch.empty((1600,), dtype=torch.float64, device=cuda), 31) * 0.05
    fref = _rand_like(coord_ext, 32) * 1e-3

    def loss():
        x = coord_ext.clone().requires_grad_(True)
        (gx,) = torch.autograd.grad(_energy(d, x, atype_ext, nlist, c), x, create_graph=True)
        return ((-gx - fref) ** 2).sum()

    params = list(d.sea.filter_layers.parameters())
    L = loss()
    grads = torch.autograd.grad(L, params)
    gen = np.random.default_rng(8)
    h = 1e-5
    gmax = max(gr.abs().max().item() for gr in grads)
    checked = 0
    for pi in gen.choice(len(params), size=8, replace=False):
        p, gr = params[pi], grads[pi]
        k = int(gen.integers(p.numel()))
        old = p.view(-1)[k].item()
        with torch.no_grad():
            p.view(-1)[k] = old + h
        lp = loss().item()  # the loss itself takes a gradient: not under no_grad
        with torch.no_grad():
            p.view(-1)[k] = old - h
        lm = loss().item()
        with torch.no_grad():
            p.view(-1)[k] = old
        fd = (lp - lm) / (2 * h)
        an = gr.view(-1)[k].item()
        assert abs(an - fd) <= 1e-6 * max(abs(fd), 1e-3 * gmax), (pi, k, an, fd)
        checked += 1
    assert checked == 8


def test_cpu_tensor_is_rejected():
    from dpgb.descriptor import prod_env_mat

    x = torch.zeros((1, 6), dtype=torch.float64)
    nl = torch.full((1, 1, 2), -1, dtype=torch.int64)
    with pytest.raises(NotImplementedError):
        prod_env_mat(x, nl, torch.zeros((1, 1), dtype=torch.int64), torch.zeros((1, 2, 4), dtype=torch.float64),
                     torch.ones((1, 2, 4), dtype=torch.float64), 6.0, 0.5)


def test_table_build_on_gpu_matches_reference_tables(cuda):
    from conftest import assert_table_close
    from dpgb.tabulate import build_tables

    d = _water_desc(cuda)
    g = golden("water192_compressed")
    data, lo, up = build_tables(d, float(g["min_nbor_dist"]), float(g["extrapolate"]), float(g["stride0"]),
                                float(g["stride1"]))
    for e in range(4):
        ii, ti = e // 2, e % 2
        name = f"filter_{ti}_net_{ii}"
        assert [lo[name], up[name]] == [int(x) for x in g[f"info_{e}"][:2]]
        assert_table_close(data[name].cpu().numpy(), g[f"table_{e}"], lo[name], up[name], float(g["stride0"]),
                           float(g["stride1"]))


def test_compressed_descriptor(cuda):
    """enable_compression with dpgb's GPU tables gives the descriptor of the
    reference's own tables (installed through the block API) and stays close
    to the uncompressed net."""
    g = golden("water192_compressed")
    _, coord_ext, atype_ext, nlist = _water_inputs(cuda)
    plain = _water_desc(cuda)(coord_ext, atype_ext, nlist)[0]
    d1 = _water_desc(cuda)
    d1.enable_compression(float(g["min_nbor_dist"]), float(g["extrapolate"]), float(g["stride0"]),
                          float(g["stride1"]))
    a = d1(coord_ext, atype_ext, nlist)[0]
    d2 = _water_desc(cuda)
    names = {f"filter_{e % 2}_net_{e // 2}": e for e in range(4)}
    d2.sea.enable_compression({n: torch.as_tensor(g[f"table_{e}"]) for n, e in names.items()},
                              [float(g["extrapolate"]), float(g["stride0"]), float(g["stride1"]), -1],
                              {n: g[f"info_{e}"][0] for n, e in names.items()},
                              {n: g[f"info_{e}"][1] for n, e in names.items()})
    b = d2(coord_ext, atype_ext, nlist)[0]
    assert d1.sea.compress and d1.need_sorted_nlist_for_lower()
    assert (a - b).abs().max().item() <= 1e-10 * b.abs().max().item()
    assert (a - plain).abs().max().item() <= 1e-3 * plain.abs().max().item()
