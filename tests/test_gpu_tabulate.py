"""GPU: torch.ops.deepmd.tabulate_fusion_se_a (libdpgb) against the reference
op's golden vectors (source/tests/pt/test_tabulate_fusion_se_a.py, FP64 1e-10,
FP32 1e-5), the oracle on random inputs, the second-order finite-difference
check of source/tests/pt/tabulate_test_utils.py, and the edge cases of
source/lib/tests/test_tabulate_se_a.cc (empty neighbour axis, padding)."""
import numpy as np
import pytest

from conftest import golden

import oracle as O

pytestmark = pytest.mark.gpu


def _op():
    import torch
    from dpgb import ops

    ops.register()
    return torch.ops.deepmd.tabulate_fusion_se_a


@pytest.mark.parametrize("dtype_name,prec", [("float64", 1e-10), ("float32", 1e-5)])
def test_golden_forward_backward(cuda, dtype_name, prec):
    import torch

    dt = getattr(torch, dtype_name)
    g = golden("tabulate_se_a_op")
    table = torch.tensor(g["table"], dtype=dt, device=cuda)
    info = torch.tensor(g["table_info"], dtype=dt)
    em_x = torch.tensor(g["em_x"], dtype=dt, device=cuda, requires_grad=True)
    em = torch.tensor(g["em"], dtype=dt, device=cuda, requires_grad=True)
    out = _op()(table, info, em_x, em, int(g["last_layer_size"]))[0]
    torch.testing.assert_close(out.cpu(), torch.tensor(g["descriptor"], dtype=dt), atol=prec, rtol=prec)
    out.sum().backward()
    torch.testing.assert_close(em_x.grad.cpu(), torch.tensor(g["dy_dem_x"], dtype=dt), atol=prec, rtol=prec)
    torch.testing.assert_close(em.grad.cpu(), torch.tensor(g["dy_dem"], dtype=dt), atol=prec, rtol=prec)


def _nonuniform_like(t):
    import torch

    return torch.linspace(-0.5, 0.75, t.numel(), dtype=t.dtype, device=t.device).reshape_as(t)


def test_second_order_matches_finite_difference(cuda):
    """dz/dy of the grad-grad kernel vs central differences (eps 1e-6, FP64)."""
    import torch

    g = golden("tabulate_se_a_op")
    dt = torch.float64
    table = torch.tensor(g["table"], dtype=dt, device=cuda)
    info = torch.tensor(g["table_info"], dtype=dt)
    em_x = torch.tensor(g["em_x"], dtype=dt, device=cuda, requires_grad=True)
    em = torch.tensor(g["em"], dtype=dt, device=cuda, requires_grad=True)
    desc = _op()(table, info, em_x, em, int(g["last_layer_size"]))[0]
    dy = _nonuniform_like(desc).requires_grad_(True)
    first = torch.autograd.grad(desc, (em_x, em), grad_outputs=dy, create_graph=True, retain_graph=True)
    weights = [_nonuniform_like(x) for x in first]
    proj = sum((a * w).sum() for a, w in zip(first, weights))
    dz_dy = torch.autograd.grad(proj, dy, retain_graph=True)[0]

    def project(dyv):
        fg = torch.autograd.grad(desc, (em_x, em), grad_outputs=dyv, retain_graph=True)
        return sum((a * w).sum() for a, w in zip(fg, weights))

    ref = torch.empty_like(dy)
    eps = 1e-6
    base = dy.detach()
    for i in range(dy.numel()):
        p, m = base.clone(), base.clone()
        p.view(-1)[i] += eps
        m.view(-1)[i] -= eps
        ref.view(-1)[i] = (project(p) - project(m)) / (2 * eps)
    torch.testing.assert_close(dz_dy, ref, atol=1e-6, rtol=1e-6)


@pytest.mark.parametrize("dtype_name", ["float64", "float32"])
@pytest.mark.parametrize("nnei", [1, 7, 46, 92])
def test_random_vs_oracle(cuda, dtype_name, nnei):
    import torch

    dt = getattr(torch, dtype_name)
    npd = np.float64 if dtype_name == "float64" else np.float32
    tol = 1e-12 if dtype_name == "float64" else 2e-5
    rng = np.random.default_rng(nnei)
    # a realistic table: 100 neurons, strides 0.01/0.1, extrapolation x5
    nl = 100
    lower, upper, extrap, s0, s1 = -0.5, 2.0, 5.0, 0.01, 0.1
    nspl = int((upper - lower) / s0) + int((extrap * upper - upper) / s1) + 2
    table = rng.normal(scale=0.3, size=(nspl, 6 * nl))
    info = np.array([lower, upper, extrap * upper, s0, s1, -1.0])
    nloc = 37
    em = rng.normal(scale=0.4, size=(nloc, nnei, 4))
    em_x = rng.uniform(-0.8, 11.0, size=(nloc * nnei, 1))  # below lower, inside, beyond max
    npad = nnei // 3
    if npad:
        em[:, -npad:, :] = 0.0
        em_x.reshape(nloc, nnei)[:, -npad:] = 0.0
        em[:, -npad:, 0] = 0.0
    args = [x.astype(npd) for x in (table, info, em_x, em)]
    ref = O.tabulate_fusion_se_a(*args, nl)
    t = lambda a: torch.tensor(a, device=cuda)
    from dpgb import ops

    out = ops.tab_forward(t(args[0]), torch.tensor(args[1]), t(args[2]), t(args[3]), nl)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(out.cpu().numpy(), ref, atol=tol * scale, rtol=tol)
    dy = rng.normal(size=ref.shape).astype(npd)
    rdx, rdem = O.tabulate_fusion_se_a_grad(*args, dy)
    dx, dem = ops.tab_grad(t(args[0]), torch.tensor(args[1]), t(args[2]), t(args[3]), t(dy))
    np.testing.assert_allclose(dx.cpu().numpy(), rdx, atol=tol * np.abs(rdx).max(), rtol=tol)
    np.testing.assert_allclose(dem.cpu().numpy(), rdem, atol=tol * np.abs(rdem).max(), rtol=tol)
    dzx = rng.normal(size=em_x.shape).astype(npd)
    dzm = rng.normal(size=em.shape).astype(npd)
    rdz = O.tabulate_fusion_se_a_grad_grad(*args, dzx, dzm, nl)
    dz = ops.tab_grad_grad(t(args[0]), torch.tensor(args[1]), t(args[2]), t(args[3]), t(dzx), t(dzm), nl)
    np.testing.assert_allclose(dz.cpu().numpy(), rdz, atol=tol * np.abs(rdz).max(), rtol=tol)


def test_empty_neighbor_axis(cuda):
    import torch
    from dpgb import ops

    table = torch.zeros(4, 6 * 8, dtype=torch.float64, device=cuda)
    info = torch.tensor([0, 0.2, 0.4, 0.01, 0.1, -1], dtype=torch.float64)
    em_x = torch.zeros(0, 1, dtype=torch.float64, device=cuda)
    em = torch.zeros(3, 0, 4, dtype=torch.float64, device=cuda)
    out = ops.tab_forward(table, info, em_x, em, 8)
    assert out.shape == (3, 4, 8) and float(out.abs().sum()) == 0.0
    dx, dem = ops.tab_grad(table, info, em_x, em, torch.ones(3, 4, 8, dtype=torch.float64, device=cuda))
    assert dx.numel() == 0 and dem.numel() == 0


def test_device_contract_errors(cuda):
    import torch

    g = golden("tabulate_se_a_op")
    table = torch.tensor(g["table"], device=cuda)
    with pytest.raises(RuntimeError, match="table_info must be on the CPU"):
        _op()(table, torch.tensor(g["table_info"], device=cuda), torch.tensor(g["em_x"], device=cuda),
              torch.tensor(g["em"], device=cuda), 8)
    with pytest.raises(RuntimeError, match="must be on the same device"):
        _op()(table, torch.tensor(g["table_info"]), torch.tensor(g["em_x"]), torch.tensor(g["em"], device=cuda), 8)
