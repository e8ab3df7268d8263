"""The se_e2_a energy model and force-loss training step (dpgb.model) on the
GPU: energy / forces / virial against the reference model's outputs, the
training gradient against the reference's own FP64 autograd gradient (one
EnergyStdLoss step, tests/golden/train_grad.npz) and against central finite
differences (FP64, h = 1e-5) on the 64 recorded weights."""
import numpy as np
import pytest

from conftest import golden, water_params

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_energy_model_matches_reference(cuda):
    from dpgb.model import EnergyModelSeA

    g = golden("water192")
    m = EnergyModelSeA.from_params(water_params(), device=cuda)
    c = torch.tensor(g["coord"].reshape(1, -1), device=cuda)
    t = torch.tensor(g["atype"].reshape(1, -1), device=cuda)
    b = torch.tensor(g["box"].reshape(1, 9), device=cuda)
    out = m(c, t, b, do_atomic_virial=True)
    assert rel(out["energy"].item(), g["energy"][0]) < 1e-12
    assert rel(out["force"][0].detach().cpu().numpy(), g["force"]) < 1e-10
    assert rel(out["virial"][0].detach().cpu().numpy(), g["virial"]) < 1e-10
    assert rel(out["atom_energy"][0, :, 0].detach().cpu().numpy(), g["atom_energy"]) < 1e-10


def _train_setup(cuda):
    from dpgb import params as P
    from dpgb.model import EnergyModelSeA, EnergyStdLoss

    g = golden("train_grad")
    nf = g["coord"].shape[0]
    m = EnergyModelSeA.from_params(P.init_params(P.water_config(), seed=1), device=cuda)
    inp = {"coord": torch.tensor(g["coord"], device=cuda),
           "atype": torch.tensor(np.tile(g["atype"], (nf, 1)), device=cuda),
           "box": torch.tensor(g["box"], device=cuda)}
    label = {"energy": torch.tensor(g["energy_label"], device=cuda).reshape(nf, 1),
             "force": torch.tensor(g["force_label"], device=cuda), "find_energy": 1.0, "find_force": 1.0}
    pe, pf = g["pref"]
    loss_fn = EnergyStdLoss(1.0, pe, pe, pf, pf)
    natoms = g["atype"].shape[0]

    def loss():
        return loss_fn(inp, m, label, natoms, 1.0)[1]

    return g, m, loss


def test_force_loss_gradient_matches_reference_autograd(cuda):
    g, m, loss = _train_setup(cuda)
    L = loss()
    assert rel(L.item(), float(g["loss"])) < 1e-10
    L.backward()
    params = dict(m.named_parameters())
    for name, norm in zip(g["names"], g["norms"]):
        got = params[str(name)].grad.norm().item()
        assert abs(got - norm) <= 1e-8 * max(norm, 1e-12), (name, got, norm)
    for name, idx, val in zip(g["pick_name"], g["pick_idx"], g["pick_val"]):
        got = params[str(name)].grad.reshape(-1)[int(idx)].item()
        assert abs(got - val) <= 1e-8 * max(abs(val), 1e-6), (name, idx, got, val)


def test_force_loss_gradient_finite_difference(cuda):
    """The 64 recorded weights: autograd through the hand-written double
    backward against central differences, within 1e-6 relative."""
    g, m, loss = _train_setup(cuda)
    L = loss()
    L.backward()
    params = dict(m.named_parameters())
    h = 1e-5
    gscale = max(abs(v) for v in g["pick_val"])
    for name, idx in zip(g["pick_name"], g["pick_idx"]):
        p = params[str(name)]
        an = p.grad.reshape(-1)[int(idx)].item()
        old = p.data.reshape(-1)[int(idx)].item()
        p.data.reshape(-1)[int(idx)] = old + h
        lp = loss().item()
        p.data.reshape(-1)[int(idx)] = old - h
        lm = loss().item()
        p.data.reshape(-1)[int(idx)] = old
        fd = (lp - lm) / (2 * h)
        assert abs(an - fd) <= 1e-6 * max(abs(fd), 1e-3 * gscale), (name, idx, an, fd)
