"""Host side of dpgb.model.EnergyModelSeA, on the CPU (no kernel runs): the
state dict of the reference's se_e2_a test model (deeppot_sea.pth, as saved
in tests/golden/deeppot_sea_model.npz) loads into it with every key
matched.  The only keys of ours that this older checkpoint lacks are the
descriptor's (empty) compression tables, which the current reference block
also registers (deepmd/pt/model/descriptor/se_a.py:565-575)."""
import numpy as np
import pytest

from conftest import golden

torch = pytest.importorskip("torch")


def test_reference_state_dict_loads():
    from dpgb.descriptor import DescrptSeA
    from dpgb.model import EnergyFittingNet, EnergyModelSeA

    g = golden("deeppot_sea_model")
    d = DescrptSeA(6.0, 0.5, [46, 92], neuron=[3, 6, 12], axis_neuron=2, type_one_side=True, device="cpu")
    f = EnergyFittingNet(2, 24, [10, 10, 10], True, device="cpu")
    m = EnergyModelSeA(d, f)
    ours, ref = set(m.state_dict()), set(g.files)
    assert ref <= ours, sorted(ref - ours)
    extra = sorted(ours - ref)
    assert all(".sea.compress_data." in k or ".sea.compress_info." in k for k in extra), extra
    r = m.load_state_dict({k: torch.tensor(g[k]) for k in g.files}, strict=False)
    assert not r.unexpected_keys
    for k in g.files:
        np.testing.assert_array_equal(m.state_dict()[k].numpy(), g[k])
