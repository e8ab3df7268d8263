"""Host side of dpgb.descriptor.DescrptSeA, on the CPU (no kernel runs):
the parameter set and state-dict names follow deepmd/pt/model/network/mlp.py
(a timestep idt only on layers with a skip connection, mlp.py:89-92), the
serialised dict has the reference's layout (se_a.py:392-423 with
NetworkCollection / EmbeddingNet / NativeLayer of dpmodel/utils/network.py),
and serialise -> deserialise gives back the same module."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _desc(**kw):
    from dpgb.descriptor import DescrptSeA

    args = dict(neuron=[25, 50, 100], axis_neuron=16, type_one_side=False, resnet_dt=True, seed=3, device="cpu")
    args.update(kw)
    return DescrptSeA(6.0, 0.5, [46, 92], **args)


def test_timestep_only_where_a_skip_connection_exists():
    d = _desc()
    keys = set(d.state_dict())
    for e in range(4):
        p = f"sea.filter_layers.networks.{e}.layers."
        assert p + "0.idt" not in keys  # 1 -> 25: no skip connection
        assert p + "1.idt" in keys and p + "2.idt" in keys  # 25 -> 50, 50 -> 100: doubling skips
        assert p + "0.matrix" in keys and p + "0.bias" in keys
    flat = d.sea.flat_params().detach()
    # the kernels' layout keeps an idt slot per layer: ones where no timestep exists
    w0 = 1 * 25
    np.testing.assert_array_equal(flat[w0 + 25:w0 + 50].numpy(), np.ones(25))
    assert flat.numel() == 4 * ((25 + 25 + 25) + (25 * 50 + 50 + 50) + (50 * 100 + 100 + 100))


def test_serialised_layout_matches_the_reference():
    s = _desc().serialize()
    assert (s["@class"], s["type"], s["@version"]) == ("Descriptor", "se_e2_a", 2)
    for k in ("rcut", "rcut_smth", "sel", "neuron", "axis_neuron", "resnet_dt", "set_davg_zero",
              "activation_function", "precision", "embeddings", "env_mat", "exclude_types", "env_protection",
              "@variables", "type_map", "trainable", "type_one_side", "spin"):
        assert k in s, k
    emb = s["embeddings"]
    assert (emb["@class"], emb["@version"], emb["ndim"], emb["ntypes"]) == ("NetworkCollection", 1, 2, 2)
    assert isinstance(emb["networks"], list) and len(emb["networks"]) == 4
    net = emb["networks"][0]
    assert (net["@class"], net["@version"], net["in_dim"], net["neuron"]) == ("EmbeddingNetwork", 2, 1, [25, 50, 100])
    layers = net["layers"]
    assert [ly["use_timestep"] for ly in layers] == [False, True, True]
    assert layers[0]["@variables"]["idt"] is None
    for ly in layers:
        assert (ly["@class"], ly["@version"], ly["resnet"], ly["bias"]) == ("Layer", 2, True, True)
    assert layers[1]["@variables"]["w"].shape == (25, 50)
    assert s["@variables"]["davg"].shape == (2, 138, 4)


@pytest.mark.parametrize("resnet_dt,one_side", [(True, False), (False, True)])
def test_serialise_deserialise_round_trip(resnet_dt, one_side):
    from dpgb.descriptor import DescrptSeA

    d = _desc(resnet_dt=resnet_dt, type_one_side=one_side)
    with torch.no_grad():
        d.sea.mean.copy_(torch.randn_like(d.sea.mean))
        d.sea.stddev.copy_(torch.rand_like(d.sea.stddev) + 0.5)
    d2 = DescrptSeA.deserialize(d.serialize(), device="cpu")
    a, b = d.state_dict(), d2.state_dict()
    assert set(a) == set(b)
    for k in a:
        torch.testing.assert_close(a[k], b[k], rtol=0, atol=0)
    torch.testing.assert_close(d.sea.flat_params(), d2.sea.flat_params(), rtol=0, atol=0)
