"""Host side of the torch op boundary, on the CPU (no kernel runs): the op
registered by dpgb.ops.register() has the reference's schema
(source/op/pt/tabulate_multi_device.cc:1630-1684) and refuses CPU inputs
loudly — the product path has no CPU fallback."""
import pytest

torch = pytest.importorskip("torch")


def test_schema_and_no_cpu_fallback():
    from dpgb import ops

    ops.register()
    op = torch.ops.deepmd.tabulate_fusion_se_a
    assert str(op.default._schema) == ("deepmd::tabulate_fusion_se_a(Tensor table, Tensor table_info, "
                                       "Tensor em_x, Tensor em, int last_layer_size) -> Tensor[]")
    f64 = dict(dtype=torch.float64)
    table, info = torch.zeros(4, 48, **f64), torch.tensor([0.0, 1.0, 2.0, 0.1, 0.2, -1.0], **f64)
    with pytest.raises(NotImplementedError):
        op(table, info, torch.zeros(6, 1, **f64), torch.zeros(2, 3, 4, **f64), 8)
