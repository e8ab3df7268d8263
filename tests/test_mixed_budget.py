"""CPU: the per-stage error budget of the mixed-precision form
(tests/mixed_budget.py), on the 192-atom water box with the water model's
energy scaled to ~1 eV/A RMS forces (dpgb.params.scale_energy).  It shows
which roundings the split-BF16 operands are there for: with every GEMM
operand in one BF16 rounding the force error exceeds the 1e-3 eV/A bound;
as built it is a fraction of it.  The table printed by `pytest -s` is the
budget quoted in the design notes."""
import numpy as np
import pytest

import mixed_budget as B

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def system():
    from dpgb import params as P, synth

    p = P.scale_energy(P.init_params(P.water_config(), seed=1), P.WATER_FORCE_SCALE)
    coord, atype, box = synth.water_box(4, seed=0)
    return p, coord, atype, box


def test_stage_budget(system):
    p, coord, atype, box = system
    cases = {
        "env FP32": {"env": "fp32"},
        "embedding activations BF16": {"emb_op": "bf16:none"},
        "embedding weights BF16": {"emb_op": "none:bf16"},
        "embedding gradient operands BF16": {"emb_grad": "bf16"},
        "embedding tanh.approx": {"emb_tanh": "approx"},
        "D BF16": {"D": "bf16"},
        "fitting layer 1 weights BF16": {"fit1_op": "none:bf16"},
        "fitting layer 1 gradient BF16": {"fit1_grad": "bf16"},
        "fitting layers 2-3 activations BF16": {"fit_op": "bf16:none"},
        "fitting gradient operands BF16": {"fit_grad": "bf16"},
        "fitting tanh.approx": {"fit_tanh": "approx"},
        "all BF16 (no splits)": B.ALL_BF16,
        "as built": B.AS_BUILT,
    }
    rms, out = B.budget(p, coord, atype, box, cases)
    print(f"\nRMS force {rms:.3f} eV/A")
    for k, (rmse, rel, de) in out.items():
        print(f"  {k:38s} F-RMSE {rmse:.2e} eV/A ({rel:.1e} of RMS)  |dE| {de:.1e} eV/atom")
    assert 0.5 < rms < 2.0
    assert out["env FP32"][0] < 1e-6
    assert out["all BF16 (no splits)"][0] > 1e-3       # one BF16 rounding per operand misses the bound
    assert out["fitting layer 1 weights BF16"][0] > 1e-3  # the largest single term
    assert out["as built"][0] < 6e-4                     # the mixed form as built meets it with room
    assert out["as built"][2] < 1e-3
