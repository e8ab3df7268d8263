"""Host side of dpgb.train on the CPU: the exponential learning-rate
schedule against the reference's LearningRateExp (values recorded in
tests/golden/train_steps.npz for six schedules: stepped, warmup by steps and
by ratio, smooth, a given decay rate with stop_lr as the floor, and the
automatic decay_steps of a short run), the lcurve.out header and rows
against the text written by the reference's print_header /
print_on_training, the batch walk of FrameSet, and the loss terms' on/off
and not-found rules."""
import ast
import re

import numpy as np
import pytest

from conftest import golden

torch = pytest.importorskip("torch")


def test_lr_schedule_matches_reference():
    from dpgb.train import LearningRateExp

    g = golden("train_steps")
    for case, steps, want in zip(g["lr_cases"], g["lr_case_steps"], g["lr_case_values"]):
        kw = dict(ast.literal_eval(str(case)))
        lr = LearningRateExp(**kw)
        got = np.array([lr.value(int(t)) for t in steps])
        np.testing.assert_allclose(got, want, rtol=1e-15, atol=0, err_msg=str(kw))


def test_lr_of_the_training_case():
    from dpgb.train import LearningRateExp

    g = golden("train_steps")
    lr = LearningRateExp(start_lr=1e-3, stop_lr=1e-5, num_steps=len(g["lr"]))
    assert lr.decay_steps == 1
    np.testing.assert_allclose([lr.value(t) for t in range(len(g["lr"]))], g["lr"], rtol=1e-15)


def test_lr_argument_errors():
    from dpgb.train import LearningRateExp

    with pytest.raises(ValueError):
        LearningRateExp(1e-3, 100, stop_lr=1e-5, stop_lr_ratio=1e-2)
    with pytest.raises(ValueError):
        LearningRateExp(1e-3, 100)
    with pytest.raises(ValueError):
        LearningRateExp(1e-3, 100, stop_lr=1e-5, warmup_steps=100)
    with pytest.raises(ValueError):
        LearningRateExp(1e-3, 100, stop_lr=1e-5, decay_steps=0)


def _parse_rows(text):
    rows = []
    for line in text.splitlines():
        if line.startswith("#"):
            continue
        f = line.split()
        rows.append((int(f[0]), [float(x) for x in f[1:-1]], float(f[-1])))
    return rows


def test_lcurve_text_matches_reference():
    """Header byte for byte; each row re-printed from its own numbers with
    lcurve_row gives the reference's line byte for byte."""
    from dpgb.train import lcurve_header, lcurve_row

    g = golden("train_steps")
    text = str(g["lcurve"])
    names = [str(k) for k in g["fig_names"]]
    lines = text.splitlines(keepends=True)
    figs = dict.fromkeys(names, 0.0)
    assert lcurve_header(figs, figs) == "".join(lines[:2])
    for line, (step, vals, lr) in zip(lines[2:], _parse_rows(text)):
        val = {k: vals[2 * i] for i, k in enumerate(names)}
        trn = {k: vals[2 * i + 1] for i, k in enumerate(names)}
        assert lcurve_row(step, lr, trn, val) == line
    # without validation data: one column per figure
    h = lcurve_header(figs, {})
    assert h.splitlines()[0] == "# step " + "".join("   %11s" % (k + "_trn") for k in names) + "   lr      "
    assert lcurve_row(12, 3.5e-4, dict(zip(names, [1.0, 2.0, 3.0])), {}) == (
        "     12      1.00e+00      2.00e+00      3.00e+00    3.5e-04\n")


def test_frameset_batches():
    from dpgb.train import FrameSet

    nf, na = 6, 4
    coord = np.arange(nf * na * 3, dtype=np.float64).reshape(nf, na * 3)
    fs = FrameSet(coord, np.zeros(na, dtype=np.int64), np.tile(np.eye(3).reshape(9) * 10, (nf, 1)),
                  energy=np.arange(nf), force=np.zeros((nf, na, 3)), batch_size=4)
    first = [fs.next_batch("cpu") for _ in range(3)]
    got = [b[0]["coord"][:, 0].numpy() / (na * 3) for b in first]
    np.testing.assert_array_equal(got[0], [0, 1, 2, 3])
    np.testing.assert_array_equal(got[1], [0, 1, 2, 3])  # frames 4-5 do not fill a batch: next pass
    inp, lab = first[0]
    assert lab["find_energy"] == 1.0 and lab["find_force"] == 1.0 and lab["find_virial"] == 0.0
    assert lab["energy"].shape == (4, 1) and inp["atype"].shape == (4, na)
    sh = FrameSet(coord, np.zeros(na, dtype=np.int64), batch_size=2, seed=3)
    seen = np.concatenate([sh.next_batch("cpu")[0]["coord"][:, 0].numpy() / (na * 3) for _ in range(3)])
    assert sorted(seen.tolist()) == list(range(nf))
    with pytest.raises(ValueError):
        FrameSet(coord, np.zeros(na, dtype=np.int64), batch_size=7)


def test_loss_terms_follow_reference_rules():
    """A term is on only when both prefactors are nonzero; a label without
    its find flag adds nothing and displays NaN (deepmd/pt/loss/ener.py:
    160-162, deepmd/pt/loss/loss.py:74-84)."""
    from dpgb.model import EnergyStdLoss

    on = EnergyStdLoss(1.0, 0.02, 1.0, 1000.0, 1.0, 0.0, 1.0)
    assert on.has_e and on.has_f and not on.has_v

    def model(**kw):
        return {"energy": torch.ones(2, 1, dtype=torch.float64), "force": torch.zeros(2, 3, 3, dtype=torch.float64)}

    label = {"energy": torch.zeros(2, 1, dtype=torch.float64), "force": torch.ones(2, 3, 3, dtype=torch.float64),
             "find_energy": 1.0}
    _, loss, more = on({}, model, label, 3, 1.0)
    assert float(more["rmse_e"]) == pytest.approx(1.0 / 3)
    assert np.isnan(float(more["rmse_f"]))
    assert float(loss) == pytest.approx(float(np.float32(1) / np.float32(3)) * 0.02)
