"""Training loop (dpgb.train.Trainer) on the GPU against six Adam steps of
the reference's own training parts (tests/golden/train_steps.npz): the
learning rate and FP64 loss of every step, the weights after the last step
(per-tensor norms and 64 entries), and lcurve.out (header byte for byte,
each displayed figure equal to the reference's at the file's 3 significant
digits)."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _frames():
    """The 16 water frames the fixture was generated on (192 atoms each)."""
    from dpgb import synth

    frames = [synth.water_box(4, seed=100 + k) for k in range(16)]
    coord = np.stack([f[0].reshape(-1) for f in frames])
    return coord, frames[0][1], np.stack([f[2].reshape(-1) for f in frames])


def _close_fields(got: str, want: str):
    """Same layout; every number equal to within one unit of its last
    printed digit (the two sides' FP64 sums differ in the last bits)."""
    gl, wl = got.splitlines(), want.splitlines()
    assert len(gl) == len(wl)
    assert gl[:2] == wl[:2]
    for a, b in zip(gl[2:], wl[2:]):
        assert len(a) == len(b), (a, b)
        fa, fb = a.split(), b.split()
        assert fa[0] == fb[0]
        for x, y in zip(fa[1:], fb[1:]):
            if x != y:
                ulp = 10.0 ** (int(y.split("e")[1]) - (2 if len(y.split("e")[0]) == 4 else 1))
                assert abs(float(x) - float(y)) <= ulp * 1.0001, (a, b)


def test_six_adam_steps_match_reference(cuda, tmp_path):
    from dpgb import params as P
    from dpgb.model import EnergyModelSeA
    from dpgb.train import FrameSet, LearningRateExp, Trainer

    g = golden("train_steps")
    coord, atype, box = _frames()
    e, f = g["energy_label"], g["force_label"]
    train = FrameSet(coord[:12], atype, box[:12], energy=e[:12], force=f[:12], batch_size=4)
    valid = FrameSet(coord[12:], atype, box[12:], energy=e[12:], force=f[12:], batch_size=4)
    m = EnergyModelSeA.from_params(P.init_params(P.water_config(), seed=1), device=cuda)
    lcurve = tmp_path / "lcurve.out"
    tr = Trainer(m, LearningRateExp(start_lr=1e-3, stop_lr=1e-5, num_steps=6), train, valid,
                 loss_params=dict(start_pref_e=0.02, limit_pref_e=1.0, start_pref_f=1000.0, limit_pref_f=1.0),
                 disp_freq=2, disp_file=str(lcurve))
    for k in range(6):
        tr.step()
        assert tr.last_lr == pytest.approx(float(g["lr"][k]), rel=1e-15)
        assert abs(float(tr.last_loss) - g["loss"][k]) <= 1e-9 * abs(g["loss"][k]), (k, float(tr.last_loss))
    params = {k: p.detach().cpu().numpy().reshape(-1) for k, p in m.named_parameters()}
    for name, norm in zip(g["names"], g["norms"]):
        got = np.linalg.norm(params[str(name)])
        assert abs(got - norm) <= 1e-10 * norm, (name, got, norm)
    for name, idx, val in zip(g["pick_name"], g["pick_idx"], g["pick_val"]):
        got = params[str(name)][int(idx)]
        assert abs(got - val) <= 1e-10 * max(abs(val), 1e-3), (name, idx, got, val)
    _close_fields(lcurve.read_text(), str(g["lcurve"]))
    assert [r["step"] for r in tr.history] == [1, 2, 4, 6]


def test_training_lowers_the_loss(cuda):
    """Twenty steps at a constant rate of 1e-4 on one batch of 4 frames: the
    displayed loss falls at every step (the reference's loop on the same
    case falls from 1.35 to 0.21)."""
    from dpgb import params as P
    from dpgb.model import EnergyModelSeA
    from dpgb.train import FrameSet, LearningRateExp, Trainer

    g = golden("train_steps")
    coord, atype, box = _frames()
    data = FrameSet(coord[:4], atype, box[:4], energy=g["energy_label"][:4], force=g["force_label"][:4],
                    batch_size=4)
    m = EnergyModelSeA.from_params(P.init_params(P.water_config(), seed=1), device=cuda)
    tr = Trainer(m, LearningRateExp(start_lr=1e-4, stop_lr=1e-4, num_steps=20), data, disp_freq=1,
                 disp_file=None, loss_params=dict(start_pref_e=0.02, limit_pref_e=0.02, start_pref_f=1000.0,
                                                  limit_pref_f=1000.0))
    hist = tr.run()
    assert len(hist) == 20
    r = [h["trn"]["rmse"] for h in hist]
    assert all(b < a for a, b in zip(r, r[1:])), r
    assert abs(r[0] - 1.35) < 0.01 and r[-1] < 0.25 * r[0], r


def test_float32_training_step_tracks_float64(cuda):
    """The reference's single-precision option (descriptor and fitting
    ``precision: float32``): the force-loss gradient of the FP32 model
    against the FP64 model's on the same weights — per-tensor norms within
    1e-3 relative, the loss within 1e-5 — and six Adam steps giving the
    FP64 trajectory's losses within 1e-3."""
    import torch

    from dpgb import params as P
    from dpgb.model import EnergyModelSeA
    from dpgb.train import FrameSet, LearningRateExp, Trainer

    g = golden("train_steps")
    coord, atype, box = _frames()
    e, f = g["energy_label"], g["force_label"]
    out = {}
    for prec in ("float64", "float32"):
        m = EnergyModelSeA.from_params(P.init_params(P.water_config(), seed=1), device=cuda, precision=prec)
        tr = Trainer(m, LearningRateExp(start_lr=1e-3, stop_lr=1e-5, num_steps=6),
                     FrameSet(coord[:12], atype, box[:12], energy=e[:12], force=f[:12], batch_size=4),
                     loss_params=dict(start_pref_e=0.02, limit_pref_e=1.0, start_pref_f=1000.0, limit_pref_f=1.0),
                     disp_freq=10 ** 9, disp_file=None)
        losses, norms = [], None
        for k in range(6):
            tr.step()
            losses.append(float(tr.last_loss))
            if k == 0:
                norms = {n: float(p.grad.double().norm()) for n, p in m.named_parameters() if p.grad is not None}
        out[prec] = (np.array(losses), norms)
    l64, n64 = out["float64"]
    l32, n32 = out["float32"]
    assert abs(l32[0] - l64[0]) <= 1e-5 * abs(l64[0])
    vmax = max(n64.values())
    for name, v in n64.items():
        assert abs(n32[name] - v) <= 1e-3 * max(v, 1e-3 * vmax), (name, n32[name], v)
    np.testing.assert_allclose(l32, l64, rtol=1e-3)
    np.testing.assert_allclose(l64, g["loss"], rtol=1e-9)
