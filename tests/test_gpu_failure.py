"""GPU: failure detection without a GPU fault.

* Non-finite input coordinates (NaN, +-inf) are an error of the call
  (DPGB_EINVAL), through the host API (dpgb_deeppot_compute), the device API
  (reported by dpgb_deeppot_check_status), an open-boundary frame and a
  batch; the handle computes correctly right after.
* A bounded device-side wait that nothing completes gives up after its
  limit (about 1 ms here), the call returns DPGB_ETIMEOUT, and the CUDA
  context keeps working (an evaluation right after matches the oracle)."""
import numpy as np
import pytest

from conftest import water_params

pytestmark = pytest.mark.gpu

EINVAL, ETIMEOUT = -1, -5


def _small():
    from dpgb import synth

    return synth.water_box(3, seed=3)  # 81 atoms


def _oracle_energy(params, coord, atype, box):
    import oracle as O

    return O.OracleModel(params).evaluate(coord, atype, box)["energy"]


@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_nonfinite_coordinates_host_api(cuda, bad):
    from dpgb._lib import DpgbError
    from dpgb.deeppot import DeepPot

    p = water_params()
    coord, atype, box = _small()
    dp = DeepPot(p, "fp64")
    c = coord.copy()
    c[17, 1] = bad
    with pytest.raises(DpgbError) as ei:
        dp.eval(c.reshape(1, -1), box, atype)
    assert ei.value.code == EINVAL and "non-finite" in str(ei.value)
    e, _, _ = dp.eval(coord.reshape(1, -1), box, atype)  # the handle still works
    assert abs(e[0] - _oracle_energy(p, coord, atype, box)) <= 1e-10 * abs(e[0])


def test_nonfinite_coordinates_device_api_and_skin(cuda):
    import torch

    from dpgb._lib import DpgbError
    from dpgb.deeppot import DeepPot

    coord, atype, box = _small()
    for skin in (0.0, 1.0):
        dp = DeepPot(water_params(), "mixed")
        dp.set_skin(skin, 5)
        x = torch.tensor(coord.reshape(1, -1), device="cuda")
        dp.eval_device(x, box, atype)
        dp.check_status()
        x[0, 40] = float("nan")
        dp.eval_device(x, box, atype)
        with pytest.raises(DpgbError) as ei:
            dp.check_status()
        assert ei.value.code == EINVAL
        x = torch.tensor(coord.reshape(1, -1), device="cuda")
        out = dp.eval_device(x, box, atype)
        dp.check_status()
        assert torch.isfinite(out["force"]).all()


def test_nonfinite_open_boundary_and_batch(cuda):
    from dpgb import params as P, synth
    from dpgb._lib import DpgbError
    from dpgb.deeppot import DeepPot

    coord, atype, _ = _small()
    dp = DeepPot(water_params(), "fp64")
    c = coord.copy()
    c[3, 0] = np.inf
    with pytest.raises(DpgbError) as ei:
        dp.eval(c.reshape(1, -1), None, atype)
    assert ei.value.code == EINVAL
    dp.eval(coord.reshape(1, -1), None, atype)
    rng = np.random.default_rng(1)
    frames = [synth.fcc_alloy_frame(n, rng) for n in (32, 108)]
    b = DeepPot(P.init_params(P.alloy_config(), seed=2), "fp64").batch(frames)
    cs = [f[0].copy() for f in frames]
    cs[1][5, 2] = np.nan
    with pytest.raises(DpgbError) as ei:
        b.eval(cs)
    assert ei.value.code == EINVAL
    b.eval([f[0] for f in frames])


def test_bounded_wait_times_out_and_context_survives(cuda):
    from dpgb import _lib
    from dpgb.deeppot import DeepPot

    rc = _lib.lib().dpgb_selftest_wait_timeout(1.0, None)
    assert rc == ETIMEOUT
    assert "timed out" in _lib.lib().dpgb_last_error().decode()
    p = water_params()
    coord, atype, box = _small()
    e, _, _ = DeepPot(p, "mixed").eval(coord.reshape(1, -1), box, atype)
    assert abs(e[0] - _oracle_energy(p, coord, atype, box)) <= 1e-4 * abs(e[0])
