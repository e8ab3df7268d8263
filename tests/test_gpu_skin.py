"""Neighbour-list reuse with a skin (dpgb_deeppot_set_skin): candidates within
rcut + skin, rebuilt every k calls or when an atom has moved more than
skin / 2, the list at rcut selected from them each call.  Against a fresh
list every call on the same coordinates:

* FP64: bitwise on the calls that build, to rounding (1e-12) in between
  (the reused wrap offsets move coordinates by an ulp);
* atoms drifting across the periodic faces, and a caller that re-wraps
  them, keep matching (the displacement check forces the rebuild);
* candidate rows too narrow for the pairs within rcut + skin are widened
  and the call repeated;
* several frames at once, and the mixed form through the device API.
"""
import dataclasses

import numpy as np
import pytest

from conftest import water_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _system(n=8, seed=11):
    from dpgb import synth

    return synth.water_box(n, seed=seed)


def _pair(params, precision, skin, every):
    from dpgb.deeppot import DeepPot

    fresh = DeepPot(params, precision)
    reuse = DeepPot(params, precision)
    reuse.set_skin(skin, every)
    return fresh, reuse


def test_skin_random_walk_fp64(cuda):
    c, t, box = _system()
    fresh, reuse = _pair(water_params(), "fp64", 2.0, 4)
    rng = np.random.default_rng(5)
    for k in range(10):
        c = c + rng.normal(0, 0.02, size=c.shape)
        e0, f0, v0 = fresh.eval(c.reshape(1, -1), box.reshape(1, 9), t)
        e1, f1, v1 = reuse.eval(c.reshape(1, -1), box.reshape(1, 9), t)
        if k % 4 == 0:  # a build call: the same list, the same arithmetic
            np.testing.assert_array_equal(e1, e0)
            np.testing.assert_array_equal(f1, f0)
            np.testing.assert_array_equal(v1, v0)
        else:
            assert rel(e1, e0) < 1e-12
            assert rel(f1, f0) < 1e-11
            assert rel(v1, v0) < 1e-11


def test_skin_atoms_cross_the_faces(cuda):
    """A uniform drift carries atoms through the box faces; the list is
    rebuilt once an atom has moved skin / 2, and a caller that wraps its
    coordinates itself (a jump of one box length) forces a rebuild too."""
    c, t, box = _system(seed=12)
    L = box[0]
    fresh, reuse = _pair(water_params(), "fp64", 1.0, 1000)
    drift = np.array([0.13, -0.07, 0.05])
    for k in range(12):
        c = c + drift
        if k == 8:
            c = c - np.floor(c / L) * L  # the caller wraps
        e0, f0, v0 = fresh.eval(c.reshape(1, -1), box.reshape(1, 9), t)
        e1, f1, v1 = reuse.eval(c.reshape(1, -1), box.reshape(1, 9), t)
        assert rel(e1, e0) < 1e-12
        assert rel(f1, f0) < 1e-11
        assert rel(v1, v0) < 1e-11


def test_skin_candidate_rows_widen(cuda):
    """sel [10, 20] keeps a tenth of what lies within rcut + skin: the first
    candidate rows are too narrow, the call widens them and repeats."""
    from dpgb import params as P

    cfg = dataclasses.replace(P.water_config(), sel=[10, 20])
    p = P.init_params(cfg, seed=3)
    c, t, box = _system(seed=13)
    fresh, reuse = _pair(p, "fp64", 2.0, 3)
    rng = np.random.default_rng(6)
    for k in range(4):
        c = c + rng.normal(0, 0.02, size=c.shape)
        e0, f0, _ = fresh.eval(c.reshape(1, -1), box.reshape(1, 9), t)
        e1, f1, _ = reuse.eval(c.reshape(1, -1), box.reshape(1, 9), t)
        assert rel(e1, e0) < 1e-12
        assert rel(f1, f0) < 1e-11


def test_skin_two_frames(cuda):
    c, t, box = _system(seed=14)
    rng = np.random.default_rng(7)
    c2 = np.stack([c, c + rng.normal(0, 0.05, size=c.shape)])
    boxes = np.stack([box, box])
    fresh, reuse = _pair(water_params(), "fp64", 2.0, 2)
    for k in range(5):
        c2 = c2 + rng.normal(0, 0.02, size=c2.shape)
        e0, f0, v0 = fresh.eval(c2.reshape(2, -1), boxes, t)
        e1, f1, v1 = reuse.eval(c2.reshape(2, -1), boxes, t)
        assert rel(e1, e0) < 1e-12
        assert rel(f1, f0) < 1e-11
        assert rel(v1, v0) < 1e-11


def test_skin_mixed_device(cuda):
    import torch

    c, t, box = _system(seed=15)
    fresh, reuse = _pair(water_params(), "mixed", 2.0, 5)
    rng = np.random.default_rng(8)
    for k in range(7):
        c = c + rng.normal(0, 0.02, size=c.shape)
        cd = torch.from_numpy(c.reshape(1, -1)).cuda()
        o0 = fresh.eval_device(cd, box.reshape(1, 9), t)
        o1 = reuse.eval_device(cd, box.reshape(1, 9), t)
        reuse.check_status()
        f0, f1 = o0["force"].cpu().numpy(), o1["force"].cpu().numpy()
        if k % 5 == 0:
            np.testing.assert_array_equal(f1, f0)
        assert float(np.sqrt(np.mean((f1 - f0) ** 2))) <= 1e-6 * float(np.sqrt(np.mean(f0 ** 2)))
        assert rel(o1["energy"].cpu().numpy(), o0["energy"].cpu().numpy()) < 1e-6
