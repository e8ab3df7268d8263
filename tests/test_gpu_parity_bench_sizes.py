"""GPU parity at the benchmarked sizes, against the oracle (the CPU
restatement of the reference, pinned to the reference's compiled library and
golden vectors in test_oracle.py):

* 4096 H2O (12,288 atoms): the whole neighbour list bit for bit against the
  oracle's build of deepmd/pt/utils/nlist.py:49-199,304-337 on the same
  extended atoms, and the FP64 energy / forces / virial within 1e-10;
* 32,768 H2O (98,304 atoms), the compressed benchmark's skin lists: a
  20-step N(0, 0.01 A) random walk with a 2 A skin and a candidate rebuild
  every 10 steps; on every step the list selected at rcut from the stored
  candidates equals, bit for bit, a fresh list built by the oracle from the
  same coordinates;
* the 4-species fcc alloy model (rcut_smth 2, sel [60] x 4, 16 embedding
  nets), frames from each batch size bucket (<= 128, <= 512, <= 2048,
  > 2048 atoms) evaluated together in one batch, each frame against the
  oracle: FP64 within 1e-10; the mixed form within 1e-3 of the RMS force.

The extended atoms of a list are numbered e = s * natom + j (image s of atom
j); the oracle builds its list on coord[j] + shift[s] in the library's image
order (DeepPot.last_nlist), so the two lists compare index for index."""
import numpy as np
import pytest

from conftest import water_params

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def oracle_list(nl_info, atype, rcut, sel):
    """The oracle's list on the library's own extended atoms of frame 0."""
    import oracle as O

    _, coord, shift = nl_info
    natom = atype.shape[0]
    ext = (coord[None, :natom, :] + shift[0][:, None, :]).reshape(-1, 3)
    ext_t = np.tile(np.asarray(atype, np.int32), shift.shape[1])
    return O.build_nlist_pt(ext, ext_t, natom, rcut, sel)


def test_water12288_nlist_and_fp64_vs_oracle(cuda):
    import oracle as O
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    params = water_params()
    c = params.config
    coord, atype, box = synth.water_box(16, seed=0)
    dp = DeepPot(params, "fp64")
    e, f, v = dp.eval(coord.reshape(1, -1), box.reshape(1, 9), atype)
    info = dp.last_nlist()
    nl = info[0]
    assert nl.shape == (atype.size, c.nnei)
    ref = oracle_list(info, atype, c.rcut, c.sel)
    np.testing.assert_array_equal(nl, ref)
    assert (nl >= 0).sum() > 80 * atype.size  # ~90 real neighbours per atom
    r = O.OracleModel(params).evaluate(coord, atype, box)
    assert rel(e[0], r["energy"]) < 1e-10
    assert rel(f[0], r["force"]) < 1e-10
    assert rel(v[0], r["virial"]) < 1e-10


def test_water98304_skin_lists_bit_exact_every_step(cuda):
    import torch

    from dpgb import synth
    from dpgb.deeppot import DeepPot

    params = water_params()
    c = params.config
    coord, atype, box = synth.water_box(32, seed=0)
    dp = DeepPot(params, "mixed")
    dp.set_skin(2.0, 10)
    x = torch.tensor(coord.reshape(1, -1), dtype=torch.float64, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(1234)
    out = None
    for step in range(20):
        if step:
            x.add_(torch.randn(x.shape, dtype=x.dtype, device="cuda", generator=gen), alpha=0.01)
        out = dp.eval_device(x, box.reshape(1, 9), atype, out=out)
        dp.check_status()
        info = dp.last_nlist()
        ref = oracle_list(info, atype, c.rcut, c.sel)
        np.testing.assert_array_equal(info[0], ref, err_msg=f"step {step}")


@pytest.fixture(scope="module")
def alloy():
    from dpgb import params as P, synth

    rng = np.random.default_rng(21)
    # one frame per size bucket: 108, 500, 2048 and 4000 atoms (whole fcc cells)
    frames = [synth.fcc_alloy_frame(n, rng) for n in (108, 500, 2048, 4000)]
    return P.init_params(P.alloy_config(), seed=3), frames


def test_alloy_buckets_fp64_and_mixed_vs_oracle(cuda, alloy):
    import oracle as O
    from dpgb.deeppot import DeepPot

    params, frames = alloy
    om = O.OracleModel(params)
    refs = [om.evaluate(c, t, b) for c, t, b in frames]
    for prec in ("fp64", "mixed"):
        dp = DeepPot(params, prec)
        e, f, v = dp.batch(frames).eval([c for c, _, _ in frames])
        for k, r in enumerate(refs):
            if prec == "fp64":
                assert rel(e[k], r["energy"]) < 1e-10, k
                assert rel(f[k], r["force"]) < 1e-10, k
                assert rel(v[k], r["virial"]) < 1e-10, k
            else:
                rms = float(np.sqrt(np.mean(r["force"] ** 2)))
                rmse = float(np.sqrt(np.mean((f[k] - r["force"]) ** 2)))
                assert rmse <= 1e-3 * rms, (k, rmse, rms)
                assert abs(e[k] - r["energy"]) / len(frames[k][1]) <= 1e-4 * max(1.0, abs(r["energy"]) / len(
                    frames[k][1])), k
