"""DescrptSeA with precision="mixed" (dpgb's option): the block runs on the
mixed form's kernels — the tcgen05 embedding (split BF16, FP32 accumulation)
or, compressed, the fused FP32 table kernels — through
dpgb_deeppot_descrpt_fwd / _bwd.  Against the FP64 descriptor on the same
weights and inputs (two frames of 648 atoms): the descriptor within 2e-4 of
its largest entry, rot_mat likewise, sw identical, and dE/d coordinates of
a linear read-out of the descriptor within 1e-3 of its RMS; compressed
likewise against the FP64 compressed descriptor.  The backward needs the
forward to be the handle's latest evaluation."""
import numpy as np
import pytest

from conftest import golden, water_params

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _desc(cuda, precision):
    from dpgb.descriptor import DescrptSeA

    p = water_params()
    c = p.config
    d = DescrptSeA(rcut=c.rcut, rcut_smth=c.rcut_smth, sel=c.sel, neuron=c.neuron, axis_neuron=c.axis_neuron,
                   type_one_side=c.type_one_side, resnet_dt=c.resnet_dt, precision=precision, device=cuda)
    sd = {k[len("atomic_model.descriptor."):]: torch.as_tensor(v) for k, v in p.to_state_dict().items()
          if k.startswith("atomic_model.descriptor.")}
    d.load_state_dict(sd, strict=False)
    return d


def _inputs(cuda):
    from dpgb import nlist as N, synth

    frames = [synth.water_box(6, seed=40 + k) for k in range(2)]
    coord = torch.tensor(np.stack([f[0] for f in frames]), dtype=torch.float64, device=cuda)
    atype = torch.tensor(np.stack([f[1] for f in frames]), device=cuda)
    p = water_params()
    ext, ext_t, _, nl = N.extend_input_and_build_neighbor_list(coord, atype, p.config.rcut, p.config.sel,
                                                               np.stack([f[2].reshape(9) for f in frames]))
    return ext.reshape(2, -1), ext_t.long(), nl.long()


def _compare(d64, dmx, ext, ext_t, nl):
    w = torch.randn(d64.get_dim_out(), dtype=torch.float64, device=ext.device,
                    generator=torch.Generator(ext.device).manual_seed(5))
    out = {}
    for name, d in (("f64", d64), ("mixed", dmx)):
        x = ext.clone().requires_grad_(True)
        D, rot, _, _, sw = d(x, ext_t, nl)
        (g,) = torch.autograd.grad((D * w).sum(), x)
        out[name] = (D.detach(), rot.detach(), sw.detach(), g)
    D0, r0, s0, g0 = out["f64"]
    D1, r1, s1, g1 = out["mixed"]
    assert D1.dtype == torch.float64 and D1.shape == D0.shape and r1.shape == r0.shape
    assert (D1 - D0).abs().max().item() <= 2e-4 * D0.abs().max().item()
    assert (r1 - r0).abs().max().item() <= 2e-4 * r0.abs().max().item()
    torch.testing.assert_close(s1, s0, rtol=0, atol=0)
    rms = g0.pow(2).mean().sqrt().item()
    assert (g1 - g0).pow(2).mean().sqrt().item() <= 1e-3 * rms, ((g1 - g0).pow(2).mean().sqrt().item(), rms)


def test_mixed_descriptor_tracks_float64(cuda):
    ext, ext_t, nl = _inputs(cuda)
    _compare(_desc(cuda, "float64"), _desc(cuda, "mixed"), ext, ext_t, nl)


def test_mixed_compressed_descriptor_tracks_float64(cuda):
    g = golden("water192_compressed")
    ext, ext_t, nl = _inputs(cuda)
    ds = []
    for prec in ("float64", "mixed"):
        d = _desc(cuda, prec)
        d.enable_compression(float(g["min_nbor_dist"]), float(g["extrapolate"]), float(g["stride0"]),
                             float(g["stride1"]))
        ds.append(d)
    _compare(ds[0], ds[1], ext, ext_t, nl)


def test_mixed_backward_needs_the_latest_forward(cuda):
    from dpgb import _lib

    ext, ext_t, nl = _inputs(cuda)
    d = _desc(cuda, "mixed")
    x = ext.clone().requires_grad_(True)
    D = d(x, ext_t, nl)[0]
    d(ext, ext_t, nl)  # a second forward of the same handle
    with pytest.raises(_lib.DpgbError):
        torch.autograd.grad(D.sum(), x)
