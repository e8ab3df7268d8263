"""Generate the golden fixtures under tests/golden/ from the reference.

Run in the build container only (it reads the read-only reference tree and
runs the reference's own code; the GPU machine has neither):

    python tests/golden/make_golden.py

Sources of each fixture:

* ``tabulate_se_a_op.npz`` — the inline arrays of the reference op test
  source/tests/pt/test_tabulate_fusion_se_a.py (read as data with ``ast``).
* ``deeppot_sea_case.npz`` / ``deeppot_sea_model.npz`` — the three blocks of
  source/tests/infer/deeppot-testcase.yaml and the weights of the TorchScript
  model source/tests/infer/deeppot_sea.pth (state dict, loaded on CPU).
* ``env_mat_a.npz``, ``fmt_nlist.npz``, ``prod_force_a.npz``,
  ``prod_virial_a.npz`` — the inline golden arrays of source/lib/tests/*.cc
  together with the inputs those tests derive (ghost copy and candidate list),
  reproduced by calling the reference's own CPU library (oracle/_ref).
* ``water192.npz`` — the reference PyTorch model (deepmd.pt, eager FP64 on
  CPU) on the 64-molecule water box with the seeded water-model weights:
  energy, forces, virial, atomic energy/virial, the typed neighbour list, the
  environment matrix and the descriptor of the first atoms.
* ``water192_compressed.npz`` — the same model after the reference's
  ``enable_compression`` (coarse strides so the fixture stays small): the
  tables, table_info and the compressed energy/forces/virial.
* ``train_grad.npz`` — one force-loss step of the reference model: the loss
  and its parameter gradient (norms and 64 entries).
* ``train_steps.npz`` — six Adam steps of the reference's training loop
  (its LearningRateExp, EnergyStdLoss and torch Adam + LambdaLR): rates,
  losses, displayed figures, final weights (norms and 64 entries) and the
  lcurve.out text of its print_header / print_on_training.
"""
from __future__ import annotations

import ast
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
# the reference checkout to read (required: the fixtures come from it)
REF = os.environ.get("DPGB_REFERENCE", "")
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "deepmd-kit_gb300"))


def _read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def cpp_vector(text, name):
    m = re.search(r"std::vector<\w+>\s+" + name + r"\s*=\s*\{([^}]*)\}", text)
    if m is None:
        raise KeyError(name)
    body = re.sub(r"//[^\n]*", "", m.group(1))
    return np.array([float(x) for x in body.replace("\n", " ").split(",") if x.strip()])


def py_test_arrays(rel):
    tree = ast.parse(_read(rel))
    out = {}
    for node in ast.walk(tree):
        if not (isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Attribute)):
            continue
        name, v = node.targets[0].attr, node.value
        shape = None
        if isinstance(v, ast.Call) and isinstance(v.func, ast.Attribute) and v.func.attr == "reshape":
            shape = tuple(ast.literal_eval(a) for a in v.args)
            v = v.func.value
        if isinstance(v, ast.Call) and isinstance(v.func, ast.Attribute) and v.func.attr == "tensor":
            arr = np.array(ast.literal_eval(v.args[0]), dtype=np.float64)
            out[name] = arr.reshape(shape) if shape else arr
        elif isinstance(v, ast.Constant) and name not in out:
            out[name] = v.value
    return out


def make_tabulate():
    a = py_test_arrays("source/tests/pt/test_tabulate_fusion_se_a.py")
    np.savez_compressed(os.path.join(HERE, "tabulate_se_a_op.npz"),
                        table=a["table_tensor"], table_info=a["table_info_tensor"],
                        em_x=a["em_x_tensor"], em=a["em_tensor"],
                        last_layer_size=a["last_layer_size"],
                        descriptor=a["expected_descriptor_tensor"],
                        dy_dem_x=a["expected_dy_dem_x"], dy_dem=a["expected_dy_dem"])


def _yaml_blocks(text):
    """The three result blocks of deeppot-testcase.yaml (a fixed layout)."""
    blocks = []
    for chunk in text.split("\n  - coord:")[1:]:
        chunk = "coord:" + chunk
        rec = {}
        for key in ("coord", "atype", "box", "atomic_energy", "force", "atomic_virial"):
            m = re.search(r"(?m)^\s*" + key + r":\s*(null|\[[^\]]*\])", chunk)
            if m is None:
                raise KeyError(key)
            rec[key] = None if m.group(1) == "null" else np.array(
                [float(x) for x in m.group(1).strip("[]").replace("\n", " ").split(",") if x.strip()])
        blocks.append(rec)
    return blocks


def make_deeppot_case():
    import torch

    blocks = _yaml_blocks(_read("source/tests/infer/deeppot-testcase.yaml"))
    out = {}
    for i, b in enumerate(blocks):
        for k, v in b.items():
            out[f"b{i}_{k}"] = np.zeros(0) if v is None else v
    np.savez_compressed(os.path.join(HERE, "deeppot_sea_case.npz"), nblock=len(blocks), **out)
    m = torch.jit.load(os.path.join(REF, "source/tests/infer/deeppot_sea.pth"), map_location="cpu")
    sd = {k: v.numpy() for k, v in m.state_dict().items() if "._networks." not in k}
    np.savez_compressed(os.path.join(HERE, "deeppot_sea_model.npz"), **sd)


def _lib_test_setup(posi, atype, box, rc, rc_smth, sel):
    import oracle as O

    ext, ext_t, mapping, rows, counts = O.ref_copy_coord_build_nlist(posi, atype, box, rc, legacy=True)
    nloc = len(atype)
    nnei = int(sum(sel))
    avg = np.zeros((len(sel), nnei, 4))
    std = np.ones((len(sel), nnei, 4))
    em, der, rij, nl = O.prod_env_mat_a_ref(ext, ext_t, rows, counts, avg, std, nloc, rc, rc_smth, sel)
    return dict(coord_ext=ext, atype_ext=ext_t, mapping=mapping, rows=rows, counts=counts,
                em=em, em_deriv=der, rij=rij, nlist=nl)


def make_lib_tests():
    posi = None
    t_env = _read("source/lib/tests/test_env_mat_a.cc")
    posi = cpp_vector(t_env, "posi")
    atype = cpp_vector(t_env, "atype").astype(np.int32)
    box = np.array([13., 0, 0, 0, 13., 0, 0, 0, 13.])
    s = _lib_test_setup(posi, atype, box, 6.0, 0.8, [10, 10])
    np.savez_compressed(os.path.join(HERE, "env_mat_a.npz"), posi=posi, atype=atype, box=box,
                        rc=6.0, rc_smth=0.8, sel=np.array([10, 10]),
                        expected_env=cpp_vector(t_env, "expected_env"), **s)

    t_fmt = _read("source/lib/tests/test_fmt_nlist.cc")
    s = _lib_test_setup(posi, atype, box, 6.0, 0.8, [10, 10])
    np.savez_compressed(os.path.join(HERE, "fmt_nlist.npz"), posi=posi, atype=atype, box=box,
                        rc=6.0, sel=np.array([10, 10]),
                        expect_nlist_cpy=cpp_vector(t_fmt, "expect_nlist_cpy").astype(np.int32), **s)

    for name, fname in (("prod_force_a", "test_prod_force_a.cc"), ("prod_virial_a", "test_prod_virial_a.cc")):
        txt = _read("source/lib/tests/" + fname)
        s = _lib_test_setup(posi, atype, box, 6.0, 0.8, [5, 5])
        nloc, nnei = s["nlist"].shape
        net_deriv = 10 - np.arange(nloc * nnei * 4) * 0.01
        extra = {}
        if name == "prod_force_a":
            extra["expected_force"] = cpp_vector(txt, "expected_force")
        else:
            extra["expected_virial"] = cpp_vector(txt, "expected_virial")
            extra["expected_atom_virial"] = cpp_vector(txt, "expected_atom_virial")
        np.savez_compressed(os.path.join(HERE, name + ".npz"), posi=posi, atype=atype, box=box,
                            rc=6.0, rc_smth=0.8, sel=np.array([5, 5]), net_deriv=net_deriv,
                            **extra, **s)


def _reference_model(params, compress=None):
    import torch
    import refshim

    refshim.install()
    from deepmd.pt.model.model import get_model

    c = params.config
    cfg = {"type_map": [str(i) for i in range(c.ntypes)],
           "descriptor": {"type": "se_e2_a", "sel": list(c.sel), "rcut_smth": c.rcut_smth,
                          "rcut": c.rcut, "neuron": list(c.neuron), "axis_neuron": c.axis_neuron,
                          "type_one_side": c.type_one_side, "resnet_dt": c.resnet_dt,
                          "precision": "float64", "seed": 1},
           "fitting_net": {"neuron": list(c.fit_neuron), "resnet_dt": c.fit_resnet_dt,
                           "precision": "float64", "seed": 1}}
    model = get_model(cfg)
    sd = model.state_dict()
    for k, v in params.to_state_dict().items():
        assert k in sd, k
        sd[k] = torch.as_tensor(v, dtype=sd[k].dtype).reshape(sd[k].shape)
    for k in list(sd):
        if "._networks." in k:
            sd[k] = sd[k.replace("._networks.", ".networks.")]
    model.load_state_dict(sd)
    if compress is not None:
        model.atomic_model.enable_compression(*compress)
    return model


def _run_reference(model, coord, atype, box):
    import torch
    from deepmd.pt.utils.nlist import extend_input_and_build_neighbor_list

    c = torch.as_tensor(coord.reshape(1, -1), dtype=torch.float64)
    t = torch.as_tensor(atype.reshape(1, -1), dtype=torch.int64)
    b = torch.as_tensor(box.reshape(1, 9), dtype=torch.float64)
    ret = model.forward(c, t, b, do_atomic_virial=True)
    ext, ext_t, mapping, nlist = extend_input_and_build_neighbor_list(
        c, t, model.get_rcut(), model.get_sel(), mixed_types=True, box=b)
    nlist = model.format_nlist(ext, ext_t, nlist)
    return ret, ext, ext_t, mapping, nlist


def _shift_order(box, rcut):
    """The image order the reference's (unstable) CPU argsort produced."""
    import torch
    from deepmd.pt.utils.region import to_face_distance

    cell = torch.as_tensor(box.reshape(1, 3, 3))
    nbuff = torch.ceil(rcut / to_face_distance(cell)).to(torch.int64).amax(0)
    xi = [torch.arange(-n, n + 1, dtype=torch.int64) for n in nbuff.tolist()]
    eye = torch.eye(3, dtype=torch.float64)
    xyz = (xi[0].view(-1, 1, 1, 1) * eye[0] + xi[1].view(1, -1, 1, 1) * eye[1]
           + xi[2].view(1, 1, -1, 1) * eye[2]).view(-1, 3)
    return torch.argsort(torch.linalg.norm(xyz, dim=-1)).numpy()


def make_water():
    import torch
    from dpgb import params as P, synth

    torch.set_num_threads(os.cpu_count() or 1)
    cfg = P.water_config()
    params = P.init_params(cfg, seed=1)
    coord, atype, box = synth.water_box(4, seed=0)
    model = _reference_model(params)
    ret, ext, ext_t, mapping, nlist = _run_reference(model, coord, atype, box)
    from deepmd.pt.model.descriptor.env_mat import prod_env_mat

    desc = model.atomic_model.descriptor
    em, diff, sw = prod_env_mat(ext, nlist, ext_t[:, :192], desc.sea.mean, desc.sea.stddev,
                                cfg.rcut, cfg.rcut_smth)
    d, rot, _, _, _ = desc(ext, ext_t, nlist)
    nkeep = 8
    np.savez_compressed(
        os.path.join(HERE, "water192.npz"), coord=coord, atype=atype, box=box,
        params_seed=1, coord_seed=0,
        energy=ret["energy"].detach().numpy().reshape(-1),
        force=ret["force"].detach().numpy().reshape(-1, 3),
        virial=ret["virial"].detach().numpy().reshape(-1),
        atom_energy=ret["atom_energy"].detach().numpy().reshape(-1),
        atom_virial=ret["atom_virial"].detach().numpy().reshape(-1, 9),
        nlist=nlist.numpy().reshape(192, -1).astype(np.int32),
        mapping=mapping.numpy().reshape(-1).astype(np.int32),
        coord_ext=ext.detach().numpy().reshape(-1, 3),
        shift_order=_shift_order(box, cfg.rcut),
        env_mat=em.detach().numpy().reshape(192, -1, 4)[:nkeep],
        sw=sw.detach().numpy().reshape(192, -1)[:nkeep],
        descriptor=d.detach().numpy().reshape(192, -1)[:nkeep],
        rot_mat=rot.detach().numpy().reshape(192, cfg.ng, 3)[:nkeep])
    return params, coord, atype, box


def make_water_compressed(params, coord, atype, box):
    # coarse strides keep the four tables small (the production strides are
    # 0.01 / 0.1; the algorithm is the same)
    min_nbor_dist, extrap, s1, s2 = 0.8, 5, 0.1, 1.0
    model = _reference_model(params, compress=(min_nbor_dist, extrap, s1, s2, -1))
    ret, *_ = _run_reference(model, coord, atype, box)
    sea = model.atomic_model.descriptor.sea
    tabs = {f"table_{e}": t.detach().numpy() for e, t in enumerate(sea.compress_data)}
    infos = {f"info_{e}": t.detach().numpy() for e, t in enumerate(sea.compress_info)}
    np.savez_compressed(
        os.path.join(HERE, "water192_compressed.npz"), min_nbor_dist=min_nbor_dist,
        extrapolate=extrap, stride0=s1, stride1=s2,
        energy=ret["energy"].detach().numpy().reshape(-1),
        force=ret["force"].detach().numpy().reshape(-1, 3),
        virial=ret["virial"].detach().numpy().reshape(-1), **tabs, **infos)


def make_pth():
    """A frozen model file as the reference's `dp --pt freeze` writes it
    (deepmd/pt/entrypoints/main.py freeze: torch.jit.script + torch.jit.save
    of the model get_model builds, model_def_script included): the reference
    test model deeppot_sea (weights of deeppot_sea_model.npz, type map O H),
    for the model-file reader and the DeepPot plugin backend."""
    import torch
    from conftest import deeppot_sea_params

    params = deeppot_sea_params()
    model = _reference_model(params)
    script = __import__("json").loads(model.model_def_script)
    script["type_map"] = ["O", "H"]
    model.model_def_script = __import__("json").dumps(script)
    model.eval()
    torch.jit.save(torch.jit.script(model), os.path.join(HERE, "deeppot_sea.pth"))


TRAIN_FRAMES = 16      # water frames of the force-loss training case (a batch of 16)
TRAIN_PREF = (0.02, 1000.0)  # energy and force prefactors (start == limit)


def train_frames():
    from dpgb import synth

    frames = [synth.water_box(4, seed=100 + k) for k in range(TRAIN_FRAMES)]
    coord = np.stack([f[0].reshape(-1) for f in frames])
    return coord, frames[0][1], np.stack([f[2].reshape(-1) for f in frames])


def make_train_grad():
    """One force-loss training step of the reference (deepmd.pt EnergyModel +
    EnergyStdLoss, FP64 autograd) on water frames labelled by a second,
    differently seeded model: the loss, the per-tensor gradient norms and 64
    gradient entries (tensor name, flat index, value)."""
    import refshim
    import torch

    refshim.install()
    from deepmd.pt.loss import EnergyStdLoss
    from dpgb import params as P

    torch.set_num_threads(os.cpu_count() or 1)
    cfg = P.water_config()
    coord, atype, box = train_frames()
    nf, nloc = coord.shape[0], atype.shape[0]
    teacher = _reference_model(P.init_params(cfg, seed=2))
    inp = {"coord": torch.as_tensor(coord), "atype": torch.as_tensor(np.tile(atype, (nf, 1)), dtype=torch.int64),
           "box": torch.as_tensor(box)}
    ref = teacher.forward(**inp)
    label = {"energy": ref["energy"].detach(), "force": ref["force"].detach(), "find_energy": 1.0,
             "find_force": 1.0}
    student = _reference_model(P.init_params(cfg, seed=1))
    loss_fn = EnergyStdLoss(starter_learning_rate=1.0, start_pref_e=TRAIN_PREF[0], limit_pref_e=TRAIN_PREF[0],
                            start_pref_f=TRAIN_PREF[1], limit_pref_f=TRAIN_PREF[1])
    _, loss, _ = loss_fn(inp, student, label, nloc, 1.0)
    loss.backward()
    names, norms, pick_name, pick_idx, pick_val = [], [], [], [], []
    rng = np.random.default_rng(64)
    grads = {k: p.grad.detach().numpy().reshape(-1) for k, p in student.named_parameters() if p.grad is not None}
    for k in sorted(grads):
        names.append(k)
        norms.append(float(np.linalg.norm(grads[k])))
    keys = sorted(grads)
    for _ in range(64):
        k = keys[int(rng.integers(len(keys)))]
        i = int(rng.integers(grads[k].size))
        pick_name.append(k)
        pick_idx.append(i)
        pick_val.append(grads[k][i])
    np.savez_compressed(
        os.path.join(HERE, "train_grad.npz"), coord=coord, atype=atype, box=box, pref=np.array(TRAIN_PREF),
        energy_label=ref["energy"].detach().numpy().reshape(-1), force_label=ref["force"].detach().numpy(),
        loss=float(loss.detach()), names=np.array(names), norms=np.array(norms), pick_name=np.array(pick_name),
        pick_idx=np.array(pick_idx), pick_val=np.array(pick_val))


TRAIN_STEPS = 6        # Adam steps of the training-loop case
TRAIN_BATCH = 4        # frames per batch: frames 0-11 train, 12-15 validate
TRAIN_LOOP_PREF = dict(start_pref_e=0.02, limit_pref_e=1.0, start_pref_f=1000.0, limit_pref_f=1.0)
TRAIN_LR = dict(start_lr=1e-3, stop_lr=1e-5, num_steps=TRAIN_STEPS)
TRAIN_DISP_FREQ = 2
TRAIN_LR_CASES = (   # schedules whose values the fixture also records
    dict(start_lr=1e-3, stop_lr=3.51e-8, num_steps=1000000, decay_steps=5000),
    dict(start_lr=2e-3, stop_lr_ratio=1e-4, num_steps=200000, decay_steps=5000, warmup_steps=500,
         warmup_start_factor=0.1),
    dict(start_lr=1e-3, stop_lr=1e-6, num_steps=50000, decay_steps=1000, smooth=True),
    dict(start_lr=1e-3, stop_lr=1e-5, num_steps=300000, decay_steps=2000, decay_rate=0.95),
    dict(start_lr=1e-3, stop_lr=1e-7, num_steps=400, decay_steps=5000),
    dict(start_lr=5e-4, stop_lr=1e-8, num_steps=20000, decay_steps=100000, warmup_ratio=0.05),
)


def make_train_steps():
    """Six Adam steps of the reference's training loop, assembled from its
    own parts as deepmd/pt/train/training.py:1074-1130, 1201-1213 and
    1385-1427 assemble them: deepmd.pt EnergyModel + EnergyStdLoss (FP64),
    LearningRateExp (start 1e-3, stop 1e-5 over 6 steps), torch Adam with
    the default betas behind a LambdaLR of lr(step) / start_lr.  Frames
    0-11 train in batches of 4 in order; frames 12-15 are one validation
    batch.  Recorded: the rate, loss and figures of every step, the
    parameter norms and 64 entries after the last step, and the lcurve.out
    text written by the reference's own print_header / print_on_training
    (display every 2 steps and at step 1, validation figures included)."""
    import io

    import refshim
    import torch

    refshim.install()
    from deepmd.dpmodel.utils.learning_rate import LearningRateExp
    from deepmd.pt.loss import EnergyStdLoss
    from deepmd.pt.train.training import Trainer
    from dpgb import params as P

    torch.set_num_threads(os.cpu_count() or 1)
    cfg = P.water_config()
    coord, atype, box = train_frames()
    nf, nloc = coord.shape[0], atype.shape[0]
    teacher = _reference_model(P.init_params(cfg, seed=2))
    at = torch.as_tensor(np.tile(atype, (nf, 1)), dtype=torch.int64)
    ref = teacher.forward(torch.as_tensor(coord), at, torch.as_tensor(box))
    e_lab, f_lab = ref["energy"].detach(), ref["force"].detach()
    student = _reference_model(P.init_params(cfg, seed=1))
    lr = LearningRateExp(**TRAIN_LR)
    loss_fn = EnergyStdLoss(starter_learning_rate=lr.start_lr, **TRAIN_LOOP_PREF)
    opt = torch.optim.Adam(student.parameters(), lr=lr.value(0), betas=(0.9, 0.999), weight_decay=0.0)
    for g in opt.param_groups:
        g["initial_lr"] = lr.start_lr
    sched = torch.optim.lr_scheduler.LambdaLR(opt, lambda s: lr.value(s) / lr.start_lr, last_epoch=-1)

    def batch(lo):
        sl = slice(lo, lo + TRAIN_BATCH)
        inp = {"coord": torch.as_tensor(coord[sl]), "atype": at[sl], "box": torch.as_tensor(box[sl])}
        lab = {"energy": e_lab[sl], "force": f_lab[sl], "find_energy": 1.0, "find_force": 1.0}
        return inp, lab

    class _Fmt:
        multi_task = False

    fout = io.StringIO()
    lrs, losses, figs = [], [], []
    keys = None
    ntrain = 12
    for step in range(TRAIN_STEPS):
        opt.zero_grad(set_to_none=True)
        inp, lab = batch((step * TRAIN_BATCH) % ntrain)
        cur = sched.get_last_lr()[0]
        _, loss, more = loss_fn(inp, student, lab, nloc, cur)
        loss.backward()
        opt.step()
        sched.step()
        trn = {k: float(more[k]) for k in sorted(more) if "l2_" not in k}
        keys = sorted(trn)
        lrs.append(cur)
        losses.append(float(loss.detach()))
        figs.append([trn[k] for k in keys])
        shown = step + 1
        if shown % TRAIN_DISP_FREQ == 0 or shown == 1:
            vinp, vlab = batch(ntrain)
            _, _, vmore = loss_fn(vinp, student, vlab, nloc, cur)
            val = {k: float(vmore[k]) for k in sorted(vmore) if "l2_" not in k}
            if shown == 1:
                Trainer.print_header(_Fmt(), fout, trn, val)
            Trainer.print_on_training(_Fmt(), fout, shown, cur, trn, val)
    params = {k: p.detach().numpy().reshape(-1) for k, p in student.named_parameters() if p.numel() > 0}
    names = sorted(params)
    rng = np.random.default_rng(65)
    pick_name, pick_idx, pick_val = [], [], []
    for _ in range(64):
        k = names[int(rng.integers(len(names)))]
        i = int(rng.integers(params[k].size))
        pick_name.append(k)
        pick_idx.append(i)
        pick_val.append(params[k][i])
    cases, case_steps, case_lr = [], [], []
    for kw in TRAIN_LR_CASES:
        sched_c = LearningRateExp(**kw)
        cases.append(repr(sorted(kw.items())))
        steps = [0, 1, 99, 100, 101, 4999, 5000, 5001, 123456, kw["num_steps"] - 1, kw["num_steps"],
                 2 * kw["num_steps"]]
        case_steps.append(steps)
        case_lr.append([sched_c.value(t) for t in steps])
    np.savez_compressed(
        os.path.join(HERE, "train_steps.npz"), lr_cases=np.array(cases), lr_case_steps=np.array(case_steps),
        lr_case_values=np.array(case_lr), energy_label=e_lab.numpy().reshape(-1), force_label=f_lab.numpy(),
        lr=np.array(lrs), loss=np.array(losses), fig_names=np.array(keys), figs=np.array(figs),
        names=np.array(names), norms=np.array([np.linalg.norm(params[k]) for k in names]),
        pick_name=np.array(pick_name), pick_idx=np.array(pick_idx), pick_val=np.array(pick_val),
        lcurve=np.array(fout.getvalue()))


if __name__ == "__main__":
    import oracle as O

    if not os.path.isdir(os.path.join(REF, "source")):
        sys.exit("make_golden: set DPGB_REFERENCE to the deepmd-kit reference checkout")

    O.build_ref()
    make_tabulate()
    make_deeppot_case()
    make_lib_tests()
    p, c, t, b = make_water()
    make_water_compressed(p, c, t, b)
    make_train_grad()
    make_train_steps()
    make_pth()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
