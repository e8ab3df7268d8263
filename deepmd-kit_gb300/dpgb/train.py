"""Force-loss training of the se_e2_a energy model: Adam steps on the
exponential learning-rate schedule, energy / force / virial prefactors
interpolated by the learning rate, and the learning curve written as
``lcurve.out`` in the reference's column format.

Follows ``deepmd.pt`` training (deepmd/pt/train/training.py): the Adam
optimiser built with the configured betas and weight decay, fused on a GPU
(:1074-1130); the LambdaLR scheduler whose factor is lr(step) / start_lr
(:1201-1213); one step = zero_grad, loss through the wrapper at the
scheduler's current rate, backward, optional gradient-norm clipping,
optimizer.step, scheduler.step (:1385-1427); the displayed training figures,
either the current batch's or the average over the display interval
(``disp_avg``, :1501-1575); the validation figures as the atom-weighted
average over ``valid_numb_batch`` batches (:1576-1605); the file header and
rows (print_header / print_on_training, :2256-2320), the first row at step 1
and then every ``disp_freq`` steps.  The schedule is LearningRateExp of
deepmd/dpmodel/utils/learning_rate.py:36-200 (warmup) and :263-399 (decay).

The model is :class:`dpgb.model.EnergyModelSeA` on the dpgb descriptor
kernels (FP64, with hand-written first and second derivatives); the
optimiser is torch's Adam, the one the reference constructs.
"""
from __future__ import annotations

from typing import Dict, List, Optional

import numpy as np
import torch

from .model import EnergyModelSeA, EnergyStdLoss


class LearningRateExp:
    """Exponentially decayed learning rate with optional linear warmup
    (deepmd/dpmodel/utils/learning_rate.py:36-200, 263-399).

    Without warmup, lr(t) = start_lr * decay_rate ** floor(t / decay_steps)
    (``smooth``: t / decay_steps unfloored), never below stop_lr.  The
    decay rate, unless given, is (stop_lr / start_lr) ** (decay_steps /
    decay_total) with decay_total = num_steps - warmup_steps; a
    ``decay_steps`` not below decay_total is replaced by 100 when
    decay_total // 10 > 100, else by decay_total // 100 + 1.  During the
    warmup the rate rises linearly from warmup_start_factor * start_lr."""

    def __init__(self, start_lr: float, num_steps: int, stop_lr: Optional[float] = None,
                 stop_lr_ratio: Optional[float] = None, decay_steps: int = 5000,
                 decay_rate: Optional[float] = None, warmup_steps: int = 0,
                 warmup_ratio: Optional[float] = None, warmup_start_factor: float = 0.0,
                 smooth: bool = False):
        if stop_lr is not None and stop_lr_ratio is not None:
            raise ValueError("stop_lr and stop_lr_ratio are mutually exclusive")
        if stop_lr is None and stop_lr_ratio is None:
            raise ValueError("Either stop_lr or stop_lr_ratio must be provided")
        self.stop_lr = start_lr * stop_lr_ratio if stop_lr_ratio is not None else stop_lr
        if warmup_steps != 0 and warmup_ratio is not None:
            raise ValueError("warmup_steps and warmup_ratio are mutually exclusive")
        self.warmup_steps = int(warmup_ratio * num_steps) if warmup_ratio is not None else warmup_steps
        if num_steps < 0:
            raise ValueError("num_steps must be non-negative")
        if self.warmup_steps < 0:
            raise ValueError("warmup_steps must be non-negative")
        if num_steps > 0 and self.warmup_steps >= num_steps:
            raise ValueError("warmup_steps must be smaller than num_steps")
        if num_steps == 0 and self.warmup_steps != 0:
            raise ValueError("warmup_steps must be 0 when num_steps is 0")
        self.warmup_start_lr = warmup_start_factor * start_lr
        self.start_lr = start_lr
        self.num_steps = num_steps
        self.decay_num_steps = num_steps - self.warmup_steps
        if decay_steps <= 0:
            raise ValueError(f"decay_steps ({decay_steps}) must be positive.")
        total = self.decay_num_steps
        self.decay_steps = decay_steps
        if decay_rate is None and decay_steps >= total:
            self.decay_steps = 100 if total // 10 > 100 else total // 100 + 1
        self.min_lr = self.stop_lr
        if decay_rate is not None:
            self.decay_rate = float(decay_rate)
        elif total == 0:
            self.decay_rate = 1.0
        else:
            self.decay_rate = float(np.exp(np.log(max(self.stop_lr, 1e-10) / start_lr) / (total / self.decay_steps)))
        self.smooth = smooth

    def _decay(self, step: float) -> float:
        e = step / self.decay_steps if self.smooth else float(step // self.decay_steps)
        return max(float(self.start_lr * np.power(np.float64(self.decay_rate), np.float64(e))), self.min_lr)

    def value(self, step) -> float:
        step = float(step)
        if self.warmup_steps == 0:
            return self._decay(step)
        if step < self.warmup_steps:
            return self.warmup_start_lr + (self.start_lr - self.warmup_start_lr) * (step / self.warmup_steps)
        return self._decay(max(step - self.warmup_steps, 0.0))


def lcurve_header(train_results: Dict[str, float], valid_results: Optional[Dict[str, float]]) -> str:
    """The two header lines of lcurve.out (training.py:2256-2286): ``# step``,
    one column per sorted figure name (``<name>_val <name>_trn`` with
    validation data, ``<name>_trn`` without), then ``lr``."""
    s = "# {:5s}".format("step")
    for k in sorted(train_results):
        s += ("   %11s %11s" % (k + "_val", k + "_trn")) if valid_results else ("   %11s" % (k + "_trn"))
    s += "   {:8s}\n".format("lr")
    s += "# If there is no available reference data, rmse_*_{val,trn} will print nan\n"
    return s


def lcurve_row(step: int, lr: float, train_results: Dict[str, float],
               valid_results: Optional[Dict[str, float]]) -> str:
    """One lcurve.out row (training.py:2288-2320): the step in 7 columns,
    each figure as %11.2e (validation before training), the rate as %8.1e."""
    s = f"{step:7d}"
    for k in sorted(train_results):
        s += ("   %11.2e %11.2e" % (valid_results[k], train_results[k])) if valid_results else (
            "   %11.2e" % train_results[k])
    return s + f"   {lr:8.1e}\n"


class FrameSet:
    """Labelled frames of one system, served in batches of ``batch_size``
    frames: coord [nf, natoms*3], atype [natoms] or [nf, natoms], box [nf, 9]
    (or None), and any of energy [nf], force [nf, natoms, 3], virial [nf, 9].
    Batches walk the frames in order, reshuffled each pass when a seed is
    given.  A batch is the reference's (input_dict, label_dict) pair, with
    ``find_<label>`` set to 1.0 for each label present and 0.0 otherwise.
    With ``device`` set, the frames are held there and a batch is gathered
    on that device; otherwise each batch is copied from host memory."""

    LABELS = ("energy", "force", "virial")

    def __init__(self, coord, atype, box=None, energy=None, force=None, virial=None, batch_size: int = 1,
                 seed: Optional[int] = None, device=None):
        self.coord = np.asarray(coord, dtype=np.float64)
        nf = self.coord.shape[0]
        self.coord = self.coord.reshape(nf, -1)
        natoms = self.coord.shape[1] // 3
        atype = np.asarray(atype, dtype=np.int64)
        self.atype = np.broadcast_to(atype.reshape(-1, natoms), (nf, natoms)).copy()
        self.box = None if box is None else np.asarray(box, dtype=np.float64).reshape(nf, 9)
        self.labels = {}
        for name, v in zip(self.LABELS, (energy, force, virial)):
            if v is not None:
                self.labels[name] = np.asarray(v, dtype=np.float64)
        if "energy" in self.labels:
            self.labels["energy"] = self.labels["energy"].reshape(nf, 1)
        if "force" in self.labels:
            self.labels["force"] = self.labels["force"].reshape(nf, natoms, 3)
        if "virial" in self.labels:
            self.labels["virial"] = self.labels["virial"].reshape(nf, 9)
        if batch_size < 1 or batch_size > nf:
            raise ValueError(f"batch_size {batch_size} outside 1..{nf}")
        self.nframes, self.natoms, self.batch_size = nf, natoms, batch_size
        self._rng = None if seed is None else np.random.default_rng(seed)
        self._order = np.arange(nf)
        self._pos = nf  # start a new pass on the first call
        self.resident = device
        if device is not None:
            self._dev = {"coord": torch.as_tensor(self.coord, device=device),
                         "atype": torch.as_tensor(self.atype, device=device),
                         "box": None if self.box is None else torch.as_tensor(self.box, device=device)}
            self._dev.update({k: torch.as_tensor(v, device=device) for k, v in self.labels.items()})

    def next_batch(self, device) -> tuple:
        if self._pos + self.batch_size > self.nframes:
            self._order = self._rng.permutation(self.nframes) if self._rng is not None else np.arange(self.nframes)
            self._pos = 0
        idx = self._order[self._pos:self._pos + self.batch_size]
        self._pos += self.batch_size
        if self.resident is not None:
            sl = slice(int(idx[0]), int(idx[0]) + len(idx)) if np.all(np.diff(idx) == 1) else None
            take = (lambda t: t[sl]) if sl is not None else (
                lambda t: t.index_select(0, torch.as_tensor(idx, device=t.device)))
            inp = {k: None if self._dev[k] is None else take(self._dev[k]) for k in ("coord", "atype", "box")}
            label = {k: take(self._dev[k]) for k in self.labels}
            for k in self.LABELS:
                label["find_" + k] = 1.0 if k in self.labels else 0.0
            return inp, label
        inp = {"coord": torch.as_tensor(self.coord[idx], device=device),
               "atype": torch.as_tensor(self.atype[idx], device=device),
               "box": None if self.box is None else torch.as_tensor(self.box[idx], device=device)}
        label = {k: torch.as_tensor(v[idx], device=device) for k, v in self.labels.items()}
        for k in self.LABELS:
            label["find_" + k] = 1.0 if k in self.labels else 0.0
        return inp, label


class Trainer:
    """Adam training of an EnergyModelSeA on one FrameSet (training.py:
    1074-1130, 1385-1427, 1501-1720).

    ``loss_params`` are EnergyStdLoss's (start/limit prefactors of energy,
    force and virial); the loss's starter learning rate is the schedule's
    start_lr, as the reference sets it.  ``step()`` runs one optimisation
    step and returns the figures it displayed, if any; ``run(n)`` runs n
    steps, writing lcurve rows to ``disp_file`` when it is set."""

    def __init__(self, model: EnergyModelSeA, lr: LearningRateExp, train: FrameSet,
                 valid: Optional[FrameSet] = None, loss_params: Optional[dict] = None, disp_freq: int = 1000,
                 disp_file: Optional[str] = "lcurve.out", disp_avg: bool = False, valid_numb_batch: int = 1,
                 gradient_max_norm: float = 0.0, adam_beta1: float = 0.9, adam_beta2: float = 0.999,
                 weight_decay: float = 0.0, start_step: int = 0):
        self.model, self.lr_schedule, self.train_data, self.valid_data = model, lr, train, valid
        self.loss = EnergyStdLoss(starter_learning_rate=lr.start_lr, **(loss_params or {}))
        self.device = next(model.parameters()).device
        self.disp_freq, self.disp_file, self.disp_avg = disp_freq, disp_file, disp_avg
        self.valid_numb_batch = valid_numb_batch
        self.gradient_max_norm = gradient_max_norm
        self.optimizer = torch.optim.Adam(model.parameters(), lr=lr.value(start_step),
                                          betas=(float(adam_beta1), float(adam_beta2)),
                                          weight_decay=float(weight_decay), fused=self.device.type != "cpu")
        base = float(lr.start_lr)
        for group in self.optimizer.param_groups:
            group["initial_lr"] = base
        self.scheduler = torch.optim.lr_scheduler.LambdaLR(self.optimizer, lambda s: lr.value(s) / base,
                                                           last_epoch=start_step - 1)
        self.step_id = start_step
        if disp_file:  # a fresh run truncates the curve, a restart appends (training.py:1336-1346)
            open(disp_file, "w" if start_step == 0 else "a").close()
        self._accu: Dict[str, float] = {}
        self._accu_n = 0
        self._header_due = True
        self.history: List[dict] = []
        self.last_lr, self.last_loss = None, None

    def _valid_results(self, cur_lr: float) -> Dict[str, float]:
        if self.valid_data is None:
            return {}
        sums: Dict[str, float] = {}
        total = 0
        for _ in range(self.valid_numb_batch):
            inp, label = self.valid_data.next_batch(self.device)
            natoms = int(inp["atype"].shape[-1])
            _, _, more = self.loss(inp, self.model, label, natoms, cur_lr)
            total += natoms
            for k, v in more.items():
                sums[k] = sums.get(k, 0.0) + float(v) * natoms
        return {k: v / total for k, v in sums.items()}

    def step(self) -> Optional[dict]:
        """One training step; returns {"step", "lr", "trn", "val"} on the
        display steps (the first and every disp_freq-th), else None."""
        self.model.train()
        self.optimizer.zero_grad(set_to_none=True)
        inp, label = self.train_data.next_batch(self.device)
        cur_lr = self.scheduler.get_last_lr()[0]
        _, loss, more = self.loss(inp, self.model, label, int(inp["atype"].shape[-1]), cur_lr)
        loss.backward()
        self.last_lr, self.last_loss = cur_lr, loss.detach()
        if self.gradient_max_norm > 0.0:
            total_norm = torch.nn.utils.clip_grad_norm_(self.model.parameters(), self.gradient_max_norm)
            if not torch.isfinite(total_norm):
                raise FloatingPointError(f"non-finite gradient norm {float(total_norm)} at step {self.step_id}")
        self.optimizer.step()
        self.scheduler.step()
        step_no = self.step_id + 1
        self.step_id = step_no
        more = {k: float(v) for k, v in more.items()}
        if self.disp_avg:
            self._accu_n += 1
            for k, v in more.items():
                self._accu[k] = self._accu.get(k, 0.0) + v
        if step_no % self.disp_freq != 0 and step_no != 1:
            return None
        self.model.eval()
        if self.disp_avg:
            trn = {k: v / self._accu_n for k, v in sorted(self._accu.items())}
            self._accu, self._accu_n = {}, 0
        else:
            trn = dict(sorted(more.items()))
        val = self._valid_results(cur_lr)
        rec = {"step": step_no, "lr": cur_lr, "trn": trn, "val": val}
        self.history.append(rec)
        if self.disp_file:
            with open(self.disp_file, "a") as f:
                if self._header_due:
                    f.write(lcurve_header(trn, val))
                f.write(lcurve_row(step_no, cur_lr, trn, val))
        self._header_due = False
        return rec

    def run(self, num_steps: Optional[int] = None) -> List[dict]:
        n = self.lr_schedule.num_steps - self.step_id if num_steps is None else num_steps
        for _ in range(n):
            self.step()
        return self.history
