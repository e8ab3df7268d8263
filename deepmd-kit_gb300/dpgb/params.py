"""se_e2_a model parameters in the reference's own parameterisation.

A :class:`SeAParams` holds the descriptor statistics (``mean``/``stddev``), the
embedding nets, the per-type energy fitting nets and the per-type energy bias,
with the shapes and key names of the reference PyTorch model
(``deepmd/pt/model/descriptor/se_a.py:534-576``,
``deepmd/pt/model/task/fitting.py:528-547``, ``deepmd/pt/model/network/mlp.py:71-163``),
so a reference ``state_dict`` converts both ways (:meth:`from_state_dict`,
:meth:`to_state_dict`).  :func:`init_params` draws the seeded random
initialisation used for the synthetic water / alloy systems.
"""
from __future__ import annotations

import dataclasses
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

MAX_TYPES = 8
MAX_LAYERS = 6

_DESC = "atomic_model.descriptor.sea."
_FIT = "atomic_model.fitting_net."


@dataclasses.dataclass
class SeAConfig:
    """Hyper-parameters of a se_e2_a energy model (DescrptSeA + EnerFitting)."""

    sel: List[int]
    rcut: float = 6.0
    rcut_smth: float = 0.5
    neuron: List[int] = dataclasses.field(default_factory=lambda: [25, 50, 100])
    axis_neuron: int = 16
    type_one_side: bool = False
    resnet_dt: bool = False
    fit_neuron: List[int] = dataclasses.field(default_factory=lambda: [240, 240, 240])
    fit_resnet_dt: bool = True
    exclude_types: List[Tuple[int, int]] = dataclasses.field(default_factory=list)
    activation_function: str = "tanh"

    @property
    def ntypes(self) -> int:
        return len(self.sel)

    @property
    def nnei(self) -> int:
        return int(sum(self.sel))

    @property
    def ng(self) -> int:
        return int(self.neuron[-1])

    @property
    def dim_descrpt(self) -> int:
        return self.ng * self.axis_neuron

    @property
    def nnets(self) -> int:
        return self.ntypes if self.type_one_side else self.ntypes * self.ntypes

    def net_index(self, neighbor_type: int, center_type: int) -> int:
        """Embedding-net index of a (neighbour, centre) type pair
        (se_a.py:805-808: ``ii = e // ntypes`` neighbour, ``ti = e % ntypes``)."""
        if self.type_one_side:
            return neighbor_type
        return neighbor_type * self.ntypes + center_type

    def pair_mask(self) -> Optional[np.ndarray]:
        if not self.exclude_types:
            return None
        m = np.ones((self.ntypes, self.ntypes), dtype=np.int32)
        for a, b in self.exclude_types:
            m[a, b] = 0
            m[b, a] = 0
        return m

    def validate(self) -> None:
        if self.ntypes > MAX_TYPES:
            raise ValueError(f"at most {MAX_TYPES} types are supported")
        if len(self.neuron) > MAX_LAYERS or len(self.fit_neuron) > MAX_LAYERS:
            raise ValueError(f"at most {MAX_LAYERS} layers per net")
        if self.activation_function != "tanh":
            raise ValueError("only the tanh activation of se_e2_a is implemented")
        if self.rcut_smth >= self.rcut:
            raise ValueError("rmin should be less than rmax.")
        if self.axis_neuron > self.ng:
            raise ValueError("axis_neuron must not exceed the last embedding width")


def _layer_shapes(nin: int, widths: Sequence[int]):
    out = []
    for w in widths:
        out.append((nin, w))
        nin = w
    return out


def _has_idt(resnet_dt: bool, nin: int, nout: int) -> bool:
    # MLPLayer: use_timestep only when a skip connection exists (mlp.py:90-92)
    return resnet_dt and (nout == nin or nout == 2 * nin)


@dataclasses.dataclass
class SeAParams:
    """FP64 parameters. Layer lists are ``[(matrix, bias, idt_or_None), ...]``."""

    config: SeAConfig
    mean: np.ndarray                      # [ntypes, nnei, 4]
    stddev: np.ndarray                    # [ntypes, nnei, 4]
    emb: List[List[Tuple[np.ndarray, np.ndarray, Optional[np.ndarray]]]]
    fit: List[List[Tuple[np.ndarray, Optional[np.ndarray], Optional[np.ndarray]]]]
    bias_atom_e: np.ndarray               # [ntypes]
    out_bias: np.ndarray                  # [ntypes]
    tables: Optional[List[np.ndarray]] = None        # per net [nspline, 6*ng]
    table_info: Optional[List[np.ndarray]] = None    # per net [6]

    @property
    def compressed(self) -> bool:
        return self.tables is not None

    def atom_ener_bias(self) -> np.ndarray:
        return (self.bias_atom_e + self.out_bias).astype(np.float64)

    # ---- conversion to / from the reference state dict ----
    @classmethod
    def from_state_dict(cls, sd: Dict[str, "np.ndarray"], config: SeAConfig) -> "SeAParams":
        def g(k):
            v = sd[k]
            return v.detach().cpu().numpy().astype(np.float64) if hasattr(v, "detach") else np.asarray(v, np.float64)

        c = config
        emb = []
        for e in range(c.nnets):
            layers = []
            for l, (nin, nout) in enumerate(_layer_shapes(1, c.neuron)):
                p = f"{_DESC}filter_layers.networks.{e}.layers.{l}."
                idt = g(p + "idt") if (p + "idt") in sd else None
                layers.append((g(p + "matrix"), g(p + "bias"), idt))
            emb.append(layers)
        fit = []
        for t in range(c.ntypes):
            layers = []
            shapes = _layer_shapes(c.dim_descrpt, c.fit_neuron) + [(c.fit_neuron[-1] if c.fit_neuron else c.dim_descrpt, 1)]
            for l, _ in enumerate(shapes):
                p = f"{_FIT}filter_layers.networks.{t}.layers.{l}."
                idt = g(p + "idt") if (p + "idt") in sd else None
                bias = g(p + "bias") if (p + "bias") in sd else None
                layers.append((g(p + "matrix"), bias, idt))
            fit.append(layers)
        bias_atom_e = g(_FIT + "bias_atom_e").reshape(-1)
        out_bias = np.zeros(c.ntypes)
        if "atomic_model.out_bias" in sd:
            out_bias = g("atomic_model.out_bias").reshape(-1)[: c.ntypes]
        return cls(c, g(_DESC + "mean"), g(_DESC + "stddev"), emb, fit, bias_atom_e, out_bias)

    def to_state_dict(self) -> Dict[str, np.ndarray]:
        c = self.config
        sd = {_DESC + "mean": self.mean, _DESC + "stddev": self.stddev}
        for e, layers in enumerate(self.emb):
            for l, (w, b, idt) in enumerate(layers):
                p = f"{_DESC}filter_layers.networks.{e}.layers.{l}."
                sd[p + "matrix"] = w
                sd[p + "bias"] = b
                if idt is not None:
                    sd[p + "idt"] = idt
        for t, layers in enumerate(self.fit):
            for l, (w, b, idt) in enumerate(layers):
                p = f"{_FIT}filter_layers.networks.{t}.layers.{l}."
                sd[p + "matrix"] = w
                if b is not None:
                    sd[p + "bias"] = b
                if idt is not None:
                    sd[p + "idt"] = idt
        sd[_FIT + "bias_atom_e"] = self.bias_atom_e.reshape(c.ntypes, 1)
        sd["atomic_model.out_bias"] = self.out_bias.reshape(1, c.ntypes, 1)
        return sd


def init_params(config: SeAConfig, seed: int = 1) -> SeAParams:
    """Seeded random initialisation: matrices ~ N(0, 1/(fan_in+fan_out)),
    biases ~ N(0, 1), idt ~ N(0.1, 0.001) (the default normal init of
    mlp.py:149-163); mean 0, stddev 1, energy bias 0."""
    config.validate()
    rng = np.random.default_rng(seed)
    c = config

    def layer(nin, nout, resnet_dt, bias=True):
        w = rng.normal(0.0, 1.0 / np.sqrt(nin + nout), size=(nin, nout))
        b = rng.normal(0.0, 1.0, size=(nout,)) if bias else None
        idt = rng.normal(0.1, 0.001, size=(nout,)) if _has_idt(resnet_dt, nin, nout) else None
        return (w, b, idt)

    emb = [[layer(nin, nout, c.resnet_dt) for nin, nout in _layer_shapes(1, c.neuron)]
           for _ in range(c.nnets)]
    fit = []
    for _ in range(c.ntypes):
        layers = [layer(nin, nout, c.fit_resnet_dt) for nin, nout in _layer_shapes(c.dim_descrpt, c.fit_neuron)]
        nlast = c.fit_neuron[-1] if c.fit_neuron else c.dim_descrpt
        layers.append(layer(nlast, 1, False))
        fit.append(layers)
    mean = np.zeros((c.ntypes, c.nnei, 4))
    std = np.ones((c.ntypes, c.nnei, 4))
    return SeAParams(c, mean, std, emb, fit, np.zeros(c.ntypes), np.zeros(c.ntypes))


# Factor that brings the seeded random-init water model's forces on the
# synthetic water boxes (RMS 3.8e-4 eV/A) to about 1 eV/A RMS, the magnitude
# of forces in trained liquid-water models; see scale_energy.
WATER_FORCE_SCALE = 2650.0


def scale_energy(params: SeAParams, factor: float) -> SeAParams:
    """A copy of ``params`` whose energy is ``factor`` times the original:
    the output layer of every fitting net (matrix and bias) and the per-type
    energy biases are scaled, so forces and virials scale by the same factor
    while the descriptor and hidden layers are unchanged.  Used to test
    mixed-precision errors against absolute force bounds at a realistic
    force magnitude."""
    fit = []
    for layers in params.fit:
        w, b, idt = layers[-1]
        fit.append(list(layers[:-1]) + [(w * factor, None if b is None else b * factor, idt)])
    return dataclasses.replace(params, fit=fit, bias_atom_e=params.bias_atom_e * factor,
                               out_bias=params.out_bias * factor)


def water_config() -> SeAConfig:
    """The water model: rcut 6, rcut_smth 0.5, sel [46, 92], embedding
    [25, 50, 100] tanh, type_one_side false, axis 16, fitting [240]*3."""
    return SeAConfig(sel=[46, 92], rcut=6.0, rcut_smth=0.5, neuron=[25, 50, 100],
                     axis_neuron=16, type_one_side=False, fit_neuron=[240, 240, 240])


def alloy_config() -> SeAConfig:
    """The fcc alloy model: rcut 6, rcut_smth 2, sel [60]*4."""
    return SeAConfig(sel=[60, 60, 60, 60], rcut=6.0, rcut_smth=2.0, neuron=[25, 50, 100],
                     axis_neuron=16, type_one_side=False, fit_neuron=[240, 240, 240])
