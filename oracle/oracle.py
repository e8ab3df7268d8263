"""Test infrastructure only: Python front end of the CPU oracle.

Loads ``oracle/liboracle.so`` (the plain-C restatement in dpgb_oracle.c,
compiled by :func:`build`) and, when present, ``oracle/_ref/libdeepmd_ref.so``
(the reference's own CPU library compiled from its sources by build_ref.sh).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker; the product never imports it.

numpy restatements here cite the reference file:line they follow.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libdeepmd_ref.so")
MAX_TYPES = 8
MAX_LAYERS = 6

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile the C restatement (seconds).  Returns the library path."""
    src = os.path.join(HERE, "dpgb_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-fopenmp", "-std=c11", "-shared",
                               "-o", LIB_PATH, src, "-lm"])
    return LIB_PATH


def build_ref() -> Optional[str]:
    """Compile the reference CPU library when DPGB_REFERENCE names a
    reference checkout (else nothing is built and None is returned)."""
    script = os.path.join(HERE, "build_ref.sh")
    ref = os.environ.get("DPGB_REFERENCE", "")
    if not ref or not os.path.isdir(os.path.join(ref, "source", "lib", "src")):
        return None
    probe = os.path.join(HERE, "_ref", "abi_probe_reference.txt")
    if not os.path.exists(REF_PATH) or not os.path.exists(probe) or os.path.getmtime(REF_PATH) < os.path.getmtime(
            os.path.join(HERE, "ref_shim.cc")):
        subprocess.check_call(["bash", script])
    return REF_PATH


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.orc_num_threads.restype = C.c_int
    return _lib


def ref_lib():
    """The reference's own compiled CPU library, or None when unavailable
    (for example on a machine without the reference tree)."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            try:
                build_ref()
            except Exception:
                return None
        if not os.path.exists(REF_PATH):
            return None
        try:
            _ref = C.CDLL(REF_PATH)
        except OSError:
            return None
    return _ref


def _p(a: np.ndarray):
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.float32:
        return a.ctypes.data_as(_fp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    raise TypeError(a.dtype)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# --------------------------------------------------------------------------
# tabulate_fusion_se_a
def tabulate_fusion_se_a(table, info, em_x, em, last_layer_size, is_sorted=True, use_ref=False):
    dt = np.float64 if np.asarray(table).dtype == np.float64 else np.float32
    sfx = "f64" if dt == np.float64 else "f32"
    table, info, em_x, em = (_c(x, dt) for x in (table, info, em_x, em))
    nloc, nnei = em.shape[0], em.shape[1]
    out = np.zeros((nloc, 4, last_layer_size), dt)
    fn = getattr(ref_lib(), f"ref_tabulate_fusion_se_a_{sfx}") if use_ref else getattr(lib(), f"orc_tabulate_fusion_se_a_{sfx}")
    fn(_p(out), _p(table), _p(info), _p(em_x), _p(em), nloc, nnei, last_layer_size, int(is_sorted))
    return out


def tabulate_fusion_se_a_grad(table, info, em_x, em, dy, is_sorted=True, use_ref=False):
    dt = np.float64 if np.asarray(table).dtype == np.float64 else np.float32
    sfx = "f64" if dt == np.float64 else "f32"
    table, info, em_x, em, dy = (_c(x, dt) for x in (table, info, em_x, em, dy))
    nloc, nnei = em.shape[0], em.shape[1]
    nl = dy.shape[-1]
    dx = np.zeros(em_x.shape, dt)
    dem = np.zeros(em.shape, dt)
    fn = getattr(ref_lib(), f"ref_tabulate_fusion_se_a_grad_{sfx}") if use_ref else getattr(lib(), f"orc_tabulate_fusion_se_a_grad_{sfx}")
    fn(_p(dx), _p(dem), _p(table), _p(info), _p(em_x), _p(em), _p(dy), nloc, nnei, nl, int(is_sorted))
    return dx, dem


def tabulate_fusion_se_a_grad_grad(table, info, em_x, em, dz_dx, dz_dem, last_layer_size,
                                   is_sorted=True, use_ref=False):
    dt = np.float64 if np.asarray(table).dtype == np.float64 else np.float32
    sfx = "f64" if dt == np.float64 else "f32"
    table, info, em_x, em, dz_dx, dz_dem = (_c(x, dt) for x in (table, info, em_x, em, dz_dx, dz_dem))
    nloc, nnei = em.shape[0], em.shape[1]
    out = np.zeros((nloc, 4, last_layer_size), dt)
    fn = getattr(ref_lib(), f"ref_tabulate_fusion_se_a_grad_grad_{sfx}") if use_ref else getattr(lib(), f"orc_tabulate_fusion_se_a_grad_grad_{sfx}")
    fn(_p(out), _p(table), _p(info), _p(em_x), _p(em), _p(dz_dx), _p(dz_dem), nloc, nnei,
       last_layer_size, int(is_sorted))
    return out


# --------------------------------------------------------------------------
# region / ghosts / neighbour lists
def table_env_range(davg, dstd, min_nbor_dist, rcut_smth, rcut):
    """Per-type tabulation range (deepmd/utils/tabulate.py:468-498
    _get_env_mat_range, then the per-type min/max of build() 91-96)."""
    x = float(min_nbor_dist)
    if x < rcut_smth:
        sw = 1.0
    elif x < rcut:
        uu = (x - rcut_smth) / (rcut - rcut_smth)
        sw = uu * uu * uu * (-6 * uu * uu + 15 * uu - 10) + 1
    else:
        sw = 0.0
    davg = np.asarray(davg, dtype=np.float64)
    dstd = np.asarray(dstd, dtype=np.float64)
    lower = np.floor(-davg[:, 0] / dstd[:, 0])
    upper = np.ceil(((1 / x) * sw - davg[:, 0]) / dstd[:, 0])
    if lower.ndim > 1:
        lower = np.min(lower, axis=tuple(range(1, lower.ndim)))
        upper = np.max(upper, axis=tuple(range(1, upper.ndim)))
    return lower, upper


def table_build(layers, lower, upper, extrapolate, stride0, stride1):
    """One net's table (deepmd/utils/tabulate.py:128-148 grid, 275-370
    _build_lower; node values/derivatives as tabulate_math.py:353-470, tanh,
    no timestep).  layers = [(W [nin, nout], b [nout]), ...]."""
    xx = np.arange(lower, upper, stride0, dtype=np.float64)
    xx = np.append(xx, np.arange(upper, extrapolate * upper, stride1, dtype=np.float64))
    xx = np.append(xx, np.array([extrapolate * upper], dtype=np.float64))
    nspline = int((upper - lower) / stride0 + (extrapolate * upper - upper) / stride1)
    y = xx.reshape(-1, 1)
    d1 = np.ones_like(y)
    d2 = np.zeros_like(y)
    for W, b in layers:
        z = y @ W + b
        z1 = d1 @ W
        z2 = d2 @ W
        t = np.tanh(z)
        g = 1 - t * t
        ny, n1, n2 = t, g * z1, g * z2 - 2 * t * g * z1 * z1
        nin, nout = W.shape
        if nout == nin:
            ny, n1, n2 = ny + y, n1 + d1, n2 + d2
        elif nout == 2 * nin:
            ny = ny + np.concatenate([y, y], 1)
            n1 = n1 + np.concatenate([d1, d1], 1)
            n2 = n2 + np.concatenate([d2, d2], 1)
        y, d1, d2 = ny, n1, n2
    ng = y.shape[1]
    tt = np.full((nspline, ng), stride1)
    tt[: int((upper - lower) / stride0), :] = stride0
    v0, v1 = y[:nspline], y[1:nspline + 1]
    a0, a1 = d1[:nspline], d1[1:nspline + 1]
    s0, s1 = d2[:nspline], d2[1:nspline + 1]
    hh = v1 - v0
    out = np.zeros((nspline, 6 * ng))
    out[:, 0::6] = v0
    out[:, 1::6] = a0
    out[:, 2::6] = 0.5 * s0
    out[:, 3::6] = (1 / (2 * tt ** 3)) * (20 * hh - (8 * a1 + 12 * a0) * tt - (3 * s0 - s1) * tt * tt)
    out[:, 4::6] = (1 / (2 * tt ** 4)) * (-30 * hh + (14 * a1 + 16 * a0) * tt + (3 * s0 - 2 * s1) * tt * tt)
    out[:, 5::6] = (1 / (2 * tt ** 5)) * (12 * hh - 6 * (a1 + a0) * tt + (s1 - s0) * tt * tt)
    return out


def normalize_coord(coord: np.ndarray, box: np.ndarray) -> np.ndarray:
    """deepmd/pt/utils/region.py:86-105: wrap into the cell."""
    cell = box.reshape(3, 3)
    rec = np.linalg.inv(cell)
    inter = coord.reshape(-1, 3) @ rec
    inter = np.remainder(inter, 1.0)
    return inter @ cell


def to_face_distance(box: np.ndarray) -> np.ndarray:
    """deepmd/pt/utils/region.py:50-83."""
    cell = box.reshape(3, 3)
    vol = np.linalg.det(cell)
    return np.array([vol / np.linalg.norm(np.cross(cell[1], cell[2])),
                     vol / np.linalg.norm(np.cross(cell[2], cell[0])),
                     vol / np.linalg.norm(np.cross(cell[0], cell[1]))])


def ghost_shifts(box: np.ndarray, rcut: float, order: Optional[np.ndarray] = None) -> np.ndarray:
    """Integer image shifts of deepmd/pt/utils/nlist.py:470-497 in the order
    the reference sorts them by norm.  ``order`` overrides the permutation of
    equal-norm images (the reference's sort is not stable); by default a
    stable sort is used."""
    nbuff = np.ceil(rcut / to_face_distance(box)).astype(np.int64)
    rng = [np.arange(-n, n + 1) for n in nbuff]
    xyz = (rng[0].reshape(-1, 1, 1, 1) * np.eye(3)[0] + rng[1].reshape(1, -1, 1, 1) * np.eye(3)[1]
           + rng[2].reshape(1, 1, -1, 1) * np.eye(3)[2]).reshape(-1, 3)
    if order is None:
        order = np.argsort(np.linalg.norm(xyz, axis=-1), kind="stable")
    return xyz[np.asarray(order)]


def extend_coord_with_ghosts(coord, atype, box, rcut, order=None):
    """deepmd/pt/utils/nlist.py:424-513: all periodic images, image-major."""
    coord = coord.reshape(-1, 3)
    nloc = coord.shape[0]
    if box is None:
        return coord.copy(), np.asarray(atype, np.int32).copy(), np.arange(nloc, dtype=np.int32)
    shifts = ghost_shifts(box, rcut, order)
    shift_vec = shifts @ box.reshape(3, 3)
    ext = (coord[None, :, :] + shift_vec[:, None, :]).reshape(-1, 3)
    ext_t = np.tile(np.asarray(atype, np.int32), shifts.shape[0])
    mapping = np.tile(np.arange(nloc, dtype=np.int32), shifts.shape[0])
    return ext, ext_t, mapping


def build_nlist_pt(coord_ext, atype_ext, nloc, rcut, sel):
    coord_ext = _c(coord_ext, np.float64).reshape(-1, 3)
    atype_ext = _c(atype_ext, np.int32)
    sel = _c(sel, np.int32)
    nnei = int(sel.sum())
    out = np.empty((nloc, nnei), np.int32)
    lib().orc_build_nlist_pt(_p(out), _p(coord_ext), _p(atype_ext), nloc, coord_ext.shape[0],
                             C.c_double(rcut), _p(sel), len(sel))
    return out


def format_nlist_cpp(coord_ext, atype_ext, rows, counts, nloc, rcut, sel, use_ref=False):
    coord_ext = _c(coord_ext, np.float64).reshape(-1, 3)
    atype_ext = _c(atype_ext, np.int32)
    rows = _c(rows, np.int32)
    counts = _c(counts, np.int32)
    sel = _c(sel, np.int32)
    out = np.empty((nloc, int(sel.sum())), np.int32)
    if use_ref:
        ref_lib().ref_format_nlist_f64(_p(out), _p(coord_ext), _p(atype_ext), _p(rows), _p(counts),
                                       rows.shape[1], nloc, coord_ext.shape[0], C.c_double(rcut),
                                       _p(sel), len(sel))
    else:
        lib().orc_format_nlist_cpp(_p(out), _p(coord_ext), _p(atype_ext), _p(rows), _p(counts),
                                   rows.shape[1], nloc, coord_ext.shape[0], C.c_double(rcut),
                                   _p(sel), len(sel))
    return out


def env_mat_a(coord_ext, atype_ext, nlist, davg, dstd, rcut, rcut_smth):
    coord_ext = _c(coord_ext, np.float64).reshape(-1, 3)
    atype_ext = _c(atype_ext, np.int32)
    nlist = _c(nlist, np.int32)
    nloc, nnei = nlist.shape
    em = np.empty((nloc, nnei, 4))
    der = np.empty((nloc, nnei, 4, 3))
    rij = np.empty((nloc, nnei, 3))
    lib().orc_env_mat_a(_p(em), _p(der), _p(rij), _p(coord_ext), _p(atype_ext), _p(nlist),
                        _p(_c(davg, np.float64)), _p(_c(dstd, np.float64)), nloc, nnei,
                        C.c_double(rcut), C.c_double(rcut_smth))
    return em, der, rij


def prod_env_mat_a_ref(coord_ext, atype_ext, rows, counts, davg, dstd, nloc, rcut, rcut_smth, sel):
    """The reference prod_env_mat_a_cpu (source/lib/src/prod_env_mat.cc:14)."""
    coord_ext = _c(coord_ext, np.float64).reshape(-1, 3)
    sel = _c(sel, np.int32)
    nnei = int(sel.sum())
    em = np.empty((nloc, nnei, 4))
    der = np.empty((nloc, nnei, 4, 3))
    rij = np.empty((nloc, nnei, 3))
    nl = np.empty((nloc, nnei), np.int32)
    rows = _c(rows, np.int32)
    ref_lib().ref_prod_env_mat_a_f64(_p(em), _p(der), _p(rij), _p(nl), _p(coord_ext),
                                     _p(_c(atype_ext, np.int32)), _p(rows), _p(_c(counts, np.int32)),
                                     rows.shape[1], _p(_c(davg, np.float64)), _p(_c(dstd, np.float64)),
                                     nloc, coord_ext.shape[0], C.c_double(rcut), C.c_double(rcut_smth),
                                     _p(sel), len(sel))
    return em, der, rij, nl


def prod_force_a(net_deriv, env_deriv, nlist, nall, use_ref=False):
    nlist = _c(nlist, np.int32)
    nloc, nnei = nlist.shape
    f = np.zeros((nall, 3))
    nd, ed = _c(net_deriv, np.float64), _c(env_deriv, np.float64)
    if use_ref:
        ref_lib().ref_prod_force_a_f64(_p(f), _p(nd), _p(ed), _p(nlist), nloc, nall, nnei, 1)
    else:
        lib().orc_prod_force_a(_p(f), _p(nd), _p(ed), _p(nlist), nloc, nall, nnei)
    return f


def prod_virial_a(net_deriv, env_deriv, rij, nlist, nall, use_ref=False):
    nlist = _c(nlist, np.int32)
    nloc, nnei = nlist.shape
    v = np.zeros(9)
    av = np.zeros((nall, 9))
    args = (_p(v), _p(av), _p(_c(net_deriv, np.float64)), _p(_c(env_deriv, np.float64)),
            _p(_c(rij, np.float64)), _p(nlist), nloc, nall, nnei)
    if use_ref:
        ref_lib().ref_prod_virial_a_f64(*args)
    else:
        lib().orc_prod_virial_a(*args)
    return v, av


def prod_force_grad_a(grad, env_deriv, nlist, use_ref=False):
    nlist = _c(nlist, np.int32)
    nloc, nnei = nlist.shape
    out = np.zeros((nloc, 4 * nnei))
    g, ed = _c(grad, np.float64), _c(env_deriv, np.float64)
    if use_ref:
        ref_lib().ref_prod_force_grad_a_f64(_p(out), _p(g), _p(ed), _p(nlist), nloc, nnei, 1)
    else:
        lib().orc_prod_force_grad_a(_p(out), _p(g), _p(ed), _p(nlist), nloc, nnei)
    return out


def prod_virial_grad_a(grad, env_deriv, rij, nlist, use_ref=False):
    nlist = _c(nlist, np.int32)
    nloc, nnei = nlist.shape
    out = np.zeros((nloc, 4 * nnei))
    args = (_p(out), _p(_c(grad, np.float64)), _p(_c(env_deriv, np.float64)),
            _p(_c(rij, np.float64)), _p(nlist), nloc, nnei)
    if use_ref:
        ref_lib().ref_prod_virial_grad_a_f64(*args)
    else:
        lib().orc_prod_virial_grad_a(*args)
    return out


def ref_copy_coord_build_nlist(coord, atype, box, rc, legacy=True, mem_nall=None, mem_nbor=512):
    """The reference's own ghost copy + candidate list (legacy grid version of
    its unit tests, or copy_coord_cpu + build_nlist_cpu)."""
    coord = _c(coord, np.float64).reshape(-1, 3)
    nloc = coord.shape[0]
    mem_nall = mem_nall or nloc * 64
    out_c = np.zeros((mem_nall, 3))
    out_t = np.zeros(mem_nall, np.int32)
    mp = np.zeros(mem_nall, np.int32)
    rows = np.full((nloc, mem_nbor), -1, np.int32)
    counts = np.zeros(nloc, np.int32)
    fn = ref_lib().ref_copy_coord_build_nlist if legacy else ref_lib().ref_copy_coord_cpu_build_nlist_cpu
    nall = fn(_p(out_c), _p(out_t), _p(mp), _p(rows), _p(counts), mem_nall, mem_nbor, _p(coord),
              _p(_c(atype, np.int32)), nloc, _p(_c(box, np.float64)), C.c_double(rc))
    if nall < 0:
        raise RuntimeError("reference buffers too small")
    return out_c[:nall], out_t[:nall], mp[:nall], rows, counts


# --------------------------------------------------------------------------
# the full model
class _Model(C.Structure):
    _fields_ = [
        ("ntypes", C.c_int),
        ("sel", C.c_int * MAX_TYPES),
        ("rcut", C.c_double),
        ("rcut_smth", C.c_double),
        ("type_one_side", C.c_int),
        ("n_emb", C.c_int),
        ("emb_neuron", C.c_int * MAX_LAYERS),
        ("axis_neuron", C.c_int),
        ("n_fit", C.c_int),
        ("fit_neuron", C.c_int * MAX_LAYERS),
        ("dim_descrpt", C.c_int),
        ("davg", _dp),
        ("dstd", _dp),
        ("emb_w", (_dp * MAX_LAYERS) * (MAX_TYPES * MAX_TYPES)),
        ("emb_b", (_dp * MAX_LAYERS) * (MAX_TYPES * MAX_TYPES)),
        ("emb_idt", (_dp * MAX_LAYERS) * (MAX_TYPES * MAX_TYPES)),
        ("fit_w", (_dp * (MAX_LAYERS + 1)) * MAX_TYPES),
        ("fit_b", (_dp * (MAX_LAYERS + 1)) * MAX_TYPES),
        ("fit_idt", (_dp * (MAX_LAYERS + 1)) * MAX_TYPES),
        ("atom_ener_bias", _dp),
        ("pair_mask", _ip),
        ("table", _dp * (MAX_TYPES * MAX_TYPES)),
        ("table_info", (C.c_double * 6) * (MAX_TYPES * MAX_TYPES)),
        ("compressed", C.c_int),
    ]


class OracleModel:
    """Packs a dpgb.params.SeAParams into the oracle's C struct (keeps the
    numpy buffers alive)."""

    def __init__(self, params):
        c = params.config
        self.params = params
        self._keep = []
        m = _Model()
        m.ntypes = c.ntypes
        for i, s in enumerate(c.sel):
            m.sel[i] = s
        m.rcut, m.rcut_smth = c.rcut, c.rcut_smth
        m.type_one_side = int(c.type_one_side)
        m.n_emb = len(c.neuron)
        for i, w in enumerate(c.neuron):
            m.emb_neuron[i] = w
        m.axis_neuron = c.axis_neuron
        m.n_fit = len(c.fit_neuron)
        for i, w in enumerate(c.fit_neuron):
            m.fit_neuron[i] = w
        m.dim_descrpt = c.dim_descrpt
        m.davg = self._ptr(params.mean)
        m.dstd = self._ptr(params.stddev)
        for e, layers in enumerate(params.emb):
            for l, (w, b, idt) in enumerate(layers):
                m.emb_w[e][l] = self._ptr(w)
                m.emb_b[e][l] = self._ptr(b)
                m.emb_idt[e][l] = self._ptr(idt)
        for t, layers in enumerate(params.fit):
            for l, (w, b, idt) in enumerate(layers):
                m.fit_w[t][l] = self._ptr(w)
                m.fit_b[t][l] = self._ptr(b)
                m.fit_idt[t][l] = self._ptr(idt)
        m.atom_ener_bias = self._ptr(params.atom_ener_bias())
        pm = c.pair_mask()
        m.pair_mask = self._ptr(pm) if pm is not None else C.cast(None, _ip)
        if params.compressed:
            m.compressed = 1
            for e, (tab, info) in enumerate(zip(params.tables, params.table_info)):
                m.table[e] = self._ptr(tab)
                for k in range(6):
                    m.table_info[e][k] = float(info[k])
        self.struct = m

    def _ptr(self, a):
        if a is None:
            return C.cast(None, _dp)
        a = np.ascontiguousarray(a)
        self._keep.append(a)
        return _p(a)

    def energy_force_ext(self, coord_ext, atype_ext, nlist, nloc):
        coord_ext = _c(coord_ext, np.float64).reshape(-1, 3)
        atype_ext = _c(atype_ext, np.int32)
        nlist = _c(nlist, np.int32)
        nall = coord_ext.shape[0]
        c = self.params.config
        ae = np.zeros(nloc)
        f = np.zeros((nall, 3))
        v = np.zeros(9)
        av = np.zeros((nall, 9))
        desc = np.zeros((nloc, c.dim_descrpt))
        rot = np.zeros((nloc, c.ng, 3))
        rc = lib().orc_se_a_energy_force(C.byref(self.struct), _p(coord_ext), _p(atype_ext),
                                         _p(nlist), nloc, nall, _p(ae), _p(f), _p(v), _p(av),
                                         _p(desc), _p(rot))
        if rc != 0:
            raise RuntimeError(f"oracle failed ({rc})")
        return dict(atom_energy=ae, force_ext=f, virial=v, atom_virial_ext=av,
                    descriptor=desc, rot_mat=rot)

    def evaluate(self, coord, atype, box, order=None):
        """E, F, V of one periodic (or open, box=None) frame, following
        EnergyModel.forward (deepmd/pt/model/model/make_model.py:136-220):
        normalise, extend with ghosts, build the typed neighbour list,
        evaluate on extended atoms and reduce onto local atoms."""
        c = self.params.config
        coord = np.asarray(coord, np.float64).reshape(-1, 3)
        nloc = coord.shape[0]
        if box is not None:
            coord = normalize_coord(coord, np.asarray(box, np.float64))
        ext, ext_t, mapping = extend_coord_with_ghosts(coord, atype, box, c.rcut, order)
        nlist = build_nlist_pt(ext, ext_t, nloc, c.rcut, c.sel)
        r = self.energy_force_ext(ext, ext_t, nlist, nloc)
        force = np.zeros((nloc, 3))
        np.add.at(force, mapping, r["force_ext"])
        av = np.zeros((nloc, 9))
        np.add.at(av, mapping, r["atom_virial_ext"])
        return dict(energy=float(r["atom_energy"].sum()), atom_energy=r["atom_energy"], force=force,
                    virial=r["virial"], atom_virial=av, nlist=nlist, coord_ext=ext,
                    atype_ext=ext_t, mapping=mapping, descriptor=r["descriptor"],
                    rot_mat=r["rot_mat"])
