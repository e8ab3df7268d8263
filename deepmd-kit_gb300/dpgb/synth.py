"""Seeded synthetic systems standing in for real trajectories.

* :func:`water_box` — n^3 water molecules: O on a cubic lattice of spacing
  3.1 A jittered U(+-0.3 A) per axis, two H at 0.9572 A with an H-O-H angle
  of 104.52 deg under a uniformly random rotation; periodic cubic box of
  3.1*n A; types O=0, H=1, atoms ordered O,H,H per molecule.
* :func:`fcc_alloy_frame` — a periodic fcc crystal (a = 4.05 A) of a whole
  number of 4-atom cells with 4 species drawn with Dirichlet(1,1,1,1)
  fractions and N(0, 0.05 A) jitter.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np


def _random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices from uniform unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], axis=1)


def water_box(n: int, seed: int = 0, spacing: float = 3.1, jitter: float = 0.3,
              bond: float = 0.9572, angle_deg: float = 104.52
              ) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Returns (coord [3*n^3, 3] f64, atype [3*n^3] int32, box [9] f64)."""
    rng = np.random.default_rng(seed)
    g = np.arange(n, dtype=np.float64)
    ox = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    ox = (ox + 0.5) * spacing + rng.uniform(-jitter, jitter, size=ox.shape)
    nmol = ox.shape[0]
    half = math.radians(angle_deg) / 2.0
    tmpl = bond * np.array([[math.sin(half), 0.0, math.cos(half)],
                            [-math.sin(half), 0.0, math.cos(half)]])
    rot = _random_rotations(rng, nmol)
    hpos = ox[:, None, :] + np.einsum("mij,hj->mhi", rot, tmpl)
    coord = np.concatenate([ox[:, None, :], hpos], axis=1).reshape(-1, 3)
    atype = np.tile(np.array([0, 1, 1], dtype=np.int32), nmol)
    L = spacing * n
    box = np.array([L, 0, 0, 0, L, 0, 0, 0, L], dtype=np.float64)
    return coord, atype, box


def _grid_dims(ncell: int) -> Tuple[int, int, int]:
    """Three factors of ncell as close to a cube as possible."""
    best = (ncell, 1, 1)
    best_score = float("inf")
    for a in range(1, int(round(ncell ** (1 / 3))) + 2):
        if ncell % a:
            continue
        rest = ncell // a
        for b in range(a, int(math.isqrt(rest)) + 1):
            if rest % b:
                continue
            c = rest // b
            score = max(a, b, c) / min(a, b, c)
            if score < best_score:
                best, best_score = (a, b, c), score
    return best


def fcc_alloy_frame(natoms_target: int, rng: np.random.Generator, a: float = 4.05,
                    ntypes: int = 4, jitter: float = 0.05
                    ) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    ncell = max(1, int(round(natoms_target / 4)))
    nx, ny, nz = _grid_dims(ncell)
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    cells = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz),
                                 indexing="ij"), -1).reshape(-1, 1, 3)
    coord = ((cells + basis[None]) * a).reshape(-1, 3)
    coord = coord + rng.normal(0.0, jitter, size=coord.shape)
    frac = rng.dirichlet(np.ones(ntypes))
    atype = rng.choice(ntypes, size=coord.shape[0], p=frac).astype(np.int32)
    box = np.diag([nx * a, ny * a, nz * a]).reshape(-1).astype(np.float64)
    return coord, atype, box


def fcc_alloy_batch(nframes: int = 512, seed: int = 0, lo: int = 32, hi: int = 4000
                    ) -> List[Tuple[np.ndarray, np.ndarray, np.ndarray]]:
    """Frames with atom counts log-uniform in [lo, hi] (rounded to 4-atom cells)."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(lo), math.log(hi), size=nframes))
    return [fcc_alloy_frame(int(c), rng) for c in counts]
