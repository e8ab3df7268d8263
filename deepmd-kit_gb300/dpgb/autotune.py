"""Launch-configuration autotuning: per size bucket of a batched evaluation,
the work-item size of the persistent embedding / table kernels.

The registry follows deepmd/kernels/autotune.py:1-87: a kernel family
registers a tuner under a name (a repeated name replaces it), and
:func:`run_autotune` calls every registered tuner once for a deployment
shape; a tuner that fails leaves the default launch configuration in place
and logs why.

The batch tuner (family ``"batch_tiles"``) sweeps, one bucket at a time
(largest atom share first, the others held at their best so far), the rows
per work item — 0 (the default split) and 32 ... 1024 — and times each
setting by replaying the whole batched evaluation from its CUDA graph
(CUDA events, median of the replays).  A setting replaces the incumbent
only when it is faster by more than ``min_gain``.  Winners are cached in a
JSON file (``DPGB_AUTOTUNE_CACHE``, default
``~/.cache/dpgb/autotune.json``) under a key made of the GPU's name, the
model's shape (not its weights) and the batch's bucket populations, so a
deployment sweeps once per shape.
"""
from __future__ import annotations

import json
import logging
import os
import statistics
from typing import Callable, Dict, List, Optional, Sequence

log = logging.getLogger(__name__)

BUCKETS = 4
BUCKET_LIMITS = (128, 512, 2048, None)  # atoms per frame: <= 128, <= 512, <= 2048, more
CANDIDATES = (0, 32, 64, 128, 256, 512, 1024)

Tuner = Callable[..., Optional[dict]]
_TUNERS: Dict[str, Tuner] = {}


def register_autotuner(name: str, tuner: Tuner) -> None:
    """Register a kernel family's tuner; a repeated name replaces the old one."""
    _TUNERS[name] = tuner


def run_autotune(target, *args, **kwargs) -> Dict[str, Optional[dict]]:
    """Call every registered tuner on ``target``; returns each family's
    result (None where the tuner failed and the defaults stay)."""
    out = {}
    for name, tuner in _TUNERS.items():
        try:
            out[name] = tuner(target, *args, **kwargs)
        except Exception:  # a failed sweep keeps the default configuration
            log.warning("autotuner %r failed; keeping the default launch configuration", name, exc_info=True)
            out[name] = None
    return out


def cache_path() -> str:
    return os.environ.get("DPGB_AUTOTUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "dpgb",
                                                                 "autotune.json")


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(path: str, key: str, value: dict) -> None:
    d = _load(path)
    d[key] = value
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def batch_key(device_name: str, shape_key: str, frames: Sequence[int], atoms: Sequence[int]) -> str:
    return f"batch_tiles|{device_name}|{shape_key}|frames{list(frames)}|atoms{list(atoms)}"


def graph_timer(batch, coord, reps: int = 5, warmup: int = 2):
    """A timer of one tile setting: the batch's evaluation captured in a CUDA
    graph (re-captured for the new items) and replayed; the median replay
    time in ms, by CUDA events on the current stream."""
    import torch

    out = {}

    def time_tiles(tiles: List[int]) -> float:
        batch.set_tiles(tiles)
        o = out.get("o")
        o = batch.eval_device(coord, out=o, use_graph=True)  # re-cut items, plain evaluation + capture
        out["o"] = o
        for _ in range(warmup):
            batch.eval_device(coord, out=o, use_graph=True)
        stream = torch.cuda.current_stream()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for a, b in ev:
            a.record(stream)
            batch.eval_device(coord, out=o, use_graph=True)
            b.record(stream)
        torch.cuda.synchronize()
        return statistics.median(a.elapsed_time(b) for a, b in ev)

    return time_tiles


def sweep_tiles(frames: Sequence[int], atoms: Sequence[int], time_tiles: Callable[[List[int]], float],
                candidates: Sequence[int] = CANDIDATES, min_gain: float = 0.01) -> dict:
    """Coordinate sweep of the rows per work item, bucket by bucket (largest
    atom share first; empty buckets keep 0).  Returns {"tiles", "ms",
    "default_ms", "trials": [[tiles, ms], ...]}."""
    best = [0] * BUCKETS
    best_ms = default_ms = time_tiles(list(best))
    trials = [[list(best), best_ms]]
    for k in sorted((k for k in range(BUCKETS) if frames[k] > 0), key=lambda k: -atoms[k]):
        for c in candidates:
            if c == best[k]:
                continue
            trial = list(best)
            trial[k] = int(c)
            ms = time_tiles(trial)
            trials.append([trial, ms])
            if ms < best_ms * (1.0 - min_gain):
                best, best_ms = trial, ms
    return {"tiles": best, "ms": best_ms, "default_ms": default_ms, "trials": trials}


def tune_batch(batch, coord=None, *, time_tiles=None, device_name: Optional[str] = None,
               cache: Optional[str] = None, force: bool = False, **sweep_kw) -> dict:
    """Tiles for ``batch`` (a DeepPotBatch): from the cache when its key is
    there (unless ``force``), else swept (``coord``: the CUDA coordinates to
    time on) and stored.  The batch is left set to the winners.  Returns the
    cache entry plus ``"cached": bool``."""
    frames, atoms = batch.buckets()
    if device_name is None:
        import torch

        device_name = torch.cuda.get_device_name()
    key = batch_key(device_name, batch.dp.shape_key, frames, atoms)
    path = cache or cache_path()
    if not force:
        hit = _load(path).get(key)
        if hit and isinstance(hit.get("tiles"), list) and len(hit["tiles"]) == BUCKETS:
            batch.set_tiles(hit["tiles"])
            return dict(hit, cached=True)
    if time_tiles is None:
        if coord is None:
            raise ValueError("tune_batch: coordinates are needed to time a sweep")
        time_tiles = graph_timer(batch, coord)
    res = sweep_tiles(frames, atoms, time_tiles, **sweep_kw)
    batch.set_tiles(res["tiles"])
    _store(path, key, res)
    return dict(res, cached=False)


register_autotuner("batch_tiles", tune_batch)
