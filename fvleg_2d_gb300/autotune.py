"""Autotuner of the stage kernel's work decomposition.

The fused stage kernel has two knobs (``cato_gpu_set_plan``): the CTA width ``threads`` (tile
width + 2 ghost columns per side) and ``rows_per_cta``, the rows one CTA marches over.  Wide
strips cut the x-halo re-computation and deep marches the y-halo, but both reduce the number of
CTAs available to fill the 152 SMs; the best point depends on the grid, the scheme and the
precision.  The tuner times each candidate on a scratch instance of the same grid (CUDA events,
a warm-up step then ``steps`` steps) and caches the winner per (scheme, precision, grid-size
class) in a JSON file (``$CATO_TUNE_CACHE``, default ``~/.cache/cato_gb300/tune.json``).
"""
from __future__ import annotations

import json
import math
import os

from .config import SchemeConfig

CANDIDATES = [(64, 8), (64, 16), (64, 32), (128, 8), (128, 16), (128, 32), (128, 64),
              (256, 16), (256, 32), (256, 64)]


def _cache_path() -> str:
    return os.environ.get("CATO_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "cato_gb300", "tune.json"))


def key(cfg: SchemeConfig) -> str:
    size_class = int(round(math.log2(max(1, cfg.ni * cfg.nj)) * 2))  # half-octave buckets
    return (f"{cfg.flux_solver}|{cfg.limiter}|{cfg.integration_strategy}|{cfg.precision}|"
            f"{size_class}|{min(cfg.ni, cfg.nj) // 64}")


def load_cache() -> dict:
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(c: dict) -> None:
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path + ".tmp", "w") as f:
            json.dump(c, f, indent=1)
        os.replace(path + ".tmp", path)
    except OSError:
        pass


def tune(cfg: SchemeConfig, prims, steps: int = 2, candidates=None, use_cache: bool = True):
    """Return ((threads, rows_per_cta), table of ms per step per candidate)."""
    from .fluid import Fluid

    k = key(cfg)
    cache = load_cache() if use_cache else {}
    if use_cache and k in cache:
        e = cache[k]
        return (e["threads"], e["rows_per_cta"]), e.get("table", {})
    table = {}
    f = Fluid(cfg).initialize(*prims)
    for threads, rows in candidates or CANDIDATES:
        if threads - 2 * cfg.ghost_layers() > cfg.ni + 2 * cfg.ghost_layers() and threads > 64:
            continue
        f.set_plan(threads, min(rows, cfg.nj))
        f.run_timed(1)
        ms, _ = f.run_timed(steps)
        table[f"{threads}x{rows}"] = ms / steps
    f.close()
    best = min(table, key=table.get)
    threads, rows = (int(x) for x in best.split("x"))
    if use_cache:
        cache[k] = {"threads": threads, "rows_per_cta": rows, "table": table}
        save_cache(cache)
    return (threads, rows), table
