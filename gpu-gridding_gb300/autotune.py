"""Autotuner for the launch and decomposition parameters of gridding plans.

A plan's speed on a given GPU depends on a handful of settings that change
no placement, norm or skip count (gg_tuning in the C header):

* ``tile_u``        -- tile width (32, 16 or 8 cells; 2048-cell tiles),
* ``slice_staging`` -- kernel slices staged in shared memory or read through L1,
* ``items_per_cta`` -- how finely heavy tiles are split into work items,
* ``sort_detail``   -- record order within a tile (plane + offset class,
  plane only, or visibility order),
* ``ctas_per_sm``   -- resident gridding CTAs per SM (0 = as many as fit),
* ``plane_group_mb`` -- kernel bytes per gridding pass (0 = half of L2),
* ``tile_order``    -- tiles taken by distance from the centre or row by row,
* ``lane_groups``   -- on 32-wide tiles, each consumer warp takes records
  whole (1) or as two half-warp streams (2).
* ``tile_phases``   -- 1, 2, 4 or 8 tile grids offset by a fraction of a tile
  width; each visibility is gridded on the one that cuts its footprint
  into the fewest tile columns (the later grids' tiles as partial tiles
  added after the pass).

:func:`search` runs a coordinate search over them with a caller-supplied
timing function; :func:`autotune` times real gridding calls of a workload
on the current GPU and keeps the winner in a JSON cache keyed by the
workload's shape -- grid size G, w-planes P, largest support s_max,
oversampling os and a power-of-two bucket of the visibility count -- and by
the GPU's name, so later runs pick it up without timing.

The cache file is ``$GPUGRID_TUNE_CACHE`` if set, else
``~/.cache/gpugrid/tuning.json``.  A missing or unreadable file is treated as
empty; writes go to a temporary file that then replaces the cache.
"""
from __future__ import annotations

import json
import math
import os
import tempfile
from typing import Callable, Dict, Iterable, Optional

import numpy as np

CACHE_ENV = "GPUGRID_TUNE_CACHE"
CACHE_VERSION = 8

#: The plan's settings before any tuning (each call chooses shape/staging).
DEFAULT_TUNING = {"tile_u": 0, "slice_staging": -1, "items_per_cta": 4,
                  "sort_detail": 2, "ctas_per_sm": 0, "plane_group_mb": 0,
                  "tile_order": 0, "lane_groups": 0, "tile_phases": 0}

#: Values tried per setting, in search order.
SEARCH_SPACE = (
    (("tile_u", "slice_staging"),
     [(0, -1), (32, 0), (32, 1), (16, 0), (16, 1), (8, 0), (8, 1)]),
    (("items_per_cta",), [(2,), (4,), (8,), (16,)]),
    (("sort_detail",), [(2,), (1,), (0,)]),
    (("ctas_per_sm",), [(0,), (1,)]),
    (("plane_group_mb",), [(0,), (16,), (32,), (48,), (64,), (96,),
                           (1 << 20,)]),
    (("tile_order",), [(0,), (1,)]),
    (("lane_groups",), [(0,), (2,)]),
    (("tile_phases",), [(0,), (2,), (4,), (8,)]),
)


def default_cache_path() -> str:
    p = os.environ.get(CACHE_ENV)
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "gpugrid",
                        "tuning.json")


def n_bucket(num_points: int) -> int:
    """Power-of-two bucket of a visibility count: floor(log2(N)), 0 for
    N <= 1."""
    n = int(num_points)
    return 0 if n <= 1 else int(math.floor(math.log2(n)))


def tuning_key(grid_size: int, num_w_planes: int, max_support: int,
               oversample: int, num_points: int, precision: str = "f",
               num_grids: int = 1) -> str:
    """Cache key of a workload shape: (G, P, s_max, os, N-bucket), plus the
    precision and, for batched calls, the number of grids."""
    key = (f"G{int(grid_size)}-P{int(num_w_planes)}-s{int(max_support)}"
           f"-os{int(oversample)}-N2^{n_bucket(num_points)}-{precision}")
    if num_grids > 1:
        key += f"-C{int(num_grids)}"
    return key


class TuningCache:
    """JSON file of tuned settings: {"version": 2, "devices": {name: {key:
    {setting: value, ..., "ms": t}}}}."""

    def __init__(self, path: Optional[str] = None):
        self.path = path or default_cache_path()
        self.data = {"version": CACHE_VERSION, "devices": {}}
        self.load()

    def load(self) -> None:
        try:
            with open(self.path, "r", encoding="utf-8") as f:
                d = json.load(f)
        except (OSError, ValueError):
            return
        if (isinstance(d, dict) and d.get("version") == CACHE_VERSION
                and isinstance(d.get("devices"), dict)):
            self.data = d

    def get(self, device: str, key: str) -> Optional[dict]:
        e = self.data["devices"].get(device, {}).get(key)
        if not isinstance(e, dict):
            return None
        try:
            return {k: int(e[k]) for k in DEFAULT_TUNING} | (
                {"ms": float(e["ms"])} if "ms" in e else {})
        except (KeyError, TypeError, ValueError):
            return None

    def put(self, device: str, key: str, entry: dict) -> None:
        self.data["devices"].setdefault(device, {})[key] = dict(entry)

    def save(self) -> None:
        d = os.path.dirname(os.path.abspath(self.path))
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=".tuning.", dir=d)
        try:
            with os.fdopen(fd, "w", encoding="utf-8") as f:
                json.dump(self.data, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)
        except BaseException:
            try:
                os.unlink(tmp)
            except OSError:
                pass
            raise


def search(measure: Callable[[dict], float],
           space: Iterable = SEARCH_SPACE,
           start: Optional[dict] = None, sweeps: int = 3) -> tuple:
    """Coordinate search: for each group of settings in turn, try its
    values with the others at their best so far and keep the fastest;
    sweep the groups again while a sweep changes the best (at most
    ``sweeps`` times: the settings interact, e.g. the tile width that is
    fastest with several plane groups need not be with one).  Each tuning
    is measured once.  ``measure(tuning) -> ms`` (inf for a failed
    configuration).  Returns (best tuning, its ms, {repr(tuning): ms} of
    every trial)."""
    best = dict(start or DEFAULT_TUNING)
    trials: Dict[str, float] = {}
    space = list(space)

    def timed(t):
        k = json.dumps(t, sort_keys=True)
        if k not in trials:
            trials[k] = float(measure(dict(t)))
        return trials[k]

    best_ms = timed(best)
    for _ in range(max(1, sweeps)):
        before = dict(best)
        for names, values in space:
            for vals in values:
                t = dict(best)
                t.update(zip(names, vals))
                ms = timed(t)
                if ms < best_ms:
                    best, best_ms = t, ms
        if best == before:
            break
    return best, best_ms, trials


def _device_name(torch) -> str:
    return torch.cuda.get_device_name(torch.cuda.current_device())


#: Settings the host-pointer calls are re-timed over, starting from the
#: plan's tuning: where the grid is the caller's host memory used in place,
#: the tile order and the plane groups change how its pages are touched,
#: and the tile phases' reduction reads and writes it after the gridding
#: launch (so fewer phases than the device plan's can pay).
HOST_SEARCH = (("tile_order", (0, 1)), ("plane_group_mb", (None, 1 << 20)),
               ("tile_phases", (None, 1, 2)))


def autotune_host(pkg, call: Callable[[], object], base: dict,
                  steps: int = 3) -> dict:
    """Tune the host-pointer entry points of the current device by timing
    ``call`` (one host-pointer gridding call on the caller's production
    buffers) with ``base`` and its variants over :data:`HOST_SEARCH`
    (``None`` = the base value); applies the fastest with
    ``pkg.set_host_tuning`` and returns it with its time ("ms").  Calls
    accumulate into the caller's grid, so pass scratch buffers."""
    import time

    def measure(t):
        pkg.set_host_tuning(t)
        call()
        best = math.inf
        for _ in range(max(1, steps)):
            t0 = time.perf_counter()
            call()
            best = min(best, time.perf_counter() - t0)
        return best * 1e3

    best = dict(base)
    best_ms = measure(best)
    for name, values in HOST_SEARCH:
        for v in values:
            cand = dict(best, **{name: base[name] if v is None else v})
            if cand == best:
                continue
            ms = measure(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    pkg.set_host_tuning(best)
    return dict(best, ms=best_ms)


def autotune(pkg, plan, stack, uu, vv, ww, vis, weight, cell_size_rad,
             w_scale, grid_size, offsets=None, cache: Optional[TuningCache] = None,
             steps: int = 2, force: bool = False) -> dict:
    """Tune ``plan`` for a workload held in device tensors and apply the
    result.  ``offsets`` (num_grids + 1 channel offsets) selects batched
    calls; without it single calls are timed.  Timed calls grid into
    scratch arrays, never into the caller's.  Returns the applied tuning
    with its time ("ms"), whether it came from the cache ("cached") and the
    cache key ("key")."""
    import torch

    cache = cache if cache is not None else TuningCache()
    n = int(uu.shape[0])
    num_grids = 1 if offsets is None else len(offsets) - 1
    key = tuning_key(grid_size, stack.num_w_planes, int(max(stack.support)),
                     stack.oversample, n, stack.precision, num_grids)
    dev = _device_name(torch)
    hit = None if force else cache.get(dev, key)
    if hit is not None:
        plan.set_tuning(hit)
        return dict(hit, cached=True, key=key)

    real = torch.float32 if stack.precision == "f" else torch.float64
    G = int(grid_size)
    grids = torch.zeros((num_grids, G, G, 2), dtype=real, device=uu.device)
    norms = torch.zeros(num_grids, dtype=torch.float64, device=uu.device)
    skips = torch.zeros(num_grids, dtype=torch.int64, device=uu.device)
    stream = torch.cuda.current_stream()
    np_real = np.float32 if stack.precision == "f" else np.float64
    cell, wsc = np_real(cell_size_rad), np_real(w_scale)

    def call():
        if offsets is None:
            pkg.grid_wproj_device(plan, stack, uu, vv, ww, vis, weight, cell,
                                  wsc, G, grids[0], norms[:1], skips[:1],
                                  stream)
        else:
            pkg.grid_wproj_batched_device(plan, stack, offsets, uu, vv, ww,
                                          vis, weight, cell, wsc, G, grids,
                                          norms, skips, stream)

    def measure(t):
        try:
            plan.set_tuning(t)
            call()
            torch.cuda.synchronize()
            best = math.inf
            for _ in range(max(1, steps)):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                call()
                e1.record(stream)
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            return best
        except pkg.GridError:
            return math.inf

    best, best_ms, trials = search(measure)
    del grids
    plan.set_tuning(best)
    entry = dict(best, ms=best_ms)
    cache.put(dev, key, entry)
    cache.save()
    return dict(entry, cached=False, key=key, trials=len(trials))
