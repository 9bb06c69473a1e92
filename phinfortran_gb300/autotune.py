"""Autotuner of the large-block engine (blocks above 48).

The large-block path has two free choices that depend on the block size,
the arithmetic and the GPU: the panel width of the blocked Gauss-Jordan
inverse (wider panels mean fewer, larger block products and a longer
sequential panel factorisation) and the number of points a batch holds
(more points fill more of the GPU per launch but need more workspace).
``autotune_tiled`` times the caller's own problem on a sample of its points
for each candidate pair, keeps the fastest, and caches it per (GPU, block
sizes, L, arithmetic) in a JSON file; ``apply_tuning`` sets the cached
choice through ``pf_tiled_set_tuning`` before a run.

    from phinfortran_gb300.autotune import autotune_tiled
    best = autotune_tiled(E_sample, blocks, precision="tc", **params)
    r = transport_tdb(E, blocks, precision="tc", **params)    # runs tuned
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time

import numpy as np

from . import _abi
from .transport import TILED_ARITH, TdbBlocks, transport_tdb

PANELS = (8, 16, 32)
BATCHES = (32, 64, 128, 256)


def default_cache():
    return os.environ.get("PF_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "phinfortran_gb300", "tiled_tuning.json"))


def _key(dims, precision):
    import torch
    n, nl, nr, L = dims
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{name}|n={n}|nl={nl}|nr={nr}|L={L}|{precision}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def set_tuning(panel=0, batch=0):
    """Panel width and batch of the large-block engine (0: built-in choice)."""
    lib = _abi.load()
    rc = lib.pf_tiled_set_tuning(int(panel), int(batch))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_tiled_last_error().decode(errors="replace"))


def layout(n, nl, nr, npts, precision="fp64"):
    """(panel width, batch) a call of this shape would use now."""
    lib = _abi.load()
    p, b = C.c_int(0), C.c_int(0)
    rc = lib.pf_tiled_layout(n, nl, nr, npts, TILED_ARITH[precision], C.byref(p), C.byref(b))
    if rc != 0:
        raise _abi.PFError(rc, lib.pf_tiled_last_error().decode(errors="replace"))
    return p.value, b.value


def apply_tuning(blocks, precision="fp64", cache=None):
    """Set the cached choice for this problem shape; returns it (None: built-in)."""
    if isinstance(blocks, dict):
        blocks = TdbBlocks.from_dict(blocks)
    _, dims, _ = blocks.stacked()
    entry = _load(cache or default_cache()).get(_key(dims, precision))
    if entry is None:
        set_tuning(0, 0)
        return None
    set_tuning(entry["panel"], entry["batch"])
    return entry


def autotune_tiled(E, blocks, *, precision="fp64", panels=PANELS, batches=BATCHES, repeats=1, cache=None,
                   **params):
    """Time transport_tdb on the points E for every (panel, batch) candidate
    and keep the fastest (the built-in choice is timed too and wins ties).
    Returns dict(panel, batch, seconds, default_seconds, candidates)."""
    import torch
    if isinstance(blocks, dict):
        blocks = TdbBlocks.from_dict(blocks)
    _, dims, _ = blocks.stacked()
    n, nl, nr, L = dims
    E = np.ascontiguousarray(E, dtype=np.float64)

    def timed(panel, batch):
        set_tuning(panel, batch)
        transport_tdb(E, blocks, want_transr=False, precision=precision, **params)   # warm-up
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(repeats):
            t0 = time.perf_counter()
            transport_tdb(E, blocks, want_transr=False, precision=precision, **params)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    base = timed(0, 0)
    seen = {layout(n, nl, nr, E.size, precision)}
    results = [dict(panel=0, batch=0, seconds=base)]
    for panel in panels:
        for batch in batches:
            set_tuning(panel, batch)
            eff = layout(n, nl, nr, E.size, precision)
            if eff in seen:          # narrowed to a layout already timed
                continue
            seen.add(eff)
            results.append(dict(panel=panel, batch=batch, seconds=timed(panel, batch), effective=list(eff)))
    win = min(results, key=lambda r: r["seconds"])
    path = cache or default_cache()
    table = _load(path)
    table[_key(dims, precision)] = dict(panel=win["panel"], batch=win["batch"], seconds=win["seconds"],
                                        points=int(E.size))
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as f:
        json.dump(table, f, indent=1)
    set_tuning(win["panel"], win["batch"])
    return dict(panel=win["panel"], batch=win["batch"], seconds=win["seconds"], default_seconds=base,
                candidates=results)
