"""Autotuner for the Z-grid engine's knobs.

Picks, by measurement on the GPU, the grid cell-size multiple (cell edge relative to the
configured minimum part size), the cell order (3-D Morton cells or x-rows) with the x cell
factor of row order, the warp walk (union walk threshold) and whether see CTAs stage their
halos in shared memory.  Each candidate runs a few steps on a throwaway batch
built from the same groups (the caller's state is not advanced); the fastest candidate is
set as the library's tuning and cached per shape class (model, pass sequence, agent-count
bucket, segment-count bucket, radius / part-size ratio) in a JSON file, so later runs of the
same class reuse it without measuring.  Results do not depend on the choice except for the
float summation order (neighbour sets are exact for every grid).
"""
from __future__ import annotations

import json
import math
import os

from . import api
from .models import by_id

DEFAULT_CANDIDATES = (
    [{"cell_multiple": cm, "union_factor": 1, "stage": 0, "cell_order": 0, "x_cell_factor": 1.0}
     for cm in (1.0, 0.5)]
    + [{"cell_multiple": cm, "union_factor": 1, "stage": 0, "cell_order": 1, "x_cell_factor": xf}
       for cm in (1.0, 0.5, 0.34, 0.25) for xf in (1.0, 0.5, 0.25)]
    + [{"cell_multiple": 1.0, "union_factor": 2, "stage": 0, "cell_order": 0, "x_cell_factor": 1.0},
       {"cell_multiple": 1.0, "union_factor": 2, "stage": 1, "cell_order": 0, "x_cell_factor": 1.0}]
    # row walk with the CTA's union rows bulk-copied (TMA) into shared memory
    + [{"cell_multiple": cm, "union_factor": 1, "stage": 1, "cell_order": 1, "x_cell_factor": 0.5}
       for cm in (1.0, 0.5)]
)


def cache_path() -> str:
    base = os.environ.get("TAY_GB300_TUNING_CACHE")
    if base:
        return base
    return os.path.join(os.path.expanduser("~"), ".cache", "tay_gb300", "tuning.json")


def shape_key(groups) -> str:
    setup0 = groups[0][0]
    names = "+".join(p.name for p in setup0.passes)
    agents = sum(r.shape[0] for _, r in groups)
    radius = max(p.radius for p in setup0.passes)
    ratio = radius / setup0.part if setup0.part > 0 else 0.0
    return (f"{names}|n2^{int(math.log2(max(agents, 1)))}|s2^{int(math.log2(len(groups)))}"
            f"|r/part{round(ratio, 2)}")


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def measure(groups, tuning: dict, steps: int = 3) -> float:
    """Device ms per step of `steps` steps (after one warm-up step) with `tuning`."""
    api.set_tuning(**tuning)
    B = api.Batch(groups)
    try:
        B.push()
        B.run(1)
        ms, _ = B.run(steps)
    finally:
        B.close()
    return ms / steps


def evolve(groups, steps: int):
    """The groups' records after `steps` steps with the current tuning (a throwaway batch;
    the caller's records are not changed)."""
    B = api.Batch(groups)
    try:
        B.push()
        B.run(steps)
        return [(setup, by_id(B.fetch(k))) for k, (setup, _) in enumerate(groups)]
    finally:
        B.close()


def autotune(groups, candidates=None, steps: int = 3, use_cache: bool = True, evolve_steps: int = 0) -> dict:
    """Chooses and sets the fastest tuning for `groups` (a list of (Setup, records)),
    returns {"tuning": ..., "ms_per_step": ..., "cached": bool, "trials": [...]}.
    With evolve_steps > 0 every candidate is also timed on the state `evolve_steps` steps
    later (flocks tighten, fluids settle) and the candidate with the least summed time
    wins, so the choice holds over a run rather than only at its first step."""
    key = shape_key(groups)
    path = cache_path()
    cache = _load(path) if use_cache else {}
    if key in cache:
        api.set_tuning(**cache[key]["tuning"])
        return dict(cache[key], cached=True)
    base = api.get_tuning()
    states = [groups]
    if evolve_steps > 0:
        states.append(evolve(groups, evolve_steps))
    trials = []
    for cand in candidates or DEFAULT_CANDIDATES:
        trials.append((sum(measure(g, dict(base, **cand), steps) for g in states) / len(states), cand))
    best_ms, best = min(trials, key=lambda t: t[0])
    best = dict(base, **best)
    api.set_tuning(**best)
    entry = {"tuning": best, "ms_per_step": best_ms,
             "trials": [{"tuning": c, "ms_per_step": m} for m, c in trials]}
    if use_cache:
        cache[key] = entry
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return dict(entry, cached=False)
