"""Shared helpers for the parity tests: run the same seeded records through the GPU
engine (the Tay C API) and through the oracle, and measure the differences."""
from __future__ import annotations

import numpy as np

from oracle import pyoracle as O
from tay_gb300 import models as M

MASKS = {
    ("agent_see",): O.PASS_SEE0,
    ("agent_act",): O.PASS_ACT0,
    ("agent_see", "agent_act"): O.PASS_SEE0 | O.PASS_ACT0,
    ("boids_see",): O.PASS_SEE0,
    ("boids_see", "boids_act"): O.PASS_SEE0 | O.PASS_ACT0,
    ("sph_density",): O.PASS_SEE0,
    ("sph_density", "sph_pressure"): O.PASS_SEE0 | O.PASS_ACT0,
    ("sph_density", "sph_pressure", "sph_force"): O.PASS_SEE0 | O.PASS_ACT0 | O.PASS_SEE1,
    ("sph_density", "sph_pressure", "sph_force", "sph_integrate"): 15,
}


def normwise(a, b):
    """max |a - b| / max |b| over the whole array (normwise relative error)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.max(np.abs(b)) if b.size else 0.0
    if scale == 0.0:
        return float(np.max(np.abs(a - b))) if a.size else 0.0
    return float(np.max(np.abs(a - b)) / scale)


def oracle_run(impl, model, setup: M.Setup, recs, steps, space="z_grid", real=np.float32, threads=0):
    names = tuple(p.name for p in setup.passes)
    see = setup.passes[0].ctx
    act = setup.passes[-1].ctx
    radius = max(p.radius for p in setup.passes)
    rec_o = recs
    if real == np.float64:
        rec_o = np.zeros(recs.shape[0], O.RECORDS[np.float64][model])
        for f in recs.dtype.names:
            rec_o[f] = recs[f]
        see = see.astype(np.float64)
        act = act.astype(np.float64)
    r = impl.run(model, space, rec_o, see, act, radius, setup.part, steps, MASKS[names], threads=threads,
                 mb=setup.mb, real=real)
    return r.records
