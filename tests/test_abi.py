"""The C ABI library loads and exports every function include/*.h declares (no device
calls: these run on machines without a GPU)."""
import os
import re

import pytest

from tay_gb300 import api

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
DECL = re.compile(r"^[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", re.M)


def declared(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set()
    for m in DECL.finditer(text):
        line = m.group(0)
        if line.startswith(("typedef", "#")):
            continue
        names.add(m.group(1))
    return sorted(names)


@pytest.mark.parametrize("header", ["tay.h", "tay_gpu.h"])
def test_every_declared_function_is_exported(built, header):
    L = api.lib()
    names = declared(header)
    assert len(names) > 10
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_mirror_covers_the_headers(built):
    mirrored = {n for n, _, _ in api.TAY_SYMBOLS + api.TGPU_SYMBOLS}
    for header in ("tay.h", "tay_gpu.h"):
        missing = [n for n in declared(header) if n not in mirrored]
        assert not missing, (header, missing)


def test_device_models_are_registered(built):
    L = api.lib()
    for name, model in [("agent_see", b"test_basic"), ("agent_act", b"test_basic"), ("boids_see", b"boids"),
                        ("boids_act", b"boids"), ("sph_density", b"sph"), ("sph_pressure", b"sph"),
                        ("sph_force", b"sph"), ("sph_integrate", b"sph")]:
        assert L.tgpu_model_of(name.encode()) == model
    assert L.tgpu_model_of(b"no_such_function") is None


def test_tuning_struct_round_trips(built):
    """TgpuTuning crosses the ABI field by field (the Python mirror has the C layout): every
    field set from Python reads back unchanged, and no arguments restore the defaults."""
    try:
        api.set_tuning(stage=1, stage_cap=640, stage_cells=48, cell_multiple=0.5, union_factor=4, use_graphs=0,
                       cell_order=0, hit_masks=1, x_cell_factor=0.25, pair_list_cap=96)
        t = api.get_tuning()
        assert t == {"stage": 1, "stage_cap": 640, "stage_cells": 48, "cell_multiple": 0.5, "union_factor": 4,
                     "use_graphs": 0, "cell_order": 0, "hit_masks": 1, "x_cell_factor": 0.25, "pair_list_cap": 96}
        api.set_tuning()
        d = api.get_tuning()
        assert d["cell_order"] == 1 and d["x_cell_factor"] == 0.5 and d["pair_list_cap"] == 320
    finally:
        api.set_tuning()
