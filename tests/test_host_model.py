"""A device model the library does not ship (tests/models/model_soft.cu: soft-sphere
repulsion, func names soft_see / soft_act), built by the tests into its own shared
library against include/tay_gpu_model.cuh, registered with tgpu_register_model_library
and run through the Tay C API on TAY_GPU_Z_GRID, as a reference host brings its own model
to the OpenCL path with ocl_add_source (tay/ocl.c:274-282).

CPU: the library builds and registers; a second registration of the same func names, a
descriptor with another ABI stamp and a library without the entry point are refused.
GPU: against a float32 restatement of the model in numpy (every product, sum, square root
and division rounded separately, as the model's CUDA code rounds them): neighbour counts
and the pair counter bit for bit, forces, positions and velocities within 1e-5 after one
step and 1e-3 after ten.
"""
import ctypes
import os

import numpy as np
import pytest

from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "models", "model_soft.cu")
OUT = os.path.join(HERE, "models", "_build", "libtaymodel_soft.so")

SOFT_RECORD = np.dtype([("tag", "<u4", 2), ("p", "<f4", 4), ("v", "<f4", 4), ("f", "<f4", 4), ("id", "<i4"),
                        ("pad", "<i4")])
assert SOFT_RECORD.itemsize == 64

R, K, DT, DAMP, SIDE = 5.0, 0.5, 0.1, 0.98, 60.0


def _ctx():
    r = np.float32(R)
    return np.array([r, r * r, K, DT, DAMP, 0.0, 0.0, 0.0, SIDE, SIDE, SIDE, 0.0], np.float32)


@pytest.fixture(scope="session")
def soft_model(built):
    from tay_gb300 import _build

    _build.build_model(SRC, OUT)
    api.register_model_library(OUT)
    return OUT


def test_model_library_registers(soft_model):
    L = api.lib()
    assert L.tgpu_model_of(b"soft_see") == b"soft_spheres"
    assert L.tgpu_model_of(b"soft_act") == b"soft_spheres"
    assert L.tgpu_model_nonpoint(b"soft_see") == 0
    # the same func names a second time
    with pytest.raises(api.TayError, match="already provided"):
        api.register_model_library(soft_model)
    # a descriptor stamped with another layout
    h = ctypes.CDLL(soft_model)
    entry = h.tgpu_model_entry
    entry.restype = ctypes.c_void_p
    entry.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    abi = ctypes.c_uint()
    desc = entry(ctypes.byref(abi))
    assert L.tgpu_register_model(desc, abi.value ^ 1) != 0
    assert b"ABI" in L.tgpu_last_error()
    # a library without the entry point
    with pytest.raises(api.TayError, match="tgpu_model_entry"):
        api.register_model_library(api.LIB_PATH)


def test_model_library_func_name_clash_refused(built):
    """The same model built to claim boids_see, a func name of the library's boids model: the
    registration is refused and names both models; boids_see still selects boids."""
    from tay_gb300 import _build

    out = os.path.join(HERE, "models", "_build", "libtaymodel_soft_clash.so")
    _build.build_model(SRC, out, defines=('SOFT_SEE_NAME="boids_see"',))
    with pytest.raises(api.TayError, match="boids_see.*already provided by model 'boids'"):
        api.register_model_library(out)
    assert api.lib().tgpu_model_of(b"boids_see") == b"boids"


def _setup(passes):
    ctx = _ctx()
    lst = [M.Pass(p, p == "soft_see", ctx, R, False) for p in passes]
    return M.Setup(SOFT_RECORD, lst, R, 16)


def _records(n, seed):
    ps = W.basic_points(n, seed=seed, side=SIDE)
    rec = np.zeros(n, SOFT_RECORD)
    rec["p"] = ps.p
    rec["v"] = ps.v
    rec["id"] = np.arange(n, dtype=np.int32)
    return rec


def _restated_step(p, v, act):
    """One step of the model in float32 numpy, agents in id order: per seer, the box test of
    the reference (skip when |a - b| > r on an axis, and the seer itself), then the see
    function over the passing agents; forces summed in float64.  Returns the forces,
    counts, pair-counter value and the new positions and velocities."""
    n = p.shape[0]
    r, r2, k = np.float32(R), np.float32(R) * np.float32(R), np.float32(K)
    f = np.zeros((n, 3), np.float64)
    count = np.zeros(n, np.int32)
    pairs = 0
    for i in range(n):
        d = p[i, :3] - p[:, :3]
        box = np.all(np.abs(d) <= r, axis=1)
        box[i] = False
        pairs += int(box.sum())
        d = d[box]
        d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
        keep = (d2 < r2) & (d2 > 0)
        d, d2 = d[keep], d2[keep]
        dist = np.sqrt(d2)
        w = (k * (r - dist)) / dist
        f[i] = (w[:, None] * d).astype(np.float64).sum(axis=0)
        count[i] = keep.sum()
    if not act:
        return f, count, pairs, p, v
    f32 = f.astype(np.float32)
    v2 = v.copy()
    p2 = p.copy()
    v2[:, :3] = np.float32(DAMP) * v[:, :3] + np.float32(DT) * f32
    p2[:, :3] = p[:, :3] + np.float32(DT) * v2[:, :3]
    for a in range(3):
        lo, hi = p2[:, a] < 0.0, p2[:, a] > np.float32(SIDE)
        p2[lo, a] = 0.0
        p2[hi, a] = np.float32(SIDE)
        v2[lo | hi, a] = -v2[lo | hi, a]
    return f, count, pairs, p2, v2


@pytest.mark.gpu
def test_host_model_see_matches_restatement(gpu, soft_model):
    recs = _records(4000, 41)
    b = api.Batch([(_setup(("soft_see",)), recs)])
    try:
        b.push()
        _, pairs = b.run(1)
        out = M.by_id(b.fetch(0))
        assert api.lib().tgpu_batch_model(b.ptr) == b"soft_spheres"
    finally:
        b.close()
    f, count, ref_pairs, _, _ = _restated_step(recs["p"], recs["v"], act=False)
    got_count = out["f"][:, 3].copy().view(np.int32)
    assert count.sum() > 10_000
    assert np.array_equal(got_count, count)
    assert pairs == ref_pairs
    assert normwise(out["f"][:, :3], f) < 1e-5


@pytest.mark.gpu
def test_host_model_steps_match_restatement(gpu, soft_model):
    recs = _records(4000, 42)
    p, v = recs["p"].copy(), recs["v"].copy()
    for steps in (1, 10):
        g = M.run(_setup(("soft_see", "soft_act")), recs, steps)
        pp, vv = p.copy(), v.copy()
        for _ in range(steps):
            _, _, _, pp, vv = _restated_step(pp, vv, act=True)
        tol = 1e-5 if steps == 1 else 1e-3
        assert normwise(g["p"][:, :3], pp[:, :3]) < tol, steps
        assert normwise(g["v"][:, :3], vv[:, :3]) < tol, steps
        assert np.all(g["f"] == 0.0)
