"""GPU float results against the oracle and its FP64 build (the same algorithm in
double), errors printed (run with -s).  Tolerances hold against the FP32 oracle (1e-5
after one step, 1e-3 after many; normwise: max |gpu - ref| / max |ref|).  Against FP64 the
error is stated and bounded by what FP32 arithmetic itself costs: the GPU must be as close
to the FP64 run as the FP32 CPU run of the same algorithm is (over many steps FP32 and FP64
trajectories part as agents cross the radius at slightly different times)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise, oracle_run

pytestmark = pytest.mark.gpu


def _check(name, fields, g, o32, o64, tol, orders=None):
    """`orders`: the same FP32 run on a second CPU structure (another summation order);
    where a model amplifies rounding differences over many steps (boids: a neighbour
    crossing the radius flips a steering force), the GPU may differ from the oracle as much
    as FP32 arithmetic differs from FP64, or as two CPU structures differ from each other."""
    for f in fields:
        e32 = normwise(g[f], o32[f])
        e64 = normwise(g[f], o64[f])
        p64 = normwise(o32[f], o64[f])
        msg = f"\n[fp64] {name} {f}: gpu vs fp32 oracle {e32:.3e}, gpu vs fp64 {e64:.3e}, fp32 oracle vs fp64 {p64:.3e}"
        bound = tol
        if orders is not None:
            chaos = normwise(orders[f], o32[f])
            msg += f", fp32 CpuGrid vs CpuZGrid {chaos:.3e}"
            # the divergence FP32 itself shows (against FP64), or twice that between two
            # CPU summation orders, whichever is larger
            bound = max(tol, 2.0 * chaos, p64)
        print(msg)
        assert e32 < bound, (name, f, e32, bound)
        assert e64 <= 2.0 * p64 + 1e-6, (name, f, e64, p64)


def _xyz(rec, fields):
    return {f: (rec[f][:, :3] if rec[f].ndim > 1 else rec[f]) for f in fields}


def test_basic_config_100k_100_steps(gpu, port):
    """The first benchmark configuration at full size: 100,000 agents, radius 50, CpuGrid
    part size 50, 100 steps; positions do not depend on the see pass (bit-exact with the
    FP32 oracle), the accumulated f_buffer does."""
    ps = W.basic_points(100_000, seed=1)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    setup = M.test_setup()
    g = M.run(setup, recs, 100)
    o32 = oracle_run(port, O.MODEL_TEST, setup, recs, 100, space="grid")
    o64 = oracle_run(port, O.MODEL_TEST, setup, recs, 100, space="grid", real=np.float64)
    assert np.array_equal(g["p"][:, :3], o32["p"][:, :3])
    f = ("f_buffer",)
    _check("test model 100k x 100 steps", f, _xyz(g, f), _xyz(o32, f), _xyz(o64, f), 1e-3)


def test_boids_vs_fp64(gpu, port):
    ps = W.boids_points(100_000, seed=17, clusters=16, side=800.0)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    see = M.boids_setup(passes=("boids_see",))
    g = M.run(see, recs, 1)
    o32 = oracle_run(port, O.MODEL_BOIDS, see, recs, 1)
    o64 = oracle_run(port, O.MODEL_BOIDS, see, recs, 1, real=np.float64)
    assert np.array_equal(g["count"], o64["count"])
    f = ("coh", "ali", "sep")
    _check("boids 100k, 1 step", f, _xyz(g, f), _xyz(o32, f), _xyz(o64, f), 1e-5)
    full = M.boids_setup()
    for steps, tol in ((1, 1e-5), (20, 1e-3), (100, 1e-3)):
        try:
            api.set_tuning(cell_order=1, x_cell_factor=0.5)
            g = M.run(full, recs, steps)
        finally:
            api.set_tuning()
        o32 = oracle_run(port, O.MODEL_BOIDS, full, recs, steps)
        o64 = oracle_run(port, O.MODEL_BOIDS, full, recs, steps, real=np.float64)
        og = oracle_run(port, O.MODEL_BOIDS, full, recs, steps, space="grid")
        f = ("p", "v")
        _check(f"boids 100k, {steps} steps", f, _xyz(g, f), _xyz(o32, f), _xyz(o64, f), tol, _xyz(og, f))


def test_sph_vs_fp64(gpu, port):
    sph = W.sph_dam(16, 32, 16)
    recs = M.records(M.SPH_RECORD, sph.points.p, sph.points.v)
    setup = M.sph_setup()
    # (rho and P are per-step fields the full program's records do not carry)
    for steps, fields, tol in ((1, ("p", "v"), 1e-5), (100, ("p", "v"), 1e-3)):
        try:
            api.set_tuning(cell_order=1, cell_multiple=0.25, x_cell_factor=0.5)
            g = M.run(setup, recs, steps)
        finally:
            api.set_tuning()
        o32 = oracle_run(port, O.MODEL_SPH, setup, recs, steps)
        o64 = oracle_run(port, O.MODEL_SPH, setup, recs, steps, real=np.float64)
        _check(f"SPH 8192 particles, {steps} steps", fields, _xyz(g, fields), _xyz(o32, fields), _xyz(o64, fields), tol)


def test_full_size_boids_steps_vs_fp64(gpu, port):
    """The benchmark's 1,048,576 boids, 5 see+act steps at the default tuning, against the FP32
    oracle (CpuZGrid), its FP64 build and CpuGrid (another FP32 summation order; 2048 MB, since
    the reference's CpuGrid cannot hold this grid in 256 MB), bounded as the 100k case is."""
    ps = W.boids_points(1 << 20, seed=2)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    full = M.boids_setup(mb=256)
    g = M.run(full, recs, 5)
    o32 = oracle_run(port, O.MODEL_BOIDS, full, recs, 5)
    o64 = oracle_run(port, O.MODEL_BOIDS, full, recs, 5, real=np.float64)
    grid = M.boids_setup(mb=2048)
    og = oracle_run(port, O.MODEL_BOIDS, grid, recs, 5, space="grid")
    f = ("p", "v")
    _check("boids 1M, 5 steps", f, _xyz(g, f), _xyz(o32, f), _xyz(o64, f), 1e-3, _xyz(og, f))
