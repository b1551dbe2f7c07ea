"""GPU parity: the CUDA Z-grid path (through the Tay C API) against the oracle, on the same
seeded records.  Counts are compared bit for bit; floats with a normwise relative error
bound (max |gpu - oracle| / max |oracle|): 1e-5 after one step, 1e-3 after many."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise, oracle_run

pytestmark = pytest.mark.gpu

TOL_1STEP = 1e-5
TOL_MANY = 1e-3


def _basic(n, seed=11):
    ps = W.basic_points(n, seed=seed)
    return M.records(M.TEST_RECORD, ps.p, ps.v)


def test_basic_counts_bit_exact_one_step(gpu, port):
    recs = _basic(20000)
    setup = M.test_setup(passes=("agent_see",))
    g = M.run(setup, recs, 1)
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 1)
    assert g["b_buffer_count"].sum() > 0
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])
    assert normwise(g["b_buffer"][:, :3], o["b_buffer"][:, :3]) < TOL_1STEP
    assert np.array_equal(g["p"], o["p"]) and np.array_equal(g["v"], o["v"])


def test_basic_counts_match_cpu_simple(gpu, port):
    recs = _basic(4000, seed=3)
    setup = M.test_setup(passes=("agent_see",))
    g = M.run(setup, recs, 1)
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 1, space="simple")
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])


def test_basic_steps(gpu, port):
    recs = _basic(20000, seed=5)
    setup = M.test_setup()
    g = M.run(setup, recs, 20)
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 20)
    # positions and velocities do not depend on the see pass: bit-exact
    assert np.array_equal(g["p"][:, :3], o["p"][:, :3])
    assert np.array_equal(g["v"][:, :3], o["v"][:, :3])
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])
    assert normwise(g["f_buffer"][:, :3], o["f_buffer"][:, :3]) < TOL_MANY


def test_boids_one_step(gpu, port):
    ps = W.boids_points(30000, seed=7, clusters=8, side=400.0)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    setup = M.boids_setup(passes=("boids_see",))
    g = M.run(setup, recs, 1)
    o = oracle_run(port, O.MODEL_BOIDS, setup, recs, 1)
    assert g["count"].sum() > 0
    assert np.array_equal(g["count"], o["count"])
    for f in ("coh", "ali", "sep"):
        assert normwise(g[f][:, :3], o[f][:, :3]) < TOL_1STEP, f
    full = M.boids_setup()
    g = M.run(full, recs, 1)
    o = oracle_run(port, O.MODEL_BOIDS, full, recs, 1)
    assert normwise(g["p"][:, :3], o["p"][:, :3]) < TOL_1STEP
    assert normwise(g["v"][:, :3], o["v"][:, :3]) < TOL_1STEP
    assert np.all(g["count"] == 0)


def test_sph_one_step(gpu, port):
    """Density, pressure and acceleration after one step within 1e-5 normwise of the FP32
    oracle; the FP32 oracle's own distance from the FP64 oracle is printed beside them."""
    sph = W.sph_dam(16, 24, 16)
    recs = M.records(M.SPH_RECORD, sph.points.p, sph.points.v)
    for passes in (("sph_density",), ("sph_density", "sph_pressure", "sph_force")):
        setup = M.sph_setup(passes=passes)
        g = M.run(setup, recs, 1)
        o = oracle_run(port, O.MODEL_SPH, setup, recs, 1)
        o64 = oracle_run(port, O.MODEL_SPH, setup, recs, 1, real=np.float64)
        fields = (("rho", "rho"), ("P", "P"), ("a", "a")) if "sph_force" in passes else (("rho", "rho"),)
        for name, f in fields:
            gv = g[f][:, :3] if f == "a" else g[f]
            ov = o[f][:, :3] if f == "a" else o[f]
            wv = o64[f][:, :3] if f == "a" else o64[f]
            e, e32, e64 = normwise(gv, ov), normwise(ov, wv), normwise(gv, wv)
            print(f"SPH one step {name}: GPU vs FP32 oracle {e:.2e}; vs FP64 {e64:.2e}; FP32 oracle vs FP64 {e32:.2e}")
            assert e < TOL_1STEP, (name, e)
    setup = M.sph_setup()
    g = M.run(setup, recs, 5)
    o = oracle_run(port, O.MODEL_SPH, setup, recs, 5)
    assert normwise(g["p"][:, :3], o["p"][:, :3]) < TOL_1STEP
    assert normwise(g["v"][:, :3], o["v"][:, :3]) < TOL_MANY


def test_batch_matches_individual_runs(gpu):
    setups, recs_list = [], []
    for i, n in enumerate((1500, 4000, 2500)):
        ps = W.boids_points(n, seed=20 + i, clusters=2, side=100.0)
        recs_list.append(M.records(M.BOIDS_RECORD, ps.p, ps.v))
        setups.append(M.boids_setup(r=5.0 + 3 * i, part=5.0 + 3 * i, mb=4))
    singles = [M.run(s, r, 3) for s, r in zip(setups, recs_list)]
    states = [M.make_state(s, r) for s, r in zip(setups, recs_list)]
    for st, _ in states:
        st.start()
    api.run_batch([st for st, _ in states], 3)
    for (st, g), single in zip(states, singles):
        out = M.by_id(st.agents(g, M.BOIDS_RECORD))
        assert np.array_equal(out["p"], single["p"])
        assert np.array_equal(out["v"], single["v"])
        st.end()


@pytest.mark.parametrize("tuning", [
    {"cell_order": 1}, {"cell_order": 1, "cell_multiple": 0.34}, {"cell_order": 1, "union_factor": 2},
    {"cell_order": 1, "hit_masks": 1}, {"cell_order": 1, "hit_masks": 1, "cell_multiple": 0.5},
    {"cell_order": 1, "x_cell_factor": 0.25}, {"cell_order": 1, "cell_multiple": 0.5, "x_cell_factor": 0.5},
    {"cell_order": 1, "stage": 1}, {"cell_order": 1, "stage": 1, "x_cell_factor": 0.5, "stage_cap": 256},
    {"cell_order": 1, "x_cell_factor": 1.0},
    {"cell_order": 0}, {"cell_order": 0, "union_factor": 2}, {"cell_order": 0, "stage": 1},
    {"cell_order": 0, "cell_multiple": 0.5}, {"cell_order": 0, "cell_multiple": 1.5},
])
def test_walk_tunings_match_oracle(gpu, port, tuning):
    """Every cell order, cell size and see walk gives the oracle's neighbour counts bit for
    bit and its accumulated vectors within the one-step tolerance."""
    ps = W.boids_points(30000, seed=9, clusters=8, side=400.0)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    setup = M.boids_setup(passes=("boids_see",))
    o = oracle_run(port, O.MODEL_BOIDS, setup, recs, 1)
    try:
        api.set_tuning(**tuning)
        g = M.run(setup, recs, 1)
    finally:
        api.set_tuning()
    assert np.array_equal(g["count"], o["count"])
    assert np.array_equal(g["sep_count"], o["sep_count"])
    for f in ("coh", "ali", "sep"):
        assert normwise(g[f][:, :3], o[f][:, :3]) < TOL_1STEP, f


@pytest.mark.parametrize("order", [0, 1, "rows_staged"])
def test_cell_orders_many_steps(gpu, port, order):
    """Both cell orders over 20 see+act steps of boids and 5 SPH steps (all four passes)."""
    ps = W.boids_points(20000, seed=13, clusters=4, side=300.0)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    setup = M.boids_setup()
    sph = W.sph_dam(16, 24, 16)
    srecs = M.records(M.SPH_RECORD, sph.points.p, sph.points.v)
    ssetup = M.sph_setup()
    tuning = {"cell_order": 1, "stage": 1, "cell_multiple": 0.5} if order == "rows_staged" else {"cell_order": order}
    try:
        api.set_tuning(**tuning)
        g = M.run(setup, recs, 20)
        gs = M.run(ssetup, srecs, 5)
    finally:
        api.set_tuning()
    o = oracle_run(port, O.MODEL_BOIDS, setup, recs, 20)
    assert normwise(g["p"][:, :3], o["p"][:, :3]) < TOL_MANY
    assert normwise(g["v"][:, :3], o["v"][:, :3]) < TOL_MANY
    os_ = oracle_run(port, O.MODEL_SPH, ssetup, srecs, 5)
    assert normwise(gs["p"][:, :3], os_["p"][:, :3]) < TOL_1STEP
    assert normwise(gs["v"][:, :3], os_["v"][:, :3]) < TOL_MANY


@pytest.mark.parametrize("tuning", [
    {"cell_multiple": 1.0, "x_cell_factor": 0.5},
    {"cell_multiple": 0.5, "x_cell_factor": 0.5},
    {"cell_multiple": 0.25, "x_cell_factor": 1.0, "stage_cap": 512, "stage_cells": 256},
])
def test_staged_rows_bit_identical_full_size(gpu, tuning):
    """At the full benchmark size (2^20 boids, 64 clusters, r = cell = 10) the row walk that
    bulk-copies its union rows into shared memory visits the same candidates in the same
    order as the walk through L1, so the records after 5 see+act steps are bit-identical
    and the pair counts equal; some CTAs must have been staged."""
    ps = W.boids_points(1 << 20, seed=2)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    setup = M.boids_setup(r=10.0, part=10.0, mb=256)
    out = {}
    try:
        for st in (0, 1):
            api.set_tuning(cell_order=1, stage=st, **tuning)
            b = api.Batch([(setup, recs)])
            try:
                b.push()
                pairs = [b.run(1)[1] for _ in range(5)]
                tel = b.telemetry()
                out[st] = (b.fetch(0), pairs, tel)
            finally:
                b.close()
    finally:
        api.set_tuning()
    (r0, p0, _), (r1, p1, t1) = out[0], out[1]
    assert p0 == p1
    assert r0.tobytes() == r1.tobytes()
    assert t1["staged_ctas"] > 0


@pytest.mark.parametrize("model", ["boids", "sph"])
def test_row_walks_bit_identical(gpu, model):
    """In row order the per-lane walk, the warp-union walk (union_factor), the hit-mask walk and
    the staged walk visit each seer's neighbours in the same order, and every inlined copy of
    the see body rounds the same way: records and pair counts are bit-identical (pair lists
    off, so the SPH force pass walks too)."""
    if model == "boids":
        ps = W.boids_points(60000, seed=9, clusters=8, side=400.0)
        recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
        setup = M.boids_setup(r=10.0, part=10.0, mb=64)
    else:
        sph = W.sph_dam(32, 40, 16)
        recs = M.records(M.SPH_RECORD, sph.points.p, sph.points.v)
        setup = M.sph_setup(mb=256)
    out = []
    for tuning in ({"union_factor": 1}, {"union_factor": 64}, {"hit_masks": 1}, {"stage": 1}):
        api.set_tuning(cell_order=1, pair_list_cap=0, **tuning)
        try:
            b = api.Batch([(setup, recs)])
            try:
                b.push()
                pairs = [b.run(1)[1] for _ in range(4)]
                out.append((b.fetch(0).tobytes(), pairs, b.telemetry()))
            finally:
                b.close()
        finally:
            api.set_tuning()
    assert out[1][2]["union_warps"] > 0
    for rec, pairs, _ in out[1:]:
        assert pairs == out[0][1]
        assert rec == out[0][0]


@pytest.mark.parametrize("tuning", [
    {"cell_order": 1}, {"cell_order": 1, "x_cell_factor": 0.25}, {"cell_order": 1, "cell_multiple": 0.5},
    {"cell_order": 1, "union_factor": 4}, {"cell_order": 1, "stage": 1, "x_cell_factor": 0.25},
    {"cell_order": 1, "hit_masks": 1, "x_cell_factor": 0.5},
])
def test_rows_with_long_gaps_match_oracle(gpu, port, tuning):
    """Agents in two slabs at the ends of x, so every occupied row has a gap of dozens of
    cells (written by the warp together, short gaps by their own lane): the lookups of a
    seer's own range, a warp's union and a CTA's staged union must find exactly the
    oracle's neighbours."""
    ps = W.basic_points(20000, seed=17)
    p = ps.p.copy()
    x = p[:, 0] / 1000.0 * 60.0
    p[:, 0] = np.where(np.arange(p.shape[0]) % 2 == 0, x, 940.0 + x)
    recs = M.records(M.TEST_RECORD, p, ps.v)
    setup = M.test_setup(passes=("agent_see",))
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 1)
    try:
        api.set_tuning(**tuning)
        g = M.run(setup, recs, 1)
    finally:
        api.set_tuning()
    assert g["b_buffer_count"].sum() > 0
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])
    assert normwise(g["b_buffer"][:, :3], o["b_buffer"][:, :3]) < TOL_1STEP


def test_batched_workload_full_size_equals_single_states(gpu):
    """The full batched workload (512 boids states, N log-uniform in [1000, 65536], about
    8.2 M agents, radius U[5, 20]) advanced by tay_run_batch for 2 steps: every state's
    records equal those of the same state run alone through tay_run, bit for bit (same
    segment grid and order, written through by the batched see pass)."""
    bb = W.batched_boids(states=512, seed=4)
    setups, recs_list = [], []
    for ps, r, _side in bb.states:
        recs_list.append(M.records(M.BOIDS_RECORD, ps.p, ps.v))
        setups.append(M.boids_setup(r=r, part=r, mb=4))
    assert sum(r.shape[0] for r in recs_list) > 8_000_000
    states = [M.make_state(s, r) for s, r in zip(setups, recs_list)]
    for st, _ in states:
        st.start()
    api.run_batch([st for st, _ in states], 2)
    for k, ((st, g), s, r) in enumerate(zip(states, setups, recs_list)):
        out = M.by_id(st.agents(g, M.BOIDS_RECORD))
        st.end()
        st.close()
        if k % 8 == 0:  # every 8th state alone (64 single runs keep the test short)
            single = M.run(s, r, 2)
            assert out.tobytes() == single.tobytes(), k
