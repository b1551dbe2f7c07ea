"""Edge cases and full sizes on the GPU, against the oracle: a single agent, coincident
agents, neighbours exactly at the radius (the reference's test is inclusive,
tay/space.c:62-68), a flat axis (zero extent), coordinates far from the origin, tiny and
large states in one batch, a push that spreads the agents (the grid budget follows one
run later), the benchmark workloads at full size (1,048,576 boids and 524,288 SPH
particles, one step), and an 8M-agent state (the largest indices of one segment)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise, oracle_run

pytestmark = pytest.mark.gpu


def _test_records(p, v=None):
    n = p.shape[0]
    p4 = np.zeros((n, 4), np.float32)
    p4[:, :3] = p
    v4 = np.zeros((n, 4), np.float32)
    if v is not None:
        v4[:, :3] = v
    return M.records(M.TEST_RECORD, p4, v4)


def _see_counts(recs, radius=50.0, part=50.0, tuning=None):
    setup = M.test_setup(radius=radius, part=part, passes=("agent_see",))
    try:
        if tuning:
            api.set_tuning(**tuning)
        return M.run(setup, recs, 1), setup
    finally:
        api.set_tuning()


@pytest.mark.parametrize("tuning", [{"cell_order": 0}, None])
def test_single_agent(gpu, port, tuning):
    recs = _test_records(np.array([[10.0, 20.0, 30.0]], np.float32), np.array([[1.0, 0.0, 0.0]], np.float32))
    g, _ = _see_counts(recs, tuning=tuning)
    assert g["b_buffer_count"][0] == 0
    full = M.test_setup()
    out = M.run(full, recs, 3)
    assert np.allclose(out["p"][0, :3], [13.0, 20.0, 30.0])


@pytest.mark.parametrize("tuning", [{"cell_order": 0}, None])
def test_coincident_agents(gpu, port, tuning):
    p = np.zeros((700, 3), np.float32) + np.float32(123.25)
    recs = _test_records(p)
    g, setup = _see_counts(recs, tuning=tuning)
    assert np.all(g["b_buffer_count"] == 699)
    assert np.all(g["b_buffer"][:, :3] == 0.0)


@pytest.mark.parametrize("tuning", [{"cell_order": 0}, None, {"cell_order": 1, "x_cell_factor": 0.25}])
def test_neighbours_exactly_at_the_radius(gpu, port, tuning):
    """A lattice with spacing equal to the radius: the 26 lattice neighbours are at |d| = r
    on every axis they differ in, and the inclusive test counts them."""
    s = np.arange(12, dtype=np.float32) * np.float32(50.0)
    p = np.stack(np.meshgrid(s, s, s, indexing="ij"), -1).reshape(-1, 3)
    recs = _test_records(p)
    g, setup = _see_counts(recs, tuning=tuning)
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 1)
    inner = np.all((p > 0) & (p < 550), axis=1)
    assert np.all(g["b_buffer_count"][inner] == 26)
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])


def test_flat_axis(gpu, port):
    ps = W.basic_points(20000, seed=71)
    p = ps.p[:, :3].copy()
    p[:, 2] = 500.0
    recs = _test_records(p, ps.v[:, :3])
    g, setup = _see_counts(recs)
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 1)
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])


@pytest.mark.parametrize("tuning", [{"cell_order": 0}, None])
def test_far_from_origin(gpu, port, tuning):
    """Coordinates near 1e6 with radius 5: float spacing there is 1/16, so cell
    coordinates round; the neighbour sets must still equal the oracle's."""
    ps = W.basic_points(20000, seed=72, side=400.0)
    p = ps.p[:, :3] + np.float32(1.0e6)
    recs = _test_records(p)
    g, setup = _see_counts(recs, radius=5.0, part=5.0, tuning=tuning)
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 1, space="simple")
    assert g["b_buffer_count"].sum() > 0
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])


def test_push_that_spreads_the_agents(gpu, port):
    """A push after a group's first does not wait for its extent: the grid budget it sizes
    (cells per axis, hence key width and radix passes) follows one run later.  The agents
    spread to 8 times their extent between runs; the run right after the push (old budget,
    cells enlarged to cover the new box) and the next one (new budget: wider keys, one radix
    pass more) both give the oracle's neighbour counts."""
    ps = W.basic_points(20000, seed=73, side=300.0)
    recs = _test_records(ps.p[:, :3])
    setup = M.test_setup(radius=20.0, part=20.0, passes=("agent_see",))
    b = api.Batch([(setup, recs)])
    try:
        b.push()
        b.run(1)
        before = b.launches_per_step()
        recs["p"][:, :3] *= np.float32(8.0)
        b.push()
        launches = []
        for k in (1, 2):
            b.run(1)
            launches.append(b.launches_per_step())
            g = M.by_id(b.fetch(0))
            # the see pass adds to the counters: after k runs, k oracle steps
            o = oracle_run(port, O.MODEL_TEST, setup, recs, k, space="simple")
            assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"]), k
        assert launches[0] == before and launches[1] == before + 1, (before, launches)
    finally:
        b.close()


def test_tiny_and_large_states_in_one_batch(gpu):
    sizes = (1, 2, 50000, 3, 20000)
    setups, recs_list = [], []
    for i, n in enumerate(sizes):
        ps = W.boids_points(n, seed=80 + i, clusters=2, side=150.0)
        recs_list.append(M.records(M.BOIDS_RECORD, ps.p, ps.v))
        setups.append(M.boids_setup(mb=8))
    singles = [M.run(s, r, 2) for s, r in zip(setups, recs_list)]
    states = [M.make_state(s, r) for s, r in zip(setups, recs_list)]
    for st, _ in states:
        st.start()
    api.run_batch([st for st, _ in states], 2)
    for (st, g), single in zip(states, singles):
        out = M.by_id(st.agents(g, M.BOIDS_RECORD))
        assert np.array_equal(out["p"], single["p"])
        assert np.array_equal(out["v"], single["v"])
        st.end()


def test_full_size_boids_one_step(gpu, port):
    """The benchmark's 1,048,576-boid workload, one see pass, autotuner's default walk."""
    ps = W.boids_points(1 << 20, seed=2)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    setup = M.boids_setup(passes=("boids_see",), mb=256)
    try:
        api.set_tuning(cell_order=1, x_cell_factor=0.25)
        g = M.run(setup, recs, 1)
    finally:
        api.set_tuning()
    o = oracle_run(port, O.MODEL_BOIDS, setup, recs, 1, threads=0)
    assert g["count"].sum() > 10_000_000
    assert np.array_equal(g["count"], o["count"])
    assert np.array_equal(g["sep_count"], o["sep_count"])
    for f in ("coh", "ali", "sep"):
        assert normwise(g[f][:, :3], o[f][:, :3]) < 1e-5, f


def test_full_size_sph_density(gpu, port):
    """The 524,288-particle dam break, density pass."""
    sph = W.sph_dam(64, 128, 64)
    recs = M.records(M.SPH_RECORD, sph.points.p, sph.points.v)
    setup = M.sph_setup(passes=("sph_density",), mb=512)
    try:
        api.set_tuning(cell_order=1, cell_multiple=0.25, x_cell_factor=0.5)
        g = M.run(setup, recs, 1)
    finally:
        api.set_tuning()
    o = oracle_run(port, O.MODEL_SPH, setup, recs, 1, threads=0)
    assert normwise(g["rho"], o["rho"]) < 1e-5


@pytest.mark.parametrize("tuning", [{"cell_order": 0}, None])
def test_eight_million_agents_counts_bit_exact(gpu, port, tuning):
    """One state of 8,388,608 test agents (uniform, about 20 neighbours each): agent, cell,
    CTA, tile and table indices at their largest for one segment; neighbour counts equal
    the oracle's bit for bit in both cell orders."""
    n = 8 << 20
    ps = W.basic_points(n, seed=71, side=7400.0)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    g, setup = _see_counts(recs, tuning=tuning)
    o = oracle_run(port, O.MODEL_TEST, setup, recs, 1)
    assert g.shape[0] == n
    assert g["b_buffer_count"].mean() > 10
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])
    assert normwise(g["b_buffer"][:, :3], o["b_buffer"][:, :3]) < 1e-5
