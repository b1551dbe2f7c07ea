"""GPU parity of states whose groups are mixed by their see passes (seer group != seen
group, several see passes per group: test/test_combo.c:114-119, tay/state_compile.c:
109-120), of the device-resident host API (lazy fetch, pushes only of changed groups),
against the oracle and the reference's golden vectors."""
import ctypes
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise

pytestmark = pytest.mark.gpu

COMBO = [("see", 0, 0, False), ("see", 0, 1, False), ("see", 1, 1, False), ("see", 1, 0, False)]
COMBO_FULL = COMBO + [("act", 0), ("act", 1)]
BOIDS_PAIR = [("see", 0, 1, False), ("see", 1, 0, False), ("act", 0), ("act", 1)]
FUNCS = {O.MODEL_TEST: (("agent_see", "agent_act"), M.TEST_RECORD),
         O.MODEL_BOIDS: (("boids_see", "boids_act"), M.BOIDS_RECORD)}


def _test_groups(na=12000, nb=8000):
    a = W.basic_points(na, seed=41)
    b = W.basic_points(nb, seed=42)
    return [M.records(M.TEST_RECORD, a.p, a.v), M.records(M.TEST_RECORD, b.p, b.v)]


def _gpu(model, recs, passes, see, act, radius, steps, part=None):
    funcs, dtype = FUNCS[model]
    return M.run_groups(dtype, funcs, recs, passes, see, act, radius, part or radius, steps)


def _oracle(port, model, recs, passes, see, act, radius, steps, part=None):
    res = port.run_groups(model, "z_grid", recs, passes, see, act, radius, part or radius, steps, threads=0)
    return [r.records for r in res]


@pytest.mark.parametrize("order", [0, 1])
def test_combo_see_counts_bit_exact(gpu, port, order):
    recs = _test_groups()
    see, act = M.test_contexts()
    try:
        api.set_tuning(cell_order=order)
        g = _gpu(O.MODEL_TEST, recs, COMBO, see, act, 50.0, 1)
    finally:
        api.set_tuning()
    o = _oracle(port, O.MODEL_TEST, recs, COMBO, see, act, 50.0, 1)
    for k in range(2):
        assert g[k]["b_buffer_count"].sum() > 0
        assert np.array_equal(g[k]["b_buffer_count"], o[k]["b_buffer_count"]), k
        assert normwise(g[k]["b_buffer"][:, :3], o[k]["b_buffer"][:, :3]) < 1e-5, k


def test_combo_full_steps(gpu, port):
    recs = _test_groups()
    see, act = M.test_contexts()
    g = _gpu(O.MODEL_TEST, recs, COMBO_FULL, see, act, 50.0, 10)
    o = _oracle(port, O.MODEL_TEST, recs, COMBO_FULL, see, act, 50.0, 10)
    for k in range(2):
        # positions and velocities do not depend on the see passes in the test model
        assert np.array_equal(g[k]["p"][:, :3], o[k]["p"][:, :3])
        assert np.array_equal(g[k]["v"][:, :3], o[k]["v"][:, :3])
        assert normwise(g[k]["f_buffer"][:, :3], o[k]["f_buffer"][:, :3]) < 1e-3, k


def test_boids_two_flocks(gpu, port):
    a = W.boids_points(15000, seed=43, clusters=4, side=250.0)
    b = W.boids_points(10000, seed=44, clusters=4, side=250.0)
    recs = [M.records(M.BOIDS_RECORD, a.p, a.v), M.records(M.BOIDS_RECORD, b.p, b.v)]
    ctx = M.boids_context()
    see_only = BOIDS_PAIR[:2]
    g = _gpu(O.MODEL_BOIDS, recs, see_only, ctx, ctx, 10.0, 1)
    o = _oracle(port, O.MODEL_BOIDS, recs, see_only, ctx, ctx, 10.0, 1)
    for k in range(2):
        assert g[k]["count"].sum() > 0
        assert np.array_equal(g[k]["count"], o[k]["count"]), k
        assert np.array_equal(g[k]["sep_count"], o[k]["sep_count"]), k
        for f in ("coh", "ali", "sep"):
            assert normwise(g[k][f][:, :3], o[k][f][:, :3]) < 1e-5, (k, f)
    g = _gpu(O.MODEL_BOIDS, recs, BOIDS_PAIR, ctx, ctx, 10.0, 5)
    o = _oracle(port, O.MODEL_BOIDS, recs, BOIDS_PAIR, ctx, ctx, 10.0, 5)
    for k in range(2):
        assert normwise(g[k]["p"][:, :3], o[k]["p"][:, :3]) < 1e-5, k
        assert normwise(g[k]["v"][:, :3], o[k]["v"][:, :3]) < 1e-3, k


GG = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_groups.npz"))
GG_NAMES = sorted({k.split("__")[0] for k in GG.files if "z_grid" in k or k.startswith("boids")})


@pytest.mark.parametrize("name", GG_NAMES)
def test_groups_match_reference_golden(gpu, name):
    """The GPU path against outputs of the reference library itself."""
    model, _, steps, ngroups = (int(x) for x in GG[f"{name}__meta"])
    radius = float(GG[f"{name}__params"][0])
    recs = [GG[f"{name}__in{k}"] for k in range(ngroups)]
    passes = [("see", int(s), int(t), bool(ss)) if see else ("act", int(s)) for see, s, t, ss in GG[f"{name}__passes"]]
    g = _gpu(model, recs, passes, GG[f"{name}__see"], GG[f"{name}__act"], radius, steps)
    for k in range(ngroups):
        want = GG[f"{name}__out{k}"]
        if model == O.MODEL_TEST:
            assert np.array_equal(g[k]["b_buffer_count"], want["b_buffer_count"])
            assert np.array_equal(g[k]["p"], want["p"])
            assert normwise(g[k]["b_buffer"][:, :3], want["b_buffer"][:, :3]) < 1e-5
            assert normwise(g[k]["f_buffer"][:, :3], want["f_buffer"][:, :3]) < 1e-3
        else:
            assert normwise(g[k]["p"][:, :3], want["p"][:, :3]) < 1e-5
            assert normwise(g[k]["v"][:, :3], want["v"][:, :3]) < 1e-3


def _negate_velocities(st, g, dtype):
    n = st.L.tay_get_agent_count(st.ptr, g)
    p = st.agent_ptr(g, 0)
    recs = np.frombuffer(ctypes.string_at(p, n * dtype.itemsize), dtype=dtype).copy()
    recs["v"][:, :3] *= -1.0
    ctypes.memmove(p, recs.ctypes.data, recs.nbytes)
    return recs


def test_device_resident_runs_and_lazy_fetch(gpu, port):
    """Runs chain on the device without host copies; tay_get_agent fetches; host edits
    reach the device only after tay_mark_agents_changed."""
    ps = W.basic_points(20000, seed=45)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    setup = M.test_setup()
    st, g = M.make_state(setup, recs)
    st.start()
    st.run(3)
    st.run(2)
    five = M.by_id(st.agents(g, setup.dtype))
    assert np.array_equal(five["p"], M.run(setup, recs, 5)["p"])
    # an edit without mark_changed stays on the host: the device continues unedited
    _negate_velocities(st, g, setup.dtype)
    st.run(1)
    six = M.by_id(st.agents(g, setup.dtype))
    ref6 = port.run(O.MODEL_TEST, "z_grid", five, setup.passes[0].ctx, setup.passes[-1].ctx, 50.0, 50.0, 1,
                    O.PASS_SEE0 | O.PASS_ACT0).records
    assert np.array_equal(six["p"][:, :3], ref6["p"][:, :3])
    # with mark_changed the edit is pushed
    edited = M.by_id(_negate_velocities(st, g, setup.dtype))
    st.mark_changed(g)
    st.run(2)
    out = M.by_id(st.agents(g, setup.dtype))
    ref = port.run(O.MODEL_TEST, "z_grid", edited, setup.passes[0].ctx, setup.passes[-1].ctx, 50.0, 50.0, 2,
                   O.PASS_SEE0 | O.PASS_ACT0).records
    assert np.array_equal(out["p"][:, :3], ref["p"][:, :3])
    assert np.array_equal(out["v"][:, :3], ref["v"][:, :3])
    st.end()
    st.close()


def test_single_group_pass_list_outside_the_programs(gpu, port):
    """A single group whose pass list no fused program covers (two see passes, then the
    act) runs as a state batch, one kernel per pass."""
    ps = W.basic_points(10000, seed=46)
    recs = [M.records(M.TEST_RECORD, ps.p, ps.v)]
    see, act = M.test_contexts()
    passes = [("see", 0, 0, False), ("see", 0, 0, True), ("act", 0)]
    g = _gpu(O.MODEL_TEST, recs, passes, see, act, 50.0, 4)
    o = _oracle(port, O.MODEL_TEST, recs, passes, see, act, 50.0, 4)
    assert np.array_equal(g[0]["p"][:, :3], o[0]["p"][:, :3])
    assert normwise(g[0]["f_buffer"][:, :3], o[0]["f_buffer"][:, :3]) < 1e-3


@pytest.mark.parametrize("host_loop", ["read", "e2e"])
def test_write_through_equals_one_run(gpu, host_loop):
    """A host that reads its agents after every run gets them written through by the run's
    last pass (from the fused see+act kernel's epilogue for one group, after the step for a
    state batch);
    with or without pushing them back each step, the records equal one uninterrupted
    run's, bit for bit."""
    ps = W.basic_points(30000, seed=47)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    setup = M.test_setup()
    a = M.run(setup, recs, 6)
    b = M.run(setup, recs, 6, host_loop=host_loop)
    assert a.tobytes() == b.tobytes()
    bp = W.boids_points(40000, seed=48, clusters=4, side=300.0)
    brecs = M.records(M.BOIDS_RECORD, bp.p, bp.v)
    bsetup = M.boids_setup()
    a = M.run(bsetup, brecs, 6)
    b = M.run(bsetup, brecs, 6, host_loop=host_loop)
    assert a.tobytes() == b.tobytes()
    groups = _test_groups()
    see, act = M.test_contexts()
    a = _gpu(O.MODEL_TEST, groups, COMBO_FULL, see, act, 50.0, 4)
    funcs, dtype = FUNCS[O.MODEL_TEST]
    b = M.run_groups(dtype, funcs, groups, COMBO_FULL, see, act, 50.0, 50.0, 4, host_loop=host_loop)
    for x, y in zip(a, b):
        assert x.tobytes() == y.tobytes()


def test_engine_write_through_equals_fetch(gpu):
    """Engine ABI: after a run with write-through into page-locked memory, the buffer holds
    exactly what tgpu_batch_fetch returns; pageable memory is refused."""
    ps = W.boids_points(50000, seed=49, clusters=4, side=300.0)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    setup = M.boids_setup()
    b = api.Batch([(setup, recs)])
    L = api.lib()
    host = L.tgpu_host_alloc(recs.nbytes)
    try:
        b.push()
        with pytest.raises(api.TayError):
            b.write_through(0, recs.ctypes.data)  # pageable
        b.write_through(0, host)
        b.run(3)
        got = np.frombuffer(ctypes.string_at(host, recs.nbytes), dtype=recs.dtype).copy()
        assert got.tobytes() == b.fetch(0).tobytes()
        b.write_through(0, None)
        b.run(1)
        stale = np.frombuffer(ctypes.string_at(host, recs.nbytes), dtype=recs.dtype)
        assert stale.tobytes() == got.tobytes()  # turned off: the buffer keeps the last write
    finally:
        b.close()
        L.tgpu_host_free(host)
