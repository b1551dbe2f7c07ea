"""The oracle restatement pinned against the reference: against the committed golden
vectors (generated by the reference library itself, tests/golden/make_golden.py) and,
where the reference source tree is present, against the reference run live."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import workloads as W

from parity import normwise

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")
SPACE_NAME = {v: k for k, v in O.SPACE.items()}


def _golden():
    g = np.load(GOLDEN)
    names = sorted({k.split("__")[0] for k in g.files})
    return g, names


GOLD, GOLD_NAMES = _golden()


def same_records(model, a, b):
    """Bit-for-bit equality of every field the reference defines.  The reference's test
    model leaves the w components of b_buffer and f_buffer undefined (its float4 helpers
    return structs whose w is never set, test/taystd.c:109-135), and the box model also
    those of min and max, so those floats are excluded for these models."""
    if model not in (O.MODEL_TEST, O.MODEL_BOX):
        return a.tobytes() == b.tobytes()
    for f in a.dtype.names:
        x, y = a[f], b[f]
        if f in ("b_buffer", "f_buffer", "min", "max"):
            x, y = x[:, :3], y[:, :3]
        if np.ascontiguousarray(x).tobytes() != np.ascontiguousarray(y).tobytes():
            return False
    return True


@pytest.mark.parametrize("name", GOLD_NAMES)
def test_port_bit_exact_with_golden(port, name):
    model, space, steps, mask = (int(x) for x in GOLD[f"{name}__meta"])
    radius, part = (float(x) for x in GOLD[f"{name}__params"])
    rec_in = GOLD[f"{name}__in"]
    r = port.run(model, SPACE_NAME[space], rec_in, GOLD[f"{name}__see"], GOLD[f"{name}__act"], radius, part, steps,
                 mask, threads=3)
    want = GOLD[f"{name}__out"]
    assert same_records(model, r.records, want), name


def test_reference_counts_identical_across_structures():
    """The reference's own property: Simple, Grid and ZGrid see the same pairs."""
    c = [GOLD[f"test_see_{s}__out"]["b_buffer_count"] for s in ("simple", "grid", "z_grid")]
    assert c[0].sum() > 0
    assert np.array_equal(c[0], c[1]) and np.array_equal(c[0], c[2])


@pytest.mark.parametrize("threads", [1, 4])
def test_port_thread_count_does_not_change_results(port, threads):
    ps = W.basic_points(3000, seed=9)
    rec = O.make_records(O.MODEL_TEST, ps.p, ps.v)
    see, act = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32)
    a = port.run(O.MODEL_TEST, "z_grid", rec, see, act, 50.0, 50.0, 5, 3, threads=threads).records
    b = port.run(O.MODEL_TEST, "z_grid", rec, see, act, 50.0, 50.0, 5, 3, threads=2).records
    assert same_records(O.MODEL_TEST, a, b)


def test_port_pair_counter_matches_counts(port):
    ps = W.basic_points(3000, seed=10)
    rec = O.make_records(O.MODEL_TEST, ps.p, ps.v)
    see, act = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32)
    r = port.run(O.MODEL_TEST, "grid", rec, see, act, 50.0, 50.0, 1, O.PASS_SEE0, threads=4)
    assert r.pairs == int(r.records["b_buffer_count"].sum())


def test_fp64_oracle_agrees_with_fp32(port):
    ps = W.basic_points(3000, seed=12)
    rec32 = O.make_records(O.MODEL_TEST, ps.p, ps.v)
    rec64 = O.make_records(O.MODEL_TEST, ps.p, ps.v, real=np.float64)
    see32, act32 = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32)
    see64, act64 = see32.astype(np.float64), act32.astype(np.float64)
    a = port.run(O.MODEL_TEST, "z_grid", rec32, see32, act32, 50.0, 50.0, 10, 3, threads=4).records
    b = port.run(O.MODEL_TEST, "z_grid", rec64, see64, act64, 50.0, 50.0, 10, 3, threads=4, real=np.float64).records
    assert np.array_equal(a["b_buffer_count"], b["b_buffer_count"])
    assert normwise(a["f_buffer"][:, :3], b["f_buffer"][:, :3]) < 1e-5


@pytest.mark.skipif(O.reference() is None, reason="reference source tree not built on this machine")
@pytest.mark.parametrize("model,space", [(O.MODEL_TEST, "grid"), (O.MODEL_BOIDS, "z_grid"), (O.MODEL_SPH, "grid")])
def test_port_bit_exact_with_live_reference(port, model, space):
    if model == O.MODEL_TEST:
        ps = W.basic_points(2500, seed=13)
        rec = O.make_records(model, ps.p, ps.v)
        see, act, radius, mask, steps = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32), 50.0, 3, 4
    elif model == O.MODEL_BOIDS:
        ps = W.boids_points(2500, seed=14, clusters=3, side=150.0)
        rec = O.make_records(model, ps.p, ps.v)
        see = act = O.boids_context(np.float32)
        radius, mask, steps = 10.0, 3, 4
    else:
        s = W.sph_dam(7, 7, 7)
        rec = O.make_records(model, s.points.p, s.points.v)
        see = act = O.sph_context(np.float32)
        radius, mask, steps = 0.04, 15, 4
    a = port.run(model, space, rec, see, act, radius, radius, steps, mask, threads=3).records
    b = O.reference().run(model, space, rec, see, act, radius, radius, steps, mask, threads=3).records
    assert same_records(model, a, b)


GOLDEN_GROUPS = os.path.join(os.path.dirname(__file__), "golden", "golden_groups.npz")
GG = np.load(GOLDEN_GROUPS)
GG_NAMES = sorted({k.split("__")[0] for k in GG.files})


def group_passes(table):
    """Pass tuples from the stored [is_see, seer, seen, self_see] rows."""
    return [("see", int(s), int(t), bool(ss)) if see else ("act", int(s)) for see, s, t, ss in table]


@pytest.mark.parametrize("name", GG_NAMES)
def test_port_groups_bit_exact_with_golden(port, name):
    """Two groups mixed by their see passes (the combination test's pass list)."""
    model, space, steps, ngroups = (int(x) for x in GG[f"{name}__meta"])
    radius, part = (float(x) for x in GG[f"{name}__params"])
    recs = [GG[f"{name}__in{k}"] for k in range(ngroups)]
    res = port.run_groups(model, SPACE_NAME[space], recs, group_passes(GG[f"{name}__passes"]), GG[f"{name}__see"],
                          GG[f"{name}__act"], radius, part, steps, threads=3)
    for k, r in enumerate(res):
        assert same_records(model, r.records, GG[f"{name}__out{k}"]), (name, k)
    if name.startswith("combo_see"):
        assert res[0].records["b_buffer_count"].sum() > 0


@pytest.mark.skipif(O.reference() is None, reason="reference source tree not built on this machine")
def test_port_groups_bit_exact_with_live_reference(port):
    a = W.basic_points(900, seed=31)
    b = W.basic_points(1300, seed=32)
    recs = [O.make_records(O.MODEL_TEST, a.p, a.v), O.make_records(O.MODEL_TEST, b.p, b.v)]
    passes = [("see", 1, 0, False), ("see", 0, 0, True), ("act", 1), ("see", 0, 1, False), ("act", 0)]
    see, act = np.array([60, 40, 50, 0], np.float32), O.test_act_context(np.float32)
    x = port.run_groups(O.MODEL_TEST, "z_grid", recs, passes, see, act, 50.0, 50.0, 4, threads=3)
    y = O.reference().run_groups(O.MODEL_TEST, "z_grid", recs, passes, see, act, 50.0, 50.0, 4, threads=3)
    for r, s in zip(x, y):
        assert same_records(O.MODEL_TEST, r.records, s.records)


GS = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_space.npz"))
GS_NAMES = sorted({k.split("__")[0] for k in GS.files})


def space_case(name):
    model, space, steps, mask, dims = (int(x) for x in GS[f"{name}__meta"])
    box = tuple(map(tuple, GS[f"{name}__box"])) if int(GS[f"{name}__fixed"][0]) else None
    return model, SPACE_NAME[space], steps, mask, dims, box


@pytest.mark.parametrize("name", GS_NAMES)
def test_port_space_options_bit_exact_with_golden(port, name):
    """tay_configure_space dims 1 / 2 and tay_fix_space_box."""
    model, space, steps, mask, dims, box = space_case(name)
    r = port.run(model, space, GS[f"{name}__in"], GS[f"{name}__see"], GS[f"{name}__act"], 50.0, 50.0, steps, mask,
                 threads=3, dims=dims, box=box)
    port.set_space()
    assert same_records(model, r.records, GS[f"{name}__out"]), name


def test_port_grid_overflow_is_an_error(port):
    """The 1M-boid workload on CpuGrid with 256 MB: the reference's shrink step rounds each
    axis up (tay/cpu_grid.c:100-108) and leaves more cells than its array holds, after which
    the reference indexes past the array.  The restatement reports the run as failed
    instead (the reference build itself is not run on this input); with 2048 MB the same
    grid fits."""
    ps = W.boids_points(1 << 20, seed=2)
    recs = O.make_records(O.MODEL_BOIDS, ps.p, ps.v)
    ctx = O.boids_context(np.float32)
    with pytest.raises(RuntimeError, match="0 of 1 steps"):
        port.run(O.MODEL_BOIDS, "grid", recs, ctx, ctx, 10.0, 10.0, 1, O.PASS_SEE0, mb=256)
