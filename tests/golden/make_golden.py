"""Generates the golden vectors in this folder by running the reference Tay library itself.

    python tests/golden/make_golden.py [/path/to/reference/tay/tree]

Builds the reference's own CPU path from its source tree (oracle/ref/Makefile, outputs in
oracle/_ref/) and runs each case below through the reference's public API
(tay_create_state ... tay_run ... tay_get_agent) on seeded inputs from
tay_gb300.workloads.  The outputs (AoS records in id order) are stored in golden.npz with
the inputs they came from, so the oracle restatement can be pinned against the reference
on machines where the reference source tree is absent.

Cases (small enough for CpuSimple):
  test_see_*     test model, 1500 agents in [0,1000]^3, r = 50, see pass only, 1 step,
                 CpuSimple / CpuGrid / CpuZGrid
  test_full_*    same agents, see + act, 10 steps, CpuGrid / CpuZGrid
  boids_see      2000 boids in 4 clusters, r = 10, see only, 1 step, CpuZGrid
  boids_full     same, see + act, 5 steps, CpuZGrid
  sph_density    6x6x6 lattice, density pass only, 1 step, CpuZGrid
  sph_full       8x8x8 lattice, all four passes, 5 steps, CpuZGrid

Two-group cases (golden_groups.npz; the pass list of test/test_combo.c:114-119):
  combo_see_*    test model, groups of 1200 and 800 agents, see a->a, a->b, b->b, b->a,
                 1 step, CpuSimple / CpuZGrid
  combo_full_*   the same passes + act a, act b, 5 steps, CpuGrid / CpuZGrid
  boids_pair     boids groups of 1500 and 1000, see a->b, b->a, act a, act b, 3 steps,
                 CpuZGrid

Space-option cases (golden_space.npz):
  dims2_*        test model, 2000 agents, tay_configure_space dims 2 (box test and grid
                 over x, y only), see + act, 3 steps, CpuSimple / CpuGrid
  dims1_grid     the same with dims 1, CpuGrid
  fixed_*        tay_fix_space_box [-10, 1010]^3 around the agents, see + act, 3 steps,
                 CpuGrid / CpuZGrid
  (the reference's CpuZGrid pairs nothing below 3 dims, tay/cpu_z_grid.c:254-260, so
  dims < 3 is pinned on CpuSimple / CpuGrid)
  box_see_simple  the reference's box agents (non-point group), 2000 cubes of edge 1..50
                  in [0,1000]^3, r = 50, see only, 1 step, CpuSimple
  box_full_simple the same, see + act, 5 steps
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as O  # noqa: E402
from tay_gb300 import workloads as W  # noqa: E402


def cases():
    ps = W.basic_points(1500, seed=101)
    see, act = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32)
    rec = O.make_records(O.MODEL_TEST, ps.p, ps.v)
    for space in ("simple", "grid", "z_grid"):
        yield f"test_see_{space}", O.MODEL_TEST, space, rec, see, act, 50.0, 50.0, 1, O.PASS_SEE0
    for space in ("grid", "z_grid"):
        yield f"test_full_{space}", O.MODEL_TEST, space, rec, see, act, 50.0, 50.0, 10, O.PASS_SEE0 | O.PASS_ACT0
    bp = W.boids_points(2000, seed=102, clusters=4, side=200.0)
    brec = O.make_records(O.MODEL_BOIDS, bp.p, bp.v)
    bctx = O.boids_context(np.float32)
    yield "boids_see", O.MODEL_BOIDS, "z_grid", brec, bctx, bctx, 10.0, 10.0, 1, O.PASS_SEE0
    yield "boids_full", O.MODEL_BOIDS, "z_grid", brec, bctx, bctx, 10.0, 10.0, 5, O.PASS_SEE0 | O.PASS_ACT0
    s6 = W.sph_dam(6, 6, 6)
    srec6 = O.make_records(O.MODEL_SPH, s6.points.p, s6.points.v)
    sctx = O.sph_context(np.float32)
    yield "sph_density", O.MODEL_SPH, "z_grid", srec6, sctx, sctx, 0.04, 0.04, 1, O.PASS_SEE0
    s8 = W.sph_dam(8, 8, 8)
    srec8 = O.make_records(O.MODEL_SPH, s8.points.p, s8.points.v)
    yield "sph_full", O.MODEL_SPH, "z_grid", srec8, sctx, sctx, 0.04, 0.04, 5, 15


COMBO = [("see", 0, 0, False), ("see", 0, 1, False), ("see", 1, 1, False), ("see", 1, 0, False)]
COMBO_FULL = COMBO + [("act", 0), ("act", 1)]
BOIDS_PAIR = [("see", 0, 1, False), ("see", 1, 0, False), ("act", 0), ("act", 1)]


def group_cases():
    a = W.basic_points(1200, seed=111)
    b = W.basic_points(800, seed=112)
    recs = [O.make_records(O.MODEL_TEST, a.p, a.v), O.make_records(O.MODEL_TEST, b.p, b.v)]
    see, act = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32)
    for space in ("simple", "z_grid"):
        yield f"combo_see_{space}", O.MODEL_TEST, space, recs, COMBO, see, act, 50.0, 1
    for space in ("grid", "z_grid"):
        yield f"combo_full_{space}", O.MODEL_TEST, space, recs, COMBO_FULL, see, act, 50.0, 5
    ba = W.boids_points(1500, seed=113, clusters=2, side=120.0)
    bb = W.boids_points(1000, seed=114, clusters=2, side=120.0)
    brecs = [O.make_records(O.MODEL_BOIDS, ba.p, ba.v), O.make_records(O.MODEL_BOIDS, bb.p, bb.v)]
    bctx = O.boids_context(np.float32)
    yield "boids_pair", O.MODEL_BOIDS, "z_grid", brecs, BOIDS_PAIR, bctx, bctx, 10.0, 3


def space_cases():
    ps = W.basic_points(2000, seed=121)
    rec = O.make_records(O.MODEL_TEST, ps.p, ps.v)
    see, act = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32)
    full = O.PASS_SEE0 | O.PASS_ACT0
    for space in ("simple", "grid"):
        yield f"dims2_{space}", space, rec, see, act, 3, full, 2, None
    yield "dims1_grid", "grid", rec, see, act, 3, full, 1, None
    box = ((-10.0, -10.0, -10.0), (1010.0, 1010.0, 1010.0))
    for space in ("grid", "z_grid"):
        yield f"fixed_{space}", space, rec, see, act, 3, full, 3, box


def box_cases():
    b = W.box_agents(2000, seed=122)
    rec = O.make_box_records(b.lo, b.hi, b.v)
    see, act = np.array([50, 50, 50, 0], np.float32), O.test_act_context(np.float32)
    yield "box_see_simple", "simple", rec, see, act, 1, O.PASS_SEE0, 3, None
    yield "box_full_simple", "simple", rec, see, act, 5, O.PASS_SEE0 | O.PASS_ACT0, 3, None


def pass_table(passes):
    return np.array([[1 if p[0] == "see" else 0, p[1], p[2] if p[0] == "see" else p[1], int(p[3]) if p[0] == "see" else 0]
                     for p in passes], np.int64)


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    O.build_reference(ref_root)
    ref = O.reference()
    if ref is None:
        raise SystemExit("the reference library did not build")
    out = {}
    for name, model, space, rec, see, act, radius, part, steps, mask in cases():
        r = ref.run(model, space, rec, see, act, radius, part, steps, mask, threads=4)
        out[f"{name}__in"] = rec
        out[f"{name}__out"] = r.records
        out[f"{name}__meta"] = np.array([model, O.SPACE[space], steps, mask], np.int64)
        out[f"{name}__params"] = np.array([radius, part], np.float64)
        out[f"{name}__see"] = see
        out[f"{name}__act"] = act
        print(f"{name}: {rec.shape[0]} agents, {steps} steps")
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    out = {}
    for name, model, space, recs, passes, see, act, radius, steps in group_cases():
        res = ref.run_groups(model, space, recs, passes, see, act, radius, radius, steps, threads=4)
        for k, (rec, r) in enumerate(zip(recs, res)):
            out[f"{name}__in{k}"] = rec
            out[f"{name}__out{k}"] = r.records
        out[f"{name}__meta"] = np.array([model, O.SPACE[space], steps, len(recs)], np.int64)
        out[f"{name}__passes"] = pass_table(passes)
        out[f"{name}__params"] = np.array([radius, radius], np.float64)
        out[f"{name}__see"] = see
        out[f"{name}__act"] = act
        print(f"{name}: {[r.shape[0] for r in recs]} agents, {steps} steps")
    np.savez_compressed(os.path.join(HERE, "golden_groups.npz"), **out)
    out = {}
    opt_cases = [(O.MODEL_TEST,) + c for c in space_cases()] + [(O.MODEL_BOX,) + c for c in box_cases()]
    for model, name, space, rec, see, act, steps, mask, dims, box in opt_cases:
        r = ref.run(model, space, rec, see, act, 50.0, 50.0, steps, mask, threads=4, dims=dims, box=box)
        out[f"{name}__in"] = rec
        out[f"{name}__out"] = r.records
        out[f"{name}__meta"] = np.array([model, O.SPACE[space], steps, mask, dims], np.int64)
        out[f"{name}__box"] = np.zeros((2, 3)) if box is None else np.array(box, np.float64)
        out[f"{name}__fixed"] = np.array([0 if box is None else 1], np.int64)
        out[f"{name}__see"] = see
        out[f"{name}__act"] = act
        print(f"{name}: {rec.shape[0]} agents, dims {dims}, fixed box {box is not None}")
    ref.set_space()
    np.savez_compressed(os.path.join(HERE, "golden_space.npz"), **out)


if __name__ == "__main__":
    main()
