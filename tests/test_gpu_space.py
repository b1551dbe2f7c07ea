"""GPU parity of the space options: tay_configure_space dims 1 / 2 (box test and grid over
the first dims axes, tay/space.c:62-68) and tay_fix_space_box (tay/state.c:120-125,
tay/space.c:36-48), against the reference's golden vectors and the oracle.  The
reference's own Z-grid pairs nothing below 3 dims (tay/cpu_z_grid.c:254-260), so dims
< 3 is compared with the reference's CpuGrid / CpuSimple, which implement it."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise

pytestmark = pytest.mark.gpu

GS = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_space.npz"))
GS_NAMES = sorted({k.split("__")[0] for k in GS.files if not k.startswith("box_")})
SPACE_NAME = {v: k for k, v in O.SPACE.items()}


@pytest.mark.parametrize("name", GS_NAMES)
def test_space_options_match_reference_golden(gpu, name):
    model, _, steps, mask, dims = (int(x) for x in GS[f"{name}__meta"])
    box = tuple(map(tuple, GS[f"{name}__box"])) if int(GS[f"{name}__fixed"][0]) else None
    setup = M.test_setup()
    setup.dims = dims
    setup.fixed_box = box
    rec = GS[f"{name}__in"]
    g = M.run(setup, rec, steps)
    want = GS[f"{name}__out"]
    assert np.array_equal(g["p"][:, :3], want["p"][:, :3])
    assert np.array_equal(g["v"][:, :3], want["v"][:, :3])
    assert normwise(g["f_buffer"][:, :3], want["f_buffer"][:, :3]) < 1e-3


@pytest.mark.parametrize("dims", [1, 2])
@pytest.mark.parametrize("order", [0, 1])
def test_low_dims_counts_bit_exact(gpu, port, dims, order):
    ps = W.basic_points(20000, seed=51)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    setup = M.test_setup(passes=("agent_see",), radius=20.0 if dims == 2 else 2.0, part=20.0 if dims == 2 else 2.0)
    setup.dims = dims
    try:
        api.set_tuning(cell_order=order)
        g = M.run(setup, recs, 1)
    finally:
        api.set_tuning()
    see = setup.passes[0].ctx
    r = setup.passes[0].radius
    o = port.run(O.MODEL_TEST, "grid", recs, see, see, r, r, 1, O.PASS_SEE0, dims=dims)
    port.set_space()
    assert g["b_buffer_count"].sum() > 0
    assert np.array_equal(g["b_buffer_count"], o.records["b_buffer_count"])
    assert normwise(g["b_buffer"][:, :3], o.records["b_buffer"][:, :3]) < 1e-5


def test_two_group_pass_uses_min_dims(gpu, port):
    """A dims-2 seer group over a dims-3 seen group tests two axes (min over both)."""
    a = W.basic_points(6000, seed=52)
    b = W.basic_points(5000, seed=53)
    recs = [M.records(M.TEST_RECORD, a.p, a.v), M.records(M.TEST_RECORD, b.p, b.v)]
    see, act = M.test_contexts(radius=20.0)
    st = api.State()
    ga = st.add_group(M.TEST_RECORD.itemsize, 6000, True)
    gb = st.add_group(M.TEST_RECORD.itemsize, 5000, True)
    st.configure_space(ga, api.TAY_GPU_Z_GRID, 2, 20.0, 8)
    st.configure_space(gb, api.TAY_GPU_Z_GRID, 3, 20.0, 8)
    st.add_see(ga, gb, "agent_see", 20.0, False, see)
    st.commit(ga, recs[0])
    st.commit(gb, recs[1])
    st.start()
    st.run(1)
    out = M.by_id(st.agents(ga, M.TEST_RECORD))
    st.end()
    st.close()
    # all pairs within 20 in x and y, any z
    pa, pb = recs[0]["p"][:, :3], recs[1]["p"][:, :3]
    want = np.zeros(6000, np.int64)
    for lo in range(0, 6000, 500):
        d = np.abs(pa[lo:lo + 500, None, :2] - pb[None, :, :2])
        want[lo:lo + 500] = np.all(~(d > 20.0), axis=2).sum(axis=1)
    assert np.array_equal(out["b_buffer_count"], want)
