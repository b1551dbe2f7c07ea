"""GPU parity of non-point (box) agents: the reference's box agent (test/agent.h:21-29,
test/agent.c:57-118) in a TAY_GPU_Z_GRID group, pairs by the reference's non-point test
(tay/space.c:92-103).  The reference keeps box agents in CpuSimple / trees only (its grids
take points), so the oracle here is CpuSimple: exact pair sets."""
import os

import numpy as np
import pytest

from oracle import pyoracle as O
from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise

pytestmark = pytest.mark.gpu


def _boxes(n, seed, max_size=50.0):
    b = W.box_agents(n, seed=seed, max_size=max_size)
    return M.box_records(b.lo, b.hi, b.v)


def _oracle(port, recs, setup, steps, mask):
    see = setup.passes[0].ctx
    act = setup.passes[-1].ctx
    r = setup.passes[0].radius if setup.passes[0].see else 50.0
    return port.run(O.MODEL_BOX, "simple", recs, see, act, r, r, steps, mask).records


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("max_size", [50.0, 200.0])
def test_box_counts_bit_exact(gpu, port, order, max_size):
    recs = _boxes(20000, 61, max_size)
    setup = M.box_setup(passes=("box_agent_see",))
    try:
        api.set_tuning(cell_order=order)
        g = M.run(setup, recs, 1)
    finally:
        api.set_tuning()
    o = _oracle(port, recs, setup, 1, O.PASS_SEE0)
    assert g["b_buffer_count"].sum() > 0
    assert np.array_equal(g["b_buffer_count"], o["b_buffer_count"])
    assert normwise(g["b_buffer"][:, :3], o["b_buffer"][:, :3]) < 1e-5


def test_box_steps(gpu, port):
    recs = _boxes(15000, 62)
    setup = M.box_setup()
    g = M.run(setup, recs, 10)
    o = _oracle(port, recs, setup, 10, O.PASS_SEE0 | O.PASS_ACT0)
    # the boxes' motion does not depend on the see pass: bit-exact
    for f in ("min", "max", "v"):
        assert np.array_equal(g[f][:, :3], o[f][:, :3]), f
    assert normwise(g["f_buffer"][:, :3], o["f_buffer"][:, :3]) < 1e-3


GS = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_space.npz"))
BOX_NAMES = sorted({k.split("__")[0] for k in GS.files if k.startswith("box_")})


@pytest.mark.parametrize("name", BOX_NAMES)
def test_box_matches_reference_golden(gpu, name):
    _, _, steps, mask, _ = (int(x) for x in GS[f"{name}__meta"])
    passes = ("box_agent_see", "box_agent_act") if mask & O.PASS_ACT0 else ("box_agent_see",)
    setup = M.box_setup(passes=passes)
    g = M.run(setup, GS[f"{name}__in"], steps)
    want = GS[f"{name}__out"]
    assert np.array_equal(g["b_buffer_count"], want["b_buffer_count"])
    for f in ("min", "max", "v"):
        assert np.array_equal(g[f][:, :3], want[f][:, :3]), f
    assert normwise(g["b_buffer"][:, :3], want["b_buffer"][:, :3]) < 1e-5
    assert normwise(g["f_buffer"][:, :3], want["f_buffer"][:, :3]) < 1e-3


def test_two_box_groups(gpu, port):
    """The combination test's non-point x non-point case (test/test_combo.c:13-14)."""
    recs = [_boxes(8000, 63), _boxes(6000, 64)]
    see, act = M.test_contexts()
    passes = [("see", 0, 0, False), ("see", 0, 1, False), ("see", 1, 1, False), ("see", 1, 0, False)]
    g = M.run_groups(M.BOX_RECORD, ("box_agent_see", "box_agent_act"), recs, passes, see, act, 50.0, 50.0, 1,
                     is_point=False)
    o = port.run_groups(O.MODEL_BOX, "simple", recs, passes, see, act, 50.0, 50.0, 1)
    for k in range(2):
        assert np.array_equal(g[k]["b_buffer_count"], o[k].records["b_buffer_count"]), k
        assert normwise(g[k]["b_buffer"][:, :3], o[k].records["b_buffer"][:, :3]) < 1e-5, k


def test_shape_mismatch_is_reported(gpu):
    st = api.State()
    g = st.add_group(M.TEST_RECORD.itemsize, 10, False)
    st.configure_space(g, api.TAY_GPU_Z_GRID, 3, 50.0, 8)
    see, _ = M.test_contexts()
    st.add_see(g, g, "agent_see", 50.0, False, see)
    st.start()
    assert st.L.tay_run(st.ptr, 1) == 0
    assert api.ERRORS[st.error()] == "TAY_ERROR_POINT_NONPOINT_MISMATCH"
