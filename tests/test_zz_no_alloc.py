"""The allocation-free neighbour pass (tgpu_see_noalloc), checked against the regular path.

tgpu_see_noalloc is for callers that cannot call cudaMalloc when they need the pass - a
host whose memory manager owns the device heap, a plugin that may not allocate after
initialisation, a latency-sensitive loop.  It keeps all its intermediate buffers in a
fixed array of the library's own device memory.  These tests call it twice in a row
through the C ABI on device buffers and compare each result with what the ordinary
entry point (tay_run with the test model's see pass) computes for the same agents:
neighbour counts bit for bit, displacement sums within 1e-5 normwise.  The cases cover a
small call, a call that fills the array (exactly the maximum agent count) and a call
whose grid wants more than the array's 64 cells per axis (its cells are enlarged).  A
call above the size limit is refused with a clear message.
"""
import ctypes

import numpy as np
import pytest

from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise

pytestmark = pytest.mark.gpu


def _twice_against_regular(L, torch, n, seed, radius, part):
    ps = W.basic_points(n, seed=seed)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    ref = M.run(M.test_setup(radius=radius, part=part, passes=("agent_see",)), recs, 1)

    radii = (ctypes.c_float * 4)(radius, radius, radius, 0.0)
    parts = (ctypes.c_float * 4)(part, part, part, part)
    pos = torch.from_numpy(ps.p.copy()).cuda()
    out = None
    for _ in range(2):
        out = torch.full((n, 4), -1.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = L.tgpu_see_noalloc(ctypes.c_void_p(pos.data_ptr()), n, radii, parts, ctypes.c_void_p(out.data_ptr()),
                                None)
        assert rc == 0, L.tgpu_noalloc_last_error().decode()
        o = out.cpu().numpy()
        counts = o[:, 3].copy().view(np.int32)
        assert counts.sum() > 0
        assert np.array_equal(counts, ref["b_buffer_count"])
        assert normwise(o[:, :3], ref["b_buffer"][:, :3]) < 1e-5
    return pos, out, radii, parts


def test_noalloc_matches_regular_entry_point(gpu):
    torch = pytest.importorskip("torch")
    L = api.lib()
    pos, out, radii, parts = _twice_against_regular(L, torch, 20000, 31, 50.0, 50.0)

    too_many = L.tgpu_noalloc_max_agents() + 1
    rc = L.tgpu_see_noalloc(ctypes.c_void_p(pos.data_ptr()), too_many, radii, parts, ctypes.c_void_p(out.data_ptr()),
                            None)
    assert rc != 0
    assert b"exceed the maximum" in L.tgpu_noalloc_last_error()


def test_noalloc_full_array(gpu):
    """Exactly tgpu_noalloc_max_agents() agents: every per-agent region of the array full."""
    torch = pytest.importorskip("torch")
    L = api.lib()
    n = L.tgpu_noalloc_max_agents()
    assert n == 65536
    _twice_against_regular(L, torch, n, 32, 40.0, 40.0)


def test_noalloc_axis_clamp(gpu):
    """Minimum part size 4 in a cube of side 1000 asks for 250 cells per axis; the array's
    grid holds 64, so the cells grow and the keys stay within 18 bits."""
    torch = pytest.importorskip("torch")
    L = api.lib()
    _twice_against_regular(L, torch, 30000, 33, 12.0, 4.0)
