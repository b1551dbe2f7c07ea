"""The allocation-free neighbour pass (tgpu_see_noalloc), checked against the regular path.

tgpu_see_noalloc is for callers that cannot call cudaMalloc when they need the pass - a
host whose memory manager owns the device heap, a plugin that may not allocate after
initialisation, a latency-sensitive loop.  It keeps all its intermediate buffers in a
fixed array of the library's own device memory.  This test calls it twice in a row
through the C ABI on device buffers and compares each result with what the ordinary
entry point (tay_run with the test model's see pass) computes for the same agents:
neighbour counts bit for bit, displacement sums within 1e-5 normwise.  It also checks
that a call above the size limit is refused with a clear message.
"""
import ctypes

import numpy as np
import pytest

from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

from parity import normwise

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_entry_point(gpu):
    torch = pytest.importorskip("torch")
    L = api.lib()
    n = 20000
    ps = W.basic_points(n, seed=31)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    ref = M.run(M.test_setup(passes=("agent_see",)), recs, 1)

    radii = (ctypes.c_float * 4)(50.0, 50.0, 50.0, 0.0)
    part = (ctypes.c_float * 4)(50.0, 50.0, 50.0, 50.0)
    pos = torch.from_numpy(ps.p.copy()).cuda()
    for _ in range(2):
        out = torch.full((n, 4), -1.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = L.tgpu_see_noalloc(ctypes.c_void_p(pos.data_ptr()), n, radii, part, ctypes.c_void_p(out.data_ptr()),
                                None)
        assert rc == 0, L.tgpu_noalloc_last_error().decode()
        o = out.cpu().numpy()
        counts = o[:, 3].copy().view(np.int32)
        assert counts.sum() > 0
        assert np.array_equal(counts, ref["b_buffer_count"])
        assert normwise(o[:, :3], ref["b_buffer"][:, :3]) < 1e-5

    too_many = L.tgpu_noalloc_max_agents() + 1
    rc = L.tgpu_see_noalloc(ctypes.c_void_p(pos.data_ptr()), too_many, radii, part, ctypes.c_void_p(out.data_ptr()),
                            None)
    assert rc != 0
    assert b"exceed the maximum" in L.tgpu_noalloc_last_error()
