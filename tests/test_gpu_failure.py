"""Failure detection without a GPU fault: every spin-wait in the engine's kernels is
bounded and reports through a device error word the host reads.  The radix sort's
look-back wait is made to run out (a predecessor word nothing sets); the kernel returns,
the error word says why, and the context keeps working."""
import ctypes
import time

import numpy as np
import pytest

from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W

pytestmark = pytest.mark.gpu

K_ERR_SORT_LOOKBACK = 2


def test_sort_wait_runs_out_and_reports(gpu):
    L = api.lib()
    err = ctypes.c_uint(0)
    t0 = time.perf_counter()
    assert L.tgpu_selftest_sort_wait(ctypes.byref(err)) == 0, L.tgpu_last_error()
    elapsed = time.perf_counter() - t0
    assert err.value == K_ERR_SORT_LOOKBACK
    assert elapsed < 30.0
    # the context is still usable: a normal step afterwards
    ps = W.basic_points(5000, seed=91)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    out = M.run(M.test_setup(), recs, 2)
    assert np.all(np.isfinite(out["p"][:, :3]))
