"""Host-side behaviour of the Tay C API that needs no GPU: validation errors are sticky
and reported with the reference's error codes (tay/tay.h:31-39) before any device work."""
import numpy as np
import pytest

from tay_gb300 import api
from tay_gb300 import models as M
from tay_gb300 import workloads as W


def _state(space=api.TAY_GPU_Z_GRID, passes=("agent_see", "agent_act"), n=100, is_point=True):
    st = api.State()
    g = st.add_group(M.TEST_RECORD.itemsize, n, is_point)
    st.configure_space(g, space, 3, 50.0, 8)
    see, act = M.test_contexts()
    for p in passes:
        if p.endswith("see"):
            st.add_see(g, g, p, 50.0, False, see)
        else:
            st.add_act(g, p, act)
    ps = W.basic_points(n, seed=1)
    st.commit(g, M.records(M.TEST_RECORD, ps.p, ps.v))
    return st, g


def _run_error(st):
    assert st.L.tay_run(st.ptr, 1) == 0
    return api.ERRORS[st.error()]


def test_run_before_start_is_a_state_error(built):
    st, _ = _state()
    assert _run_error(st) == "TAY_ERROR_STATE_STATUS"


def test_cpu_structure_is_not_implemented_here(built):
    st, _ = _state(space=api.TAY_CPU_Z_GRID)
    st.start()
    assert _run_error(st) == "TAY_ERROR_NOT_IMPLEMENTED"
    assert "TAY_GPU_Z_GRID" in st.message()


def test_unknown_function_name(built):
    st, _ = _state(passes=("nobody_see",))
    st.start()
    assert _run_error(st) == "TAY_ERROR_DEVICE_MODEL"


def test_non_point_group_is_rejected(built):
    st, _ = _state(is_point=False)
    st.start()
    assert _run_error(st) == "TAY_ERROR_POINT_NONPOINT_MISMATCH"


def _two_boids_groups(st):
    groups = []
    for _ in range(2):
        g = st.add_group(M.BOIDS_RECORD.itemsize, 10, True)
        st.configure_space(g, api.TAY_GPU_Z_GRID, 3, 10.0, 8)
        groups.append(g)
    return groups


def test_two_sees_of_one_group_need_an_accumulating_model(built):
    """Boids' see function starts its accumulators from zero, so one boids group cannot
    have two see passes (here over itself and over a second group); refused before any
    device work."""
    st = api.State()
    a, b = _two_boids_groups(st)
    ctx = M.boids_context()
    st.add_see(a, a, "boids_see", 10.0, False, ctx)
    st.add_see(a, b, "boids_see", 10.0, False, ctx)
    st.add_act(a, "boids_act", ctx)
    st.start()
    assert _run_error(st) == "TAY_ERROR_DEVICE_MODEL"
    assert "does not accumulate" in st.message()


def test_pass_on_a_group_of_another_state(built):
    st = api.State()
    other = api.State()
    a = st.add_group(M.TEST_RECORD.itemsize, 10, True)
    st.configure_space(a, api.TAY_GPU_Z_GRID, 3, 50.0, 8)
    b = other.add_group(M.TEST_RECORD.itemsize, 10, True)
    see, _ = M.test_contexts()
    st.add_see(a, b, "agent_see", 50.0, False, see)
    st.start()
    assert _run_error(st) == "TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE"


def test_state_pass_list_is_checked_before_device_work(built):
    """tgpu_state_create refuses unknown functions, bad group indices and passes without
    a standalone kernel before touching the device."""
    import ctypes

    L = api.lib()
    gd = (api.TgpuGroup * 2)()
    for g in gd:
        g.agent_size = 80
        g.count = 10
        g.min_part_sizes[:] = [50.0] * 4
        g.shared_megabytes = 1
    sp = (api.TgpuStatePass * 2)()
    sp[0].pass_.func_name = b"agent_see"
    sp[0].pass_.is_see = 1
    sp[0].seer_group, sp[0].seen_group = 0, 2
    sp[1].pass_.func_name = b"agent_act"
    sp[1].seer_group = 1
    out = ctypes.c_void_p()
    assert L.tgpu_state_create(gd, 2, sp, 2, ctypes.byref(out)) == 1  # TGPU_ERR_ARG
    assert b"out of range" in L.tgpu_last_error()
    sp[0].seen_group = 1
    sp[1].pass_.func_name = b"sph_integrate"
    assert L.tgpu_state_create(gd, 2, sp, 2, ctypes.byref(out)) == 2  # TGPU_ERR_UNKNOWN_FUNC


def test_group_capacity_is_enforced(built):
    st = api.State()
    g = st.add_group(80, 4, True)
    recs = np.zeros(6, M.TEST_RECORD)
    assert st.L.tay_commit_agents(st.ptr, g, recs.ctypes.data, 6) == 4
    assert api.ERRORS[st.error()] == "TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE"
    assert st.L.tay_get_agent_count(st.ptr, g) == 4


def test_start_twice_and_end_without_start(built):
    st = api.State()
    st.L.tay_simulation_end(st.ptr)
    assert api.ERRORS[st.error()] == "TAY_ERROR_STATE_STATUS"
    st2 = api.State()
    st2.L.tay_simulation_start(st2.ptr)
    st2.L.tay_simulation_start(st2.ptr)
    assert api.ERRORS[st2.error()] == "TAY_ERROR_STATE_STATUS"


def test_agents_round_trip_on_host(built):
    st = api.State()
    g = st.add_group(M.TEST_RECORD.itemsize, 50, True)
    ps = W.basic_points(50, seed=2)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    st.commit(g, recs)
    assert st.agents(g, M.TEST_RECORD).tobytes() == recs.tobytes()


def test_opencl_switch_reports_no_device(built):
    st = api.State()
    assert st.L.tay_switch_to_ocl(st.ptr) == 0
    assert st.L.tay_switch_to_host(st.ptr) == 0


def test_unsupported_pass_sequence_is_refused_before_device_work(built):
    passes = (api.TgpuPass * 1)()
    ctx = np.zeros(8, np.float32)
    passes[0].func_name = b"agent_act"
    passes[0].is_see = 0
    passes[0].context = ctx.ctypes.data
    passes[0].context_size = ctx.nbytes
    gd = (api.TgpuGroup * 1)()
    gd[0].agent_size = 80
    gd[0].count = 10
    gd[0].min_part_sizes[:] = [50.0] * 4
    gd[0].shared_megabytes = 1
    gd[0].pass_count = 1
    gd[0].passes = passes
    L = api.lib()
    import ctypes

    out = ctypes.c_void_p()
    # agent_act alone is a supported sequence; sph_force alone is not
    passes[0].func_name = b"sph_force"
    gd[0].agent_size = 72
    assert L.tgpu_batch_create(gd, 1, ctypes.byref(out)) == 3  # TGPU_ERR_PROGRAM
    assert b"not supported" in L.tgpu_last_error()
