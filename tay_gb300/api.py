"""ctypes mirror of the Tay C API (include/tay.h) and of the engine ABI (include/tay_gpu.h).

The shared library tay_gb300/libtay_gb300.so is built in-tree by tay_gb300._build.
Loading it is mandatory: there is no fallback implementation, and every entry point
raises when the library is missing or a call fails.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libtay_gb300.so")

TAY_FALSE, TAY_TRUE = 0, 1
(TAY_SPACE_NONE, TAY_CPU_SIMPLE, TAY_CPU_KD_TREE, TAY_CPU_AABB_TREE, TAY_CPU_GRID, TAY_CPU_Z_GRID,
 TAY_GPU_Z_GRID) = range(7)
ERRORS = ["TAY_ERROR_NONE", "TAY_ERROR_POINT_NONPOINT_MISMATCH", "TAY_ERROR_SPACE_INDEX_OUT_OF_RANGE",
          "TAY_ERROR_GROUP_INDEX_OUT_OF_RANGE", "TAY_ERROR_STATE_STATUS", "TAY_ERROR_NOT_IMPLEMENTED",
          "TAY_ERROR_OCL", "TAY_ERROR_CUDA", "TAY_ERROR_DEVICE_MODEL", "TAY_ERROR_BATCH"]


class Float4(ctypes.Structure):
    _pack_ = 1
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float), ("w", ctypes.c_float)]


def f4(x, y=None, z=None, w=0.0) -> Float4:
    if y is None:
        y = z = x
    return Float4(float(x), float(y), float(z), float(w))


class TayError(RuntimeError):
    pass


_VP = ctypes.c_void_p
# (name, restype, argtypes) of every exported symbol declared in include/tay.h and include/tay_gpu.h
TAY_SYMBOLS = [
    ("tay_create_state", _VP, []),
    ("tay_destroy_state", None, [_VP]),
    ("tay_switch_to_ocl", ctypes.c_int, [_VP]),
    ("tay_switch_to_host", ctypes.c_int, [_VP]),
    ("tay_get_error", ctypes.c_int, [_VP]),
    ("tay_add_group", _VP, [_VP, ctypes.c_uint, ctypes.c_uint, ctypes.c_int]),
    ("tay_configure_space", None, [_VP, _VP, ctypes.c_int, ctypes.c_int, Float4, ctypes.c_int]),
    ("tay_fix_space_box", None, [_VP, _VP, Float4, Float4]),
    ("tay_add_see", None, [_VP, _VP, _VP, _VP, ctypes.c_char_p, Float4, ctypes.c_int, _VP, ctypes.c_uint]),
    ("tay_add_act", None, [_VP, _VP, _VP, ctypes.c_char_p, _VP, ctypes.c_uint]),
    ("tay_clear_all_agents", None, [_VP, _VP]),
    ("tay_mark_agents_changed", None, [_VP, _VP]),
    ("tay_get_available_agent", _VP, [_VP, _VP]),
    ("tay_commit_available_agent", None, [_VP, _VP]),
    ("tay_get_agent", _VP, [_VP, _VP, ctypes.c_int]),
    ("tay_simulation_start", None, [_VP]),
    ("tay_run", ctypes.c_int, [_VP, ctypes.c_int]),
    ("tay_simulation_end", None, [_VP]),
    ("tay_get_ms_per_step_for_last_run", ctypes.c_double, [_VP]),
    ("tay_log", None, [_VP, ctypes.c_char_p]),
    ("ocl_add_source", None, [_VP, ctypes.c_char_p]),
    ("tay_threads_start", None, [ctypes.c_uint, ctypes.c_uint]),
    ("tay_threads_stop", None, []),
    ("tay_get_number_of_threads", ctypes.c_uint, []),
    ("tay_run_batch", ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_int]),
    ("tay_get_pairs_for_last_run", ctypes.c_ulonglong, [_VP]),
    ("tay_get_device_ms_for_last_run", ctypes.c_double, [_VP]),
    ("tay_commit_agents", ctypes.c_uint, [_VP, _VP, _VP, ctypes.c_uint]),
    ("tay_get_agent_count", ctypes.c_uint, [_VP, _VP]),
    ("tay_get_error_message", ctypes.c_char_p, [_VP]),
    ("tay_run_recorded", ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("tay_run_backward", ctypes.c_int, [ctypes.POINTER(_VP), ctypes.c_int, _VP, _VP, _VP, _VP, _VP]),
    ("tay_get_recorded_forward_ms", ctypes.c_double, []),
    ("tay_get_backward_ms", ctypes.c_double, []),
    ("tay_get_adjoint_device_bytes", ctypes.c_ulonglong, []),
]
TGPU_SYMBOLS = [
    ("tgpu_batch_create", ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(_VP)]),
    ("tgpu_batch_destroy", None, [_VP]),
    ("tgpu_state_create", ctypes.c_int, [_VP, ctypes.c_int, _VP, ctypes.c_int, ctypes.POINTER(_VP)]),
    ("tgpu_state_set_contexts", ctypes.c_int, [_VP, _VP, ctypes.c_int]),
    ("tgpu_model_nonpoint", ctypes.c_int, [ctypes.c_char_p]),
    ("tgpu_selftest_sort_wait", ctypes.c_int, [ctypes.POINTER(ctypes.c_uint)]),
    ("tgpu_batch_set_contexts", ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    ("tgpu_batch_push", ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    ("tgpu_batch_run", ctypes.c_int, [_VP, ctypes.c_int]),
    ("tgpu_batch_enqueue", ctypes.c_int, [_VP, ctypes.c_int]),
    ("tgpu_batch_sync", ctypes.c_int, [_VP]),
    ("tgpu_batch_fetch", ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    ("tgpu_batch_write_through", ctypes.c_int, [_VP, ctypes.c_int, _VP]),
    ("tgpu_batch_last_device_ms", ctypes.c_double, [_VP]),
    ("tgpu_batch_last_pairs", ctypes.c_ulonglong, [_VP]),
    ("tgpu_batch_launches_per_step", ctypes.c_int, [_VP]),
    ("tgpu_batch_model", ctypes.c_char_p, [_VP]),
    ("tgpu_batch_program", ctypes.c_int, [_VP]),
    ("tgpu_set_tuning", None, [_VP]),
    ("tgpu_get_tuning", None, [_VP]),
    ("tgpu_model_of", ctypes.c_char_p, [ctypes.c_char_p]),
    ("tgpu_register_model", ctypes.c_int, [_VP, ctypes.c_uint]),
    ("tgpu_register_model_library", ctypes.c_int, [ctypes.c_char_p]),
    ("tgpu_batch_profile", ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    ("tgpu_batch_kernel_classes", ctypes.c_int, [_VP]),
    ("tgpu_batch_telemetry", ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_int]),
    ("tgpu_batch_flush_l2", ctypes.c_int, [_VP]),
    ("tgpu_host_alloc", _VP, [ctypes.c_ulonglong]),
    ("tgpu_host_free", None, [_VP]),
    ("tgpu_adjoint_create", ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_VP)]),
    ("tgpu_adjoint_forward", ctypes.c_int, [_VP]),
    ("tgpu_adjoint_backward", ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, _VP]),
    ("tgpu_adjoint_forward_ms", ctypes.c_double, [_VP]),
    ("tgpu_adjoint_backward_ms", ctypes.c_double, [_VP]),
    ("tgpu_adjoint_device_bytes", ctypes.c_ulonglong, [_VP]),
    ("tgpu_adjoint_destroy", None, [_VP]),
    ("tgpu_batch_device_bytes", ctypes.c_ulonglong, [_VP]),
    ("tgpu_see_noalloc", ctypes.c_int, [_VP, ctypes.c_uint, ctypes.POINTER(ctypes.c_float),
                                         ctypes.POINTER(ctypes.c_float), _VP, _VP]),
    ("tgpu_noalloc_max_agents", ctypes.c_uint, []),
    ("tgpu_noalloc_last_error", ctypes.c_char_p, []),
    ("tgpu_device_count", ctypes.c_int, []),
    ("tgpu_last_error", ctypes.c_char_p, []),
]

_lib = None


def lib():
    """Loads libtay_gb300.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m tay_gb300._build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in TAY_SYMBOLS + TGPU_SYMBOLS:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class State:
    """One TayState with the reference's call sequence (test/test_basic.c:92-165)."""

    def __init__(self):
        self.L = lib()
        self.ptr = self.L.tay_create_state()
        if not self.ptr:
            raise TayError("tay_create_state failed")
        self._keep = []  # contexts are borrowed by the C side: keep them alive

    def close(self):
        if self.ptr:
            self.L.tay_destroy_state(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self):
        return self.L.tay_get_error(self.ptr)

    def message(self):
        m = self.L.tay_get_error_message(self.ptr)
        return m.decode() if m else ""

    def check(self, what):
        e = self.error()
        if e:
            raise TayError(f"{what}: {ERRORS[e] if e < len(ERRORS) else e}: {self.message()}")

    def add_group(self, agent_size, capacity, is_point=True):
        g = self.L.tay_add_group(self.ptr, agent_size, capacity, 1 if is_point else 0)
        if not g:
            self.check("tay_add_group")
        return g

    def configure_space(self, group, space_type, dims, part, mb):
        self.L.tay_configure_space(self.ptr, group, space_type, dims, part if isinstance(part, Float4) else f4(part),
                                   int(mb))

    def fix_space_box(self, group, lo, hi):
        self.L.tay_fix_space_box(self.ptr, group, lo, hi)

    def add_see(self, seer, seen, func_name, radii, self_see, ctx):
        buf = None if ctx is None else np.ascontiguousarray(ctx)
        self._keep.append(buf)
        self.L.tay_add_see(self.ptr, seer, seen, None, func_name.encode(),
                           radii if isinstance(radii, Float4) else f4(radii), 1 if self_see else 0,
                           None if buf is None else buf.ctypes.data, 0 if buf is None else buf.nbytes)

    def add_act(self, group, func_name, ctx):
        buf = None if ctx is None else np.ascontiguousarray(ctx)
        self._keep.append(buf)
        self.L.tay_add_act(self.ptr, group, None, func_name.encode(), None if buf is None else buf.ctypes.data,
                           0 if buf is None else buf.nbytes)

    def commit(self, group, records: np.ndarray):
        rec = np.ascontiguousarray(records)
        n = self.L.tay_commit_agents(self.ptr, group, rec.ctypes.data, rec.shape[0])
        if n != rec.shape[0]:
            self.check("tay_commit_agents")
        return n

    def agents(self, group, dtype) -> np.ndarray:
        """Copy of the group's committed agents, in storage (cell) order."""
        n = self.L.tay_get_agent_count(self.ptr, group)
        if n == 0:
            return np.zeros(0, dtype)
        p = self.L.tay_get_agent(self.ptr, group, 0)
        raw = ctypes.string_at(p, n * dtype.itemsize)
        return np.frombuffer(raw, dtype=dtype).copy()

    def mark_changed(self, group):
        self.L.tay_mark_agents_changed(self.ptr, group)

    def agent_ptr(self, group, index=0):
        """tay_get_agent: fetches the group's records when the device holds newer ones."""
        return self.L.tay_get_agent(self.ptr, group, index)

    def start(self):
        self.L.tay_simulation_start(self.ptr)
        self.check("tay_simulation_start")

    def run(self, steps):
        r = self.L.tay_run(self.ptr, steps)
        if r != steps:
            self.check("tay_run")
            raise TayError(f"tay_run ran {r} of {steps} steps")
        return r

    def end(self):
        self.L.tay_simulation_end(self.ptr)

    def ms_per_step(self):
        return self.L.tay_get_ms_per_step_for_last_run(self.ptr)

    def device_ms(self):
        return self.L.tay_get_device_ms_for_last_run(self.ptr)

    def pairs(self):
        return self.L.tay_get_pairs_for_last_run(self.ptr)


class TgpuPass(ctypes.Structure):
    _fields_ = [("func_name", ctypes.c_char_p), ("is_see", ctypes.c_int), ("radii", ctypes.c_float * 4),
                ("self_see", ctypes.c_int), ("context", ctypes.c_void_p), ("context_size", ctypes.c_uint)]


class TgpuGroup(ctypes.Structure):
    _fields_ = [("agent_size", ctypes.c_uint), ("count", ctypes.c_uint), ("min_part_sizes", ctypes.c_float * 4),
                ("shared_megabytes", ctypes.c_int), ("box_fixed", ctypes.c_int), ("box_min", ctypes.c_float * 4),
                ("box_max", ctypes.c_float * 4), ("pass_count", ctypes.c_int),
                ("passes", ctypes.POINTER(TgpuPass)), ("dims", ctypes.c_int)]


class TgpuStatePass(ctypes.Structure):
    _fields_ = [("pass_", TgpuPass), ("seer_group", ctypes.c_int), ("seen_group", ctypes.c_int)]


class Batch:
    """Direct use of the engine ABI (include/tay_gpu.h): one device batch of groups that
    share a model and pass sequence.  `groups` is a list of (setup, records) pairs with
    setup a tay_gb300.models.Setup."""

    def __init__(self, groups):
        self.L = lib()
        self._keep = []
        descs = (TgpuGroup * len(groups))()
        for i, (setup, recs) in enumerate(groups):
            passes = (TgpuPass * len(setup.passes))()
            for k, p in enumerate(setup.passes):
                ctx = np.ascontiguousarray(p.ctx)
                name = p.name.encode()
                self._keep += [ctx, name]
                passes[k].func_name = name
                passes[k].is_see = 1 if p.see else 0
                passes[k].radii[:] = [p.radius] * 4
                passes[k].self_see = 1 if p.self_see else 0
                passes[k].context = ctx.ctypes.data
                passes[k].context_size = ctx.nbytes
            self._keep.append(passes)
            d = descs[i]
            d.agent_size = setup.dtype.itemsize
            d.count = recs.shape[0]
            d.min_part_sizes[:] = [setup.part] * 4
            d.shared_megabytes = setup.mb
            d.box_fixed = 0
            if setup.fixed_box is not None:
                d.box_fixed = 1
                d.box_min[:3] = list(setup.fixed_box[0])
                d.box_max[:3] = list(setup.fixed_box[1])
            d.pass_count = len(setup.passes)
            d.passes = passes
            d.dims = setup.dims
        self._descs = descs
        self.ptr = ctypes.c_void_p()
        self._check(self.L.tgpu_batch_create(descs, len(groups), ctypes.byref(self.ptr)), "tgpu_batch_create")
        self.groups = groups

    def _check(self, rc, what):
        if rc != 0:
            raise TayError(f"{what}: {self.L.tgpu_last_error().decode()}")

    def push(self):
        for i, (_, recs) in enumerate(self.groups):
            r = np.ascontiguousarray(recs)
            self._check(self.L.tgpu_batch_push(self.ptr, i, r.ctypes.data), "tgpu_batch_push")

    def run(self, steps):
        self._check(self.L.tgpu_batch_run(self.ptr, steps), "tgpu_batch_run")
        return self.L.tgpu_batch_last_device_ms(self.ptr), self.L.tgpu_batch_last_pairs(self.ptr)

    def fetch(self, i):
        setup, recs = self.groups[i]
        out = np.zeros(recs.shape[0], setup.dtype)
        self._check(self.L.tgpu_batch_fetch(self.ptr, i, out.ctypes.data), "tgpu_batch_fetch")
        return out

    def write_through(self, i, host_ptr):
        """tgpu_batch_write_through: the last step of every following run stores group i's
        records into the page-locked buffer at host_ptr (an int address, e.g. from
        host_alloc); None turns it off."""
        self._check(self.L.tgpu_batch_write_through(self.ptr, i, host_ptr), "tgpu_batch_write_through")

    def profile(self, steps):
        n = self.L.tgpu_batch_kernel_classes(self.ptr)
        ms = (ctypes.c_double * n)()
        self._check(self.L.tgpu_batch_profile(self.ptr, steps, ms, n), "tgpu_batch_profile")
        return list(ms)

    def telemetry(self):
        """Counters of the last run: candidates tested, pairs, staged / global CTAs,
        union / per-lane warps, warps that replayed a pair list."""
        out = (ctypes.c_ulonglong * 8)()
        self._check(self.L.tgpu_batch_telemetry(self.ptr, out, 8), "tgpu_batch_telemetry")
        return {"candidates": out[0], "pairs": self.L.tgpu_batch_last_pairs(self.ptr), "staged_ctas": out[1],
                "global_ctas": out[2], "union_warps": out[3], "lane_warps": out[4], "replay_warps": out[5]}

    def flush_l2(self):
        self._check(self.L.tgpu_batch_flush_l2(self.ptr), "tgpu_batch_flush_l2")

    def launches_per_step(self):
        return self.L.tgpu_batch_launches_per_step(self.ptr)

    def close(self):
        if self.ptr:
            self.L.tgpu_batch_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def register_model_library(path):
    """Registers the device model of a shared library built against
    include/tay_gpu_model.cuh (tgpu_register_model_library); raises TayError when refused."""
    L = lib()
    if L.tgpu_register_model_library(os.fsencode(path)) != 0:
        raise TayError(L.tgpu_last_error().decode())


def run_batch(states, steps):
    L = lib()
    arr = (ctypes.c_void_p * len(states))(*[s.ptr for s in states])
    r = L.tay_run_batch(arr, len(states), steps)
    if r != steps:
        states[0].check("tay_run_batch")
        raise TayError("tay_run_batch failed")
    return r


class TgpuTuning(ctypes.Structure):
    _fields_ = [("stage", ctypes.c_int), ("stage_cap", ctypes.c_uint), ("stage_cells", ctypes.c_uint),
                ("cell_multiple", ctypes.c_float), ("union_factor", ctypes.c_uint), ("use_graphs", ctypes.c_int),
                ("cell_order", ctypes.c_uint), ("hit_masks", ctypes.c_uint), ("x_cell_factor", ctypes.c_float),
                ("pair_list_cap", ctypes.c_uint)]


def get_tuning() -> dict:
    t = TgpuTuning()
    lib().tgpu_get_tuning(ctypes.byref(t))
    return {f: getattr(t, f) for f, _ in TgpuTuning._fields_}


def set_tuning(**kw):
    """Sets tuning fields (stage, stage_cap, stage_cells, cell_multiple, union_factor,
    use_graphs, cell_order, hit_masks, x_cell_factor, pair_list_cap) for batches created afterwards; no arguments
    restores the defaults."""
    if not kw:
        lib().tgpu_set_tuning(None)
        return
    cur = get_tuning()
    cur.update(kw)
    t = TgpuTuning(**{k: (float(v) if k in ("cell_multiple", "x_cell_factor") else int(v)) for k, v in cur.items()})
    lib().tgpu_set_tuning(ctypes.byref(t))
