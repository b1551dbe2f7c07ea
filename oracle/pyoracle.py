"""Python access to the oracle (TEST INFRASTRUCTURE ONLY).

Two CPU implementations of the reference Tay path, with one calling convention:
  port      oracle/_build/liboracle.so - the C restatement (tay_oracle.c), FP32 and FP64
  reference oracle/_ref/libtayref.so   - the reference's own sources built by
                                         oracle/ref/Makefile (only where the reference
                                         source tree is available)

Both take AoS agent records in id order and return them in id order.  The record
layouts below mirror oracle/oracle_models.h (and, for the test model, the reference's
test/agent.h:2-10).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libtayref.so")

MODEL_TEST, MODEL_BOIDS, MODEL_SPH, MODEL_BOX = 0, 1, 2, 3
SPACE = {"simple": 1, "kd_tree": 2, "aabb_tree": 3, "grid": 4, "z_grid": 5}
PASS_SEE0, PASS_ACT0, PASS_SEE1, PASS_ACT1 = 1, 2, 4, 8


def _rec(real):
    f = "<f4" if real == np.float32 else "<f8"
    test = np.dtype([("tag", "<u4", 2), ("p", f, 4), ("v", f, 4), ("b_buffer", f, 4), ("b_buffer_count", "<i4"),
                     ("f_buffer", f, 4), ("id", "<i4")])
    boid = np.dtype([("tag", "<u4", 2), ("p", f, 4), ("v", f, 4), ("coh", f, 4), ("ali", f, 4), ("sep", f, 4),
                     ("count", "<i4"), ("sep_count", "<i4"), ("id", "<i4"), ("pad", "<i4")])
    sph = np.dtype([("tag", "<u4", 2), ("p", f, 4), ("v", f, 4), ("a", f, 4), ("rho", f), ("P", f), ("id", "<i4"),
                    ("pad", "<i4")])
    box = np.dtype([("tag", "<u4", 2), ("min", f, 4), ("max", f, 4), ("v", f, 4), ("b_buffer", f, 4),
                    ("b_buffer_count", "<i4"), ("f_buffer", f, 4), ("id", "<i4")])
    return {MODEL_TEST: test, MODEL_BOIDS: boid, MODEL_SPH: sph, MODEL_BOX: box}


RECORDS = {np.float32: _rec(np.float32), np.float64: _rec(np.float64)}
assert RECORDS[np.float32][MODEL_TEST].itemsize == 80
assert RECORDS[np.float32][MODEL_BOIDS].itemsize == 104
assert RECORDS[np.float32][MODEL_SPH].itemsize == 72
assert RECORDS[np.float32][MODEL_BOX].itemsize == 96


def boids_context(real, r=10.0, sep_r=5.0, w_sep=1.5, w_ali=1.0, w_coh=1.0, max_speed=2.0, max_force=0.03, dt=1.0):
    r = real(r)
    sep_r = real(sep_r)
    return np.array([r, r * r, sep_r * sep_r, w_sep, w_ali, w_coh, max_speed, max_force, dt, 0, 0, 0], dtype=real)


def sph_context(real, h=0.02, dx=0.01, rho0=1000.0, c0=20.0, alpha=0.05, dt=1e-4, g=(0.0, 0.0, -9.81),
                tank_min=(0.0, 0.0, 0.0), tank_max=(2.0, 1.5, 0.8)):
    """Context values are computed in float64 and rounded once to `real`."""
    m = rho0 * dx ** 3
    vals = [h, 1.0 / h, (2.0 * h) ** 2, 1.0 / (np.pi * h ** 3), m, rho0, c0 * c0 * rho0 / 7.0, c0, alpha,
            0.01 * h * h, dt, *g, *tank_min, *tank_max]
    return np.array(vals, dtype=real)


def test_act_context(real, lo=0.0, hi=1000.0):
    return np.array([lo, lo, lo, 0.0, hi, hi, hi, 0.0], dtype=real)


def make_records(model, p, v, real=np.float32):
    """AoS records for positions/velocities ([N,4] arrays); ids 0..N-1, accumulators zero."""
    n = p.shape[0]
    rec = np.zeros(n, RECORDS[real][model])
    rec["p"] = p
    rec["v"] = v
    rec["id"] = np.arange(n, dtype=np.int32)
    return rec


def make_box_records(lo, hi, v, real=np.float32):
    """Box-agent records from min / max corners and velocities ([N,4] arrays)."""
    n = lo.shape[0]
    rec = np.zeros(n, RECORDS[real][MODEL_BOX])
    rec["min"] = lo
    rec["max"] = hi
    rec["v"] = v
    rec["id"] = np.arange(n, dtype=np.int32)
    return rec


def build_port():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def build_reference(ref_root):
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={ref_root}"], check=True)


_ARGTYPES = None


def _bind(lib, name, real_c):
    fn = getattr(lib, name)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   real_c, real_c, ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_int,
                   ctypes.POINTER(ctypes.c_double)]
    return fn


@dataclass
class RunResult:
    records: np.ndarray
    ms_per_step: float
    pairs: int = -1  # box-test passes over the run (port only)


def _bind_groups(lib, name, real_c):
    fn = getattr(lib, name)
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, real_c, real_c, ctypes.c_int, ctypes.c_int, ctypes.c_int] + \
        [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    return fn


class _Impl:
    def __init__(self, so, names, pair_fns=None, group_names=None, space_fns=None):
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        self.lib = ctypes.CDLL(so)
        self.space_fns = {}
        for real, (nm, c) in (space_fns or {}).items():
            f = getattr(self.lib, nm)
            f.restype = None
            f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
            self.space_fns[real] = (f, c)
        self.fns = {real: _bind(self.lib, nm, c) for real, (nm, c) in names.items()}
        self.group_fns = {real: _bind_groups(self.lib, nm, c) for real, (nm, c) in (group_names or {}).items()}
        self.pair_fns = {}
        for real, nm in (pair_fns or {}).items():
            f = getattr(self.lib, nm)
            f.restype = ctypes.c_ulonglong
            f.argtypes = []
            self.pair_fns[real] = f

    def set_space(self, dims=3, box=None, real=np.float32):
        """Space options of the following runs: dims (1..3) and a fixed box ((min3, max3))."""
        f, _ = self.space_fns[real]
        lo = np.zeros(3, real) if box is None else np.asarray(box[0], real)
        hi = np.zeros(3, real) if box is None else np.asarray(box[1], real)
        f(int(dims), 0 if box is None else 1, lo.ctypes.data, hi.ctypes.data)

    def run(self, model, space, records, see_ctx, act_ctx, radius, part_size, steps, pass_mask, threads=0, mb=250,
            real=np.float32, dims=3, box=None):
        self.set_space(dims, box, real)
        fn = self.fns[real]
        rec = np.ascontiguousarray(records.copy())
        see = np.ascontiguousarray(see_ctx) if see_ctx is not None else np.zeros(4, real)
        act = np.ascontiguousarray(act_ctx) if act_ctx is not None else see
        ms = ctypes.c_double()
        sp = SPACE[space] if isinstance(space, str) else int(space)
        ran = fn(model, sp, rec.shape[0], rec.ctypes.data, see.ctypes.data, act.ctypes.data, real(radius),
                 real(part_size), mb, steps, pass_mask, threads, ctypes.byref(ms))
        if ran != steps:
            raise RuntimeError(f"oracle run failed ({ran} of {steps} steps)")
        pairs = int(self.pair_fns[real]()) if real in self.pair_fns else -1
        return RunResult(rec, ms.value, pairs)

    def run_groups(self, model, space, groups, passes, see_ctx, act_ctx, radius, part_size, steps, threads=0, mb=250,
                   real=np.float32, dims=3, box=None):
        """Several groups of one model; `groups` is a list of record arrays (id order),
        `passes` a list of ("see", seer, seen, self_see) / ("act", group) tuples.
        Returns a list of RunResult (one per group; pairs summed over all passes)."""
        self.set_space(dims, box, real)
        fn = self.group_fns[real]
        recs = [np.ascontiguousarray(r.copy()) for r in groups]
        counts = np.array([r.shape[0] for r in recs], np.int32)
        ptrs = (ctypes.c_void_p * len(recs))(*[r.ctypes.data for r in recs])
        is_see = np.array([1 if p[0] == "see" else 0 for p in passes], np.int32)
        seer = np.array([p[1] for p in passes], np.int32)
        seen = np.array([p[2] if p[0] == "see" else p[1] for p in passes], np.int32)
        self_see = np.array([int(p[3]) if p[0] == "see" else 0 for p in passes], np.int32)
        see = np.ascontiguousarray(see_ctx) if see_ctx is not None else np.zeros(4, real)
        act = np.ascontiguousarray(act_ctx) if act_ctx is not None else see
        ms = ctypes.c_double()
        sp = SPACE[space] if isinstance(space, str) else int(space)
        ran = fn(model, sp, len(recs), counts.ctypes.data, ctypes.cast(ptrs, ctypes.c_void_p), see.ctypes.data,
                 act.ctypes.data, real(radius), real(part_size), mb, steps, len(passes), is_see.ctypes.data,
                 seer.ctypes.data, seen.ctypes.data, self_see.ctypes.data, threads, ctypes.byref(ms))
        if ran != steps:
            raise RuntimeError(f"oracle group run failed ({ran} of {steps} steps)")
        pairs = int(self.pair_fns[real]()) if real in self.pair_fns else -1
        return [RunResult(r, ms.value, pairs) for r in recs]


_port = None
_ref = None


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build_port()
        _port = _Impl(PORT_SO, {np.float32: ("oracle_run_f32", ctypes.c_float),
                                np.float64: ("oracle_run_f64", ctypes.c_double)},
                      {np.float32: "oracle_last_pairs_f32", np.float64: "oracle_last_pairs_f64"},
                      {np.float32: ("oracle_run_groups_f32", ctypes.c_float),
                       np.float64: ("oracle_run_groups_f64", ctypes.c_double)},
                      {np.float32: ("oracle_set_space_f32", ctypes.c_float),
                       np.float64: ("oracle_set_space_f64", ctypes.c_double)})
    return _port


def reference():
    """The reference's own CPU path, or None when it was not built on this machine."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            return None
        _ref = _Impl(REF_SO, {np.float32: ("ref_run", ctypes.c_float)}, None,
                     {np.float32: ("ref_run_groups", ctypes.c_float)},
                     {np.float32: ("ref_set_space", ctypes.c_float)})
    return _ref


def sph_adjoint_f64(x0, v0, ctx64, steps, dl_dx=None, dl_dv=None, backward=True):
    """FP64 CPU adjoint of an SPH rollout (oracle/sph_adjoint.c): every pair within the
    support, from per-step neighbour lists, summed in ascending index order.
    x0, v0, dl_dx, dl_dv: [n, 3]; ctx64: sph_context(np.float64, ...).  Returns
    dict(dx0, dv0, dalpha, dc0, x_final, v_final); with backward=False only the forward
    rollout runs (x_final, v_final; the gradients are zero)."""
    lib = port().lib
    fn = lib.oracle_sph_adjoint_f64
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 7
    n = x0.shape[0]
    x0 = np.ascontiguousarray(x0[:, :3], np.float64)
    v0 = np.ascontiguousarray(v0[:, :3], np.float64)
    gx = np.zeros((n, 3)) if dl_dx is None else np.ascontiguousarray(dl_dx[:, :3], np.float64)
    gv = np.zeros((n, 3)) if dl_dv is None else np.ascontiguousarray(dl_dv[:, :3], np.float64)
    c = np.ascontiguousarray(ctx64, np.float64)
    dx0, dv0 = np.zeros((n, 3)), np.zeros((n, 3))
    xf, vf = np.zeros((n, 3)), np.zeros((n, 3))
    th = np.zeros(2)
    r = fn(n, x0.ctypes.data, v0.ctypes.data, c.ctypes.data, steps, gx.ctypes.data, gv.ctypes.data,
           dx0.ctypes.data if backward else None, dv0.ctypes.data, th.ctypes.data, xf.ctypes.data, vf.ctypes.data)
    if r != steps:
        raise RuntimeError("oracle_sph_adjoint_f64 failed")
    return {"dx0": dx0, "dv0": dv0, "dalpha": th[0], "dc0": th[1], "x_final": xf, "v_final": vf}
