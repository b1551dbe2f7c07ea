"""Host-side descriptions of the device models: AoS record layouts, contexts, pass lists.

Each model is registered in the library under the func names listed here; a host uses
them through the plain Tay API (tay_add_see / tay_add_act with these names), exactly as a
reference host registers its functions for the OpenCL path.

  test_basic  the reference's test agent (test/agent.h:2-19, test/agent.c:2-55):
              passes agent_see (self_see FALSE), agent_act
  boids       separation / alignment / cohesion in steering form: boids_see (self_see
              FALSE), boids_act
  sph         weakly compressible SPH: sph_density (self_see TRUE), sph_pressure,
              sph_force (self_see FALSE), sph_integrate
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import api

F4 = ("<f4", 4)

TEST_RECORD = np.dtype([("tag", "<u4", 2), ("p",) + F4, ("v",) + F4, ("b_buffer",) + F4, ("b_buffer_count", "<i4"),
                        ("f_buffer",) + F4, ("id", "<i4")])
BOIDS_RECORD = np.dtype([("tag", "<u4", 2), ("p",) + F4, ("v",) + F4, ("coh",) + F4, ("ali",) + F4,
                         ("sep",) + F4, ("count", "<i4"), ("sep_count", "<i4"), ("id", "<i4"), ("pad", "<i4")])
SPH_RECORD = np.dtype([("tag", "<u4", 2), ("p",) + F4, ("v",) + F4, ("a",) + F4, ("rho", "<f4"), ("P", "<f4"),
                       ("id", "<i4"), ("pad", "<i4")])
BOX_RECORD = np.dtype([("tag", "<u4", 2), ("min",) + F4, ("max",) + F4, ("v",) + F4, ("b_buffer",) + F4,
                       ("b_buffer_count", "<i4"), ("f_buffer",) + F4, ("id", "<i4")])
assert TEST_RECORD.itemsize == 80 and BOIDS_RECORD.itemsize == 104 and SPH_RECORD.itemsize == 72
assert BOX_RECORD.itemsize == 96


def records(dtype, p, v):
    n = p.shape[0]
    rec = np.zeros(n, dtype)
    rec["p"] = p
    rec["v"] = v
    rec["id"] = np.arange(n, dtype=np.int32)
    return rec


def box_records(lo, hi, v):
    """Box-agent records (the reference's BoxAgent, test/agent.h:21-29) from min / max
    corners and velocities ([N,4] arrays)."""
    n = lo.shape[0]
    rec = np.zeros(n, BOX_RECORD)
    rec["min"] = lo
    rec["max"] = hi
    rec["v"] = v
    rec["id"] = np.arange(n, dtype=np.int32)
    return rec


def by_id(rec):
    """Records reordered by their id field (the reference's result_index idiom)."""
    out = np.empty_like(rec)
    out[rec["id"]] = rec
    return out


def test_contexts(radius=50.0, lo=0.0, hi=1000.0):
    see = np.array([radius, radius, radius, 0.0], np.float32)           # SeeContext {float4 radii}
    act = np.array([lo, lo, lo, 0.0, hi, hi, hi, 0.0], np.float32)      # ActContext {float4 min, max}
    return see, act


def boids_context(r=10.0, sep_r=None, w_sep=1.5, w_ali=1.0, w_coh=1.0, max_speed=2.0, max_force=0.03, dt=1.0):
    """Context of the boids model: neighbour radius r, separation radius sep_r (r / 2 by
    default), weights, max speed and max steering force, time step."""
    r = np.float32(r)
    sep_r = np.float32(r / 2 if sep_r is None else sep_r)
    return np.array([r, r * r, sep_r * sep_r, w_sep, w_ali, w_coh, max_speed, max_force, dt, 0, 0, 0], np.float32)


def sph_context(h=0.02, dx=0.01, rho0=1000.0, c0=20.0, alpha=0.05, dt=1e-4, g=(0.0, 0.0, -9.81),
                tank_min=(0.0, 0.0, 0.0), tank_max=(2.0, 1.5, 0.8)):
    """Context values computed in float64 and rounded once to float32."""
    m = rho0 * dx ** 3
    vals = [h, 1.0 / h, (2.0 * h) ** 2, 1.0 / (np.pi * h ** 3), m, rho0, c0 * c0 * rho0 / 7.0, c0, alpha,
            0.01 * h * h, dt, *g, *tank_min, *tank_max]
    return np.array(vals, np.float32)


@dataclass
class Pass:
    name: str
    see: bool
    ctx: np.ndarray
    radius: float = 0.0
    self_see: bool = False


@dataclass
class Setup:
    """A one-group state: record dtype, passes, space parameters."""

    dtype: np.dtype
    passes: list
    part: float
    mb: int = 250
    fixed_box: tuple | None = None
    extra: dict = field(default_factory=dict)
    dims: int = 3
    is_point: bool = True


def test_setup(radius=50.0, part=50.0, passes=("agent_see", "agent_act"), mb=250):
    see, act = test_contexts(radius)
    lst = []
    for p in passes:
        if p == "agent_see":
            lst.append(Pass("agent_see", True, see, radius, False))
        else:
            lst.append(Pass("agent_act", False, act))
    return Setup(TEST_RECORD, lst, part, mb)


def box_setup(radius=50.0, part=50.0, passes=("box_agent_see", "box_agent_act"), mb=250):
    """The reference's box agents: a non-point group."""
    see, act = test_contexts(radius)
    lst = []
    for p in passes:
        if p == "box_agent_see":
            lst.append(Pass("box_agent_see", True, see, radius, False))
        else:
            lst.append(Pass("box_agent_act", False, act))
    return Setup(BOX_RECORD, lst, part, mb, is_point=False)


def boids_setup(r=10.0, part=10.0, passes=("boids_see", "boids_act"), mb=250):
    ctx = boids_context(r)
    lst = [Pass(p, p == "boids_see", ctx, r, False) for p in passes]
    return Setup(BOIDS_RECORD, lst, part, mb)


def sph_setup(h=0.02, part=None, passes=("sph_density", "sph_pressure", "sph_force", "sph_integrate"), mb=250,
              **ctx_kw):
    ctx = sph_context(h=h, **ctx_kw)
    r = 2.0 * h
    lst = [Pass(p, p in ("sph_density", "sph_force"), ctx, r, p == "sph_density") for p in passes]
    return Setup(SPH_RECORD, lst, part if part is not None else r, mb)


def make_state(setup: Setup, recs: np.ndarray):
    """Creates a state with one TAY_GPU_Z_GRID group holding `recs`, passes registered."""
    st = api.State()
    g = st.add_group(setup.dtype.itemsize, max(1, recs.shape[0]), setup.is_point)
    st.configure_space(g, api.TAY_GPU_Z_GRID, setup.dims, api.f4(setup.part), setup.mb)
    if setup.fixed_box is not None:
        st.fix_space_box(g, api.f4(*setup.fixed_box[0]), api.f4(*setup.fixed_box[1]))
    for p in setup.passes:
        if p.see:
            st.add_see(g, g, p.name, api.f4(p.radius, p.radius, p.radius, p.radius), p.self_see, p.ctx)
        else:
            st.add_act(g, p.name, p.ctx)
    st.commit(g, recs)
    return st, g


def _host_loop(st, gs, dtype, steps, host_loop):
    """`steps` steps through the C API: one run (host_loop None), or one run per step with
    the host reading every group after it ("read") and also marking them changed before
    it ("e2e": every step pushes and fetches)."""
    if host_loop is None:
        st.run(steps)
        return
    for _ in range(steps):
        if host_loop == "e2e":
            for g in gs:
                st.mark_changed(g)
        st.run(1)
        for g in gs:
            st.agents(g, dtype)


def run(setup: Setup, recs: np.ndarray, steps: int, host_loop=None):
    """Runs `steps` steps through the C API; returns the records ordered by id."""
    st, g = make_state(setup, recs)
    st.start()
    _host_loop(st, [g], setup.dtype, steps, host_loop)
    out = by_id(st.agents(g, setup.dtype))
    st.end()
    st.close()
    return out


def run_groups(dtype, funcs, groups, passes, see_ctx, act_ctx, radius, part, steps, mb=8, is_point=True,
               host_loop=None):
    """A state of several groups of one model mixed by its passes, through the C API.
    `funcs` = (see func name, act func name); `groups` = record arrays (id order);
    `passes` = ("see", seer, seen, self_see) / ("act", group) tuples in registration
    order.  Returns each group's records ordered by id."""
    from . import api

    st = api.State()
    gs = []
    for recs in groups:
        g = st.add_group(dtype.itemsize, recs.shape[0], is_point)
        st.configure_space(g, api.TAY_GPU_Z_GRID, 3, part, mb)
        gs.append(g)
    for p in passes:
        if p[0] == "see":
            st.add_see(gs[p[1]], gs[p[2]], funcs[0], radius, p[3], see_ctx)
        else:
            st.add_act(gs[p[1]], funcs[1], act_ctx)
    for g, recs in zip(gs, groups):
        st.commit(g, recs)
    st.start()
    _host_loop(st, gs, dtype, steps, host_loop)
    out = [by_id(st.agents(g, dtype)) for g in gs]
    st.end()
    st.close()
    return out
