#!/usr/bin/env python3
"""Benchmark of the GB300 Z-grid step on the 1M-boid workload.

Workload: 1,048,576 FP32 boids, 64 Gaussian clusters (sigma 40) with centres uniform in a
cube of side 2000, velocity = unit random direction x speed U[1, 2]; see radius 10,
separation/alignment/cohesion weights 1.5/1.0/1.0, max speed 2, dt 1; Z-grid with minimum
cell size 10 (seeded synthetic data: SplitMix64, seed 2).

One step = sort (keys, radix passes, cell table with the reorder) + the fused see+act pass.
  value   pair-interactions/s with the agents resident in HBM: pairs that passed the box
          test (device counter) / device time of the timed steps (CUDA events on the
          engine's stream), L2 flushed between steps;
  e2e     the same metric through the Tay C API with host buffers: each step is
          tay_mark_agents_changed + tay_run(state, 1) + tay_get_agent, which copies the AoS
          records host->device, runs the step and copies them back (what the OpenCL
          path's push/fetch around every run costs, tay/state.c:208-315);
  roofline  of the dominant kernel (the fused see+act pass), from a profiled leg with
          CUDA events around every kernel class on the engine's stream.
--impl reference times the CPU implementation of the same step (the oracle restatement
of the reference's CpuZGrid, all host threads) on the same workload.

Multi-GPU: the step does not shard (one state = one GPU); N ranks run N independent
replicas ("replicas only"), and value = pairs of all ranks / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_BOIDS = 1 << 20
RADIUS = 10.0
CELL = 10.0
SEED = 2
BOIDS_RECORD_BYTES = 104


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=100,
                    help="largest CPU sample: the CPU baseline and the reference arm time min(steps, this) steps "
                         "of the same workload from the same initial state (0.26 s per step on 16 Grace cores)")
    ap.add_argument("--c1", type=int, default=1, help="1 = add the 100,000-agent test model leg and its CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batched-states", type=int, default=512, help="states of the batched leg (0 = skip)")
    ap.add_argument("--sph", type=int, default=1, help="1 = add the 524,288-particle SPH leg")
    ap.add_argument("--features", type=int, default=1, help="1 = add the two-group / resident / dims-2 / box legs")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--adjoint", type=int, default=1, help="1 = add the differentiable SPH leg")
    ap.add_argument("--adjoint-steps", type=int, default=200, help="rollout steps of the differentiable SPH leg")
    ap.add_argument("--adjoint-keeps", default="2,1,0",
                    help="kept segments of each adjoint run (checkpoints every 20 steps; 0 records every step)")
    ap.add_argument("--stage", type=int, default=None, help="see kernel: 1 = stage halos in shared memory")
    ap.add_argument("--union-factor", type=int, default=None, help="see kernel: union walk threshold")
    ap.add_argument("--cell-order", type=int, default=None, help="0 = Morton cells, 1 = x-rows")
    ap.add_argument("--hit-masks", type=int, default=None, help="1 = see walk with hit masks (cell order 1)")
    ap.add_argument("--x-cell-factor", type=float, default=None, help="cell order 1: x cell / y,z cell")
    ap.add_argument("--cell-multiple", type=float, default=None, help="grid cell edge / min part size")
    return ap.parse_args()


def rank_visible_device(local, visible):
    """The device a rank keeps visible: the local rank's entry of CUDA_VISIBLE_DEVICES when
    that lists devices, else the device whose index is the local rank."""
    vis = [v.strip() for v in (visible or "").split(",") if v.strip()]
    return vis[local % len(vis)] if vis else str(local)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x):
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def wait_first(self, timeout_s=3.0):
        """Waits (bounded) until the sampler has written its first line, so that the samples
        cover the region that follows rather than the sampler's own start-up."""
        t0 = time.perf_counter()
        while self.proc is not None and time.perf_counter() - t0 < timeout_s:
            if os.path.getsize(self.path) > 0:
                return
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 7:
                    continue
                try:
                    sm.append(float(parts[0]))
                    mx.append(float(parts[1]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[3:7]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def workload():
    from tay_gb300 import models as M
    from tay_gb300 import workloads as W

    ps = W.boids_points(N_BOIDS, seed=SEED)
    recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
    setup = M.boids_setup(r=RADIUS, part=CELL, mb=256)
    return setup, recs


CONFIG = {"workload": "boids_1M_zgrid", "agents": N_BOIDS, "radius": RADIUS, "cell": CELL,
          "clusters": 64, "sigma": 40.0, "side": 2000.0, "weights": [1.5, 1.0, 1.0], "max_speed": 2.0, "dt": 1.0,
          "passes": ["boids_see", "boids_act"], "seed": SEED}


def bench_config(world):
    """The workload description both arms print (the same keys and values)."""
    return dict(CONFIG, l2="GPU arm: flushed between timed steps", parallelism=f"replicas{world}")


def batched_workload(states):
    """The batched boids workload: `states` states, N log-uniform in [1000, 65536], box side
    (125 N)^(1/3), radius U[5, 20] (cell = radius), same boids rules."""
    from tay_gb300 import models as M
    from tay_gb300 import workloads as W

    bb = W.batched_boids(states=states, seed=4)
    groups = []
    for ps, r, side in bb.states:
        recs = M.records(M.BOIDS_RECORD, ps.p, ps.v)
        groups.append((M.boids_setup(r=r, part=r, mb=4), recs))
    return groups


def batched_cpu_baseline(groups, steps=1):
    """The batched workload on the host: every state one by one on CpuZGrid (oracle
    restatement, all host threads), `steps` steps each from its initial state."""
    from oracle import pyoracle as O

    threads = os.cpu_count() or 1
    pairs, secs = 0, 0.0
    for setup, recs in groups:
        ctx = setup.passes[0].ctx
        r = O.port().run(O.MODEL_BOIDS, "z_grid", recs, ctx, ctx, setup.passes[0].radius, setup.part, steps,
                         O.PASS_SEE0 | O.PASS_ACT0, threads=threads, mb=setup.mb)
        pairs += r.pairs
        secs += r.ms_per_step * steps / 1000.0
    return {"value": pairs / secs, "unit": "pair-interactions/s", "cores": threads, "kind": "port",
            "ms_per_step": 1000.0 * secs / steps,
            "sample": f"{steps} step(s) of each of the {len(groups)} states, one state after another, on CpuZGrid "
                      f"(oracle restatement, {threads} threads)"}


def batched_vs_plain(states, steps, tune=True, cpu_steps=0):
    """Device-resident comparison on the same GPU: one batch of all states (one launch per
    kernel per step) against the states run one by one (each its own batch and step)."""
    from tay_gb300 import api, autotune

    groups = batched_workload(states)
    if tune:
        autotune.autotune(groups, use_cache=False)
    agents = sum(r.shape[0] for _, r in groups)
    B = api.Batch(groups)
    B.push()
    B.run(2)
    dev_ms, pairs = 0.0, 0
    t0 = time.perf_counter()
    for _ in range(steps):
        ms, p = B.run(1)
        dev_ms += ms
        pairs += p
    wall_b = (time.perf_counter() - t0) / steps
    B.close()
    singles = [api.Batch([g]) for g in groups]
    for s in singles:
        s.push()
        s.run(1)
    plain_steps = steps
    dev_p, pairs_p = 0.0, 0
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        for s in singles:
            ms, p = s.run(1)
            dev_p += ms
            pairs_p += p
    wall_p = (time.perf_counter() - t0) / plain_steps
    for s in singles:
        s.close()
    tuning = api.get_tuning()
    api.set_tuning()
    out = {"tuning": tuning, "states": states, "agents": agents, "steps": steps, "plain_steps": plain_steps,
           "batched_ms_per_step": wall_b * 1000.0, "batched_device_ms_per_step": dev_ms / steps,
           "batched_pairs_per_s": pairs / (wall_b * steps),
           "plain_ms_per_step": wall_p * 1000.0, "plain_device_ms_per_step": dev_p / plain_steps,
           "plain_pairs_per_s": pairs_p / (wall_p * plain_steps),
           "speedup": wall_p / wall_b}
    if cpu_steps:
        out["cpu_baseline"] = batched_cpu_baseline(groups, cpu_steps)
    return out


def sph_leg(steps, tune=True, cpu_steps=0):
    """The SPH dam break: 64x128x64 = 524,288 particles on a 0.01 lattice in a
    2.0 x 1.5 x 0.8 tank, h 0.02 (see radius 2h), four passes per step."""
    from tay_gb300 import api, autotune
    from tay_gb300 import models as M
    from tay_gb300 import workloads as W

    s = W.sph_dam(64, 128, 64)
    recs = M.records(M.SPH_RECORD, s.points.p, s.points.v)
    setup = M.sph_setup(mb=512)
    if tune:
        autotune.autotune([(setup, recs)], use_cache=False)
    B = api.Batch([(setup, recs)])
    B.push()
    B.run(2)
    dev_ms, pairs = 0.0, 0
    for _ in range(steps):
        B.flush_l2()
        ms, p = B.run(1)
        dev_ms += ms
        pairs += p
    tel = B.telemetry()  # the last step: warps that walked, and warps that replayed a pair list
    B.close()
    tuning = api.get_tuning()
    api.set_tuning()
    out = {"particles": int(recs.shape[0]), "steps": steps, "ms_per_step": dev_ms / steps,
           "pair_interactions_per_s": pairs / (dev_ms / 1000.0), "pairs_per_step": pairs / steps,
           "tuning": tuning,
           "last_step_warps": {k: tel[k] for k in ("union_warps", "lane_warps", "replay_warps")}}
    if cpu_steps:
        from oracle import pyoracle as O

        threads = os.cpu_count() or 1
        ctx = setup.passes[0].ctx
        r = O.port().run(O.MODEL_SPH, "z_grid", recs, ctx, ctx, setup.passes[0].radius, setup.part, cpu_steps, 15,
                         threads=threads, mb=setup.mb)
        secs = r.ms_per_step * cpu_steps / 1000.0
        out["cpu_baseline"] = {"value": r.pairs / secs, "unit": "pair-interactions/s", "cores": threads,
                               "kind": "port", "ms_per_step": r.ms_per_step,
                               "sample": f"{cpu_steps} steps of the 524,288-particle dam (4 passes) on CpuZGrid "
                                         f"(oracle restatement, {threads} threads)"}
    return out


def adjoint_cpu_baseline(points, tank, steps=2, instances=32):
    """The calibration rollout's forward on the host: one instance (the instances are the
    same lattice) on CpuZGrid, all four SPH passes, `steps` steps (oracle restatement, all
    host threads); the batch's time is that of its instances one after another."""
    from oracle import pyoracle as O
    from tay_gb300 import models as M

    threads = os.cpu_count() or 1
    setup = M.sph_setup(alpha=0.05, c0=20.0, tank_min=(0.0, 0.0, 0.0), tank_max=tank, mb=64)
    recs = M.records(M.SPH_RECORD, points.p, points.v)
    ctx = setup.passes[0].ctx
    r = O.port().run(O.MODEL_SPH, "z_grid", recs, ctx, ctx, setup.passes[0].radius, setup.part, steps, 15,
                     threads=threads, mb=setup.mb)
    batch_ms = r.ms_per_step * instances
    return {"value": r.pairs / (r.ms_per_step * steps / 1000.0), "unit": "pair-interactions/s", "cores": threads,
            "kind": "port", "ms_per_step": batch_ms,
            "sample": f"{steps} forward steps of one {points.n}-particle instance on CpuZGrid (oracle restatement, "
                      f"{threads} threads); ms_per_step is that of the {instances} instances one after another"}


def adjoint_leg(steps=200, every=20, instances=32, keep=1, tune=True, cpu_steps=0):
    """The differentiable SPH calibration: `instances` SPH instances of 20,480
    particles (32x40x16 lattice, spacing 0.01, h 0.02), a `steps`-step rollout, loss = MSE
    of final positions against a target rollout (alpha 0.08, c0 22, same initial state);
    gradients w.r.t. (alpha, c0) and initial velocities from the adjoint with checkpoints
    every `every` steps.  Reports forward, recorded-forward and backward device time and
    the device memory held."""
    from tay_gb300 import api, autotune
    from tay_gb300 import workloads as W
    from tay_gb300.adjoint import SphRollout

    tank = (0.64, 0.6, 0.4)
    s = W.sph_dam(32, 40, 16, tank=tank)
    inst = [(s.points, 0.05, 20.0, (0.0, 0.0, 0.0), tank) for _ in range(instances)]
    tgt_roll = SphRollout([(s.points, 0.08, 22.0, (0.0, 0.0, 0.0), tank) for _ in range(instances)], steps, every)
    target, _ = tgt_roll.forward()
    tgt_roll.close()
    groups = SphRollout(inst, steps)._groups(np.zeros((len(inst) * s.points.n, 3), np.float32),
                                             np.array([[0.05, 20.0]] * instances))
    if tune:
        autotune.autotune(groups, use_cache=False)
    # plain forward (no recording) of the same rollout, one batch, graphs
    plain = api.Batch(groups)
    plain.push()
    fwd_ms, _ = plain.run(steps)
    plain.close()
    roll = SphRollout(inst, steps, every, keep_segments=keep)
    x, _ = roll.forward()
    n = s.points.n
    g = np.zeros_like(x)
    loss = 0.0
    for k in range(instances):
        d = x[k * n:(k + 1) * n] - target[k * n:(k + 1) * n]
        loss += float(np.mean(np.sum(d.astype(np.float64) ** 2, axis=1)))
        g[k * n:(k + 1) * n] = 2.0 * d / n
    dx0, dv0, dp = roll.backward(g)
    rec_ms, bwd_ms, mem = roll.forward_ms(), roll.backward_ms(), roll.device_bytes()
    roll.close()
    tuning = api.get_tuning()
    api.set_tuning()
    out = {"instances": instances, "particles_per_instance": n, "steps": steps, "checkpoint_every": every,
           "kept_segments": keep if every else None, "tuning": tuning,
           "forward_ms": fwd_ms, "recorded_forward_ms": rec_ms, "backward_ms": bwd_ms,
           "fwd_plus_bwd_over_fwd": (rec_ms + bwd_ms) / fwd_ms, "device_bytes": mem, "loss": loss,
           "dloss_dalpha_mean": float(dp[:, 0].mean()), "dloss_dc0_mean": float(dp[:, 1].mean())}
    if cpu_steps:
        cb = adjoint_cpu_baseline(s.points, tank, cpu_steps, instances)
        cb["forward_ms_for_the_rollout_steps"] = cb["ms_per_step"] * steps
        out["cpu_baseline"] = cb
    return out


def c1_leg(steps=100, cpu_steps=100):
    """The first configuration: 100,000 test agents, positions U[0, 1000]^3, velocities
    U[-1, 1]^3 (seed 1), see radius 50 with the test model's count and displacement sum,
    act moving each agent and reflecting it at the walls, minimum part size 50, 100 steps.
    GPU: device time through the C API; CPU: the oracle restatement of CpuGrid (the
    configuration's structure) on all host threads, the same steps from the same state."""
    from oracle import pyoracle as O
    from tay_gb300 import api
    from tay_gb300 import models as M
    from tay_gb300 import workloads as W

    ps = W.basic_points(100_000, seed=1)
    recs = M.records(M.TEST_RECORD, ps.p, ps.v)
    setup = M.test_setup(radius=50.0, part=50.0, mb=64)
    st, g = M.make_state(setup, recs)
    st.start()
    st.run(3)
    st.run(steps)
    dev = st.L.tay_get_device_ms_for_last_run(st.ptr) / steps
    pairs = st.pairs() / steps
    st.end()
    st.close()
    out = {"agents": 100_000, "steps": steps, "ms_per_step": dev, "pairs_per_step": pairs,
           "pair_interactions_per_s": pairs / (dev / 1000.0), "tuning": api.get_tuning()}
    if cpu_steps:
        threads = os.cpu_count() or 1
        see, act = M.test_contexts(50.0)
        r = O.port().run(O.MODEL_TEST, "grid", recs, see, act, 50.0, 50.0, cpu_steps, O.PASS_SEE0 | O.PASS_ACT0,
                         threads=threads, mb=setup.mb)
        secs = r.ms_per_step * cpu_steps / 1000.0
        out["cpu_baseline"] = {"value": r.pairs / secs, "unit": "pair-interactions/s", "cores": threads,
                               "kind": "port", "ms_per_step": r.ms_per_step,
                               "sample": f"{cpu_steps} steps of the 100,000-agent workload on CpuGrid, part size 50 "
                                         f"(oracle restatement, {threads} threads)"}
    return out


def features_leg(setup, recs, tuning, steps=20):
    """The hot path's other shapes (the rows after the headline), each timed through the C
    API with the headline's tuning: a two-group state with the combination test's passes,
    the device-resident loop (tay_run(state, 1) with no host copies) beside the e2e loop, a
    2-D space, a fixed space box, and non-point (box) agents.  Device time per step from
    the engine's events."""
    import time

    from tay_gb300 import api
    from tay_gb300 import models as M
    from tay_gb300 import workloads as W

    api.set_tuning()
    api.set_tuning(**tuning)
    out = {"tuning": dict(tuning)}
    see, act = M.test_contexts(radius=10.0, hi=500.0)

    # two groups of 262,144, see a->a, a->b, b->b, b->a, act a, act b (test/test_combo.c)
    st = api.State()
    gs = []
    for k in range(2):
        ps = W.basic_points(1 << 18, seed=300 + k, side=500.0)
        g = st.add_group(M.TEST_RECORD.itemsize, 1 << 18, True)
        st.configure_space(g, api.TAY_GPU_Z_GRID, 3, 10.0, 64)
        st.commit(g, M.records(M.TEST_RECORD, ps.p, ps.v))
        gs.append(g)
    for a, b in ((0, 0), (0, 1), (1, 1), (1, 0)):
        st.add_see(gs[a], gs[b], "agent_see", 10.0, False, see)
    for a in (0, 1):
        st.add_act(gs[a], "agent_act", act)
    st.start()
    st.run(3)
    st.run(steps)
    dev = st.L.tay_get_device_ms_for_last_run(st.ptr) / steps
    pairs = st.pairs() / steps
    out["two_groups"] = {"agents": 2 << 18, "passes": "4 see + 2 act", "ms_per_step": dev,
                         "pair_interactions_per_s": pairs / (dev / 1000.0), "pairs_per_step": pairs}
    st.end()
    st.close()

    # device-resident loop vs the loop that copies the records both ways every step
    st, g = M.make_state(setup, recs)
    st.start()
    st.run(3)
    t0 = time.perf_counter()
    for _ in range(steps):
        st.run(1)
    resident = 1000.0 * (time.perf_counter() - t0) / steps
    st.agent_ptr(g, 0)
    t0 = time.perf_counter()
    for _ in range(steps):
        st.mark_changed(g)
        st.run(1)
        st.agent_ptr(g, 0)
    copying = 1000.0 * (time.perf_counter() - t0) / steps
    out["device_resident"] = {"agents": int(recs.shape[0]), "tay_run_1_ms": resident, "with_push_fetch_ms": copying}
    st.end()
    st.close()

    # 2-D space (dims 2): 1M agents on a 2000 x 2000 plane, radius 5
    ps = W.basic_points(1 << 20, seed=310, side=2000.0)
    ps.p[:, 2] = 0.0
    rec2 = M.records(M.TEST_RECORD, ps.p, ps.v)
    s2 = M.test_setup(radius=5.0, part=5.0, passes=("agent_see", "agent_act"), mb=64)
    s2.passes[-1].ctx[4:7] = 2000.0
    s2.dims = 2
    st, g = M.make_state(s2, rec2)
    st.start()
    st.run(3)
    st.run(steps)
    dev = st.L.tay_get_device_ms_for_last_run(st.ptr) / steps
    out["dims2"] = {"agents": 1 << 20, "ms_per_step": dev, "pair_interactions_per_s": st.pairs() / steps / (dev / 1000.0)}
    st.end()
    st.close()

    # fixed space box around the test model's walls
    ps = W.basic_points(1 << 20, seed=311, side=1000.0)
    rec3 = M.records(M.TEST_RECORD, ps.p, ps.v)
    s3 = M.test_setup(radius=10.0, part=10.0, mb=128)
    s3.fixed_box = ((0.0, 0.0, 0.0), (1000.0, 1000.0, 1000.0))
    st, g = M.make_state(s3, rec3)
    st.start()
    st.run(3)
    st.run(steps)
    dev = st.L.tay_get_device_ms_for_last_run(st.ptr) / steps
    out["fixed_box"] = {"agents": 1 << 20, "ms_per_step": dev,
                        "pair_interactions_per_s": st.pairs() / steps / (dev / 1000.0)}
    st.end()
    st.close()

    # non-point agents: 524,288 cubes of edge 1..5 in [0, 500]^3, radius 5
    bx = W.box_agents(1 << 19, seed=312, side=500.0, min_size=1.0, max_size=5.0)
    rec4 = M.box_records(bx.lo, bx.hi, bx.v)
    s4 = M.box_setup(radius=5.0, part=5.0, mb=64)
    s4.passes[-1].ctx[4:7] = 500.0
    st, g = M.make_state(s4, rec4)
    st.start()
    st.run(3)
    st.run(steps)
    dev = st.L.tay_get_device_ms_for_last_run(st.ptr) / steps
    out["box_agents"] = {"agents": 1 << 19, "ms_per_step": dev,
                         "pair_interactions_per_s": st.pairs() / steps / (dev / 1000.0)}
    st.end()
    st.close()
    api.set_tuning()
    return out


def cpu_baseline(setup, recs, steps):
    """Oracle restatement of the reference CpuZGrid step, all host threads, `steps` steps."""
    from oracle import pyoracle as O

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r = O.port().run(O.MODEL_BOIDS, "z_grid", recs, setup.passes[0].ctx, setup.passes[0].ctx, RADIUS, CELL, steps,
                     O.PASS_SEE0 | O.PASS_ACT0, threads=threads, mb=setup.mb)
    wall = time.perf_counter() - t0
    secs = r.ms_per_step * steps / 1000.0
    return {"value": r.pairs / secs, "unit": "pair-interactions/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full steps of the 1M-boid workload on CpuZGrid (oracle restatement, {threads} threads)",
            "ms_per_step": r.ms_per_step, "pairs_per_step": r.pairs / steps, "wall_s": round(wall, 2)}


def cpu_sample_steps(args):
    """Steps of the CPU sample, the same in the reference arm and in the GPU arm's CPU
    baseline: the run's own step count, bounded by --cpu-steps."""
    return max(1, min(args.steps, args.cpu_steps))


def run_reference(args, rank, world):
    if rank != 0:
        return
    setup, recs = workload()
    # warm-up: each oracle run starts from the initial records, so these only warm the
    # host (threads, caches); the timed sample is the same as the GPU arm's CPU baseline
    warm = min(args.warmup, 3)
    for _ in range(warm):
        cpu_baseline(setup, recs, 1)
    steps = cpu_sample_steps(args)
    cb = cpu_baseline(setup, recs, steps)
    line = {"metric": "pair-interactions/s", "value": cb["value"], "unit": "pair-interactions/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warm, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64, 64 Gaussian clusters of boids)", "config": bench_config(world),
            "impl": "reference", "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "pair-interactions/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference's own build (oracle/_ref) needs its source tree, absent on the GPU box; "
                    "the oracle restatement, bit-exact with it in tests, is timed instead"}
    print(json.dumps(line), flush=True)


def run_gb300(args, rank, world, D):
    from tay_gb300 import api
    from tay_gb300 import models as M

    first = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0].strip()
    gpu_index = int(first) if first.isdigit() else 0  # physical index for the clock sampler
    setup, recs = workload()
    from tay_gb300 import autotune

    api.set_tuning()  # library defaults, then the autotuner's choice or command-line overrides
    over = {k: v for k, v in (("stage", args.stage), ("union_factor", args.union_factor),
                              ("cell_multiple", args.cell_multiple), ("cell_order", args.cell_order),
                              ("hit_masks", args.hit_masks), ("x_cell_factor", args.x_cell_factor)) if v is not None}
    tuned = None
    if over:
        api.set_tuning(**over)
    elif not args.no_autotune:
        tuned = autotune.autotune([(setup, recs)], use_cache=False, evolve_steps=args.warmup + args.steps)
    B = api.Batch([(setup, recs)])
    B.push()
    # the sampler runs from the warm-up through the e2e leg (the GPU busy throughout)
    clocks = Clocks(gpu_index)
    clocks.start()
    clocks.wait_first()
    for _ in range(args.warmup):
        B.flush_l2()
        B.run(1)

    D.barrier()
    dev_ms, pairs = 0.0, 0
    for _ in range(args.steps):
        B.flush_l2()
        ms, p = B.run(1)
        dev_ms += ms
        pairs += p
    D.barrier()
    B.run(1)
    tel = B.telemetry()
    # profiled leg: per-kernel-class device time, same flush protocol, no graphs
    prof_steps = min(args.steps, 20)
    prof = [0.0] * 8
    for _ in range(prof_steps):
        B.flush_l2()
        part = B.profile(1)
        prof = [a + b for a, b in zip(prof + [0.0] * (len(part) - len(prof)), part)]
    launches = B.launches_per_step() * args.steps
    B.close()

    # e2e through the C API with host buffers (push + step + fetch every step)
    st, g = M.make_state(setup, recs)
    st.start()
    for _ in range(max(3, args.warmup // 2)):  # the same loop as timed (its step graphs exist)
        st.mark_changed(g)
        st.run(1)
        st.agent_ptr(g, 0)
    e2e_steps = min(args.steps, 50)
    D.barrier()
    t0 = time.perf_counter()
    e2e_pairs = 0
    for _ in range(e2e_steps):
        st.mark_changed(g)   # the step's inputs are the host records: pushed (H2D)
        st.run(1)
        st.agent_ptr(g, 0)   # the step's result read back into the host records (D2H)
        e2e_pairs += st.pairs()
    e2e_s = time.perf_counter() - t0
    D.barrier()
    st.end()
    st.close()
    clk = clocks.stop()

    secs = D.max(dev_ms / 1000.0)
    all_pairs = D.sum(pairs)
    e2e_s = D.max(e2e_s)
    e2e_pairs = D.sum(e2e_pairs)

    peak, peak_kind = peaks()
    see_ms = prof[4] / prof_steps
    # algorithmic bytes of one fused see+act launch: every agent's seen fields (position
    # and velocity, 32 B) read once and its new position and velocity (32 B) written once
    see_bytes = N_BOIDS * 64
    achieved = see_bytes / (see_ms / 1000.0) / 1e9
    step_ms = sum(prof) / prof_steps
    # whole-step algorithmic bytes, counted as if see and act were separate passes (the
    # accumulators written and read back): per agent, key from position 16 B, key + index
    # write 8 B, reorder of the 36 B state read + write, see 32 B seen + 40 B accumulators,
    # act 2 x 36 B state + 40 B accumulators = 280 B
    step_bytes = N_BOIDS * (16 + 8 + 2 * 36 + (32 + 40) + (2 * 36 + 40))
    see_name = "see_rows_kernel<boids::SeeAct>" if api.get_tuning().get("cell_order") == 1 else "see_kernel<boids::SeeAct>"
    # instruction-issue floor of the see kernel: every lane of every scheduler busy (152 SMs
    # x 4 schedulers x 32 lanes per cycle at the sampled SM clock), 10 thread instructions
    # per candidate box-tested (load, three subtractions, three compares, self test, loop)
    # and 30 per pair that passed the box test (the see body with its distance test and
    # accumulates); candidates and pairs from the device counters of the last step
    sm_hz = 1e6 * (clk["sm_mhz"] or clk["sm_max_mhz"] or 2070.0)
    floor_ms = 1000.0 * (10.0 * tel["candidates"] + 30.0 * tel["pairs"]) / (152 * 4 * 32 * sm_hz)
    traffic = None
    tp = os.path.join(ROOT, "profiles", "see_boids_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        if tj.get("kernel", see_name) == see_name:
            traffic = tj.get("dram_bytes_per_launch")
    if rank == 0:
        line = {
            "metric": "pair-interactions/s", "value": all_pairs / secs, "unit": "pair-interactions/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64, 64 Gaussian clusters of boids)",
            "config": bench_config(world),
            "steps_per_s": args.steps / secs,
            "pairs_per_step": all_pairs / world / args.steps,
            "e2e": {"value": e2e_pairs / e2e_s, "unit": "pair-interactions/s",
                    "h2d_bytes_per_step": N_BOIDS * BOIDS_RECORD_BYTES,
                    "d2h_bytes_per_step": N_BOIDS * BOIDS_RECORD_BYTES, "steps": e2e_steps,
                    "ms_per_step": 1000.0 * e2e_s / e2e_steps},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": see_name, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": see_bytes, "launch_ms": see_ms},
            "issue_roofline": {"bound": "issue", "kernel": see_name, "floor_ms": floor_ms, "launch_ms": see_ms,
                               "frac": floor_ms / see_ms, "instructions_per_candidate": 10,
                               "instructions_per_pair": 30, "candidates": tel["candidates"], "pairs": tel["pairs"]},
            "step_roofline": {"achieved": step_bytes / (step_ms / 1000.0) / 1e9, "unit": "GB/s",
                              "frac": step_bytes / (step_ms / 1000.0) / 1e9 / peak,
                              "algorithmic_bytes_per_step": step_bytes, "profiled_step_ms": step_ms},
            "kernel_ms": {"box": prof[0] / prof_steps, "sort": prof[1] / prof_steps,
                          "cell_table_reorder": (prof[2] + prof[3]) / prof_steps,
                          "see_act": prof[4] / prof_steps},
            "clocks": clk,
            "tuning": api.get_tuning(),
            "autotune": None if tuned is None else {"trials": tuned["trials"], "ms_per_step": tuned["ms_per_step"]},
            "telemetry": tel,
        }
        cpu = not args.no_cpu_baseline and world == 1
        if args.c1:
            line["c1"] = c1_leg(cpu_steps=100 if cpu else 0)
        if args.batched_states > 0:
            line["batched"] = batched_vs_plain(args.batched_states, min(args.steps, 20), not args.no_autotune,
                                               cpu_steps=1 if cpu else 0)
        if args.sph:
            line["sph"] = sph_leg(min(args.steps, 20), not args.no_autotune, cpu_steps=2 if cpu else 0)
        if args.adjoint:
            tune = not args.no_autotune
            for i, keep in enumerate(int(k) for k in args.adjoint_keeps.split(",") if k.strip()):
                name = "adjoint_record_all" if keep == 0 else ("adjoint" if i == 0 else f"adjoint_keep{keep}")
                line[name] = adjoint_leg(steps=args.adjoint_steps, every=0 if keep == 0 else 20, keep=max(keep, 1),
                                         tune=tune, cpu_steps=2 if cpu and i == 0 else 0)
        if args.features:
            line["features"] = features_leg(setup, recs, line["tuning"])
        if cpu:
            line["cpu_baseline"] = cpu_baseline(setup, recs, cpu_sample_steps(args))
        # the benchmark spec's targets in one short object at the end of the line
        tg = {"step_ms": round(line["ms_per_step"], 4), "see_launch_ms": round(see_ms, 4),
              "see_issue_frac": round(floor_ms / see_ms, 3), "see_hbm_frac": round(achieved / peak, 4)}
        if "batched" in line:
            tg["batched_speedup"] = round(line["batched"]["speedup"], 2)
        for k in line:
            if k.startswith("adjoint"):
                tg[k + "_fwd_bwd_over_fwd"] = round(line[k]["fwd_plus_bwd_over_fwd"], 3)
        line["targets"] = tg
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        # one GPU per rank, chosen before anything initialises CUDA
        os.environ["CUDA_VISIBLE_DEVICES"] = rank_visible_device(local, os.environ.get("CUDA_VISIBLE_DEVICES"))
    D = Dist(world)
    try:
        run_gb300(args, rank, world, D)
    finally:
        D.close()


if __name__ == "__main__":
    main()
