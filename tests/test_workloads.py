"""Seeded workload generators: SplitMix64 known answers and the workload shapes."""
import numpy as np

from tay_gb300 import workloads as W


def test_splitmix64_known_answers():
    # SplitMix64 from state 0 (Steele, Lea, Flood 2014): published first outputs
    z = W.splitmix64(0, 3)
    assert [int(x) for x in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_streams_are_reproducible_and_offsettable():
    a = W.splitmix64(7, 10)
    b = W.splitmix64(7, 5, offset=5)
    assert np.array_equal(a[5:], b)
    s = W.Stream(3)
    u = s.uniform(1000)
    assert u.min() >= 0.0 and u.max() < 1.0


def test_workload_shapes():
    ps = W.basic_points(1000, seed=1)
    assert ps.p.shape == (1000, 4) and ps.p.dtype == np.float32
    assert ps.p[:, :3].min() >= 0 and ps.p[:, :3].max() <= 1000
    assert np.all(np.abs(ps.v[:, :3]) <= 1.0)
    b = W.boids_points(4096, seed=2)
    speed = np.linalg.norm(b.v[:, :3], axis=1)
    assert speed.min() >= 0.999 and speed.max() <= 2.001
    s = W.sph_dam(64, 128, 64)
    assert s.points.n == 524288
    assert s.points.p[:, :3].max() < 1.29 and s.points.p[:, :3].min() > 0.0
    bb = W.batched_boids(states=16, seed=4)
    ns = [st[0].n for st in bb.states]
    assert min(ns) >= 1000 and max(ns) <= 65536
    assert all(5.0 <= st[1] <= 20.0 for st in bb.states)
