"""Seeded synthetic workloads for the Tay grid step.

Every generator draws from SplitMix64 (Steele, Lea, Flood 2014: state += 0x9E3779B97F4A7C15,
then two xor-shift-multiply rounds), one 64-bit draw per scalar, so the same seed produces
the same arrays on every machine.  A uniform float in [0, 1) is the top 24 bits of a draw
times 2^-24 (exact in float32).  Gaussians use Box-Muller in float64, rounded to float32.

Workloads (all FP32, 3-D point agents):
  basic_points N agents uniform in [0, 1000]^3, velocities uniform in [-1, 1]^3.  The
               reference's own generator normalises velocities to unit length
               (test/test.c:172-203); this one keeps them un-normalised.
  boids_points 64 Gaussian clusters (sigma 40) with centres uniform in [0, 2000]^3;
               velocity = unit random direction * speed uniform in [1, 2].
  sph_dam      a nx*ny*nz lattice block (spacing dx) in the corner of a tank.
  batched_boids  S states, N_i log-uniform in [n_lo, n_hi], uniform in a cube of side
               (125 N_i)^(1/3), see radius per state uniform in [5, 20].
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_C1 = np.uint64(0xBF58476D1CE4E5B9)
_C2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """Draws `count` SplitMix64 outputs for stream `seed`, starting at draw `offset`."""
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + i * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _C1
        z = (z ^ (z >> np.uint64(27))) * _C2
        z = z ^ (z >> np.uint64(31))
    return z


class Stream:
    """Sequential SplitMix64 stream."""

    def __init__(self, seed: int):
        self.seed = int(seed)
        self.pos = 0

    def bits(self, count: int) -> np.ndarray:
        out = splitmix64(self.seed, count, self.pos)
        self.pos += count
        return out

    def uniform(self, count: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        """float64 values lo + (hi - lo) * u with u = top24(draw) * 2^-24."""
        u = (self.bits(count) >> np.uint64(40)).astype(np.float64) * (1.0 / (1 << 24))
        return lo + (hi - lo) * u

    def normal(self, count: int) -> np.ndarray:
        u1 = self.uniform(count)
        u2 = self.uniform(count)
        r = np.sqrt(-2.0 * np.log(1.0 - u1))
        return r * np.cos(2.0 * np.pi * u2)


@dataclass
class PointSet:
    """Positions and velocities as float32 [N, 4] arrays (w = 0)."""

    p: np.ndarray
    v: np.ndarray

    @property
    def n(self) -> int:
        return int(self.p.shape[0])


def _pack4(x: np.ndarray) -> np.ndarray:
    out = np.zeros((x.shape[0], 4), dtype=np.float32)
    out[:, :3] = x.astype(np.float32)
    return out


def basic_points(n: int = 100_000, seed: int = 1, side: float = 1000.0) -> PointSet:
    s = Stream(seed)
    p = s.uniform(3 * n, 0.0, side).reshape(n, 3)
    v = s.uniform(3 * n, -1.0, 1.0).reshape(n, 3)
    return PointSet(_pack4(p), _pack4(v))


def boids_points(n: int = 1 << 20, seed: int = 2, clusters: int = 64, sigma: float = 40.0,
                 side: float = 2000.0) -> PointSet:
    s = Stream(seed)
    centres = s.uniform(3 * clusters, 0.0, side).reshape(clusters, 3)
    owner = np.arange(n) % clusters
    p = centres[owner] + sigma * s.normal(3 * n).reshape(n, 3)
    d = s.normal(3 * n).reshape(n, 3)
    d /= np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-12)
    speed = s.uniform(n, 1.0, 2.0)
    return PointSet(_pack4(p), _pack4(d * speed[:, None]))


@dataclass
class BoxSet:
    lo: np.ndarray   # [N, 4] float32 min corners
    hi: np.ndarray   # [N, 4] float32 max corners
    v: np.ndarray    # [N, 4] float32 velocities


def box_agents(n: int = 10_000, seed: int = 3, side: float = 1000.0, min_size: float = 1.0,
               max_size: float = 50.0, speed: float = 1.0) -> BoxSet:
    """Cubes of edge U[min_size, max_size] placed inside [0, side]^3 with velocity of the given
    speed in a uniform random direction (the reference's non-point test population,
    test/test.c:133-170, with its sizes 1..50 and speed 1)."""
    s = Stream(seed)
    size = s.uniform(n, min_size, max_size)
    u = s.uniform(3 * n, 0.0, 1.0).reshape(n, 3)
    lo = u * (side - size[:, None])
    hi = lo + size[:, None]
    d = s.uniform(3 * n, -1.0, 1.0).reshape(n, 3)
    d *= speed / np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-12)
    return BoxSet(_pack4(lo), _pack4(hi), _pack4(d))


@dataclass
class SphSetup:
    points: PointSet
    tank_min: tuple
    tank_max: tuple
    dx: float


def sph_dam(nx: int = 64, ny: int = 128, nz: int = 64, dx: float = 0.01,
            tank=(2.0, 1.5, 0.8)) -> SphSetup:
    """Lattice block of nx*ny*nz particles at spacing dx, in the tank's x-min/y-min/z-min
    corner, offset half a spacing from the walls.  Velocities start at zero."""
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    p = (p + 0.5) * dx
    n = p.shape[0]
    return SphSetup(PointSet(_pack4(p), np.zeros((n, 4), np.float32)),
                    (0.0, 0.0, 0.0), tuple(float(t) for t in tank), dx)


@dataclass
class BatchedBoids:
    states: list  # list of (PointSet, radius, side)


def batched_boids(states: int = 512, seed: int = 4, n_lo: int = 1000, n_hi: int = 65536,
                  volume_per_agent: float = 125.0, r_lo: float = 5.0, r_hi: float = 20.0) -> BatchedBoids:
    s = Stream(seed)
    logn = s.uniform(states, math.log(n_lo), math.log(n_hi))
    radii = s.uniform(states, r_lo, r_hi)
    out = []
    for i in range(states):
        n = int(round(math.exp(logn[i])))
        side = (volume_per_agent * n) ** (1.0 / 3.0)
        p = s.uniform(3 * n, 0.0, side).reshape(n, 3)
        d = s.normal(3 * n).reshape(n, 3)
        d /= np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-12)
        speed = s.uniform(n, 1.0, 2.0)
        out.append((PointSet(_pack4(p), _pack4(d * speed[:, None])), float(np.float32(radii[i])), side))
    return BatchedBoids(out)
