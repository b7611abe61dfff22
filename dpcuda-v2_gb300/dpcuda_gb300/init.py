"""Seeded initial states in the reference's own random streams.

`random_uniform` reproduces the reference's RandomUniform functor
(include/functors.h:17-33): element i draws from thrust's default engine
(minstd, a = 48271, m = 2^31 - 1) seeded with seed + seed_offset + seed + i,
advanced by seed + seed_offset + i draws, and maps the next draw onto [lo, hi)
with uniform_real_distribution's (u - 1) / (m - 1) rule.  The jump-ahead is
vectorised: the engine's state after z steps is x * a^z mod m, and a^(2^b)
mod m is the same for every element, so one pass over the 32 bits of z
serves the whole array.

`disk_packing` is the bidisperse start of Disk::initializeFromConfig
(src/particles/disk/disk.cu:98-141): the first floor(n * count_ratio) disks
have diameter size_ratio, the rest diameter 1, in a square box at packing
fraction phi, positions from `random_uniform`.
"""
from __future__ import annotations

import numpy as np

_A = 48271
_M = 2147483647


def random_uniform(n: int, lo: float, hi: float, seed_offset: int, seed: int) -> np.ndarray:
    n = int(n)
    i = np.arange(n, dtype=np.uint64)
    k = (np.uint64(int(seed + seed_offset) & 0xFFFFFFFF) + i) & np.uint64(0xFFFFFFFF)
    s = (np.uint64(int(seed) & 0xFFFFFFFF) + k) & np.uint64(0xFFFFFFFF)
    x = s % np.uint64(_M)
    x[x == 0] = 1
    acc = np.ones(n, dtype=np.uint64)
    mul = _A
    for b in range(32):
        bit = ((k >> np.uint64(b)) & np.uint64(1)).astype(bool)
        acc[bit] = (acc[bit] * np.uint64(mul)) % np.uint64(_M)
        mul = (mul * mul) % _M
    st = (acc * x) % np.uint64(_M)
    st = (st * np.uint64(_A)) % np.uint64(_M)
    u = (st - np.uint64(1)).astype(np.float64)
    u /= (1.0 + float(_M - 2))
    return u * (hi - lo) + lo


def disk_packing(n: int, phi: float, seed: int, size_ratio: float = 1.4,
                 count_ratio: float = 0.5) -> dict:
    n = int(n)
    n_large = int(n * count_ratio)
    r = np.full(n, 0.5)
    r[:n_large] = size_ratio / 2.0
    a = 0.0
    for v in r.tolist():   # sequential sum, as the host computes the area
        a += v * v
    box = (a * np.pi / phi) ** 0.5
    x = random_uniform(n, 0.0, box, 0, seed)
    y = random_uniform(n, 0.0, box, n, seed)
    return dict(x=x, y=y, r=r, m=np.ones(n), box=box)


def bumpy_vertex_radius(min_diameter: float, n_vertices_small: int, seg: float) -> float:
    """Vertex radius of the reference's rigid bumpy bodies
    (src/particles/rigid_bumpy/rigid_bumpy.cu:570-610): adjacent vertices of
    the smallest body, on a circle of diameter min_diameter, sit seg vertex
    diameters apart."""
    ang = 2.0 * np.pi / n_vertices_small
    return min_diameter / (1.0 + seg / np.sin(ang / 2.0)) / 2.0


def bumpy_packing(n_bodies: int, phi: float, seed: int, n_small: int = 20, seg: float = 0.9,
                  size_ratio: float = 1.4, count_ratio: float = 0.5) -> dict:
    """Bidisperse rigid bumpy bodies (RigidBumpy::initializeFromConfig,
    src/particles/rigid_bumpy/rigid_bumpy.cu:138-230): body radii 0.5 and
    size_ratio / 2, n_small vertices on the small bodies and
    floor(n_small * size_ratio) on the large ones, one vertex radius from
    bumpy_vertex_radius, vertex energy scale (2 r_v / d_min)^2, box at packing
    fraction phi of the body discs, positions and angles from random_uniform
    (angles share the positions' x stream, as the reference's offsets do)."""
    n = int(n_bodies)
    n_large = int(n * count_ratio)
    r = np.full(n, 0.5)
    r[:n_large] = size_ratio / 2.0
    a = 0.0
    for v in r.tolist():
        a += v * v
    box = (a * np.pi / phi) ** 0.5
    x = random_uniform(n, 0.0, box, 0, seed)
    y = random_uniform(n, 0.0, box, n, seed)
    th = random_uniform(n, 0.0, 2 * np.pi, 0, seed)
    n_lg = int(n_small * size_ratio)
    nvb = np.where(r == size_ratio / 2.0, n_lg, n_small).astype(np.int64)
    rv = bumpy_vertex_radius(1.0, n_small, seg)
    e_c = (2.0 * rv / 1.0) ** 2
    return dict(x=x, y=y, th=th, r=r, nvb=nvb, nv=int(nvb.sum()), box=box, rv=rv, e_c=e_c, seg=seg)
