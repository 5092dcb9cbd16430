"""Seeded synthetic scenes (particle initial states) used by the tests and the
benchmark.

Random numbers come from SplitMix64 (G. L. Steele, D. Lea, C. H. Flood, "Fast
splittable pseudorandom number generators", OOPSLA 2014) used as a counter-based
generator: draw ``i`` of stream ``seed`` is ``mix64(seed * 2**32 + i + 1) *
golden-ratio increment``; the same function is implemented on the device for
particle spawning (``csrc/fsim_common.cuh``), so host and device draws agree.

Dam-break seeding rule: fluid cells are the interior (non-wall) cells whose
centre lies in the block; every fluid cell gets 8 particles, one per 2x2x2
sub-cell, at the sub-cell centre plus a uniform jitter of up to +-0.5 sub-cell
width (scaled by 0.999 so a jittered particle never leaves its sub-cell after
rounding to FP32).  Velocities and APIC matrices start at zero.  Positions are
generated in FP64 and returned as FP32, which is what both the CUDA path and the
oracles (promoted back to FP64) receive.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(counter: np.ndarray) -> np.ndarray:
    """SplitMix64 output for the given 64-bit counters (vectorised, wraps mod 2**64)."""
    with np.errstate(over="ignore"):
        z = counter.astype(np.uint64) * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, start: int, count: int) -> np.ndarray:
    """``count`` doubles in [0, 1) from stream ``seed`` starting at draw ``start``."""
    ctr = (np.uint64(seed) << np.uint64(32)) + np.arange(start + 1, start + count + 1, dtype=np.uint64)
    bits = splitmix64(ctr) >> np.uint64(11)
    return bits.astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class GridSpec:
    """A MAC grid over [0, dims] with ``resolution`` cells per unit length
    (MacGrid ctor semantics, macGrid.cpp:9-13)."""

    resolution: float
    dims: tuple = (1.0, 1.0, 1.0)
    two_d: bool = False  # 2D mode: z is 3 cells of dims[2] / 3

    @property
    def h(self) -> float:
        return 1.0 / float(np.float32(self.resolution))

    @property
    def hz(self) -> float:
        return self.dims[2] / 3 if self.two_d else self.h

    @property
    def shape(self) -> tuple:
        h = self.h
        return (int(self.dims[0] / h), int(self.dims[1] / h), 3 if self.two_d else int(self.dims[2] / h))


def dam_break(grid: GridSpec, block_lo=(0.0, 0.0, 0.0), block_hi=(0.4, 0.6, 1.0), seed: int = 0,
              jitter: bool = True) -> np.ndarray:
    """FP32 particle positions (n, 3) for a dam-break block, 8 per fluid cell."""
    h = grid.h
    nx, ny, nz = grid.shape
    axes = []
    for a, n in enumerate((nx, ny, nz)):
        idx = np.arange(1, n - 1)
        centre = (idx + 0.5) * h
        axes.append(idx[(centre >= block_lo[a]) & (centre <= block_hi[a])])
    ix, iy, iz = np.meshgrid(*axes, indexing="ij")
    cells = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    sub = np.array([[sx, sy, sz] for sx in (0.25, 0.75) for sy in (0.25, 0.75) for sz in (0.25, 0.75)])
    pos = (cells[:, None, :] + sub[None, :, :]).reshape(-1, 3)
    if jitter:
        u = uniform01(seed, 0, pos.size).reshape(-1, 3)
        pos = pos + (u - 0.5) * 0.5 * 0.999
    return (pos * h).astype(np.float32)


def dam_break_2d(grid: GridSpec, block_lo=(0.0, 0.0), block_hi=(0.4, 0.6), seed: int = 0) -> np.ndarray:
    """FP32 positions (n, 3) for a 2D-mode dam break: interior cells of the x-y
    plane whose centre lies in the block, 4 particles per cell (2x2 sub-cells,
    +-0.5 sub-cell jitter), all at z = dims[2] / 2 (HashedParticles' zConst
    plane, simulationManager.cpp:27)."""
    assert grid.two_d
    h = grid.h
    nx, ny, _ = grid.shape
    axes = []
    for a, n in enumerate((nx, ny)):
        idx = np.arange(1, n - 1)
        centre = (idx + 0.5) * h
        axes.append(idx[(centre >= block_lo[a]) & (centre <= block_hi[a])])
    ix, iy = np.meshgrid(*axes, indexing="ij")
    cells = np.stack([ix.ravel(), iy.ravel()], axis=1).astype(np.float64)
    sub = np.array([[sx, sy] for sx in (0.25, 0.75) for sy in (0.25, 0.75)])
    xy = (cells[:, None, :] + sub[None, :, :]).reshape(-1, 2)
    u = uniform01(seed, 0, xy.size).reshape(-1, 2)
    xy = (xy + (u - 0.5) * 0.5 * 0.999) * h
    z = np.full((xy.shape[0], 1), grid.dims[2] / 2)
    return np.concatenate([xy, z], axis=1).astype(np.float32)


def fill_below(grid: GridSpec, y_top: float, seed: int = 0) -> np.ndarray:
    """All interior cells with centre below ``y_top`` (the 256^3 APIC scene)."""
    return dam_break(grid, (0.0, 0.0, 0.0), (grid.dims[0], y_top, grid.dims[2]), seed=seed)


@dataclass
class Scene:
    name: str
    grid: GridSpec
    transfer: int
    dt: float
    steps: int
    flip_ratio: float = 0.95
    gravity: float = -9.81
    block_lo: tuple = (0.0, 0.0, 0.0)
    block_hi: tuple = (0.4, 0.6, 1.0)
    seed: int = 0
    max_iters: int = 200
    tol: float = 1e-6
    notes: str = ""
    extras: dict = field(default_factory=dict)

    def positions(self) -> np.ndarray:
        return dam_break(self.grid, self.block_lo, self.block_hi, self.seed)

    @property
    def particle_r(self) -> float:
        return self.grid.h / 4.0


PIC, FLIP, APIC = 0, 1, 2

# The workloads the benchmark and the parity tests are defined on.
SCENES = {
    "dam32_flip": Scene("dam32_flip", GridSpec(32), FLIP, 1.0 / 120.0, 100),
    "dam128_pic": Scene("dam128_pic", GridSpec(128), PIC, 1.0 / 240.0, 200),
    "dam128_flip": Scene("dam128_flip", GridSpec(128), FLIP, 1.0 / 240.0, 200),
    "dam128_apic": Scene("dam128_apic", GridSpec(128), APIC, 1.0 / 240.0, 200),
    "fill256_apic": Scene("fill256_apic", GridSpec(256), APIC, 1.0 / 480.0, 500,
                          block_hi=(1.0, 0.5, 1.0), max_iters=2000),
}


def moving_sphere_x(t: float, base=(0.5, 0.6, 0.5), amp: float = 0.1) -> tuple:
    """Sphere centre of the 256^3 scene: x = 0.5 + 0.1 sin(pi t)."""
    return (base[0] + amp * math.sin(math.pi * t), base[1], base[2])
