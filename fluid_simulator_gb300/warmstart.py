"""Training data and training loop of the learned pressure warm start.

The network (fsim_net_* in include/fsim.h, kernels in csrc/k_conv.cu and
csrc/k_net.cu) maps a pressure problem -- the solver's right-hand side scaled
by its RMS over fluid cells, plus one-hot fluid / solid / air cell types -- to
a pressure guess.  Its training pairs come from the plain solver: each problem
(cell types + rhs) is solved by the library's own PCG to a tight tolerance, and
the solution is the target.  Training runs entirely on the GPU through the
library's forward / backward kernels and Adam.

Problems are synthetic and seeded: a pool whose surface height varies smoothly
over (x, z), floating blobs, solid spheres inside, solid walls; the rhs is the
discrete divergence of a Gaussian-smoothed N(0, 1) face-velocity field,
restricted to fluid cells.  Units are the solver's integer-stencil units
(dt = rho h^2 makes the scale dt / (rho h^2) equal to one).
"""
from __future__ import annotations

import math

import numpy as np

from . import native as N


def _smooth(a: np.ndarray, sigma: float) -> np.ndarray:
    """Periodic Gaussian filter through the FFT (no scipy needed)."""
    out = np.fft.fftn(a)
    for ax, n in enumerate(a.shape):
        k = np.fft.fftfreq(n)
        g = np.exp(-2.0 * (math.pi * sigma * k) ** 2)
        shape = [1] * a.ndim
        shape[ax] = n
        out = out * g.reshape(shape)
    return np.real(np.fft.ifftn(out))


def make_problem(n: int, seed: int):
    """One synthetic pressure problem on an n^3 grid: (flags uint8, rhs float64)."""
    rng = np.random.default_rng(seed)
    x, y, z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    hgt = _smooth(rng.standard_normal((n, n)), n / 8)
    hgt = (hgt - hgt.min()) / max(hgt.max() - hgt.min(), 1e-9)
    level = rng.uniform(0.25, 0.6) + 0.25 * (hgt - 0.5)
    fluid = y < (level[:, None, :] * n)
    blobs = _smooth(rng.standard_normal((n, n, n)), max(n / 16, 1.5))
    fluid |= blobs > np.quantile(blobs, 0.97)
    solid = np.zeros((n, n, n), bool)
    for _ in range(rng.integers(0, 3)):
        c = rng.uniform(0.2, 0.8, 3) * n
        r = rng.uniform(0.05, 0.15) * n
        solid |= (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 < r * r
    border = (x == 0) | (y == 0) | (z == 0) | (x == n - 1) | (y == n - 1) | (z == n - 1)
    solid |= border
    flags = np.full((n, n, n), N.AIR, np.uint8)
    flags[fluid] = N.WATER
    flags[solid] = N.SOLID
    sig = 3.0
    u = [_smooth(rng.standard_normal((n + 1, n, n)), sig),
         _smooth(rng.standard_normal((n, n + 1, n)), sig),
         _smooth(rng.standard_normal((n, n, n + 1)), sig)]
    div = (u[0][1:] - u[0][:-1]) + (u[1][:, 1:] - u[1][:, :-1]) + (u[2][:, :, 1:] - u[2][:, :, :-1])
    rhs = np.where(flags == N.WATER, -div, 0.0)
    return flags, rhs


def solver_fluid(flags: np.ndarray) -> np.ndarray:
    """Cells the pressure solver treats as unknowns (water, not on the border)."""
    f = flags == N.WATER
    f[0, :, :] = f[-1, :, :] = False
    f[:, 0, :] = f[:, -1, :] = False
    f[:, :, 0] = f[:, :, -1] = False
    return f


def net_input(flags: np.ndarray, rhs: np.ndarray):
    """Network input [d, h, w, 4] and the rhs RMS it was scaled by."""
    fl = solver_fluid(flags)
    b = np.where(fl, rhs, 0.0)
    cnt = max(int(fl.sum()), 1)
    rms = math.sqrt(float((b * b).sum()) / cnt) or 1.0
    x = np.zeros(flags.shape + (4,), np.float32)
    x[..., 0] = b / rms
    x[..., 1] = fl
    x[..., 2] = flags == N.SOLID
    x[..., 3] = ~fl & (flags != N.SOLID)
    return x, rms


class ProblemSolver:
    """Solves problems with the library's plain PCG (FP64-accurate mixed precision)."""

    def __init__(self, n: int, tol: float = 1e-9):
        self.n = n
        self.tol = tol
        self.params = N.default_params(resolution=n, tol=tol, tol_mode=N.TOL_REL_L2, max_iters=4000)
        self.sim = N.Simulation(n, self.params)
        self.dt = 1.0 / float(n * n)  # rho h^2 with rho = 1, h = 1/n: scale 1

    def solve(self, flags, rhs, *, warm: int = N.WARM_ZERO, tol: float | None = None, backoff: bool = False):
        p = N.default_params(resolution=self.n, tol=self.tol if tol is None else tol, tol_mode=N.TOL_REL_L2,
                             max_iters=4000, warm_start=warm, timing=True, learned_backoff=backoff)
        self.sim.set_params(p)
        self.sim.set_grid(N.F_FLAGS, flags)
        self.sim.set_grid(N.F_PRESSURE, np.zeros(flags.shape, np.float32))
        return self.sim.solve_pressure(rhs, self.dt, tol_mode=N.TOL_REL_L2, tol=self.tol if tol is None else tol,
                                       max_iters=4000)


def make_dataset(n: int, count: int, seed: int = 0, solver: ProblemSolver | None = None):
    """count problems on n^3: inputs [count, n, n, n, 4], targets [count, n, n, n], masks."""
    solver = solver or ProblemSolver(n)
    xs = np.zeros((count, n, n, n, 4), np.float32)
    ts = np.zeros((count, n, n, n), np.float32)
    ms = np.zeros((count, n, n, n), np.uint8)
    for i in range(count):
        flags, rhs = make_problem(n, seed * 100003 + i)
        p, _ = solver.solve(flags, rhs)
        x, rms = net_input(flags, rhs)
        xs[i] = x
        ts[i] = np.where(x[..., 1] > 0, p / rms, 0.0)
        ms[i] = x[..., 1] > 0
    return xs, ts, ms


def scene_dataset(sim: N.Simulation, dt: float, steps: int, every: int, obstacles_fn=None):
    """(input, target, mask) pairs from a running simulation: every `every` steps
    the step's own solve (rhs = FSIM_F_DIVERGENCE, pressure = FSIM_F_PRESSURE,
    solved by the plain PCG to the simulation's tolerance) becomes one pair."""
    xs, ts, ms = [], [], []
    scale = dt / (sim.params.fluid_density * sim.h * sim.h)
    t = 0.0
    for s in range(steps):
        if obstacles_fn is not None:
            sim.set_obstacles(obstacles_fn(t))
        sim.step(dt)
        t += dt
        if s % every != every - 1:
            continue
        flags = sim.grid(N.F_FLAGS)
        b = sim.grid(N.F_DIVERGENCE).astype(np.float64)
        phi = sim.grid(N.F_PRESSURE).astype(np.float64)
        x, rms = net_input(flags, b)
        xs.append(x)
        ts.append(np.where(x[..., 1] > 0, phi * scale / rms, 0.0).astype(np.float32))
        ms.append((x[..., 1] > 0).astype(np.uint8))
    return np.stack(xs), np.stack(ts), np.stack(ms)


def target_scale(ts: np.ndarray, ms: np.ndarray) -> float:
    v = ts[ms > 0]
    return float(np.sqrt(np.mean(v * v))) if v.size else 1.0


def train(net: N.WarmStartNet, xs, ts, ms, *, iters: int, batch: int, lr: float = 1e-3, seed: int = 0,
          device: str = "cuda", log_every: int = 0):
    """Adam on random mini-batches, data resident on the GPU; returns the loss history."""
    import torch

    gen = np.random.default_rng(seed)
    X = torch.from_numpy(xs).to(device)
    T = torch.from_numpy(ts).to(device)
    M = torch.from_numpy(ms).to(device)
    hist = []
    for it in range(iters):
        idx = torch.from_numpy(gen.choice(xs.shape[0], size=batch, replace=False)).to(device)
        xb = X.index_select(0, idx).contiguous()
        tb = T.index_select(0, idx).contiguous()
        mb = M.index_select(0, idx).contiguous()
        torch.cuda.synchronize()
        loss = net.train_step(xb, tb, mb, lr)
        hist.append(loss)
        if log_every and it % log_every == 0:
            print(f"iter {it} loss {loss:.4e}", flush=True)
    return hist


def time_forward(size: int, iters: int = 5, seed: int = 1):
    """CUDA-event time of one network forward pass on a size^3 volume (random input)."""
    import torch

    net = N.WarmStartNet(seed=seed)
    x = torch.zeros((1, size, size, size, 4), device="cuda")
    x[..., 0] = torch.randn((1, size, size, size), device="cuda")
    x[..., 1] = 1.0
    net.forward(x)  # workspace allocation
    torch.cuda.synchronize()
    times = []
    for _ in range(iters):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        net.forward(x)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    net.close()
    return times


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description="warm-start network utilities")
    sub = ap.add_subparsers(dest="cmd", required=True)
    f = sub.add_parser("forward", help="time the forward pass")
    f.add_argument("--size", type=int, default=256)
    f.add_argument("--iters", type=int, default=5)
    a = ap.parse_args()
    if a.cmd == "forward":
        t = time_forward(a.size, a.iters)
        print(f"forward {a.size}^3 ms: " + " ".join(f"{v:.3f}" for v in t), flush=True)
