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

    def solve(self, flags, rhs, *, warm: int = N.WARM_ZERO, tol: float | None = None, backoff: bool = False,
              precond: int = N.PRECOND_MG):
        p = N.default_params(resolution=self.n, tol=self.tol if tol is None else tol, tol_mode=N.TOL_REL_L2,
                             max_iters=4000, warm_start=warm, timing=True, learned_backoff=backoff, precond=precond)
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


def pool_from_arrays(xs, ts, ms, device: str = "cuda"):
    """A resident training pool (types uint8, scaled rhs, scaled target) from
    network inputs [count, d, h, w, 4], targets and fluid masks."""
    import torch

    types = np.where(ms > 0, 0, np.where(xs[..., 2] > 0, 2, 1)).astype(np.uint8)
    rhs = np.where(ms > 0, xs[..., 0], 0.0).astype(np.float32)
    return (torch.from_numpy(types).to(device), torch.from_numpy(rhs).to(device),
            torch.from_numpy(np.ascontiguousarray(ts, np.float32)).to(device))


def train_pool(net: N.WarmStartNet, pool, *, iters: int, batch: int, lr: float = 1e-3, seed: int = 0,
               report_every: int = 0, log=print):
    """Adam on random mini-batches of a resident pool (fsim_net_train_batch: the
    library gathers each batch on the device; the host never waits inside the
    loop).  Returns the loss history (one value per iteration)."""
    import torch

    types, rhs, target = pool
    count = types.shape[0]
    gen = np.random.default_rng(seed)
    idx = np.stack([gen.choice(count, size=batch, replace=count < batch) for _ in range(iters)]).astype(np.int32)
    idx_d = torch.from_numpy(idx).to(types.device)
    losses = torch.zeros(iters, dtype=torch.float32, device=types.device)
    for it in range(iters):
        net.train_batch(types, rhs, target, idx_d[it], lr, losses[it:it + 1])
        if report_every and (it + 1) % report_every == 0:
            net.synchronize()
            log(f"iter {it + 1} loss {float(losses[it - report_every + 1:it + 1].mean()):.4f}")
    net.synchronize()
    return losses.cpu().numpy().tolist()


def train(net: N.WarmStartNet, xs, ts, ms, *, iters: int, batch: int, lr: float = 1e-3, seed: int = 0,
          device: str = "cuda", log_every: int = 0):
    """Adam on random mini-batches of (inputs, targets, masks) arrays, moved to
    the GPU once; returns the loss history."""
    return train_pool(net, pool_from_arrays(xs, ts, ms, device), iters=iters, batch=batch, lr=lr, seed=seed,
                      report_every=log_every)


# ---------------------------------------------------------------- training protocol
# The learned warm start's training protocol: 20k (rhs, pressure) pairs on 64^3
# volumes from dam-break runs (the 32^3 FLIP run embedded in a 64^3 solid box;
# 64^3 windows of the 128^3 PIC / FLIP / APIC runs) and from random masks with
# the statistics of the precision study (Gaussian-filtered N(0, 1) noise,
# sigma 6 cells, thresholded to 40-70 % fluid, solid walls; rhs the divergence
# of an N(0, 1) face-velocity field smoothed with sigma 3 cells); batch 8, 20k
# Adam iterations at lr 1e-3; loss = relative residual + 0.1 relative L2 error.
PROTO_N = 64


def _smooth_batch(a: np.ndarray, sigma: float, threads: int = -1) -> np.ndarray:
    """Periodic Gaussian filter over the last three axes of a float32 batch
    (scipy's threaded FFT when available, else numpy)."""
    try:
        import scipy.fft as sf

        fwd = lambda x: sf.rfftn(x, axes=(1, 2, 3), workers=threads)  # noqa: E731
        inv = lambda x, shp: sf.irfftn(x, s=shp, axes=(1, 2, 3), workers=threads)  # noqa: E731
    except ImportError:
        fwd = lambda x: np.fft.rfftn(x, axes=(1, 2, 3))  # noqa: E731
        inv = lambda x, shp: np.fft.irfftn(x, s=shp, axes=(1, 2, 3))  # noqa: E731
    shp = a.shape[1:]
    f = fwd(a)
    for ax, n in enumerate(shp):
        k = np.fft.rfftfreq(n) if ax == 2 else np.fft.fftfreq(n)
        g = np.exp(-2.0 * (math.pi * sigma * k) ** 2).astype(np.float32)
        sh = [1, 1, 1, 1]
        sh[ax + 1] = k.size
        f = f * g.reshape(sh)
    return inv(f, shp).astype(np.float32)


def mask_problems(n: int, count: int, seed: int, threads: int = -1):
    """count random-mask problems on n^3: (flags uint8 [count, n, n, n], rhs float32).
    Mask: N(0, 1) noise filtered with sigma = 6 cells, fluid where it is below
    the quantile of a fluid fraction drawn from [0.4, 0.7]; the border is solid.
    rhs: -div of an N(0, 1) face field, smoothed with sigma = 3 cells (the
    filter commutes with the difference operator), on fluid cells only."""
    rng = np.random.default_rng(seed)
    noise = _smooth_batch(rng.standard_normal((count, n, n, n), dtype=np.float32), 6.0, threads)
    frac = rng.uniform(0.4, 0.7, count)
    flags = np.full((count, n, n, n), N.AIR, np.uint8)
    for i in range(count):
        k = int(frac[i] * (n ** 3 - 1))
        thr = np.partition(noise[i].ravel(), k)[k]
        flags[i][noise[i] < thr] = N.WATER
    flags[:, 0] = flags[:, -1] = N.SOLID
    flags[:, :, 0] = flags[:, :, -1] = N.SOLID
    flags[:, :, :, 0] = flags[:, :, :, -1] = N.SOLID
    rhs = np.where(flags == N.WATER, random_divergence(rng, count, n, threads), 0.0).astype(np.float32)
    return flags, rhs


def random_divergence(rng, count: int, n: int, threads: int = -1) -> np.ndarray:
    """-div of an N(0, 1) face-velocity field smoothed with sigma = 3 cells,
    [count, n, n, n] float32 (the smoothing is applied to the divergence of the
    white-noise field: the filter commutes with the difference operator)."""
    ux = rng.standard_normal((count, n + 1, n, n), dtype=np.float32)
    uy = rng.standard_normal((count, n, n + 1, n), dtype=np.float32)
    uz = rng.standard_normal((count, n, n, n + 1), dtype=np.float32)
    div = (ux[:, 1:] - ux[:, :-1]) + (uy[:, :, 1:] - uy[:, :, :-1]) + (uz[:, :, :, 1:] - uz[:, :, :, :-1])
    return -_smooth_batch(div, 3.0, threads)


def crop_problem(flags: np.ndarray, rhs: np.ndarray, origin, n: int = PROTO_N):
    """An n^3 window of a larger problem as a well-posed problem of its own:
    cells outside the source grid are solid; on the window's faces, solid
    cells stay solid and every other cell becomes air (the cut fluid meets a
    free surface there), so no fluid region is left without a Dirichlet
    boundary."""
    fl = np.full((n, n, n), N.SOLID, np.uint8)
    b = np.zeros((n, n, n))
    src = [slice(max(o, 0), min(o + n, s)) for o, s in zip(origin, flags.shape)]
    dst = [slice(sl.start - o, sl.stop - o) for sl, o in zip(src, origin)]
    fl[tuple(dst)] = flags[tuple(src)]
    b[tuple(dst)] = rhs[tuple(src)]
    for ax in range(3):
        for idx in (0, n - 1):
            face = [slice(None)] * 3
            face[ax] = idx
            f = fl[tuple(face)]
            f[f != N.SOLID] = N.AIR
    b[fl != N.WATER] = 0.0
    return fl, b


def dam_snapshots(res: int, transfer: int, dt: float, steps: int, every: int):
    """(flags, rhs) of a dam-break run every `every` steps: the problems its
    solver saw (the rhs taken as the right-hand side of a problem in the
    solver's integer-stencil units; its overall scale does not matter, the
    network sees it divided by its RMS)."""
    from .scenes import GridSpec, dam_break

    p = N.default_params(transfer=transfer, resolution=res, tol=1e-6, max_iters=200)
    sim = N.Simulation(res, p)
    sim.set_particles(dam_break(GridSpec(res), seed=0))
    out = []
    for s in range(steps):
        sim.step(dt)
        if s % every == every - 1:
            out.append((sim.grid(N.F_FLAGS), sim.grid(N.F_DIVERGENCE).astype(np.float64)))
    sim.close()
    return out


def protocol_problems(total: int = 20000, seed: int = 5, log=print):
    """Generator of the training problems (flags, rhs) on 64^3, in blocks."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os

    n = PROTO_N
    made = 0
    # config 1: 32^3 FLIP dam break, dt 1/120, 100 steps, every step, embedded in a 64^3 solid box
    blocks = []
    for fl, b in dam_snapshots(32, N.FLIP, 1.0 / 120.0, 100, 1):
        f64 = np.full((n, n, n), N.SOLID, np.uint8)
        b64 = np.zeros((n, n, n))
        f64[16:48, 16:48, 16:48] = fl
        b64[16:48, 16:48, 16:48] = b
        blocks.append((f64, b64))
    yield blocks
    made += len(blocks)
    log(f"config-1 snapshots: {len(blocks)}")
    # config 2: 128^3 dam break, PIC / FLIP / APIC, dt 1/240, 200 steps: the 8 octants every 4th step
    for transfer in (N.PIC, N.FLIP, N.APIC):
        blocks = []
        for fl, b in dam_snapshots(128, transfer, 1.0 / 240.0, 200, 4):
            for o in range(8):
                org = (64 * (o >> 2), 64 * ((o >> 1) & 1), 64 * (o & 1))
                cf_, cb_ = crop_problem(fl, b, org)
                if (cf_ == N.WATER).sum() >= 1000:
                    blocks.append((cf_, cb_))
        yield blocks
        made += len(blocks)
        log(f"config-2 windows (transfer {transfer}): {len(blocks)}")
    # random masks for the rest, synthesised on the host cores by a process
    # pool (spawned: this process already uses the GPU) while the GPU solves
    # the previous blocks
    block = 64
    nblocks = (max(total - made, 0) + block - 1) // block
    workers = max(1, min(8, (os.cpu_count() or 2) - 1))
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        futs = [ex.submit(mask_problems, n, block, seed * 1000003 + k, 1) for k in range(min(nblocks, 2 * workers))]
        for k in range(nblocks):
            fl, b = futs[k].result()
            futs[k] = None
            if k + 2 * workers < nblocks:
                futs.append(ex.submit(mask_problems, n, block, seed * 1000003 + k + 2 * workers, 1))
            cnt = min(block, total - made)
            yield [(fl[i], b[i].astype(np.float64)) for i in range(cnt)]
            made += cnt
            if made >= total:
                break


def build_pool(total: int = 20000, seed: int = 5, tol: float = 1e-8, log=print):
    """Solve every training problem with the plain solver (multigrid PCG to
    relative residual `tol`) and keep the pool on the GPU: types, rhs / rms,
    pressure / rms ([total, 64, 64, 64] each).  Returns (pool, info)."""
    import time

    import torch

    n = PROTO_N
    types = torch.empty((total, n, n, n), dtype=torch.uint8, device="cuda")
    rhs = torch.empty((total, n, n, n), dtype=torch.float32, device="cuda")
    target = torch.empty((total, n, n, n), dtype=torch.float32, device="cuda")
    solver = ProblemSolver(n, tol=tol)
    t0 = time.time()
    i = 0
    iters = []
    skipped = 0
    sources = {}
    for block in protocol_problems(total, seed, log):
        for flags, b in block:
            if i >= total:
                break
            p, st = solver.solve(flags, b)
            if not st.converged:
                skipped += 1
                continue
            x, rms = net_input(flags, b)
            fl = x[..., 1] > 0
            types[i] = torch.from_numpy(np.where(fl, 0, np.where(flags == N.SOLID, 2, 1)).astype(np.uint8))
            rhs[i] = torch.from_numpy(x[..., 0])
            target[i] = torch.from_numpy(np.where(fl, p / rms, 0.0).astype(np.float32))
            iters.append(st.pcg_iterations)
            i += 1
        if i and i % 2000 < len(block):
            log(f"pool: {i} problems solved, {time.time() - t0:.0f} s")
    solver.sim.close()
    info = {"problems": i, "skipped_not_converged": skipped, "grid": [n, n, n], "solver_tol": tol,
            "solver_iterations_mean": round(float(np.mean(iters)), 2), "seconds": round(time.time() - t0, 1)}
    return (types[:i], rhs[:i], target[:i]), info


def save_params(net: N.WarmStartNet, path: str, meta: dict):
    import json

    np.savez_compressed(path, theta=net.params(), out_scale=np.float32(net.out_scale),
                        meta=np.array(json.dumps(meta)))


def load_net(path: str) -> N.WarmStartNet:
    z = np.load(path)
    net = N.WarmStartNet(seed=1, out_scale=float(z["out_scale"]))
    net.set_params(z["theta"])
    return net


def run_protocol(out: str, total: int = 20000, iters: int = 20000, batch: int = 8, lr: float = 1e-3,
                 seed: int = 5, log=print):
    """The whole training protocol on the GPU; saves the parameters to `out`."""
    import time

    pool, info = build_pool(total, seed, log=log)
    log(f"pool: {info}")
    types, _, tgt = pool
    v = tgt[types == 0]
    sc = float((v * v).mean().sqrt()) if v.numel() else 1.0
    net = N.WarmStartNet(seed=1, out_scale=sc)
    t0 = time.time()
    hist = train_pool(net, pool, iters=iters, batch=batch, lr=lr, seed=seed, report_every=1000, log=log)
    train_s = time.time() - t0
    meta = {"pool": info, "iters": iters, "batch": batch, "lr": lr, "loss": "relative residual + 0.1 relative L2",
            "out_scale": sc, "loss_first_100": float(np.mean(hist[:100])),
            "loss_last_100": float(np.mean(hist[-100:])), "train_seconds": round(train_s, 1),
            "loss_curve_every_500": [round(float(np.mean(hist[k:k + 500])), 4) for k in range(0, iters, 500)]}
    save_params(net, out, meta)
    net.close()
    return meta


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
    pr = sub.add_parser("protocol", help="build the training pool, train, save the parameters")
    pr.add_argument("--out", required=True)
    pr.add_argument("--problems", type=int, default=20000)
    pr.add_argument("--iters", type=int, default=20000)
    pr.add_argument("--batch", type=int, default=8)
    pr.add_argument("--lr", type=float, default=1e-3)
    a = ap.parse_args()
    if a.cmd == "protocol":
        import json

        def log(msg):
            print(msg, flush=True)

        meta = run_protocol(a.out, a.problems, a.iters, a.batch, a.lr, log=log)
        print(json.dumps(meta), flush=True)
    if a.cmd == "forward":
        t = time_forward(a.size, a.iters)
        print(f"forward {a.size}^3 ms: " + " ".join(f"{v:.3f}" for v in t), flush=True)
