"""Particle sources against the oracle (Simulator::spawnParticles,
simulator.cpp:106-125; SphericalParticleSource, obstacles.hpp:46-57).

The emission angles come from different generators (SplitMix64 on the GPU, the
C library's rand() in the reference), so particles are compared by the rules
they must satisfy, not one by one: the emitted count floor(rate dt + carried
fraction) and the carried fraction bit-exact step after step, every new
particle on the sphere of radius r_source + r_particle around the source,
moving along the outward normal at the source's speed, with C = 0.  The disc
source (an extension of the 256^3 workload, in the oracle too) emits 8
particles in every covered cell of its row: the cells it fills agree exactly."""
import numpy as np
import pytest

from fluid_simulator_gb300 import native as N
from fluid_simulator_gb300.scenes import GridSpec, dam_break
from oracle import oracle as O

from parity_util import make_pair

pytestmark = pytest.mark.gpu

DT = 1.0 / 120.0


def _sphere_rules(pos, vel, c, centre, radius, speed, name):
    d = pos.astype(np.float64) - np.asarray(centre)
    dist = np.linalg.norm(d, axis=1)
    assert np.abs(dist - radius).max() <= 2e-6, f"{name}: particles off the emission sphere"
    nrm = d / dist[:, None]
    v = vel.astype(np.float64)
    assert np.abs(np.linalg.norm(v, axis=1) - abs(speed)).max() <= 2e-6 * abs(speed), f"{name}: speed"
    assert np.abs(v - speed * nrm).max() <= 1e-5 * abs(speed), f"{name}: velocity not along the normal"
    assert not np.asarray(c).any(), f"{name}: new particles carry C"


def test_spherical_source_count_fraction_and_placement(gpu, port_lib):
    pos = dam_break(GridSpec(32), (0, 0, 0), (0.4, 0.3, 1.0), seed=1)
    g, o = make_pair(pos, 32, N.FLIP, spawning=True)
    centre, r_src, rate, speed = (0.6, 0.7, 0.45), 0.06, 1234.5, 0.8
    g.set_obstacles([N.obstacle(N.OBS_SOURCE, centre, r=r_src, spawn_rate=rate, spawn_speed=speed, frac=0.3)])
    o.set_obstacles([O.obstacle(O.OBS_SOURCE, centre, r=r_src, spawn_rate=rate, spawn_speed=speed, frac=0.3)])
    radius = r_src + g.params.particle_r
    frac = 0.3
    n_init = g.n
    for step in range(6):
        n0 = g.n
        g.stage(N.STAGE_SPAWN, DT)
        o.stage(O.STAGE_SPAWN, DT)
        want = int(rate * DT + frac)
        frac = rate * DT + frac - want
        assert g.n - n0 == want and o.n == g.n, f"step {step}: emitted {g.n - n0}, oracle {o.n - n0}, want {want}"
        assert g.obstacles()[0].last_spawn_fraction == o.obstacles()[0].last_spawn_fraction == frac
        gp, gv, gc = g.particles()
        op, ov, oc = o.particles()
        _sphere_rules(gp[n0:], gv[n0:], gc[n0:], centre, radius, speed, f"GPU step {step}")
        _sphere_rules(op[n0:], ov[n0:], oc[n0:], centre, radius, speed, f"oracle step {step}")
        # the particles that were there before any emission are untouched
        assert np.array_equal(gp[:n_init].astype(np.float64), op[:n_init])


def test_disc_source_fills_the_same_cells(gpu, port_lib):
    pos = dam_break(GridSpec(32), (0, 0, 0), (0.4, 0.3, 1.0), seed=2)
    g, o = make_pair(pos, 32, N.FLIP, spawning=True)
    h = 1.0 / 32
    g.set_obstacles([N.obstacle(N.OBS_DISC_SOURCE, (0.5, 0.95, 0.5), r=4 * h, spawn_speed=-1.0)])
    o.set_obstacles([O.obstacle(O.OBS_DISC_SOURCE, (0.5, 0.95, 0.5), r=4 * h, spawn_speed=-1.0)])
    for step in range(2):
        n0 = g.n
        g.stage(N.STAGE_SPAWN, DT)
        o.stage(O.STAGE_SPAWN, DT)
        assert g.n == o.n and g.n - n0 > 0
        gp, gv, _ = g.particles()
        op, ov, _ = o.particles()
        cells_g = np.floor(gp[n0:].astype(np.float64) / h).astype(int)
        cells_o = np.floor(op[n0:] / h).astype(int)
        ug, cg = np.unique(cells_g, axis=0, return_counts=True)
        uo, co = np.unique(cells_o, axis=0, return_counts=True)
        assert np.array_equal(ug, uo) and (cg == 8).all() and (co == 8).all()
        assert (ug[:, 1] == int(0.95 * 32)).all()
        assert np.array_equal(gv[n0:], np.tile(np.float32([0.0, -1.0, 0.0]), (g.n - n0, 1)))
