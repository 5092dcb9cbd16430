"""The headless fluid renderer (include/fsim_render.h) against the CPU
restatement of the reference's shaders (oracle/render_oracle.c).

The reference renders with OpenGL, which does not exist where these tests run,
so the oracle is pinned by analytic cases here (the depth of a sprite's front
point, an empty frame) instead of by reference images.  Tolerances: the sprite
depth buffer is bit-exact (the same FP32 operations, no FMA contraction on
either side, correctly rounded sqrt and division); the smoothed depth agrees
to 2e-6; thickness (atomic sums in any order) to 1e-5 relative on 99.9 % of
the pixels (the rest took the other kernel size at an integer boundary of the
shaders' int(extent * width)); the shaded frame, whose normals difference
neighbouring depths, to 2e-3 on 99.5 % of the pixels."""
import ctypes as C

import numpy as np
import pytest

from fluid_simulator_gb300 import native as N
from fluid_simulator_gb300.scenes import GridSpec, dam_break
from oracle import oracle as O

W, H = 161, 121


def scene_particles(seed=0, res=16):
    """Dam-break positions with a density per particle (a fifth of them spray)."""
    pos = dam_break(GridSpec(res), (0, 0, 0), (0.5, 0.6, 1.0), seed=seed)
    rng = np.random.default_rng(seed)
    dens = rng.uniform(0.0, 6.0, pos.shape[0]).astype(np.float32)
    vel = rng.uniform(0.0, 1.0, pos.shape[0]).astype(np.float32)
    return np.concatenate([pos, vel[:, None], dens[:, None]], axis=1).astype(np.float32)


def scene_camera(w=W, h=H):
    eye = (1.6, 1.1, 2.0)
    yaw, pitch = N.look_at_angles(eye, (0.4, 0.3, 0.5))
    return N.camera(eye, yaw, pitch, fov=40.0, aspect=w / h, near=0.05, far=20.0)


def test_oracle_single_sprite_front_depth():
    """A sprite straight ahead: the centre pixel holds the window depth of the
    sphere's front point, and the covered pixels form a disc."""
    n = 101
    cam = N.camera((0.0, 0.0, 0.0), -90.0, 0.0, fov=40.0, aspect=1.0, near=0.05, far=20.0)
    prm = N.default_render_params(particle_radius=0.05, spray_enabled=0, transparency_enabled=0, noise_enabled=0)
    D = 2.0
    pts = np.array([[0.0, 0.0, -D, 0.0, 3.0]], np.float32)
    out = O.render_frame(pts, cam, prm, n, n)
    raw = out["raw_depth"]
    P = np.array(cam.proj, np.float64).reshape(4, 4).T  # column-major storage
    z = -D + 0.05
    clip = P @ np.array([0.0, 0.0, z, 1.0])
    assert abs(raw[n // 2, n // 2] - (clip[2] / clip[3] * 0.5 + 0.5)) < 1e-6
    covered = raw < 1.0
    # sprite radius in pixels: r / (D tan(fov/2)) * n/2
    rpx = 0.05 / (D * np.tan(np.radians(20.0))) * n / 2
    assert abs(covered.sum() - np.pi * rpx * rpx) < 2 * np.pi * rpx
    assert np.array_equal(covered, covered[::-1, :]) and np.array_equal(covered, covered[:, ::-1])
    # nearest point in the middle, depth grows outwards
    assert raw[n // 2, n // 2] == raw[covered].min()


def test_oracle_empty_frame_is_background():
    cam = scene_camera()
    prm = N.default_render_params(background=(0.1, 0.2, 0.3, 1.0))
    out = O.render_frame(np.zeros((0, 5), np.float32), cam, prm, W, H)
    assert np.all(out["depth"] == 1.0)
    assert np.all(out["color"] == np.array([0.1, 0.2, 0.3, 1.0], np.float32))


def _compare(img_g, img_o, tol, frac, name):
    d = np.abs(img_g.astype(np.float64) - img_o.astype(np.float64))
    bad = (d > tol).mean()
    assert bad <= frac, f"{name}: {bad:.4%} of values differ by more than {tol} (max {d.max():.3e})"
    return float(d.max())


@pytest.mark.gpu
@pytest.mark.parametrize("bilateral,spray,transparency,noise", [(0, 1, 1, 1), (1, 1, 1, 1), (0, 0, 0, 0),
                                                                (1, 0, 1, 0)])
def test_render_matches_oracle(gpu, port_lib, bilateral, spray, transparency, noise):
    pts = scene_particles()
    cam = scene_camera()
    prm = N.default_render_params(particle_radius=1 / 64, smoothing_size=0.08, transparency_blur_size=0.08,
                                  bilateral_filter=bilateral, spray_enabled=spray, transparency_enabled=transparency,
                                  noise_enabled=noise, noise_scale=9.0, noise_offset=0.37, blur_depth_falloff=300.0,
                                  background=(0.05, 0.05, 0.08, 1.0))
    # lights around the unit box
    for l, p in enumerate([(3, 3, 3, 1), (3, 3, -3, 1), (-3, 3, -3, 1), (-3, 3, 3, 1)]):
        prm.lights[l].position[:] = p
        prm.lights[l].power_density[:] = (8.0, 8.0, 8.0)
    r = N.Renderer(W, H)
    r.frame(pts, cam, prm)
    ms, launches = r.stats()
    assert launches >= 7
    ref = O.render_frame(pts, cam, prm, W, H)
    raw = r.read(N.IMG_RAW_DEPTH)
    assert (raw < 1).sum() > 0.1 * W * H  # the fluid covers a good part of the frame
    assert np.array_equal(raw, ref["raw_depth"])
    depth = r.read(N.IMG_DEPTH)
    assert np.array_equal(depth < 1, ref["depth"] < 1)
    _compare(depth, ref["depth"], 2e-6, 0.0, "depth")
    if transparency:
        th = r.read(N.IMG_THICKNESS)
        scale = float(ref["thickness"].max())
        assert scale > 0
        # a pixel whose projected kernel extent sits on an integer (the shaders'
        # int(extent * width)) can take the next kernel size on one side
        _compare(th / scale, ref["thickness"] / scale, 1e-5, 0.001, "thickness")
    nd = r.read(N.IMG_NORMAL_DEPTH)
    _compare(nd, ref["normal_depth"], 2e-3, 0.005, "normal + depth")
    col = r.read(N.IMG_COLOR)
    _compare(col, ref["color"], 2e-3, 0.005, "colour")
    r.close()


@pytest.mark.gpu
def test_render_scene_depth_occludes(gpu, port_lib):
    """A scene depth image (another object nearer than the fluid on the left half)
    hides the fluid there in the thickness and in the composite, as the reference's
    depth test against the render target does."""
    import torch

    pts = scene_particles(seed=2)
    cam = scene_camera()
    prm = N.default_render_params(particle_radius=1 / 64, smoothing_size=0.08, transparency_blur_size=0.08,
                                  noise_enabled=0, background=(0.0, 0.0, 0.0, 1.0))
    scene = np.ones((H, W), np.float32)
    scene[:, : W // 2] = 0.5  # nearer than anything in the fluid
    r = N.Renderer(W, H)
    r.frame(pts, cam, prm, scene_depth=torch.from_numpy(scene).cuda())
    ref = O.render_frame(pts, cam, prm, W, H, scene_depth=scene)
    col = r.read(N.IMG_COLOR)
    assert np.all(col[:, : W // 2] == np.array([0, 0, 0, 1], np.float32))
    _compare(col, ref["color"], 2e-3, 0.005, "colour")
    r.close()


@pytest.mark.gpu
def test_render_ctx_equals_frame_of_gfx_buffer(gpu):
    """fsim_render_ctx renders exactly what fsim_fill_gfx publishes."""
    grid = GridSpec(32)
    pos = dam_break(grid, seed=0)
    sim = N.Simulation(32, N.default_params(transfer=N.FLIP, resolution=32))
    sim.set_particles(pos)
    for _ in range(3):
        sim.step(1 / 120)
    cam = scene_camera()
    prm = N.default_render_params(particle_radius=1 / 128, smoothing_size=0.05, transparency_blur_size=0.05)
    r = N.Renderer(W, H)
    r.frame_sim(sim, cam, prm)
    a = r.read(N.IMG_COLOR)
    raw_a = r.read(N.IMG_RAW_DEPTH)
    r.frame(sim.gfx(), cam, prm)
    assert np.array_equal(raw_a, r.read(N.IMG_RAW_DEPTH))
    assert np.allclose(a, r.read(N.IMG_COLOR), atol=1e-6)
    r.close()
    sim.close()
