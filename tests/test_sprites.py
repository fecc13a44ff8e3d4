"""Headless particle sprites (particleSpriteGeom.{vert,geom,frag}) against their CPU restatement.

CPU: the restatement's closed-form cases -- a lone sprite's disc area and centre colour, and the
nearer of two sprites winning.  GPU: pbd_render_sprites bit-identical to the restatement (images
and depths), on a small scene and on a 1,000,000-particle state."""
import numpy as np
import pytest


def _lone(pbd, col_x, size=97):   # odd: a pixel centre on the sprite centre
    pos = np.array([[0.0, 0.0, 0.0, 1.0]], np.float32)
    col = np.array([[col_x, 0.0, 0.0, 1.0]], np.float32)
    cam = pbd.camera(eye=(0.0, 0.0, 10.0), center=(0.0, 0.0, 0.0), width=size, height=size)
    return pos, col, cam


def test_lone_sprite_disc_and_centre_colour(pbd, oracle_mod):
    pos, col, cam = _lone(pbd, 1.0)
    rgba, depth = oracle_mod.render_sprites(pos, col, cam)
    covered = depth < 1.0
    r_px = 0.5 / (10.0 * np.tan(np.pi / 8)) * cam.width / 2        # projected radius in pixels
    assert abs(covered.sum() - np.pi * r_px ** 2) < 2 * np.pi * r_px + 4
    h, w = cam.height, cam.width
    # centre: N = L = V = R = +z, colour (0, 0, 1): 0.3 c + 0.7 c + 0.2 = (0.2, 0.2, 1.2)
    c = rgba[h // 2, w // 2]
    assert tuple(c) == (51, 51, 255, 255)
    assert tuple(rgba[0, 0]) == (0, 0, 0, 255) and depth[0, 0] == 1.0


def test_nearer_sprite_wins(pbd, oracle_mod):
    pos = np.array([[0.0, 0.0, 0.0, 1.0], [0.1, 0.0, 1.0, 1.0]], np.float32)
    col = np.array([[0.0, 0, 0, 1], [1.0, 0, 0, 1]], np.float32)
    cam = pbd.camera(eye=(0.0, 0.0, 10.0), center=(0.0, 0.0, 0.0), width=64, height=64)
    rgba, depth = oracle_mod.render_sprites(pos, col, cam)
    only_back = oracle_mod.render_sprites(pos[:1], col[:1], cam)[1]
    assert depth[32, 32] < only_back[32, 32]                          # the z = 1 sprite is in front
    assert rgba[32, 32, 2] == 255 and rgba[32, 32, 0] < 200            # with the blue colour


def _gpu_vs_oracle(pbd, oracle_mod, pos, col, cam):
    sim = pbd.Sim(pbd.default_params(), len(pos))
    sim.add_particles(pos, np.zeros_like(pos), col)
    a_rgba, a_depth = sim.render(cam)
    b_rgba, b_depth = oracle_mod.render_sprites(pos, col, cam)
    assert (a_depth < 1).sum() > 0
    assert np.array_equal(a_depth, b_depth)
    assert np.array_equal(a_rgba, b_rgba)
    return a_rgba


@pytest.mark.gpu
def test_gpu_sprites_small_scene_bit_identical(need_gpu, pbd, scenes, oracle_mod):
    pos, _ = scenes.lattice(10, 8, 10, spacing=0.9, seed=3)
    col = np.random.default_rng(3).uniform(0, 1, size=pos.shape).astype(np.float32)
    cam = pbd.camera(eye=(25.0, 14.0, 30.0), center=(7.0, 5.0, 7.0), width=320, height=240)
    _gpu_vs_oracle(pbd, oracle_mod, pos, col, cam)
    # close up: sprites tens of pixels wide, the eye inside the box
    cam2 = pbd.camera(eye=(6.0, 5.0, 12.0), center=(6.0, 5.0, 0.0), width=200, height=150)
    _gpu_vs_oracle(pbd, oracle_mod, pos, col, cam2)


@pytest.mark.gpu
def test_gpu_sprites_million_particles_bit_identical(need_gpu, pbd, scenes, oracle_mod):
    w = scenes.WORKLOADS["fluid_1m"]
    params = scenes.workload_params(pbd, w["box"], 1000.0)
    params.lambda_epsilon = 0.1
    pos, vel = scenes.lattice(*w["shape"], seed=w["seed"])
    sim = pbd.Sim(params, len(pos))
    sim.add_particles(pos, vel)
    sim.step(20)
    x = sim.state()["x"]
    sim.close()
    col = np.random.default_rng(4).uniform(0, 1, size=x.shape).astype(np.float32)
    cam = pbd.camera(eye=(180.0, 120.0, 200.0), center=(64.0, 30.0, 64.0), width=640, height=480)
    _gpu_vs_oracle(pbd, oracle_mod, x, col, cam)
