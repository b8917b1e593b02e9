"""Seeded inputs and host-side camera helpers (no GPU)."""
import math

import numpy as np
import pytest

from spacetime_gb300 import api, scene, ship, workloads


def test_sky_seeded_and_shaped():
    a = scene.make_sky(256, 128, n_stars=300, seed=5)
    b = scene.make_sky(256, 128, n_stars=300, seed=5)
    c = scene.make_sky(256, 128, n_stars=300, seed=6)
    assert a.shape == (128, 256, 3) and a.dtype == np.float32
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert (a > 0).all()
    # log-normal background: median log near mu = -6
    assert abs(np.median(np.log(a[..., 1])) + 6.0) < 0.1


def test_volume_grid():
    v = scene.make_volume(inner=2.32, outer=25.0, nr=32, nphi=16, nz=8, scale_height=0.05, seed=7)
    assert v.shape == (32, 16, 8)
    assert v.density.shape == (8, 16, 32) and v.density.dtype == np.float32
    assert math.isclose(v.density.max(), 1.0, rel_tol=1e-6)
    assert v.density.min() >= 0.0
    assert math.isclose(v.z_max, 3 * 0.05 * 25.0, rel_tol=1e-6)
    v2 = scene.make_volume(inner=2.32, outer=25.0, nr=32, nphi=16, nz=8, scale_height=0.05, seed=7)
    assert np.array_equal(v.density, v2.density)


def test_camera_basis_and_lens():
    cam = scene.Camera.look_at((0, -30, 3), (0, 0, 0), (0, 0, 1.0), api.Lens(24).fov_factor)
    assert math.isclose(cam.fov_factor, 0.75)
    B = np.stack([cam.fwd, cam.right, cam.up_local])
    assert np.allclose(B @ B.T, np.eye(3), atol=1e-12)
    assert np.allclose(cam.fwd, -cam.pos / np.linalg.norm(cam.pos))


def test_kerr_argument_error():
    with pytest.raises(ValueError):
        api.Kerr(1.0, 1.5)
    assert api.Kerr(1.0, 0.6).a == 0.6


def test_render_rejects_kerr_before_gpu():
    with pytest.raises(TypeError):
        api.render(scene.Camera.look_at((0, -30, 3), (0, 0, 0), (0, 0, 1.0), 0.75), api.Kerr(1.0, 0.5),
                   np.zeros((4, 8, 3), np.float32))


def test_free_fall_track():
    cams = ship.free_fall_track(30.0, 1.5, 12)
    r = np.array([np.linalg.norm(c.pos) for c in cams])
    assert math.isclose(r[0], 30.0, rel_tol=1e-12)
    assert np.all(np.diff(r) < 0) and r[-1] <= 1.6
    speeds = np.array([np.linalg.norm(c.velocity) for c in cams])
    assert speeds[0] < 1e-9 and np.all(speeds < 1.0)
    # falling straight in: the velocity points along the view direction
    for c in cams[1:]:
        v = c.velocity / np.linalg.norm(c.velocity)
        assert v @ c.fwd > 0.999


def test_ship_mass_shell():
    s = ship.ShipState.at_rest(np.array([20.0, 0.0, 1.0]), 1.0)
    for _ in range(20):
        ship.step_ship(s, 1.0, 0.5)
        u = ship.ks_raise(s.x, 1.0, s.p_t, s.p)
        assert abs(ship.ks_gdot(s.x, 1.0, u, u) + 1.0) < 1e-10


def test_workload_shapes():
    w = workloads.config1(nr=16, nphi=8, nz=4)
    assert (w.width, w.height) == (1920, 1080) and w.bh.a == 0.9
    assert abs(np.linalg.norm(w.cam.pos[[0, 2]]) - math.hypot(math.sqrt(15 ** 2 + 0.81) * math.sin(math.radians(80)),
                                                               15 * math.cos(math.radians(80)))) < 1e-9
