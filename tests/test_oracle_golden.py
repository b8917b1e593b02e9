"""The FP64 oracle pinned to SpaceTime.jl's own known-answer tests
(test/runtests.jl), restated here against the oracle's C entry points.
The reference (Julia + Metal) cannot run in this environment, so these
executable physics statements, plus the committed golden render, are the pin.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import scene


def _axes(pos, up=(0.0, 0.0, 1.0)):
    fwd = -np.asarray(pos, float) / np.linalg.norm(pos)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    return fwd, right, np.cross(right, fwd)


def _ks_metric(pos, M):
    r = np.linalg.norm(pos)
    l = np.r_[1.0, np.asarray(pos) / r]
    return np.diag([-1.0, 1, 1, 1]) + (2 * M / r) * np.outer(l, l)


# test/runtests.jl:67-85
@pytest.mark.parametrize("r,beta", [(30.0, (0.5, 0.0, 0.0)), (5.0, (-0.6, 0.2, 0.1)),
                                    (2.6, (0.3, -0.3, 0.2)), (100.0, (0.0, 0.0, 0.9))])
def test_boosted_tetrad_orthonormal(oracle_lib, r, beta):
    d = np.array([1.0, 0.3, -0.2])
    pos = r * d / np.linalg.norm(d)
    fwd, right, up = _axes(pos)
    u, Ef, Er, Eu = O.camera_tetrad(pos, fwd, right, up, 1.0, 0.0, beta)
    T = np.stack([u, Ef, Er, Eu], axis=1)
    assert np.abs(T.T @ _ks_metric(pos, 1.0) @ T - np.diag([-1.0, 1, 1, 1])).max() < 1e-12


# test/runtests.jl:87-100
@pytest.mark.parametrize("bf", [0.5, -0.5])
def test_flat_space_doppler(oracle_lib, bf):
    pos = np.array([1.0e6, 0.0, 0.0])
    u, Ef, _, _ = O.camera_tetrad(pos, [-1.0, 0, 0], [0, -1.0, 0], [0, 0, 1.0], 1.0, 0.0, (bf, 0.0, 0.0))
    q = Ef - u
    xh = pos / np.linalg.norm(pos)
    p_t = -q[0] + (2.0 / np.linalg.norm(pos)) * (q[0] + xh @ q[1:])
    g = 1.0 / math.sqrt(1.0 - bf * bf)
    assert abs(1.0 / abs(p_t) - g * (1.0 + bf)) <= 1e-5


# test/runtests.jl:102-110
def test_zero_boost_is_unboosted_bitwise(oracle_lib):
    pos = np.array([10.0, 1.0, 0.5])
    fwd, right, up = _axes(pos)
    t0 = O.camera_tetrad(pos, fwd, right, up, 1.0, 0.0, (0.0, 0.0, 0.0))
    t1 = O.camera_tetrad(pos, fwd, right, up, 1.0)
    for a, b in zip(t0, t1):
        assert np.array_equal(a, b)


def _shifts(R, W=24, H=14, fov=0.5):
    pos = np.array([R, 0.0, 0.0])
    fwd, right, up = _axes(pos)
    u4, Ef, Er, Eu = O.camera_tetrad(pos, fwd, right, up, 1.0)
    g = np.zeros((W, H))
    for i in range(1, W + 1):
        for j in range(1, H + 1):
            uu = (i - 0.5 - W / 2 + 0.5) / (H / 2)     # sensor_coordinate, src/camera.jl:391-396
            vv = (j - 0.5 - H / 2 + 0.5) / (H / 2)
            d = right * uu * fov + up * vv * fov + fwd
            d /= np.linalg.norm(d)
            q = (d @ fwd) * Ef + (d @ right) * Er + (d @ up) * Eu - u4
            _, pt = O.init_photon(pos, q, 1.0, 0.0)
            g[i - 1, j - 1] = 1.0 / min(max(abs(pt), 0.05), 20.0)
    return g


# test/runtests.jl:113-141
@pytest.mark.parametrize("R", [20.0, 6.0, 3.0])
def test_per_ray_shift_static(oracle_lib, R):
    g = _shifts(R)
    assert g.max() - g.min() < 1e-7
    assert abs(g[0, 0] - 1 / math.sqrt(1 - 2 / R)) <= 1e-7 * (1 / math.sqrt(1 - 2 / R))


def test_per_ray_shift_inside_freeze_radius(oracle_lib):
    g = _shifts(2.1)
    assert (g.max() - g.min()) / g.mean() > 0.5
    assert g.min() > 1 / math.sqrt(1 - 2 / 2.1)


# test/runtests.jl:143-186 (beaming through the CPU renderer's rules)
def test_camera_velocity_beams(oracle_lib):
    pos = np.array([20.0, 0.0, 0.0])
    v = np.array([-0.6, 0.0, 0.0])
    still = scene.Camera.look_at(pos, (0, 0, 0), (0, 0, 1.0), 0.5)
    moving = scene.Camera.look_at(pos, (0, 0, 0), (0, 0, 1.0), 0.5, velocity=v)
    assert np.allclose(scene.camera_beta(moving), [0.6, 0.0, 0.0], atol=1e-12)
    bg = np.empty((32, 64, 3), np.float32)
    bg[:] = (0.05, 0.05, 0.08)
    means = []
    for cam in (still, moving):
        sc = O.Scene(cam=cam, M=1.0, a=0.0, sky=bg, width=28, height=16, semantics=O.SEM_RENDER,
                     integrator=O.INT_TSIT5, relativistic=True, rtol=1e-8, atol=1e-10)
        img, _ = sc.render()
        means.append(img.astype(np.float64).mean())
    assert means[1] > 1.5 * means[0]


# test/runtests.jl:188-200 (src/utils.jl:31-37)
def test_shadow_radius(oracle_lib):
    assert math.isclose(O.shadow_radius(1e6, 1.0, 1.0) * 1.0, 3 * math.sqrt(3) / 1e6, rel_tol=1e-6)
    assert O.shadow_radius(5.0, 1.0, 1.0) == math.inf


# test/runtests.jl:576-594
def test_horizon_and_photon_orbit(oracle_lib):
    assert math.isclose(O.horizon_radius(1.0, 0.0), 2.0)
    assert math.isclose(O.horizon_radius(1.0, 0.6), 1.0 + math.sqrt(1 - 0.36))
    assert math.isclose(O.horizon_radius(1.0, 1.0), 1.0)
    assert math.isclose(O.photon_orbit_min(1.0, 0.0), 3.0)
    assert abs(O.photon_orbit_min(1.0, 1.0) - 1.0) < 1e-9
    assert O.photon_orbit_min(1.0, 0.9) < O.photon_orbit_min(1.0, 0.5)
    for a in (0.0, 0.3, 0.6, 0.9, 0.99):
        assert O.photon_orbit_min(1.0, a) >= O.horizon_radius(1.0, a) - 1e-12


# test/runtests.jl:596-608
def test_kerr_rhs_reduces_to_schwarzschild(oracle_lib):
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(5000):
        s = rng.standard_normal(6) * 3
        if s[:3] @ s[:3] < 4:
            continue
        k = O.rhs(True, s, -1.0, 1.0, 0.0)
        c = O.rhs(False, s, -1.0, 1.0, 0.0)
        worst = max(worst, float(np.max(np.abs(k - c) / np.maximum(np.abs(c), 1e-3))))
    assert worst < 1e-9


# test/runtests.jl:610-641
@pytest.mark.parametrize("a", [0.0, 0.5, 0.9, 0.998])
def test_lz_conservation(oracle_lib, a):
    assert O.lz_drift(a, 0.005, 20000) < 1e-8


# test/runtests.jl:643-656
def test_metric_inverse(oracle_lib):
    q = np.array([12.0, 3.0, 2.0])
    for a in (0.0, 0.9):
        assert np.abs(O.metric(1.0, a, q) @ O.metric_inverse(1.0, a, q) - np.eye(4)).max() < 1e-13
    q2 = np.array([6.0, 2.0, 1.5])
    assert np.allclose(O.metric_inverse(1.0, 1e-300, q2), O.metric_inverse(1.0, 0.0, q2), rtol=1e-12)


# test/runtests.jl:30-38 (sensor_coordinate signs), in the CPU convention
def test_sensor_coordinate_signs():
    def sc(i, j, w, h):
        return (i - 0.5 - w / 2 + 0.5) / (h / 2), (j - 0.5 - h / 2 + 0.5) / (h / 2)
    u, v = sc(1, 1, 10, 10)
    assert u < 0 and v < 0
    u, v = sc(10, 10, 10, 10)
    assert u > 0 and v > 0


def test_blackbody_lut_two_restatements_agree(oracle_lib):
    a = O.blackbody_lut(6500.0)
    b = scene.blackbody_lut(6500.0)
    assert np.abs(a - b).max() < 1e-5
    # the white point renders neutral: T(208) = 500 + 29500*208/1023 ~ 6498 K
    assert np.abs(a[208] - 1.0).max() < 2e-3


def test_sim_hash_bit_exact(oracle_lib):
    def h(x, y, z):
        m = 0xffffffff
        v = ((x & m) * 0x8da6b343 & m) ^ ((y & m) * 0xd8163841 & m) ^ ((z & m) * 0xcb1ab31f & m)
        v ^= v >> 13
        v = (v * 0x9e3779b9) & m
        v ^= v >> 16
        return np.float32(v & 0x00ffffff) * np.float32(5.9604645e-8)
    rng = np.random.default_rng(3)
    for x, y, z in rng.integers(-2 ** 31, 2 ** 31 - 1, size=(500, 3)):
        assert O.sim_hash(int(x), int(y), int(z)) == h(int(x), int(y), int(z))


def test_isco_values(oracle_lib):
    r, E, L = O.isco(1.0, 0.0)
    assert math.isclose(r, 6.0, rel_tol=1e-12)
    assert math.isclose(E, math.sqrt(8.0 / 9.0), rel_tol=1e-12)
    r9 = O.isco(1.0, 0.9)[0]
    assert abs(r9 - 2.32088) < 1e-4
