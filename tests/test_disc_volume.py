"""The gas grid generator, a numpy restatement of DiscVolume(disc; ...)
(src/disc_volume.jl:175-464), checked on the facts its construction fixes
(no GPU).  The reference draws its 64^3 noise lattice from a Julia RNG stream
this cannot reproduce, so the checks are structural, on the same formulas:
value noise interpolates the lattice, fBm is a normalised average of octaves,
Worley noise measures distances to one feature point per cell, erosion is the
cloud remap, the azimuthal seam is crossfaded onto the phi - 2 pi branch over
18 deg, the haze envelope closes to zero at the grid edge, and with no
turbulence the grid is the radial profile times the Gaussian slab."""
import math

import numpy as np
import pytest

from spacetime_gb300 import scene


@pytest.fixture(scope="module")
def lat():
    return np.random.default_rng(11).random((64, 64, 64), dtype=np.float32)


def test_value_noise_interpolates_the_lattice(lat):
    i = np.array([0, 5, 63, 64, -1, 130])
    j = np.array([3, 7, 0, 1, 2, 5])
    k = np.array([9, 0, 63, 2, -3, 4])
    got = scene._value_noise(lat, i.astype(float), j.astype(float), k.astype(float))
    np.testing.assert_array_equal(got, lat[i % 64, j % 64, k % 64].astype(np.float64))
    # midpoint along x: smoothstep(1/2) = 1/2, the plain average
    mid = scene._value_noise(lat, np.array([2.5]), np.array([4.0]), np.array([6.0]))
    assert math.isclose(mid[0], 0.5 * (float(lat[2, 4, 6]) + float(lat[3, 4, 6])), rel_tol=1e-12)


def test_fbm_is_a_normalised_average():
    const = np.full((64, 64, 64), 0.37, np.float32)
    x = np.linspace(-3, 40, 50)
    np.testing.assert_allclose(scene._fbm(const, x, 2 * x, -x, 4, 0.5, 2.1), np.float32(0.37), rtol=1e-12)


def test_worley_ranges_and_feature_points(lat):
    rng = np.random.default_rng(2)
    x, y, z = (rng.uniform(-20, 20, 500) for _ in range(3))
    for ridge in (True, False):
        w = scene._worley(lat, x, y, z, ridge=ridge)
        assert (w >= 0).all() and (w <= 1).all()
    # at a cell's own feature point F1 = 0: billow = 1 - F1 = 1
    cx, cy, cz = 4, -2, 7
    px = cx + float(lat[cx % 64, cy % 64, cz % 64])
    py = cy + float(lat[(cx + 17) % 64, (cy + 31) % 64, (cz + 7) % 64])
    pz = cz + float(lat[(cx + 43) % 64, (cy + 11) % 64, (cz + 29) % 64])
    b = scene._worley(lat, np.array([px]), np.array([py]), np.array([pz]), ridge=False)
    assert math.isclose(b[0], 1.0, abs_tol=1e-12)


def test_erosion_zero_is_the_base_and_erosion_carves(lat):
    rng = np.random.default_rng(3)
    ls, u, zh = rng.uniform(1, 3, 400), rng.uniform(0, 20, 400), rng.uniform(-6, 6, 400)
    base = scene._fbm(lat, 10 * ls, 6 * u, zh, 4, 0.5, 2.1)
    np.testing.assert_array_equal(scene._shape_coverage(lat, ls, u, zh, 4, 0.5, 2.1, 0.0, 4.0, 3, False), base)
    carved = scene._shape_coverage(lat, ls, u, zh, 4, 0.5, 2.1, 0.9, 4.0, 3, False)
    assert (carved <= base + 1e-12).all() and (carved == 0).any()


def test_no_turbulence_is_profile_times_slab():
    inner, outer, h = 2.32, 25.0, 0.05
    v = scene.make_volume(inner=inner, outer=outer, nr=24, nphi=8, nz=9, scale_height=h, turbulence=0.0)
    nz, nphi, nr = v.density.shape
    s = np.exp(math.log(inner) + np.arange(nr) / (nr - 1) * (math.log(outer) - math.log(inner)))
    z = -v.z_max + np.arange(nz) / (nz - 1) * 2 * v.z_max
    ref = scene.disc_radial_profile(s, inner, outer)[None, :] * np.exp(-z[:, None] ** 2 / (2 * (h * s[None, :]) ** 2))
    ref = (ref / ref.max()).astype(np.float32)
    for j in range(nphi):
        np.testing.assert_allclose(v.density[:, j, :], ref, rtol=2e-6, atol=1e-7)


def test_haze_closes_at_the_grid_edge():
    """haze adds haze * exp(-z^2 / 2 (haze_height H)^2) * window: at the
    midplane the window is 1 (the column gains a factor 1 + haze), at |z| =
    z_max it is 0 (nothing added), so against the plain grid -- each
    normalised by its own peak -- the ratio at the midplane is (1 + haze)
    times the ratio at the edge, in every radial column."""
    kw = dict(inner=3.0, outer=20.0, nr=16, nphi=4, nz=11, scale_height=0.08, turbulence=0.0)
    plain = scene.make_volume(**kw)
    hazy = scene.make_volume(**kw, haze=0.5, haze_height=4.0)
    ok = plain.density[0, 0] > 1e-20
    edge = hazy.density[0, 0][ok].astype(np.float64) / plain.density[0, 0][ok]
    mid = hazy.density[5, 0][ok].astype(np.float64) / plain.density[5, 0][ok]
    np.testing.assert_allclose(mid / edge, 1.5, rtol=1e-5)
    assert np.ptp(edge) <= 1e-5 * edge.mean()


def test_wrap_crossfade_starts_at_its_sector():
    kw = dict(inner=3.0, outer=20.0, nr=12, nphi=40, nz=6, scale_height=0.08, seed=9)
    v = scene.make_volume(**kw)
    phi = np.arange(40) / 40 * 2 * math.pi
    outside = phi <= 2 * math.pi - scene.WRAP_BLEND
    # recompute without the crossfade: identical outside the last 18 deg
    lat = np.random.default_rng(9).random((64, 64, 64), dtype=np.float32)
    nz, nphi, nr = v.density.shape
    s = np.exp(math.log(3.0) + np.arange(nr) / (nr - 1) * (math.log(20.0) - math.log(3.0)))
    z = -v.z_max + np.arange(nz) / (nz - 1) * 2 * v.z_max
    H = 0.08 * s
    u = phi[None, :, None] + 4.0 * np.log(s / 3.0)[None, None, :]
    shape = (nz, nphi, nr)
    n = scene._fbm(lat, np.broadcast_to(10 * np.log(s), shape), np.broadcast_to(6 * u, shape),
                   np.broadcast_to(2 * z[:, None, None] / H[None, None, :], shape), 4, 0.5, 2.1)
    raw = (scene.disc_radial_profile(s, 3.0, 20.0)[None, None, :] *
           np.exp(-z[:, None, None] ** 2 / (2 * H[None, None, :] ** 2)) * np.exp(6 * 0.8 * (n - 0.5)))
    raw = (raw / raw.max()).astype(np.float32)
    np.testing.assert_allclose(v.density[:, outside, :], raw[:, outside, :], rtol=1e-5, atol=1e-8)
    assert not np.allclose(v.density[:, ~outside, :], raw[:, ~outside, :], rtol=1e-5, atol=1e-8)
