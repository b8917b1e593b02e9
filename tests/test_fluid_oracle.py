"""The fluid-disc oracle (DiscFluidSim / step_sim!, src/disc_sim.jl) on the CPU.

The reference ships no tests or fixtures for the solver, so the restatement
is pinned by facts its equations fix:
- construction (src/disc_sim.jl:45-91): the midplane slice over its peak,
  the radial profile of src/disc_volume.jl:274-283 on every phi column, the
  Gaussian envelope exp(-z^2 / 2 H^2) with H = scale_height s, and the
  Keplerian shear sqrt(M / s^3) nphi / 2 pi, against numpy in float64;
- with forcing 0 from rest the velocity stays exactly zero and, with
  relax 0, one step moves each density row by dt shear(s) cells: the
  bilinear shift, its backward re-advection and the MacCormack limiter,
  restated independently in numpy float32 with the same operation order,
  agree bit for bit;
- more Jacobi sweeps leave a less divergent velocity;
- the extruded texture is the density times the envelope, exactly.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300.scene import disc_radial_profile, make_volume

INNER, OUTER = 3.0, 20.0


@pytest.fixture(scope="module")
def vol():
    return make_volume(inner=INNER, outer=OUTER, nr=40, nphi=48, nz=10, seed=3)


def test_construction(vol):
    sim = O.FluidSim(vol, INNER, OUTER, falloff=0.8)
    nr, nphi, nz = vol.shape
    mid = vol.density[(nz + 1) // 2 - 1]
    np.testing.assert_array_equal(sim.dens, mid / mid.max())
    s = np.exp(np.float64(vol.log_s_in) + np.arange(nr) / (nr - 1) * np.float64(
        np.float32(vol.log_s_out) - np.float32(vol.log_s_in)))
    prof = disc_radial_profile(s, INNER, OUTER, 1.0, 0.8).astype(np.float32)
    np.testing.assert_allclose(sim.base, np.broadcast_to(prof, (nphi, nr)), rtol=1e-6, atol=1e-12)
    H = np.float64(np.float32(vol.scale_height)) * s
    z = -np.float64(vol.z_max) + np.arange(nz)[:, None] / (nz - 1) * 2 * np.float64(vol.z_max)
    np.testing.assert_allclose(sim.env, np.exp(-z ** 2 / (2 * H ** 2)), rtol=1e-6, atol=1e-30)
    np.testing.assert_allclose(sim.shear, np.sqrt(1.0 / s ** 3) * nphi / (2 * math.pi), rtol=1e-6)
    assert np.all(sim.vu == 0) and np.all(sim.vv == 0) and sim.t == 0.0


def _shift_step(d, shear, dt):
    """One zero-velocity MacCormack step (relax 0) in numpy float32, written
    from the equations: forward sample at j - dt shear, backward at j + dt
    shear, corrected by half the round-trip error and clamped to the four
    corners of the forward footprint."""
    f32 = np.float32
    nphi, nr = d.shape
    dt = f32(dt)
    i = np.arange(1, nr + 1, dtype=np.int64)[None, :].repeat(nphi, 0)
    j = np.arange(1, nphi + 1, dtype=np.int64)[:, None].repeat(nr, 1)

    def foot(x, y):
        x = np.clip(x, f32(1), f32(nr))
        i0 = np.clip(np.floor(x).astype(np.int64), 1, nr - 1)
        tx = (x - i0.astype(f32)).astype(f32)
        yw = (y - f32(nphi) * np.floor((y - f32(1)) / f32(nphi))).astype(f32)
        j0 = np.floor(yw).astype(np.int64)
        ty = (yw - j0.astype(f32)).astype(f32)
        j0a = np.mod(j0 - 1, nphi) + 1
        j1a = np.mod(j0, nphi) + 1
        return i0, tx, j0a, j1a, ty

    def sample(f, x, y):
        i0, tx, j0a, j1a, ty = foot(x, y)
        g = lambda ii, jj: f[jj - 1, ii - 1]
        a = g(i0, j0a) + tx * (g(i0 + 1, j0a) - g(i0, j0a))
        b = g(i0, j1a) + tx * (g(i0 + 1, j1a) - g(i0, j1a))
        return (a + ty * (b - a)).astype(f32)

    x = i.astype(f32) - dt * f32(0)
    sh = shear[None, :].astype(f32)
    y = (j.astype(f32) - dt * (f32(0) + sh)).astype(f32)
    d1 = sample(d, x, y)
    yb = (j.astype(f32) - (-dt) * (f32(0) + sh)).astype(f32)
    d2 = sample(d1, x, yb)
    i0, _, j0a, j1a, _ = foot(x, y)
    g = lambda ii, jj: d[jj - 1, ii - 1]
    lo = np.minimum(np.minimum(g(i0, j0a), g(i0 + 1, j0a)), np.minimum(g(i0, j1a), g(i0 + 1, j1a)))
    hi = np.maximum(np.maximum(g(i0, j0a), g(i0 + 1, j0a)), np.maximum(g(i0, j1a), g(i0 + 1, j1a)))
    a = np.clip((d1 + f32(0.5) * (d - d2)).astype(f32), lo, hi)
    return np.maximum(a, f32(0))


def test_zero_velocity_is_a_shear_shift(vol):
    sim = O.FluidSim(vol, INNER, OUTER, forcing=0.0, relax=0.0)
    d0 = sim.dens.copy()
    sim.step(dt=0.3, jacobi=8, nsteps=1)
    assert np.all(sim.vu == 0) and np.all(sim.vv == 0)
    np.testing.assert_array_equal(sim.dens, _shift_step(d0, sim.shear, 0.3))
    # and keeps doing so
    d1 = sim.dens.copy()
    sim.step(dt=0.3, jacobi=8, nsteps=1)
    np.testing.assert_array_equal(sim.dens, _shift_step(d1, sim.shear, 0.3))
    assert sim.t == np.float32(np.float32(0.3) + np.float32(0.3))


def _div(vu, vv):
    nphi, nr = vu.shape
    ip = np.minimum(np.arange(nr) + 1, nr - 1)
    im = np.maximum(np.arange(nr) - 1, 0)
    return 0.5 * (vu[:, ip] - vu[:, im] + np.roll(vv, -1, axis=0) - np.roll(vv, 1, axis=0))


def test_more_sweeps_less_divergence(vol):
    norms = []
    for jac in (0, 2, 8, 40):
        sim = O.FluidSim(vol, INNER, OUTER)
        sim.step(dt=0.05, jacobi=jac, nsteps=3)
        norms.append(float(np.sqrt(np.mean(_div(sim.vu.astype(np.float64), sim.vv.astype(np.float64)) ** 2))))
    assert norms[0] > norms[1] > norms[2] > norms[3], norms
    assert norms[0] > 0


def test_extrusion_and_clock(vol):
    sim = O.FluidSim(vol, INNER, OUTER)
    v = sim.step(dt=0.08, jacobi=8, nsteps=5, volume=True)
    np.testing.assert_array_equal(v, sim.dens[None, :, :] * sim.env[:, None, :])
    t = np.float32(0)
    for _ in range(5):
        t = np.float32(t + np.float32(0.08))
    assert sim.t == t
    assert np.isfinite(sim.vu).all() and np.abs(sim.vu).max() > 0
    assert (sim.dens >= 0).all()
