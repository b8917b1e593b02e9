"""Procedural starfield and motion blur on the GPU, against the oracle.

Stars (starfield_mtl, src/metal.jl:652-724; starfield_color,
src/starfield.jl:83-150): FP64 renders with stars match the oracle's FP64
twin at the twin tolerances (direction median <= 1e-9 rad, radiance p99
<= 1e-5), under both rule sets, with the sky image on or off; the stars'
colour does not follow the disc's white point.

Motion blur (src/metal.jl:2130-2169, 829-857): poses that do not move
reproduce the still render bit for bit in both shutter modes; the per-pixel
shutter of one pass matches the oracle twin interpolating the same two poses
at the same hashed instants; the midpoint mode renders the stratum's pose.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Context, Starfield
from spacetime_gb300.scene import Camera, kerr_position, lens_fov

from .helpers import compare, gpu_render, oracle_scene

pytestmark = pytest.mark.gpu

FP64 = _abi.ST_PREC_FP64


def _stars(w, **kw):
    sf = dict(height=w.height, fov_factor=w.cam.fov_factor, density=96, fill=0.9, flux=0.5, psf_pixels=1.5)
    sf.update(kw)
    return sf


def _gpu_with_stars(w, sky, sf, precision=FP64):
    with Context(sky, disc=w.disc, volume=w.vol, emitter=w.emitter) as ctx:
        ctx.set_starfield(Starfield(**sf))
        return gpu_render(w, sky, precision, ctx=ctx)


def _check_twin(c, n):
    assert c["class_mismatch"] <= max(2, 2e-3 * n), c
    assert c["dir_median"] <= 1e-9 and c["rad_p99"] <= 1e-5, c


@pytest.mark.parametrize("tw", [0.0, 1.0])
def test_stars_render_rules_fp64_vs_twin(built_lib, tw):
    w = workloads.config0().scaled(160, 90)
    sky = workloads.sky(512, 256)
    sf = _stars(w, texture_weight=tw)
    g = _gpu_with_stars(w, sky, sf)
    ref, rays = oracle_scene(w, sky, O.INT_RK4, starfield=sf).render()
    c = compare(g.image, g.diag, ref, rays)
    _check_twin(c, w.width * w.height)
    # the stars are there: the star-only sky is not the image-only one
    if tw == 0.0:
        plain = gpu_render(w, sky, FP64)
        assert np.abs(g.image - plain.image).max() > 1e-3


def test_stars_kerr_draft_fp64_vs_twin(built_lib):
    w = workloads.config1_thin().scaled(160, 90)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    sky = workloads.sky(512, 256)
    sf = _stars(w, texture_weight=0.5, galactic=(0.3, 0.0, 1.0), seed=777)
    g = _gpu_with_stars(w, sky, sf)
    ref, rays = oracle_scene(w, sky, O.INT_RK4, starfield=sf).render()
    _check_twin(compare(g.image, g.diag, ref, rays), w.width * w.height)


def test_star_colour_ignores_the_disc_white_point(built_lib):
    w = workloads.config0().scaled(96, 54)
    sky = workloads.sky(512, 256)
    sf = _stars(w)
    imgs = []
    for wb in (10000.0, 4000.0):
        disc = workloads.AccretionDisc(3.0, 20.0, workloads.Blackbody(wb_temperature=wb), 0.0)
        with Context(sky, disc=disc, emitter=w.emitter) as ctx:
            ctx.set_starfield(Starfield(**sf))
            imgs.append(gpu_render(w, sky, FP64, ctx=ctx))
    a, b = imgs
    clear = ((a.diag["flags"] & (_abi.ST_RAY_CROSSED | _abi.ST_RAY_BLACK)) == 0)
    assert clear.mean() > 0.3
    np.testing.assert_array_equal(a.image[clear], b.image[clear])
    assert not np.array_equal(a.image[~clear], b.image[~clear])


def _orbit_cam(r, incl_deg, phi, a, speed=0.0):
    p0 = kerr_position(r, incl_deg, a)
    c, s = math.cos(phi), math.sin(phi)
    pos = np.array([c * p0[0] - s * p0[1], s * p0[0] + c * p0[1], p0[2]])
    cam = Camera.look_at(pos, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), lens_fov(24.0))
    cam.velocity = speed * np.array([-s, c, 0.0])
    return cam


def _motion_workload():
    w = workloads.config1_thin().scaled(96, 54)
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    return w


@pytest.mark.parametrize("per_pixel", [False, True])
def test_still_poses_reproduce_the_still_render(built_lib, per_pixel):
    w = _motion_workload()
    sky = workloads.sky(512, 256)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=FP64, samples=2, pixel_jitter=1,
                       exit_landing=1, seed=5)
        still = ctx.render_raw(w.cam, w.bh, p)
        poses = [w.cam] * (5 if per_pixel else 4)
        mo = ctx.render_motion_raw(w.cam, poses, w.bh, p, per_pixel_shutter=per_pixel)
    np.testing.assert_array_equal(mo.image, still.image)
    assert mo.stats["launches"] == 4


def test_per_pixel_shutter_fp64_vs_twin(built_lib):
    w = _motion_workload()
    a = w.bh.a
    cam0 = _orbit_cam(15.0, 80.0, 0.0, a, speed=0.3)
    cam1 = _orbit_cam(15.0, 80.0, 0.08, a, speed=0.3)
    sky = workloads.sky(512, 256)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=FP64, samples=1, pixel_jitter=0,
                       exit_landing=1)
        g = ctx.render_motion_raw(cam0, [cam0, cam1], w.bh, p, per_pixel_shutter=True, diag=True)
        g0 = ctx.render_raw(cam0, w.bh, p)
    w.cam = cam0
    ref, rays = oracle_scene(w, sky, O.INT_RK4, shutter=(104729 + 1, cam1)).render()
    _check_twin(compare(g.image, g.diag, ref, rays), w.width * w.height)
    assert np.abs(g.image - g0.image).max() > 1e-4   # the shutter moved the camera


def test_midpoint_shutter_renders_the_stratum_pose(built_lib):
    w = _motion_workload()
    a = w.bh.a
    cam0 = _orbit_cam(15.0, 80.0, 0.0, a)
    mid = _orbit_cam(15.0, 80.0, 0.05, a)
    sky = workloads.sky(512, 256)
    with Context(sky, disc=w.disc, emitter=w.emitter) as ctx:
        p = ctx.params(w.semantics, width=w.width, height=w.height, precision=FP64, samples=1, pixel_jitter=0,
                       exit_landing=1)
        g = ctx.render_motion_raw(cam0, [mid], w.bh, p)
        ref = ctx.render_raw(mid, w.bh, p)
    # same orbit radius: the same escape radius and step budget as `mid` alone
    np.testing.assert_array_equal(g.image, ref.image)
