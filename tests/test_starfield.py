"""Procedural starfield, host side: the stars' own colour table against the
reference's known answers (test/runtests.jl:461-493), the C defaults against
set_starfield!'s keyword defaults (src/metal.jl:257-267), and oracle
properties of the per-ray star sum."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.api import Starfield


def _br(lut, T, tmin=500.0, tmax=30000.0):
    n = lut.shape[0]
    i = int(np.clip(round((T - tmin) / (tmax - tmin) * (n - 1)), 0, n - 1))
    return lut[i, 2] / lut[i, 0]


def test_star_table_tracks_temperature_across_its_white_point(oracle_lib):
    lut = O.star_lut()
    assert _br(lut, 3500.0) < 0.5                       # a cool star is warm
    assert abs(_br(lut, O.STAR_WB_TEMPERATURE) - 1.0) <= 0.02   # the white point is white
    assert _br(lut, 15000.0) > 1.2                      # a hot star is blue
    sf = Starfield()
    assert sf.temp_min < O.STAR_WB_TEMPERATURE < sf.temp_max   # the default range straddles it


def test_star_table_is_not_the_discs(oracle_lib):
    # the disc's table moves with its white point; the stars' does not
    assert not np.array_equal(O.blackbody_lut(10000.0), O.blackbody_lut(4000.0))
    assert np.array_equal(O.star_lut(), O.star_lut(O.STAR_WB_TEMPERATURE))
    desat = O.star_lut(saturation=0.35)
    L = lambda t: 0.2126 * t[:, 0] + 0.7152 * t[:, 1] + 0.0722 * t[:, 2]
    np.testing.assert_allclose(L(desat), L(O.star_lut()), rtol=1e-5)


def test_c_defaults_match_set_starfield(built_lib):
    lib = _abi.load()
    c = _abi.StStarfield()
    lib.st_starfield_default(C.byref(c))
    ref = Starfield()
    for name, _ in _abi.StStarfield._fields_:
        got = list(c.galactic) if name == "galactic" else getattr(c, name)
        want = list(ref.galactic) if name == "galactic" else getattr(ref, name)
        assert got == pytest.approx(want), name


def _scene(**kw):
    w = workloads.config0().scaled(64, 36)
    sf = dict(height=36, fov_factor=w.cam.fov_factor, density=96, fill=0.9, flux=0.5, psf_pixels=1.5)
    sf.update(kw)
    return w, sf


def test_oracle_stars_only_add_light_to_escaped_rays(oracle_lib):
    w, sf = _scene()
    sky = workloads.sky(64, 32)
    base, rays = O.scene_for(w, sky, O.INT_RK4).render()
    lit, rays2 = O.scene_for(w, sky, O.INT_RK4, starfield=dict(sf, texture_weight=1.0)).render()
    np.testing.assert_array_equal(rays["flags"], rays2["flags"])
    black = (rays["flags"] & O.RAY_BLACK) > 0
    np.testing.assert_array_equal(lit[black], base[black])
    assert (lit >= base - 1e-7).all() and (lit > base + 1e-6).any()
    off, _ = O.scene_for(w, sky, O.INT_RK4, starfield=dict(sf, strength=0.0)).render()
    np.testing.assert_array_equal(off, base)


def test_oracle_shutter_to_the_same_pose_is_still(oracle_lib):
    w = workloads.config0().scaled(48, 27)
    sky = workloads.sky(64, 32)
    still, _ = O.scene_for(w, sky, O.INT_RK4).render()
    shut, _ = O.scene_for(w, sky, O.INT_RK4, shutter=(104730, w.cam)).render()
    np.testing.assert_array_equal(shut, still)
