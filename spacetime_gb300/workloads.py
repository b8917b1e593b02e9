"""Benchmark workloads of the render path, with their seeded inputs.

    config0  Schwarzschild M=1, pinhole at (0,-30,3) looking at the origin,
             up z, Lens(24), 320x180, thin disc 3-20 with Keplerian
             Planck-Doppler shading; the CPU renderer's rules.
    config1  Kerr a=0.9 M=1, static camera at KS r=15, inclination 80 deg,
             Lens(24), 1920x1080 float32 HDR, volumetric gas 256x64x32 from
             the ISCO (2.32M) to 25M, scale height 0.05 r; the kernel's rules.
    config2  240 frames 1280x720 on a radial free fall from r=30M to 1.5M
             (Schwarzschild), thin disc 3-20, per-frame Lorentz boost.
    config4  Kerr a=0.99, r=20, inclination 85 deg, boost 0.3c, 3840x2160,
             gas 512x128x64, 8 frames on a circular orbit.
All skies: 2048x1024 synthetic (scene.make_sky).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .api import AccretionDisc, Blackbody, Kerr, Schwarzschild
from .scene import Camera, Volume, kerr_position, lens_fov, make_sky, make_volume
from .ship import free_fall_track

SKY_SEED = 1234
VOL_SEED = 7

_sky_cache: dict = {}
_vol_cache: dict = {}


def sky(width=2048, height=1024, seed=SKY_SEED) -> np.ndarray:
    key = (width, height, seed)
    if key not in _sky_cache:
        _sky_cache[key] = make_sky(width, height, n_stars=20000 if width >= 1024 else 2000, seed=seed)
    return _sky_cache[key]


def volume(nr, nphi, nz, inner, outer, scale_height, seed=VOL_SEED) -> Volume:
    key = (nr, nphi, nz, inner, outer, scale_height, seed)
    if key not in _vol_cache:
        _vol_cache[key] = make_volume(inner=inner, outer=outer, nr=nr, nphi=nphi, nz=nz,
                                      scale_height=scale_height, seed=seed)
    return _vol_cache[key]


@dataclass
class Workload:
    name: str
    bh: object
    cam: Camera
    width: int
    height: int
    semantics: int
    disc: AccretionDisc | None
    emitter: int
    vol: Volume | None = None
    params: dict = field(default_factory=dict)
    cams: list | None = None  # camera track (batched frames)

    def scaled(self, width, height):
        w = Workload(**{**self.__dict__})
        w.width, w.height = width, height
        return w


def config0() -> Workload:
    cam = Camera.look_at((0.0, -30.0, 3.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), lens_fov(24.0))
    return Workload("config0-schwarzschild-320x180-thin-disc-render", Schwarzschild(1.0), cam, 320, 180,
                    _abi.ST_SEM_RENDER, AccretionDisc(3.0, 20.0, Blackbody(), 0.0), _abi.ST_EMIT_KEPLER,
                    params=dict(samples=1, pixel_jitter=0))


def config1(nr=256, nphi=64, nz=32) -> Workload:
    a = 0.9
    pos = kerr_position(15.0, 80.0, a)
    cam = Camera.look_at(pos, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), lens_fov(24.0))
    vol = volume(nr, nphi, nz, 2.32, 25.0, 0.05)
    # the gas is the disc: its AccretionDisc (ISCO to 25M) supplies the blackbody
    # table; with a volume present the thin plane is not traced (src/metal.jl:1160)
    return Workload("config1-kerr0.9-1920x1080-volume", Kerr(1.0, a), cam, 1920, 1080, _abi.ST_SEM_DRAFT,
                    AccretionDisc(2.32, 25.0, Blackbody(), 0.0), _abi.ST_EMIT_KS_EXACT, vol=vol,
                    params=dict(samples=1, pixel_jitter=0, exit_landing=1))


def config1_thin() -> Workload:
    """config1's camera and hole with the thin disc (2.32-25) instead of gas."""
    w = config1()
    w.name = "config1-kerr0.9-thin-disc"
    w.vol = None
    w.disc = AccretionDisc(2.32, 25.0, Blackbody(), 0.0)
    return w


def config1_nogas() -> Workload:
    """config1's camera and hole with neither disc nor gas: every ray escapes or
    falls in (the frame the learned surrogate serves)."""
    w = config1()
    w.name = "config1-kerr0.9-no-disc-no-gas"
    w.vol = None
    w.disc = None
    return w


def config2(nframes=240, width=1280, height=720) -> Workload:
    cams = free_fall_track(30.0, 1.5, nframes, M=1.0, incl_deg=85.0, fov=lens_fov(24.0))
    return Workload("config2-freefall-240x1280x720", Schwarzschild(1.0), cams[0], width, height,
                    _abi.ST_SEM_DRAFT, AccretionDisc(3.0, 20.0, Blackbody(), 0.0), _abi.ST_EMIT_KS_EXACT,
                    params=dict(samples=1, pixel_jitter=0, nmax=20000, exit_landing=1), cams=cams)


def config4(nframes=8, width=3840, height=2160) -> Workload:
    a = 0.99
    cams = []
    for f in range(nframes):
        phi = 2 * math.pi * f / max(nframes, 1) * 0.05
        p0 = kerr_position(20.0, 85.0, a)
        c, s = math.cos(phi), math.sin(phi)
        pos = np.array([c * p0[0] - s * p0[1], s * p0[0] + c * p0[1], p0[2]])
        cam = Camera.look_at(pos, (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), lens_fov(24.0))
        # boost 0.3c along the prograde orbital direction (world frame)
        t = np.array([-math.sin(phi), math.cos(phi), 0.0])
        cam.velocity = 0.3 * t
        cams.append(cam)
    vol = volume(512, 128, 64, 1.45, 25.0, 0.05)
    return Workload("config4-kerr0.99-3840x2160-volume-boosted", Kerr(1.0, a), cams[0], width, height,
                    _abi.ST_SEM_DRAFT, AccretionDisc(1.45, 25.0, Blackbody(), 0.0), _abi.ST_EMIT_KS_EXACT,
                    vol=vol,
                    params=dict(samples=1, pixel_jitter=0, exit_landing=1), cams=cams)
