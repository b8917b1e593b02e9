"""Seeded synthetic inputs: the equirectangular sky, the gas density grid,
the blackbody table used to colour sky stars, and the camera set-ups of the
benchmark workloads.

There is no public dataset on this path; the reference renders a JPEG star
map (assets/starmap_g4k.jpg) and DiscVolume's fBm grid
(src/disc_volume.jl:175-271).  These generators produce inputs of the same
shapes and statistics from a seed, so every consumer sees identical bytes.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


# ---------------------------------------------------------------------------
# Blackbody colour (src/blackbody.jl:15-60), numpy, for sky star colours.
# ---------------------------------------------------------------------------

def _cie_gauss(lam, mu, s1, s2):
    s = np.where(lam < mu, s1, s2)
    return np.exp(-0.5 * ((lam - mu) / s) ** 2)


def blackbody_rgb(T: np.ndarray) -> np.ndarray:
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    lam = np.arange(380.0, 780.0 + 1e-9, 5.0)
    lm = lam * 1e-9
    B = 1.0 / (lm[None, :] ** 5 * (np.exp(0.014388 / (lm[None, :] * T[:, None])) - 1.0))
    xb = 1.056 * _cie_gauss(lam, 599.8, 37.9, 31.0) + 0.362 * _cie_gauss(lam, 442.0, 16.0, 26.7) \
        - 0.065 * _cie_gauss(lam, 501.1, 20.4, 26.2)
    yb = 0.821 * _cie_gauss(lam, 568.8, 46.9, 40.5) + 0.286 * _cie_gauss(lam, 530.9, 16.3, 31.1)
    zb = 1.217 * _cie_gauss(lam, 437.0, 11.8, 36.0) + 0.681 * _cie_gauss(lam, 459.0, 26.0, 13.8)
    X, Y, Z = (B * xb).sum(1), (B * yb).sum(1), (B * zb).sum(1)
    r = np.maximum(3.2406 * X - 1.5372 * Y - 0.4986 * Z, 0.0)
    g = np.maximum(-0.9689 * X + 1.8758 * Y + 0.0415 * Z, 0.0)
    b = np.maximum(0.0557 * X - 0.2040 * Y + 1.0570 * Z, 0.0)
    m = np.maximum(np.maximum(r, g), np.maximum(b, 1e-10))
    return np.stack([r / m, g / m, b / m], axis=1)


def blackbody_lut(wb_temperature=6500.0, table_min=500.0, table_max=30000.0, table_size=1024):
    ref = blackbody_rgb(np.array([wb_temperature]))[0]
    T = np.linspace(table_min, table_max, table_size)
    return (blackbody_rgb(np.maximum(T, 1.0)) / ref[None, :]).astype(np.float32)


# ---------------------------------------------------------------------------
# Sky: 2048x1024 float32 RGB, first index phi, stored (H, W, 3) C-order,
# which is the reference's (3, W, H) column-major layout byte for byte.
# ---------------------------------------------------------------------------

def make_sky(width=2048, height=1024, n_stars=20000, seed=1234, mu=-6.0, sigma=0.5,
             pareto_alpha=1.5, star_xm=0.05, t_lo=3000.0, t_hi=12000.0) -> np.ndarray:
    """Log-normal background exp(N(mu, sigma^2)) per texel plus point stars
    placed uniformly on the sphere, Pareto(alpha, x_m) brightness and
    blackbody colour at T ~ U(t_lo, t_hi), deposited bilinearly."""
    rng = np.random.default_rng(seed)
    sky = np.exp(rng.normal(mu, sigma, size=(height, width))).astype(np.float64)
    sky = np.repeat(sky[:, :, None], 3, axis=2)
    z = rng.uniform(-1.0, 1.0, n_stars)
    phi = rng.uniform(0.0, 2.0 * math.pi, n_stars)
    theta = np.arccos(z)
    flux = star_xm * (1.0 + rng.pareto(pareto_alpha, n_stars))
    T = rng.uniform(t_lo, t_hi, n_stars)
    lut = blackbody_lut()
    idx = np.clip(np.rint((T - 500.0) / (30000.0 - 500.0) * 1023).astype(int), 0, 1023)
    col = lut[idx].astype(np.float64) * flux[:, None]
    xf = phi / (2.0 * math.pi) * (width - 1)
    yf = theta / math.pi * (height - 1)
    x0 = np.clip(np.floor(xf).astype(int), 0, width - 1)
    y0 = np.clip(np.floor(yf).astype(int), 0, height - 1)
    x1 = np.minimum(x0 + 1, width - 1)
    y1 = np.minimum(y0 + 1, height - 1)
    fx = (xf - x0)[:, None]
    fy = (yf - y0)[:, None]
    for xx, yy, w in ((x0, y0, (1 - fx) * (1 - fy)), (x1, y0, fx * (1 - fy)),
                      (x0, y1, (1 - fx) * fy), (x1, y1, fx * fy)):
        np.add.at(sky, (yy, xx), col * w)
    return np.ascontiguousarray(sky.astype(np.float32))


# ---------------------------------------------------------------------------
# Gas density grid: (nr, nphi, nz) float32 column-major, stored as a numpy
# array of shape (nz, nphi, nr) C-order (the same bytes).
# ---------------------------------------------------------------------------

def _value_noise(lat, x, y, z):
    n = lat.shape[0]
    ix, iy, iz = np.floor(x).astype(np.int64), np.floor(y).astype(np.int64), np.floor(z).astype(np.int64)
    fx, fy, fz = x - ix, y - iy, z - iz
    fx = fx * fx * (3 - 2 * fx)
    fy = fy * fy * (3 - 2 * fy)
    fz = fz * fz * (3 - 2 * fz)

    def L(i, j, k):
        return lat[i % n, j % n, k % n]

    c00 = L(ix, iy, iz) + fx * (L(ix + 1, iy, iz) - L(ix, iy, iz))
    c10 = L(ix, iy + 1, iz) + fx * (L(ix + 1, iy + 1, iz) - L(ix, iy + 1, iz))
    c01 = L(ix, iy, iz + 1) + fx * (L(ix + 1, iy, iz + 1) - L(ix, iy, iz + 1))
    c11 = L(ix, iy + 1, iz + 1) + fx * (L(ix + 1, iy + 1, iz + 1) - L(ix, iy + 1, iz + 1))
    c0 = c00 + fy * (c10 - c00)
    c1 = c01 + fy * (c11 - c01)
    return c0 + fz * (c1 - c0)


def _fbm(lat, x, y, z, octaves=4, gain=0.5, lacunarity=2.1):
    w = np.array([0.5 * gain ** k for k in range(octaves)])
    w = w / w.sum()
    out = np.zeros_like(x)
    f = 1.0
    for k in range(octaves):
        out += w[k] * _value_noise(lat, x * f + 17.0 * k, y * f + 31.0 * k, z * f + 7.0 * k)
        f *= lacunarity
    return out


@dataclass
class Volume:
    density: np.ndarray      # (nz, nphi, nr) float32 C-order == (nr, nphi, nz) column-major
    log_s_in: float
    log_s_out: float
    z_max: float
    scale_height: float
    emission_scale: float = 0.8
    opacity_scale: float = 1.2
    march_stride: int = 2

    @property
    def shape(self):
        nz, nphi, nr = self.density.shape
        return nr, nphi, nz


def disc_radial_profile(s, inner, outer, M=1.0, falloff=0.0):
    """src/disc_volume.jl:274-283: the thin disc's opacity tapers."""
    R = s / (2 * M)
    R_in, R_out = inner / (2 * M), outer / (2 * M)
    iscotaper = np.clip((R ** 2 - R_in ** 2) * 0.3, 0.0, 1.0)
    T_emit = np.exp(10.034259 - 0.375 * np.log(R ** 2))
    outertaper = np.clip(T_emit / 1000.0, 0.0, 1.0)
    dens = np.clip((R_out - R) / (R_out - R_in), 0.0, 1.0)
    return iscotaper * outertaper * (dens ** falloff if falloff != 0 else 1.0)


def make_volume(inner=3.0, outer=20.0, M=1.0, nr=192, nphi=256, nz=48, scale_height=0.08,
                turbulence=0.8, spiral_twist=4.0, seed=7, falloff=0.0,
                emission_scale=0.8, opacity_scale=1.2, march_stride=2) -> Volume:
    """Gas grid in the form of DiscVolume (src/disc_volume.jl:175-271): radial
    profile x Gaussian slab exp(-z^2/2H^2), H = scale_height*s, times the
    log-normal turbulence exp(6 t (n - 1/2)) of a seeded value-noise fBm n on
    sheared (log s, phi + twist log(s/s_in), z/H) coordinates; log-spaced s,
    periodic phi, z in +-3 H(s_out); peak-normalised."""
    rng = np.random.default_rng(seed)
    lat = rng.random((64, 64, 64))
    z_max = 3.0 * scale_height * outer
    log_in, log_out = math.log(inner), math.log(outer)
    k = np.arange(nz)[:, None, None]
    j = np.arange(nphi)[None, :, None]
    i = np.arange(nr)[None, None, :]
    z = -z_max + k / (nz - 1) * 2 * z_max
    phi = j / nphi * 2 * math.pi
    s = np.exp(log_in + i / (nr - 1) * (log_out - log_in))
    H = scale_height * s
    rho0 = disc_radial_profile(s, inner, outer, M, falloff)
    slab = np.exp(-z ** 2 / (2 * H ** 2))
    u = phi + spiral_twist * np.log(s / inner)
    shape = np.broadcast_shapes(z.shape, phi.shape, s.shape)
    X = np.broadcast_to(8.0 * np.log(s), shape)
    Y = np.broadcast_to(u * (64 / (2 * math.pi)) / 4.0, shape)
    Zc = np.broadcast_to(2.0 * z / H, shape)
    n = _fbm(lat, X, Y, Zc)
    # close the azimuthal seam: crossfade the last 18 deg onto the phi - 2 pi branch
    blend = math.radians(18.0)
    Y2 = np.broadcast_to((u - 2 * math.pi) * (64 / (2 * math.pi)) / 4.0, shape)
    n2 = _fbm(lat, X, Y2, Zc)
    wphi = np.clip((phi - (2 * math.pi - blend)) / blend, 0.0, 1.0)
    wphi = wphi * wphi * (3 - 2 * wphi)
    n = (1 - wphi) * n + wphi * n2
    turb = np.exp(6.0 * turbulence * (n - 0.5))
    dens = (rho0 * slab * turb).astype(np.float32)
    peak = dens.max()
    if peak > 0:
        dens /= peak
    return Volume(np.ascontiguousarray(dens), float(np.float32(log_in)), float(np.float32(log_out)),
                  float(np.float32(z_max)), scale_height, emission_scale, opacity_scale, march_stride)


# ---------------------------------------------------------------------------
# Cameras (src/camera.jl:36-50, src/raytrace.jl:22-29).
# ---------------------------------------------------------------------------

def _normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.linalg.norm(v)


@dataclass
class Camera:
    pos: np.ndarray
    fwd: np.ndarray
    right: np.ndarray
    up_local: np.ndarray
    fov_factor: float
    velocity: np.ndarray
    projection: int = 0
    fisheye_deg: float = 0.0
    aperture_world: float = 0.0
    focus_dist: float = 1.0

    @classmethod
    def look_at(cls, pos, target, up, fov_factor=1.0, velocity=(0.0, 0.0, 0.0)):
        pos = np.asarray(pos, dtype=np.float64)
        fwd = _normalize(np.asarray(target, dtype=np.float64) - pos)
        right = _normalize(np.cross(fwd, np.asarray(up, dtype=np.float64)))
        up_local = np.cross(right, fwd)
        return cls(pos, fwd, right, up_local, float(fov_factor), np.asarray(velocity, dtype=np.float64))


def lens_fov(focal_length_mm: float) -> float:
    """Lens(f): fov_factor = 18/f (src/raytrace.jl:22-26)."""
    return 18.0 / focal_length_mm


def camera_beta(cam: Camera) -> np.ndarray:
    """src/camera.jl:19-22."""
    return np.array([cam.velocity @ cam.fwd, cam.velocity @ cam.right, cam.velocity @ cam.up_local])


def kerr_position(r_ks: float, incl_deg: float, a: float) -> np.ndarray:
    """Cartesian KS position at Boyer-Lindquist-like (r, theta), azimuth 0."""
    th = math.radians(incl_deg)
    return np.array([math.sqrt(r_ks * r_ks + a * a) * math.sin(th), 0.0, r_ks * math.cos(th)])
