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

def _lat(lat, i, j, k):
    """Lattice value at integer cell (i, j, k), periodic in 64 (_lat,
    src/disc_volume.jl:287-288)."""
    return lat[np.mod(i, 64), np.mod(j, 64), np.mod(k, 64)]


def _value_noise(lat, x, y, z):
    """Trilinear value noise with smoothstep weights (src/disc_volume.jl:290-307)."""
    ix, iy, iz = np.floor(x).astype(np.int64), np.floor(y).astype(np.int64), np.floor(z).astype(np.int64)
    fx, fy, fz = x - ix, y - iy, z - iz
    fx = fx * fx * (3 - 2 * fx)
    fy = fy * fy * (3 - 2 * fy)
    fz = fz * fz * (3 - 2 * fz)

    def L(i, j, k):
        return _lat(lat, i, j, k)

    c00 = L(ix, iy, iz) + fx * (L(ix + 1, iy, iz) - L(ix, iy, iz))
    c10 = L(ix, iy + 1, iz) + fx * (L(ix + 1, iy + 1, iz) - L(ix, iy + 1, iz))
    c01 = L(ix, iy, iz + 1) + fx * (L(ix + 1, iy, iz + 1) - L(ix, iy, iz + 1))
    c11 = L(ix, iy + 1, iz + 1) + fx * (L(ix + 1, iy + 1, iz + 1) - L(ix, iy + 1, iz + 1))
    c0 = c00 + fy * (c10 - c00)
    c1 = c01 + fy * (c11 - c01)
    return c0 + fz * (c1 - c0)


def _fbm(lat, x, y, z, octaves=4, gain=0.5, lacunarity=2.1):
    """Octaves of value noise, each `lacunarity` finer and `gain` weaker,
    normalised by the sum of amplitudes (_fbm, src/disc_volume.jl:336-347)."""
    amp, freq, total, norm = 0.5, 1.0, 0.0, 0.0
    for _ in range(octaves):
        total = total + amp * _value_noise(lat, x * freq, y * freq, z * freq)
        norm += amp
        amp *= gain
        freq *= lacunarity
    return total / norm


VEIN_SCALE = 2.5  # src/disc_volume.jl:350


def _worley(lat, x, y, z, ridge=True):
    """Cellular noise over the 3x3x3 neighbourhood, one feature point per
    lattice cell drawn from the lattice at three offsets: F2 - F1 (scaled by
    VEIN_SCALE) for ridge, else 1 - F1, clamped to [0, 1] (_worley,
    src/disc_volume.jl:373-399)."""
    ix, iy, iz = np.floor(x).astype(np.int64), np.floor(y).astype(np.int64), np.floor(z).astype(np.int64)
    f1 = np.full(np.shape(x), np.inf)
    f2 = np.full(np.shape(x), np.inf)
    for dk in (-1, 0, 1):
        for dj in (-1, 0, 1):
            for di in (-1, 0, 1):
                cx, cy, cz = ix + di, iy + dj, iz + dk
                px = cx + _lat(lat, cx, cy, cz)
                py = cy + _lat(lat, cx + 17, cy + 31, cz + 7)
                pz = cz + _lat(lat, cx + 43, cy + 11, cz + 29)
                d = (px - x) ** 2 + (py - y) ** 2 + (pz - z) ** 2
                closer = d < f1
                f2 = np.where(closer, f1, np.where(d < f2, d, f2))
                f1 = np.where(closer, d, f1)
    f1, f2 = np.sqrt(f1), np.sqrt(f2)
    return np.clip(VEIN_SCALE * (f2 - f1), 0.0, 1.0) if ridge else np.clip(1.0 - f1, 0.0, 1.0)


def _worley_fbm(lat, x, y, z, octaves, gain=0.5, lacunarity=2.0, ridge=True):
    """Octaves of Worley noise, normalised (_worley_fbm, src/disc_volume.jl:410-422)."""
    amp, freq, total, norm = 0.5, 1.0, 0.0, 0.0
    for _ in range(octaves):
        total = total + amp * _worley(lat, x * freq, y * freq, z * freq, ridge=ridge)
        norm += amp
        amp *= gain
        freq *= lacunarity
    return total / norm


def _shape_coverage(lat, ls, u, zh, octaves, gain, lac, erosion, escale, eoct, eridge):
    """Base fBm on (10 ln s, 6 u, zh), carved by the Worley detail field with
    the cloud remap (base - e w) / (1 - e w) when erosion > 0
    (_shape_coverage, src/disc_volume.jl:454-464)."""
    n = _fbm(lat, 10.0 * ls, 6.0 * u, zh, octaves, gain, lac)
    if erosion <= 0.0:
        return n
    w = _worley_fbm(lat, escale * 10.0 * ls, escale * 6.0 * u, escale * zh, eoct, ridge=eridge)
    ew = erosion * w
    return np.clip((n - ew) / (1.0 - ew), 0.0, 1.0)


WRAP_BLEND = math.radians(18.0)  # src/disc_volume.jl:164
HAZE_WINDOW = 0.6                # src/disc_volume.jl:173


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
                emission_scale=0.8, opacity_scale=1.2, march_stride=2, noise_octaves=4, noise_gain=0.5,
                noise_lacunarity=2.1, haze=0.0, haze_height=4.0, erosion=0.0, erosion_scale=4.0,
                erosion_octaves=3, erosion_mode="billow") -> Volume:
    """The gas grid of DiscVolume(disc; ...) (src/disc_volume.jl:175-271),
    restated in numpy with the same keywords and defaults: radial profile x
    Gaussian slab exp(-z^2/2H^2), H = scale_height s (plus the windowed haze
    envelope when haze > 0), times the log-normal turbulence
    exp(6 turbulence (n - 1/2)) of the coverage field n -- value-noise fBm on
    sheared coordinates (10 ln s, 6 (phi + spiral_twist ln(s/s_in)), 2 z/H),
    optionally carved by Worley noise -- with the last 18 deg of azimuth
    crossfaded onto the phi - 2 pi branch; log-spaced s, periodic phi, z in
    +-3 H(s_out); peak-normalised.  The 64^3 noise lattice is uniform [0, 1)
    float32 from a seeded numpy generator (the reference draws it from its
    `rng` argument, a Julia stream this cannot reproduce), so the field has the
    reference's construction and statistics, not its bytes."""
    if erosion_mode not in ("vein", "billow"):
        raise ValueError(f"erosion_mode must be 'vein' or 'billow', got {erosion_mode!r}")
    eridge = erosion_mode == "vein"
    ero = min(max(float(erosion), 0.0), 0.95)
    rng = np.random.default_rng(seed)
    lat = rng.random((64, 64, 64), dtype=np.float32)
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
    if haze > 0.0:
        Hh = haze_height * H
        t = np.clip((np.abs(z / z_max) - HAZE_WINDOW) / (1.0 - HAZE_WINDOW), 0.0, 1.0)
        slab = slab + haze * np.exp(-z ** 2 / (2 * Hh ** 2)) * (1.0 - t * t * (3.0 - 2.0 * t))
    shape = np.broadcast_shapes(z.shape, phi.shape, s.shape)
    u = phi + spiral_twist * np.log(s / inner)
    ls = np.broadcast_to(np.log(s), shape)
    U = np.broadcast_to(u, shape)
    ZH = np.broadcast_to(2.0 * z / H, shape)
    args = (noise_octaves, noise_gain, noise_lacunarity, ero, erosion_scale, erosion_octaves, eridge)
    n = _shape_coverage(lat, ls, U, ZH, *args)
    # the wrap sector: crossfade onto the phi - 2 pi branch of the noise
    jw = np.nonzero(phi[0, :, 0] > 2 * math.pi - WRAP_BLEND)[0]
    if jw.size:
        n2 = _shape_coverage(lat, ls[:, jw, :], U[:, jw, :] - 2 * math.pi, ZH[:, jw, :], *args)
        w = (phi[:, jw, :] - (2 * math.pi - WRAP_BLEND)) / WRAP_BLEND
        w = w * w * (3.0 - 2.0 * w)
        n = np.array(n)
        n[:, jw, :] = (1.0 - w) * n[:, jw, :] + w * n2
    turb = np.exp(6.0 * turbulence * (n - 0.5))
    dens = (rho0 * slab * turb).astype(np.float32)
    peak = dens.max()
    if peak > 0:
        dens /= peak
    return Volume(np.ascontiguousarray(dens), float(np.float32(log_in)), float(np.float32(log_out)),
                  float(np.float32(z_max)), float(np.float32(scale_height)), emission_scale, opacity_scale,
                  march_stride)


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
