"""Free-falling camera worldline (host side, FP64), restating src/ship.jl.

    ks_gdot / ks_raise / ks_lower     src/ship.jl:22-58
    ShipState(pos, M)                 src/ship.jl:79-88
    ship_velocity(ship, M, f, r, u)   src/ship.jl:99-108
    step_ship(ship, M, dtau)          src/ship.jl:130-166 (coasting, no thrust)

The ship's beta against the local reference observer becomes the camera's
world-frame velocity, which the renderer turns into the Lorentz-boosted
tetrad (src/preview.jl:180-196).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .scene import Camera


def ks_gdot(pos, M, A, B):
    r = np.linalg.norm(pos)
    f = 2.0 * M / r
    lA = A[0] + pos @ A[1:] / r
    lB = B[0] + pos @ B[1:] / r
    return -A[0] * B[0] + A[1:] @ B[1:] + f * lA * lB


def ks_raise(pos, M, p_t, p):
    r = np.linalg.norm(pos)
    xh = pos / r
    f = 2.0 * M / r
    ell = -p_t + xh @ p
    return np.concatenate([[-p_t + f * ell], p - (f * ell) * xh])


def ks_lower(pos, M, u):
    r = np.linalg.norm(pos)
    xh = pos / r
    f = 2.0 * M / r
    lu = u[0] + xh @ u[1:]
    return -u[0] + f * lu, u[1:] + (f * lu) * xh


def _static_tetrad(pos, fwd, right, up, M):
    """Unboosted ks_camera_tetrad for a = 0 (src/preview.jl:99-110, 164-178)."""
    r = np.linalg.norm(pos)
    l = pos / r
    f = 2.0 * M / r
    E = math.sqrt(max(1.0 - 2.0 / 2.5, 1.0 - f))
    v = -math.sqrt(max(E * E - (1.0 - f), 0.0))
    w = (1.0 - E * (E - v)) / (E - v)
    lu = E + w
    u = np.concatenate([[E + f * lu], (w - f * lu) * l])

    def g(A, B):
        return -A[0] * B[0] + A[1:] @ B[1:] + f * (A[0] + l @ A[1:]) * (B[0] + l @ B[1:])

    Ef = np.concatenate([[0.0], fwd]); Ef = Ef + g(Ef, u) * u; Ef = Ef / math.sqrt(g(Ef, Ef))
    Er = np.concatenate([[0.0], right]); Er = Er + g(Er, u) * u; Er = Er - g(Er, Ef) * Ef
    Er = Er / math.sqrt(g(Er, Er))
    Eu = np.concatenate([[0.0], up]); Eu = Eu + g(Eu, u) * u; Eu = Eu - g(Eu, Ef) * Ef - g(Eu, Er) * Er
    Eu = Eu / math.sqrt(g(Eu, Eu))
    return u, Ef, Er, Eu


@dataclass
class ShipState:
    x: np.ndarray
    p: np.ndarray
    p_t: float
    tau: float = 0.0
    t: float = 0.0

    @classmethod
    def at_rest(cls, pos, M):
        pos = np.asarray(pos, dtype=np.float64)
        fwd = np.array([0.0, 0.0, 1.0]) if abs(pos[2]) < 0.9 * np.linalg.norm(pos) else np.array([1.0, 0.0, 0.0])
        right = np.cross(fwd, pos)
        right /= np.linalg.norm(right)
        up = np.cross(right, fwd)
        u = _static_tetrad(pos, fwd, right, up, M)[0]
        p_t, p = ks_lower(pos, M, u)
        return cls(pos.copy(), p, p_t)


def _ks_rhs(mu, p_t, M):
    x, p = mu[:3], mu[3:]
    r2 = x @ x
    inv_r = 1.0 / math.sqrt(r2)
    f = 2.0 * M * inv_r
    kap = (x @ p) * inv_r
    ell = -p_t + kap
    c1 = f * ell * inv_r
    c2 = f * ell * (0.5 * ell + kap) * inv_r * inv_r
    return np.concatenate([p - c1 * x, c1 * p - c2 * x])


def _rk4(mu, p_t, M, h):
    k1 = _ks_rhs(mu, p_t, M)
    k2 = _ks_rhs(mu + 0.5 * h * k1, p_t, M)
    k3 = _ks_rhs(mu + 0.5 * h * k2, p_t, M)
    k4 = _ks_rhs(mu + h * k3, p_t, M)
    return mu + (h / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)


def step_ship(ship: ShipState, M: float, dtau: float) -> ShipState:
    """Coasting geodesic step by proper time dtau with radius-adaptive RK4
    substeps and a final mass-shell renormalisation."""
    if dtau <= 0.0:
        return ship
    rem = dtau
    while rem > 1e-12:
        r = np.linalg.norm(ship.x)
        h = min(rem, 0.015 * min(max(r / M, 0.4), 30.0) * M)
        ship.t += ks_raise(ship.x, M, ship.p_t, ship.p)[0] * h
        mu = _rk4(np.concatenate([ship.x, ship.p]), ship.p_t, M, h)
        ship.x, ship.p = mu[:3], mu[3:]
        ship.tau += h
        rem -= h
    u = ks_raise(ship.x, M, ship.p_t, ship.p)
    u = u / math.sqrt(max(-ks_gdot(ship.x, M, u, u), 1e-6))
    ship.p_t, ship.p = ks_lower(ship.x, M, u)
    return ship


def ship_velocity(ship: ShipState, M, fwd, right, up):
    u = ks_raise(ship.x, M, ship.p_t, ship.p)
    u_ref, Ef, Er, Eu = _static_tetrad(ship.x, fwd, right, up, M)
    gam = -ks_gdot(ship.x, M, u, u_ref)
    beta = np.array([ks_gdot(ship.x, M, u, Ef), ks_gdot(ship.x, M, u, Er), ks_gdot(ship.x, M, u, Eu)]) / gam
    return beta, gam


def free_fall_track(r0: float, r1: float, nframes: int, M=1.0, incl_deg=85.0, fov=0.75):
    """Cameras at equal proper-time spacing on a radial free fall from rest at
    r0 down to r1, looking at the hole, each boosted by the ship's velocity."""
    th = math.radians(incl_deg)
    n = np.array([0.0, -math.sin(th), math.cos(th)])
    probe = ShipState.at_rest(r0 * n, M)
    dt_probe = 0.05
    while np.linalg.norm(probe.x) > r1:
        step_ship(probe, M, dt_probe)
    tau_end = probe.tau
    ship = ShipState.at_rest(r0 * n, M)
    cams = []
    for k in range(nframes):
        target = tau_end * k / max(nframes - 1, 1)
        step_ship(ship, M, target - ship.tau)
        cam = Camera.look_at(ship.x.copy(), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), fov)
        beta, _ = ship_velocity(ship, M, cam.fwd, cam.right, cam.up_local)
        cam.velocity = beta[0] * cam.fwd + beta[1] * cam.right + beta[2] * cam.up_local
        cams.append(cam)
    return cams
