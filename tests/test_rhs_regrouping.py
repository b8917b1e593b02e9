"""The float units' regrouped geodesic right-hand sides are the same algebra as
the reference's term-by-term form (src/metal.jl:466-508 Kerr, src/gr.jl:85-109
Schwarzschild), which the oracle restates.

The regrouping in spacetime_gb300/csrc/st_trace.cuh (rhs_kerr_f32, the float
branch of rhs_schw, ks_r2_f32) is written out here in FP64 numpy, operation
for operation, and compared with the oracle's RHS on seeded states around the
hole: in FP64 the two forms must agree to rounding (1e-12 of the largest
component), so any difference on the GPU is float rounding, not algebra.
"""
import numpy as np

from oracle import oracle as O


def ks_r2_half_w(x, y, z, a):
    """KS r^2 from the quartic with w/2 = (x^2 + y^2 + z^2 - a^2)/2."""
    wh = (x * x + y * y + z * z) * 0.5 - 0.5 * a * a
    return wh + np.sqrt(wh * wh + a * a * z * z)


def kerr_regrouped(s, pt, M, a):
    x, y, z, px, py, pz = s
    a2 = a * a
    q = a2 * z * z
    r2 = max(ks_r2_half_w(x, y, z, a), 1e-12)
    ir = 1.0 / np.sqrt(r2)
    r = r2 * ir
    isig = 1.0 / (r2 * r2 + q)
    r2a = r2 + a2
    ira = 1.0 / r2a
    A = px * x + py * y
    B = px * y - py * x
    T = (r * A + a * B) * ira
    Z = z * pz * ir
    ell = (T + Z) - pt
    rsig = r2 * r * isig
    fl = 2.0 * M * rsig * ell
    Fi = fl * ira
    Fr, Fa = Fi * r, Fi * a
    flir = fl * ir
    dldr = (A - 2.0 * r * T) * ira - Z * ir
    inner = ell * ir * (2.0 * q * isig - 0.5) + dldr
    G = fl * inner
    Gr = G * rsig
    return np.array([
        px - Fr * x - Fa * y,
        py - Fr * y + Fa * x,
        pz - flir * z,
        Gr * x + Fr * px - Fa * py,
        Gr * y + Fr * py + Fa * px,
        z * isig * (G * r * r2a - a2 * ell * fl) + flir * pz,
    ])


def schw_regrouped(s, pt, M):
    x, y, z, px, py, pz = s
    ir = 1.0 / np.sqrt(x * x + y * y + z * z)
    f = 2.0 * M * ir
    kap = (x * px + y * py + z * pz) * ir
    ell = kap - pt
    c1 = f * ell * ir
    c2 = c1 * (0.5 * ell + kap) * ir
    return np.array([px - c1 * x, py - c1 * y, pz - c1 * z,
                     c1 * px - c2 * x, c1 * py - c2 * y, c1 * pz - c2 * z])


def _states(n, seed):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        pos = rng.normal(size=3)
        pos *= rng.uniform(1.6, 60.0) / np.linalg.norm(pos)
        yield pos, rng.normal(size=3), -rng.uniform(0.3, 3.0)


def test_kerr_regrouped_matches_oracle():
    worst = 0.0
    for k, (pos, p, pt) in enumerate(_states(3000, 11)):
        a = (-0.999, -0.5, 0.3, 0.9, 0.998)[k % 5]
        s = np.concatenate([pos, p])
        ref = O.rhs(True, s, pt, 1.0, a)
        got = kerr_regrouped(s, pt, 1.0, a)
        worst = max(worst, float(np.abs(got - ref).max() / np.abs(ref).max()))
    assert worst <= 1e-12, worst


def test_kerr_regrouped_near_the_ring_and_the_plane():
    """States on the equatorial plane and just off the ring radius |(x, y)| = a,
    where Sigma and r are smallest relative to their terms."""
    worst = 0.0
    rng = np.random.default_rng(12)
    for a in (0.5, 0.9, 0.99):
        for _ in range(400):
            phi = rng.uniform(0, 2 * np.pi)
            rho = a + rng.uniform(0.05, 3.0)
            pos = np.array([rho * np.cos(phi), rho * np.sin(phi), rng.choice([0.0, rng.normal() * 0.01])])
            s = np.concatenate([pos, rng.normal(size=3)])
            pt = -rng.uniform(0.3, 3.0)
            ref = O.rhs(True, s, pt, 1.0, a)
            got = kerr_regrouped(s, pt, 1.0, a)
            worst = max(worst, float(np.abs(got - ref).max() / np.abs(ref).max()))
    assert worst <= 1e-10, worst


def test_schwarzschild_regrouped_matches_oracle():
    worst = 0.0
    for pos, p, pt in _states(2000, 13):
        s = np.concatenate([pos, p])
        ref = O.rhs(False, s, pt, 1.0, 0.0)
        got = schw_regrouped(s, pt, 1.0)
        worst = max(worst, float(np.abs(got - ref).max() / np.abs(ref).max()))
    assert worst <= 1e-12, worst
