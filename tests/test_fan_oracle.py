"""The deflection fan's twin in the oracle (orc_trace_dirs), host side: a
radially outward ray goes straight out, the escape flag is monotone in psi,
and the escape/capture transition sits at the shadow edge of a static
observer, sin(alpha) = 3 sqrt(3) M / r * sqrt(1 - 2M / r) (Synge 1966), within
the fan's own resolution and the fixed step's error."""
import math

import numpy as np

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads
from spacetime_gb300.scene import Camera


def _fan_scene(r):
    cam = Camera(np.array([r, 0.0, 0.0]), np.array([1.0, 0, 0]), np.array([0, 1.0, 0]), np.array([0, 0, 1.0]),
                 1.0, np.zeros(3))
    w = workloads.Workload("fan", workloads.Schwarzschild(1.0), cam, 4, 4, _abi.ST_SEM_DRAFT, None,
                           _abi.ST_EMIT_KS_EXACT, params=dict(samples=1, pixel_jitter=0, exit_landing=1))
    return O.scene_for(w, workloads.sky(64, 32), O.INT_RK4)


def test_fan_twin_geometry(oracle_lib):
    for r in (8.0, 30.0):
        sc = _fan_scene(r)
        n = 2048
        psi = math.pi * np.arange(n) / (n - 1)
        rays = sc.trace_dirs(np.stack([np.cos(psi), np.sin(psi), np.zeros(n)], 1))
        esc = (rays["flags"] & O.RAY_BLACK) == 0
        # straight out along the radial axis
        assert esc[0] and abs(rays["dir"][0][1]) < 1e-12 and rays["dir"][0][0] > 0.999999
        # one transition, escape below it, capture above
        k = np.nonzero(esc[:-1] != esc[1:])[0]
        assert k.size == 1 and esc[: k[0] + 1].all() and not esc[k[0] + 1:].any()
        alpha = math.asin(3 * math.sqrt(3) / r * math.sqrt(1 - 2 / r))
        psi_c = 0.5 * (psi[k[0]] + psi[k[0] + 1])
        assert abs(psi_c - (math.pi - alpha)) <= 2 * math.pi / (n - 1) + 2e-3, (r, psi_c, math.pi - alpha)
        # in-plane: no out-of-plane exit component
        assert np.abs(rays["dir"][esc][:, 2]).max() < 1e-12
