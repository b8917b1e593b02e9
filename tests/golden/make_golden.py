"""Regenerate tests/golden/oracle_renders.npz: per-ray records of the FP64
oracle's fixed-step twin on small, seeded versions of the benchmark scenes.

The reference (Julia + Metal) cannot run here, so these vectors freeze the
oracle's output: the CPU tests check the oracle still reproduces them and
the GPU tests check the CUDA path against them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from spacetime_gb300 import _abi, workloads  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_renders.npz")
SKY = dict(width=512, height=256, seed=99)


def cases():
    """name -> (workload, width, height)"""
    c0 = workloads.config0()
    d0 = workloads.config0()
    d0.semantics, d0.emitter = _abi.ST_SEM_DRAFT, _abi.ST_EMIT_KS_EXACT
    d0.params = dict(samples=1, pixel_jitter=0, exit_landing=0)
    kt = workloads.config1_thin()
    kt.params = dict(samples=1, pixel_jitter=0, exit_landing=0)
    kv = workloads.config1(nr=64, nphi=32, nz=16)
    return {
        "render_schw_kepler": (c0, 48, 27),
        "draft_schw_exact": (d0, 48, 27),
        "draft_kerr09_thin": (kt, 48, 27),
        "draft_kerr09_gas": (kv, 32, 18),
    }


def main():
    sky = workloads.sky(**SKY)
    out = {}
    for name, (w, W, H) in cases().items():
        img, rays = O.scene_for(w, sky, O.INT_RK4, width=W, height=H).render()
        out[f"{name}.rgb"] = img
        out[f"{name}.dir"] = rays["dir"]
        out[f"{name}.flags"] = rays["flags"]
        out[f"{name}.steps"] = rays["steps"]
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
