"""Train the exit-direction surrogate on the GPU and save its parameters.

    python -m spacetime_gb300.train_surrogate --samples 50331648 --steps 200000 \
        --out spacetime_gb300/data/surrogate_kerr.npy

The shipped spacetime_gb300/data/surrogate_kerr.npy was made by exactly this
command on one GB300 (label generation ~95 s, training ~85 s): FP64 labels of
Sobol-sampled rays (camera r in [4, 50] M, inclination [0, 90] deg, spin
[0, 0.99], 80% of directions in the 75-degree inward cone), AdamW on batches of
16384 with a cosine learning rate from 2e-3 to 1e-5 and weight decay 1e-6.
Training uses atomics in its weight-gradient reductions, so a rerun gives a
network of the same accuracy, not the same bits: the same command on a GB300
with the tcgen05 training GEMMs (the default) gave held-out exit-direction
errors of 9.35e-5 rad median (9.30e-5 for the shipped network), and with the
mma.sync GEMMs (SPACETIME_GB300_TRAIN_MMA=sync) 1.03e-4.  The schedule matters:
four times the steps at the same peak learning rate diverged (a loss spike
near step 100000, from which the variance output never recovered).
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from .surrogate import Surrogate


def train(samples: int, steps: int, seed: int = 1, device: int = 0, batch: int = 16384, chunk: int = 2000,
          lr_max: float = 2e-3, lr_min: float = 1e-5, weight_decay: float = 1e-6, log=print) -> Surrogate:
    s = Surrogate(device, seed=seed)
    t0 = time.time()
    s.generate(samples, offset=0, copy=False)
    log(f"labels: {samples} rays in {time.time() - t0:.1f} s")
    n = max(steps // chunk, 1)
    t0 = time.time()
    for k in range(n):
        frac = k / max(n - 1, 1)
        lr = lr_min + 0.5 * (lr_max - lr_min) * (1 + np.cos(np.pi * frac))
        h = s.train(chunk, batch=batch, lr=lr, weight_decay=weight_decay)
        if k % 10 == 0 or k == n - 1:
            log(f"step {(k + 1) * chunk} lr {lr:.2e} loss {h[-100:].mean():.4f} t {time.time() - t0:.1f}")
    return s


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=50331648)
    ap.add_argument("--steps", type=int, default=200000)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    s = train(a.samples, a.steps, seed=a.seed)
    np.save(a.out, s.get_params())
    s.close()


if __name__ == "__main__":
    main()
