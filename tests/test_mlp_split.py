"""The split-bf16 edge layers of the tensor-core network kernel, on the CPU.

sur_mlp_tc_kernel runs the network's FP32 edge layers on the tensor cores
as products of bf16 pairs (hi = bf16(v), lo = bf16(v - hi)): layer 0 as
x_hi.w_hi + x_lo.w_hi + x_hi.w_lo + b_hi + b_lo (x_lo.w_lo dropped), layer 4
with w_hi + w_lo against the bf16 activations.  oracle.mlp_oracle restates
that arithmetic (forward_split); here it is checked against the FP64 edge
layers of forward_bf16 on the shipped network and on the network's own input
distribution:
- each layer-0 pre-activation within 2^-15 of sum |x_i w_i| + |b| of the
  exact one (each term of the split carries ~2^-16; the dropped x_lo.w_lo
  term is 2^-16 of |x w|);
- the outputs: median difference <= 1e-6 of each output's scale, 99.9th
  percentile <= 5e-3 -- the tail is the occasional hidden unit whose value
  sits on a bf16 rounding boundary and rounds to the other neighbour.
"""
import os

import numpy as np

from oracle import mlp_oracle as MO

SHIPPED = os.path.join(os.path.dirname(__file__), "..", "spacetime_gb300", "data", "surrogate_kerr.npy")


def test_split_pair_represents_fp32_values():
    v = np.random.default_rng(3).normal(0, 3, 100000).astype(np.float32).astype(np.float64)
    hi, lo = MO.split_bf16(v)
    assert np.all(np.abs(hi + lo - v) <= 2.0 ** -16 * np.abs(v))


def test_split_edge_layers_against_the_fp64_edges():
    P = np.load(SHIPPED)
    rng = np.random.default_rng(11)
    # inputs like the network's: camera radius, inclination, spin normalised to [-1, 1],
    # a unit direction
    n = 4000
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    X = np.concatenate([rng.uniform(-1, 1, (n, 3)), d], axis=1).astype(np.float32)
    out_split, z0 = MO.forward_split(P, X)
    w = MO.unpack(P)
    Xd = X.astype(np.float64)
    z_exact = Xd @ w["W0"].T + w["b0"]
    bound = 2.0 ** -15 * (np.abs(Xd) @ np.abs(w["W0"]).T + np.abs(w["b0"]))
    assert np.all(np.abs(z0 - z_exact) <= bound)
    ref = MO.forward_bf16(P, X)
    cols = [0, 1, 3, 4, 5]
    e = np.abs(out_split - ref)[:, cols] / np.abs(ref[:, cols]).max(0)
    print("median", np.median(e), "p99.9", np.percentile(e, 99.9), "max", e.max())
    assert np.median(e) <= 1e-6 and np.percentile(e, 99.9) <= 5e-3
