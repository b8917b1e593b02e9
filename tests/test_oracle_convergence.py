"""Oracle self-consistency: the fixed-step FP64 twin against the adaptive
Tsit5 (rtol 1e-10) on small frames of every semantics, the committed golden
records, and a planted mistake that the parity comparison must catch."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from spacetime_gb300 import _abi, workloads

from .golden.make_golden import SKY, cases
from .helpers import angle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "oracle_renders.npz")


@pytest.fixture(scope="module")
def small_sky():
    return workloads.sky(**SKY)


@pytest.mark.parametrize("name", list(cases()))
def test_oracle_reproduces_golden(oracle_lib, small_sky, name):
    g = np.load(GOLDEN)
    w, W, H = cases()[name]
    img, rays = O.scene_for(w, small_sky, O.INT_RK4, width=W, height=H).render()
    assert np.array_equal(rays["flags"], g[f"{name}.flags"])
    assert np.array_equal(rays["steps"], g[f"{name}.steps"])
    assert np.abs(rays["dir"] - g[f"{name}.dir"]).max() < 1e-9
    np.testing.assert_allclose(img, g[f"{name}.rgb"], rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("name", list(cases()))
def test_twin_converges_to_tsit5(oracle_lib, small_sky, name):
    w, W, H = cases()[name]
    w.params = dict(w.params, exit_landing=1)
    a_img, a = O.scene_for(w, small_sky, O.INT_RK4, width=W, height=H).render()
    b_img, b = O.scene_for(w, small_sky, O.INT_TSIT5, width=W, height=H).render()
    both = ((a["flags"] & O.RAY_ESCAPED) > 0) & ((b["flags"] & O.RAY_ESCAPED) > 0)
    d = angle(a["dir"][both], b["dir"][both])
    assert np.median(d) < 1e-8
    mism = ((a["flags"] & O.RAY_BLACK) != (b["flags"] & O.RAY_BLACK)).sum()
    assert mism <= max(2, 0.002 * W * H)
    rel = np.abs(a_img - b_img).sum(-1) / np.maximum(b_img.sum(-1), 1e-6)
    assert np.median(rel) < 1e-5


def test_planted_mistake_is_caught(oracle_lib, small_sky):
    """A 1e-6 relative error in the hole's mass (planted in the oracle) must
    exceed the FP64 twin tolerance the GPU parity tests use."""
    w, W, H = cases()["draft_schw_exact"]
    _, a = O.scene_for(w, small_sky, O.INT_RK4, width=W, height=H).render()
    sc = O.scene_for(w, small_sky, O.INT_RK4, width=W, height=H)
    sc.s.M = 1.0 + 1e-6
    _, b = sc.render()
    both = ((a["flags"] & O.RAY_ESCAPED) > 0) & ((b["flags"] & O.RAY_ESCAPED) > 0)
    assert np.median(angle(a["dir"][both], b["dir"][both])) > 1e-8
