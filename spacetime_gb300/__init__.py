"""GB300 (sm_103a) implementation of SpaceTime.jl's per-pixel null-geodesic
render path behind a C ABI (include/spacetime_gb300.h)."""
from . import _abi
from .api import (AccretionDisc, Blackbody, Camera, Context, DiscFluidSim, Kerr, Lens, RenderResult,
                  Schwarzschild, Starfield, camera_tetrad, render, render_depth, render_draft, render_frames,
                  step_sim)
from .scene import Volume, make_sky, make_volume

__all__ = [
    "_abi", "AccretionDisc", "Blackbody", "Camera", "Context", "DiscFluidSim", "Kerr", "Lens", "RenderResult",
    "Schwarzschild", "Starfield", "camera_tetrad", "render", "render_depth", "render_draft", "render_frames",
    "step_sim", "Volume", "make_sky", "make_volume",
]
