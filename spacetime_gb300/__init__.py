"""GB300 (sm_103a) implementation of SpaceTime.jl's per-pixel null-geodesic
render path behind a C ABI (include/spacetime_gb300.h)."""
from . import _abi
from .api import (AccretionDisc, Blackbody, Camera, Context, Kerr, Lens, RenderResult, Schwarzschild,
                  camera_tetrad, render, render_draft, render_frames)
from .scene import Volume, make_sky, make_volume

__all__ = [
    "_abi", "AccretionDisc", "Blackbody", "Camera", "Context", "Kerr", "Lens", "RenderResult",
    "Schwarzschild", "camera_tetrad", "render", "render_draft", "render_frames", "Volume", "make_sky",
    "make_volume",
]
