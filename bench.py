"""Benchmark of the render path: Mrays/s on the 1080p Kerr a=0.9 frame.

Workload (one "step" = one full frame): Kerr a=0.9 M=1, static camera at KS
r=15 M, inclination 80 deg, Lens(24), 1920x1080 float32 HDR, volumetric gas
256x64x32 from the ISCO (2.32 M) to 25 M (scale height 0.05 r), 2048x1024
synthetic sky, kernel (render_draft_mtl) rules, samples=1 at pixel centres,
exit landing on r_escape.  All inputs are seeded synthetic data.

    value     Mrays/s with inputs resident in HBM: CUDA-event time of the trace
              launch on the library's stream, L2 flushed (256 MiB write)
              between timed steps.
    e2e       the same metric through st_render with a host output buffer
              (device->host copy of the frame inside the timed region).
    roofline  FP32 compute roof of the trace kernel (algorithmic flops per
              step counted from the source, x accepted steps, / launch time).
    cpu_baseline  the FP64 oracle (Tsit5, rtol 1e-10) on a bounded crop.

`--impl reference` times the reference's CPU path as restated by the oracle
(the reference itself is Julia + Metal and cannot run here).
Multi-GPU: replicas only (each rank renders its own frames; no collective on
the data path); value = rays of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s 1080p Kerr a=0.9: surrogate+FP32 vs plain RK4, same GB300, ≤1e-4 rad"
UNIT = "Mrays/s"
# surrogate gates (max predicted std-dev of the exit angles, rad): the widest
# that keeps the frame's exit directions inside the 1e-4 / 1e-3 rad target on
# the no-disc 1080p frame, and a wider one that serves about half of it
SIGMA_TARGET = 2e-4
SIGMA_WIDE = 4e-4

# Algorithmic flops, counted from spacetime_gb300/csrc/st_trace.cuh (every
# add, mul, div, sqrt, rsqrt, rcp, exp, log, atan2 counted as one).
FLOPS_RHS_KERR = 126
FLOPS_RHS_SCHW = 34
FLOPS_RK4_UPDATE = 74
# One gas sample (march_gas + sample_volume, FP64 form): 52 for every sample
# (position and its cylinder radius and angle, the log-radial grid index, the
# trilinear density) plus 77 for an emitting one (blackbody temperature, the
# emitter's redshift, the colour-table index, Planck factor, absorption,
# compositing); 62 % of the config-1 frame's samples emit, so 52 + 0.62 * 77.
FLOPS_GAS_SAMPLE = 100


def flops_per_step(kerr: bool) -> int:
    return 4 * (FLOPS_RHS_KERR if kerr else FLOPS_RHS_SCHW) + FLOPS_RK4_UPDATE


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, path: str | None = None):
        self.index = index
        self.rows = []
        self.proc = None
        self.path = path

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        if self.path:
            with open(self.path, "w") as f:
                f.write(self.FIELDS + "\n")
                for r in self.rows:
                    f.write(",".join(r) + "\n")
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        load = [s for s in sm if s > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def config1_workload(W: int = 1920, H: int = 1080) -> str:
    return (f"config1: Kerr a=0.9 M=1, static camera r=15 M i=80 deg, Lens(24), {W}x{H}, "
            "gas 256x64x32 ISCO-25M h=0.05r, sky 2048x1024, kernel rules, samples=1")


def measure_fp32_peak(device: int, iters: int = 100000):
    """(TFLOP/s, ms) of the library's FP32 FMA-chain ceiling kernel, or (None, 0)."""
    import ctypes as C
    from spacetime_gb300 import _abi
    tf, ms = C.c_double(0.0), C.c_double(0.0)
    try:
        rc = _abi.load().st_measure_fp32_peak(device, iters, C.byref(tf), C.byref(ms))
    except Exception:
        return None, 0.0
    return (tf.value, ms.value) if rc == 0 and tf.value > 0 else (None, 0.0)


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _strided_dirs(w, FW: int, FH: int, n_rays: int):
    """Camera-frame directions (cf, cr, cu) of a strided pixel sample of the
    whole frame, about n_rays of them, as the pinhole camera maps pixel centres
    (src/metal.jl:863-872, 907-949): a sample of rays of every length."""
    import numpy as np
    stride = max(1, math.ceil(math.sqrt(FW * FH / max(n_rays, 1))))
    i = np.arange(stride // 2, FW, stride)
    j = np.arange(stride // 2, FH, stride)
    I, J = np.meshgrid(i, j)
    u = (I + 0.5 - FW / 2.0) / (FH / 2.0) * w.cam.fov_factor
    v = (J + 0.5 - FH / 2.0) / (FH / 2.0) * w.cam.fov_factor
    nu = np.sqrt(u * u + v * v + 1.0)
    return np.stack([1.0 / nu, u / nu, v / nu], -1).reshape(-1, 3), stride


def cpu_baseline(seconds_target: float = 15.0, threads: int | None = None, gpu_frame=None,
                 gpu_diag=None, workload: str = "config1", frame_size=(1920, 1080), rate_hint=None,
                 twin: bool = True) -> dict:
    """The CPU path timed on the host cores: the oracle's restatement of the
    reference's CPU renderer loop -- DifferentialEquations-style Tsit5 at the
    reference's own tolerances (reltol = abstol = 1e-6, src/raytrace.jl:369-373)
    under the kernel's rules -- on a strided pixel sample of the whole frame,
    sized for ~10-30 s of host work, so the rate covers rays of every length.  When the
    GPU frame and its per-ray records are given, a central crop rendered by the
    oracle at rtol 1e-10 also yields the GPU path's exit-direction and radiance
    error against it."""
    from oracle import oracle as O
    from spacetime_gb300 import workloads
    FW, FH = frame_size
    w = {"config1": workloads.config1, "config1_thin": workloads.config1_thin,
         "config1_nogas": workloads.config1_nogas,
         "config2": lambda: workloads.config2(nframes=240), "config4": workloads.config4}[workload]()
    w = w.scaled(FW, FH)
    threads = threads or os.cpu_count() or 1
    sky = workloads.sky()
    tol = dict(rtol=1e-6, atol=1e-6)

    sc = O.scene_for(w, sky, O.INT_TSIT5, **tol)

    def run(n):
        dirs, stride = _strided_dirs(w, FW, FH, n)
        t0 = time.perf_counter()
        sc.trace_dirs(dirs, nthreads=threads)
        return dirs.shape[0], stride, time.perf_counter() - t0

    if rate_hint:
        rate = rate_hint
    else:
        n0, _, t0 = run(4000)
        rate = n0 / max(t0, 1e-6)
    n, stride, dt = run(int(min(max(rate * seconds_target, 2000), 400000)))
    out = {"value": n / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port", "rate_rays_per_s": n / dt,
           "sample": f"pixels on a stride-{stride} grid over the whole {FW}x{FH} frame ({workload}; {n} rays), "
                     f"FP64 Tsit5 reltol = abstol = 1e-6 (the reference renderer's), {dt:.1f} s on {threads} threads"}
    if twin:
        # the same CPU restatement with the GPU path's own integrator: the
        # oracle's FP64 RK4 twin of the kernel (its step rule and stopping
        # rules), on a strided sample sized for about half the Tsit5 time
        tw = O.scene_for(w, sky, O.INT_RK4)

        def run_twin(m):
            dirs, st = _strided_dirs(w, FW, FH, m)
            t1 = time.perf_counter()
            tw.trace_dirs(dirs, nthreads=threads)
            return dirs.shape[0], st, time.perf_counter() - t1

        m0, _, s0 = run_twin(2000)
        mt, st_t, dtt = run_twin(int(min(max(m0 / max(s0, 1e-6) * seconds_target / 2, 2000), 400000)))
        out["fp64_rk4_twin"] = {
            "value": mt / dtt / 1e6, "unit": UNIT, "cores": threads,
            "sample": f"pixels on a stride-{st_t} grid over the whole {FW}x{FH} frame ({mt} rays), the oracle's "
                      f"FP64 RK4 twin of the kernel (the GPU path's step and stopping rules), {dtt:.1f} s on "
                      f"{threads} threads"}
    if gpu_frame is not None:
        import numpy as np
        cw, ch = 596, 335
        c0, r0 = (FW - cw) // 2, (FH - ch) // 2
        ref, rays = O.scene_for(w, sky, O.INT_TSIT5, rect=(c0, cw, r0, ch)).render(nthreads=threads)
        g = gpu_frame[r0:r0 + ch, c0:c0 + cw].astype(np.float64)
        d = gpu_diag[r0:r0 + ch, c0:c0 + cw]
        both = ((d["flags"] & 1) > 0) & ((rays["flags"] & O.RAY_ESCAPED) > 0)
        a = d["dir"][both]
        b = rays["dir"][both]
        ang = 2 * np.arcsin(np.clip(np.linalg.norm(a - b, axis=-1) / 2, 0, 1))
        rel = np.abs(g - ref).sum(-1) / np.maximum(ref.sum(-1), 1e-6)
        out["accuracy_vs_oracle"] = {
            "oracle": f"Tsit5 rtol 1e-10 on the central {cw}x{ch} crop",
            "rays": int(cw * ch), "escaped_both": int(both.sum()),
            "dir_median_rad": float(np.median(ang)), "dir_p99_rad": float(np.percentile(ang, 99)),
            "radiance_rel_median": float(np.median(rel)), "radiance_rel_p99": float(np.percentile(rel, 99)),
            "class_mismatch": int((((d["flags"] & 8) > 0) != ((rays["flags"] & O.RAY_BLACK) > 0)).sum())}
    return out


# crops of the 1920x1080 frame the oracle renders for the accuracy figures:
# (col0, cols, row0, rows) -- the central 240x135 (shadow, photon ring, the
# densest gas) and a 3x3 grid of 80x45 tiles spread over the frame
CROPS = [((1920 - 240) // 2, 240, (1080 - 135) // 2, 135)] + [
    (c, 80, r, 45) for c in (160, 920, 1680) for r in (90, 517, 945)]


def _crop_stack(img, diag=None):
    import numpy as np
    im = np.concatenate([img[r0:r0 + rh, c0:c0 + cw].reshape(-1, 3) for c0, cw, r0, rh in CROPS])
    if diag is None:
        return im
    return im, np.concatenate([diag[r0:r0 + rh, c0:c0 + cw].reshape(-1) for c0, cw, r0, rh in CROPS])


def _errors(img, diag, ref, rays, served=None):
    """Exit-direction error (rad) over rays both sides call escaped, relative
    radiance error (L1 over RGB / oracle L1) over all rays; with `served`,
    the same over the surrogate-served rays alone."""
    import numpy as np
    from oracle import oracle as O

    def ang(a, b):
        return 2 * np.arcsin(np.clip(np.linalg.norm(a - b, axis=-1) / 2, 0, 1))

    esc = ((diag["flags"] & 1) > 0) & ((rays["flags"] & O.RAY_ESCAPED) > 0)
    d = ang(diag["dir"][esc].astype(np.float64), rays["dir"][esc])
    rel = np.abs(img.astype(np.float64) - ref).sum(-1) / np.maximum(ref.sum(-1), 1e-6)
    out = {"rays": int(img.shape[0]), "escaped_both": int(esc.sum()),
           "dir_median_rad": float(np.median(d)) if d.size else None,
           "dir_p99_rad": float(np.percentile(d, 99)) if d.size else None,
           "radiance_rel_median": float(np.median(rel)), "radiance_rel_p99": float(np.percentile(rel, 99)),
           "class_mismatch": int((((diag["flags"] & 8) > 0) != ((rays["flags"] & O.RAY_BLACK) > 0)).sum())}
    if served is not None and served.any():
        se = served & esc
        ds = ang(diag["dir"][se].astype(np.float64), rays["dir"][se]) if se.any() else np.zeros(1)
        out["served"] = {"rays": int(served.sum()), "captured_in_oracle": int((served & ~esc).sum()),
                         "dir_median_rad": float(np.median(ds)), "dir_p99_rad": float(np.percentile(ds, 99)),
                         "dir_max_rad": float(ds.max()),
                         "radiance_rel_median": float(np.median(rel[served])),
                         "radiance_rel_p99": float(np.percentile(rel[served], 99))}
    return out


def headline_block(ctx_cls, device: int, flush, sigma: float, reps: int = 5) -> dict:
    """The metric's comparison on one GB300: surrogate + FP32 against the plain
    FP64-guarded RK4 path and plain FP32 RK4, each frame 1920x1080 with config
    1's camera and hole (Kerr a=0.9, r=15 M, i=80 deg, Lens(24), kernel rules,
    exit landing), on three scenes: the gas (config 1 itself), the thin disc
    (2.32-25 M) and neither.  Each arm: device time per frame (L2 flushed),
    Mrays/s, surrogate-served fraction, and errors against the FP64 oracle's
    Tsit5 (rtol 1e-10) on crops of the timed frame itself (CROPS); for the
    surrogate arm also the served rays alone."""
    import numpy as np
    import torch
    from oracle import oracle as O
    from spacetime_gb300 import _abi, workloads
    from spacetime_gb300.surrogate import load_trained
    sky = workloads.sky()
    sur = load_trained(device)
    guards = dict(r_guard=3.0, crit_band=0.05, crit_r=4.0, renorm_every=256)
    arms = {"plain_fp32": dict(precision=_abi.ST_PREC_FP32),
            "fp32_fp64_guarded": dict(precision=_abi.ST_PREC_FP32_GUARDED, **guards),
            "fp32_df_guarded": dict(precision=_abi.ST_PREC_FP32_GUARDED_DF, **guards),
            "surrogate_fp32": dict(precision=_abi.ST_PREC_FP32, surrogate=1, surrogate_sigma=sigma),
            "surrogate_fp32_wide_gate": dict(precision=_abi.ST_PREC_FP32, surrogate=1,
                                             surrogate_sigma=SIGMA_WIDE)}
    out = {"frame": "1920x1080, config 1's camera and hole (Kerr a=0.9, r=15 M, i=80 deg, Lens(24)), kernel "
                    "rules, exit landing; the shipped surrogate network",
           "sigma_gate_rad": sigma, "sigma_gate_wide_rad": SIGMA_WIDE,
           "gates": "surrogate_fp32: the widest gate that keeps the frame's exit directions inside the target "
                    "(median 1e-4, p99 1e-3 rad); surrogate_fp32_wide_gate: a gate that serves about half the "
                    "no-disc frame and misses the target",
           "errors_on": "crops of the timed frame: central 240x135 + nine 80x45 tiles (64,800 rays), "
                        "against the FP64 oracle's Tsit5 (rtol 1e-10)"}
    for wname, make in (("config1_gas", workloads.config1), ("config1_thin_disc", workloads.config1_thin),
                        ("config1_no_disc_no_gas", workloads.config1_nogas)):
        w = make()
        ctx = ctx_cls(sky, disc=w.disc, volume=w.vol, emitter=w.emitter, device=device)
        ctx.set_surrogate(sur)
        refs = [O.scene_for(w, sky, O.INT_TSIT5, rect=rect).render() for rect in CROPS]
        ref = np.concatenate([r[0].reshape(-1, 3) for r in refs]).astype(np.float64)
        rays = np.concatenate([r[1].reshape(-1) for r in refs])
        block = {}
        for name, kw in arms.items():
            if kw.get("surrogate") and w.vol is not None:
                # the gate serves no ray of a gas frame (each ray's gas line integral
                # needs its integrated path), so st_render refuses the combination;
                # surrogate + FP32 on this frame is the plain FP32 path
                block[name] = {**block["plain_fp32"], "served_fraction": 0.0,
                               "note": "st_render refuses the surrogate with gas (ST_EUNSUPPORTED): every ray "
                                       "starts inside the gas slab and needs its integrated path; the numbers are "
                                       "the plain FP32 arm's"}
                continue
            p = ctx.params(w.semantics, width=1920, height=1080, **w.params, **kw)
            ctx.render_device(w.cam, w.bh, p)
            ts = []
            for _ in range(reps):
                flush.zero_()
                torch.cuda.synchronize()
                _, st = ctx.render_device(w.cam, w.bh, p)
                ts.append(st["kernel_ms"])
            ms = float(np.median(ts))  # median of the frames: one slow frame does not move the ratios
            r = ctx.render_raw(w.cam, w.bh, p, diag=True)
            img, diag = _crop_stack(r.image, r.diag)
            served = (diag["flags"] & _abi.ST_RAY_SURROGATE) > 0 if kw.get("surrogate") else None
            block[name] = {"value": 1920 * 1080 / (ms * 1e-3) / 1e6, "ms_per_step": ms,
                           "ms_range": [float(min(ts)), float(max(ts))],
                           "served_fraction": st["surrogate_rays"] / (1920 * 1080),
                           "steps_per_frame": st["steps"], "fp64_steps_per_frame": st["fp64_steps"],
                           "errors": _errors(img, diag, ref, rays, served)}
        sv, sw, pl, gd = (block[k]["value"] for k in ("surrogate_fp32", "surrogate_fp32_wide_gate", "plain_fp32",
                                                          "fp32_fp64_guarded"))
        block["surrogate_vs_fp32_fp64_guarded"] = sv / gd
        block["surrogate_vs_plain_fp32"] = sv / pl
        block["surrogate_wide_gate_vs_fp32_fp64_guarded"] = sw / gd
        block["surrogate_wide_gate_vs_plain_fp32"] = sw / pl
        block["plain_fp32_vs_fp32_fp64_guarded"] = pl / gd
        block["plain_fp32_vs_fp32_df_guarded"] = pl / block["fp32_df_guarded"]["value"]
        out[wname] = block
        ctx.close()
    sur.close()
    return out


def layered_variant(ctx_cls, device: int, flush, reps: int = 3) -> dict:
    """The layered engine on a Schwarzschild frame: config 0's camera and hole
    (static camera at r = 30 M, Lens(24)) with the kernel's rules and its thin
    disc (3-20 M, exact emitter) at 1920x1080, FP32.  The full per-pixel trace
    against the layered frame (fan-driven sky, disc layer at the display and
    at half resolution, the latter also with the foveated ring pass at the
    display resolution for rays of periapsis below 6 M): time per frame with the fans built (first frame at a
    radius) and cached (every later frame at that radius), and the radiance
    difference from the full trace."""
    import numpy as np
    import torch
    from spacetime_gb300 import _abi, workloads
    w = workloads.config0().scaled(1920, 1080)
    w.semantics = _abi.ST_SEM_DRAFT
    w.emitter = _abi.ST_EMIT_KS_EXACT
    w.params = dict(samples=1, pixel_jitter=0, exit_landing=1)
    ctx = ctx_cls(workloads.sky(), disc=w.disc, emitter=w.emitter, device=device)
    p = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32, **w.params)
    out = {"workload": "config0 camera and hole (Schwarzschild, static r=30 M, Lens(24)), 1920x1080, kernel rules, "
                       "thin disc 3-20 M exact emitter, FP32"}

    def timed(fn):
        ts = []
        for _ in range(reps):
            flush.zero_()
            torch.cuda.synchronize()
            r = fn()
            ts.append(r.stats["kernel_ms"])
        return r, float(np.mean(ts))

    full, ms_full = timed(lambda: ctx.render_raw(w.cam, w.bh, p))
    out["full_trace"] = {"ms_per_step": ms_full, "value": 1920 * 1080 / (ms_full * 1e-3) / 1e6,
                         "steps": full.stats["steps"]}
    lum = np.maximum(full.image.astype(np.float64).sum(-1), 1e-6)
    for name, size, ring in (("layered", None, 0.0), ("layered_half_res_layer", (960, 540), 0.0),
                             ("layered_half_res_layer_ring", (960, 540), 6.0)):
        # a radius not yet seen: the fans are built with the frame
        from spacetime_gb300.scene import Camera
        other = Camera.look_at((0.0, -25.0, 3.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), w.cam.fov_factor)
        ctx.render_layered_raw(other, w.bh, p, layer_size=size, ring_rmin=ring)
        torch.cuda.synchronize()
        cold = ctx.render_layered_raw(w.cam, w.bh, p, layer_size=size, ring_rmin=ring)
        lay, ms = timed(lambda: ctx.render_layered_raw(w.cam, w.bh, p, layer_size=size, ring_rmin=ring))
        rel = np.abs(lay.image.astype(np.float64) - full.image).sum(-1) / lum
        out[name] = {"ms_per_step": ms, "value": 1920 * 1080 / (ms * 1e-3) / 1e6,
                     "ms_first_frame_at_radius": cold.stats["kernel_ms"], "steps": lay.stats["steps"],
                     "speedup_vs_full_trace": ms_full / ms,
                     "radiance_rel_vs_full_median": float(np.median(rel)),
                     "radiance_rel_vs_full_p99": float(np.percentile(rel, 99))}
    ctx.close()
    return out


def features_variant(ctx_cls, device: int, flush, reps: int = 3) -> dict:
    """The draft renderer's optional features on config 1's 1920x1080 frame
    (Kerr a=0.9 with gas, FP32), device time per frame beside the plain frame
    of the same passes: procedural stars; 4 jittered passes plain, with a
    per-pixel motion-blur shutter (camera_at moving the camera 0.2 M along
    its right axis), and with adaptive refinement (refine 3); depth buckets
    (10, one pass)."""
    import numpy as np
    import torch
    from spacetime_gb300 import _abi, workloads
    from spacetime_gb300.api import Starfield
    from spacetime_gb300.scene import Camera
    w = workloads.config1()
    ctx = ctx_cls(workloads.sky(), disc=w.disc, volume=w.vol, emitter=w.emitter, device=device)
    base = dict(w.params)

    def params(**kw):
        q = dict(base)
        q.update(kw)
        return ctx.params(w.semantics, width=1920, height=1080, precision=_abi.ST_PREC_FP32, **q)

    def timed(fn):
        fn()
        ts = []
        for _ in range(reps):
            flush.zero_()
            torch.cuda.synchronize()
            ts.append(fn().stats["kernel_ms"])
        return float(np.median(ts))

    out = {"workload": "config1 camera, hole and gas, 1920x1080, kernel rules, FP32"}
    one = params()
    out["plain_1_pass_ms"] = timed(lambda: ctx.render_raw(w.cam, w.bh, one))
    out["depth_buckets_10_ms"] = timed(lambda: ctx.render_depth_raw(w.cam, w.bh, one, 10))
    ctx.set_starfield(Starfield(height=1080, fov_factor=w.cam.fov_factor))
    out["starfield_1_pass_ms"] = timed(lambda: ctx.render_raw(w.cam, w.bh, one))
    ctx.set_starfield(None)
    four = params(samples=2, pixel_jitter=1, seed=3)
    out["plain_4_passes_ms"] = timed(lambda: ctx.render_raw(w.cam, w.bh, four))
    c = w.cam
    poses = [Camera(c.pos + (0.2 * m / 4) * c.right, c.fwd, c.right, c.up_local, c.fov_factor, c.velocity)
             for m in range(5)]
    out["motion_blur_4_passes_ms"] = timed(lambda: ctx.render_motion_raw(c, poses, w.bh, four,
                                                                          per_pixel_shutter=True))
    ref = params(samples=2, pixel_jitter=1, seed=3, refine=3)
    r = ctx.render_raw(w.cam, w.bh, ref)
    out["refine_3_ms"] = timed(lambda: ctx.render_raw(w.cam, w.bh, ref))
    out["refine_3_rays_per_pixel"] = r.stats["rays"] / (1920 * 1080)
    ctx.close()
    return out


def fluid_variant(ctx_cls, device: int, steps: int = 200) -> dict:
    """The live fluid disc (DiscFluidSim / step_sim!, dt 0.08, jacobi 8) on two
    grids: config 1's gas grid (256 x 64 x 32, ISCO to 25 M) and the
    reference's default DiscVolume grid (192 x 256 x 48, 3-20 M).  Device time
    per step through the CUDA graph and as plain stream launches (4 kernels a
    step), and the oracle's single-thread CPU time per step."""
    import time

    import numpy as np
    from oracle import oracle as O
    from spacetime_gb300 import workloads
    from spacetime_gb300.api import AccretionDisc, Blackbody, DiscFluidSim
    from spacetime_gb300.scene import make_volume
    out = {}
    for name, vol, disc in (
            ("config1_grid_256x64x32", workloads.config1().vol, AccretionDisc(2.32, 25.0, Blackbody(), 0.0)),
            ("default_grid_192x256x48", make_volume(inner=3.0, outer=20.0, nr=192, nphi=256, nz=48, seed=3),
             AccretionDisc(3.0, 20.0, Blackbody(wb_temperature=10000.0), 0.8))):
        ctx = ctx_cls(workloads.sky(256, 128), disc=disc, volume=vol, device=device)
        sim = DiscFluidSim(ctx, vol, disc)
        sim.step(dt=0.08, nsteps=20, graph=True, timed=True)          # warm-up (and graph build)
        ms_graph = sim.step(dt=0.08, nsteps=steps, graph=True, timed=True) / steps
        sim.step(dt=0.08, nsteps=20, graph=False, timed=True)
        ms_plain = sim.step(dt=0.08, nsteps=steps, graph=False, timed=True) / steps
        nr, nphi, nz = vol.shape
        orc = O.FluidSim(vol, disc.inner_radius, disc.outer_radius, falloff=disc.density_falloff)
        t0 = time.perf_counter()
        orc.step(dt=0.08, jacobi=8, nsteps=5, volume=True)
        cpu_ms = (time.perf_counter() - t0) * 1e3 / 5
        # algorithmic bytes: every field read and written once per kernel, the texture written once
        n = nr * nphi
        algo = (19 * n + n * nz) * 4
        out[name] = {"us_per_step_graph": ms_graph * 1e3, "us_per_step_stream": ms_plain * 1e3,
                     "launches_per_step": 4, "algorithmic_bytes_per_step": algo,
                     "achieved_GBs_graph": algo / (ms_graph * 1e-3) / 1e9,
                     "oracle_cpu_ms_per_step_1_thread": cpu_ms,
                     "speedup_vs_oracle": cpu_ms / ms_graph}
        sim.close()
        ctx.close()
    return out


# dram__bytes_read.sum + dram__bytes_write.sum of the 1920x1080 config-1 FP32 launch
# (26.27 MB read, 0.12 MB written; profiles/trace_fp32_kerr_gas_1080p_dram.md)
TRACE_1080P_DRAM_BYTES = 26_271_744 + 124_672


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    per_step = []
    base = None
    # each step a bounded sample: the whole run stays near two minutes of host work
    secs = max(1.0, min(args.ref_seconds, 120.0 / max(args.warmup + args.steps, 1)))
    rate = None
    for k in range(args.warmup + args.steps):
        b = cpu_baseline(seconds_target=secs, threads=threads, rate_hint=rate, twin=False)
        rate = b["rate_rays_per_s"]
        if k >= args.warmup:
            per_step.append(b["value"])
            base = b
    value = statistics.median(per_step)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": config1_workload(1920, 1080), "sample": base["sample"]},
        "cpu_baseline": {**base, "value": value},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def track_accuracy(ctx, w, p, track_img, workload: str) -> dict:
    """Errors of timed track frames against the FP64 oracle's Tsit5 (rtol
    1e-10) on crops of those frames: config 4, frame 0 -- the central 480x270
    and a 3x3 grid of 160x90 tiles of the 3840x2160 frame; config 2, frames
    0, 120 and 239 (r = 30 M, mid-fall, inside the horizon) -- the central
    320x180 of each.  Radiance from the track's own output; exit directions
    from a single-frame render of the same camera with per-ray records (the
    same kernel; tracks and single frames are tested equal).  Each frame is
    also scored against the oracle's fixed-step FP64 twin of the kernel's
    rules: from inside the horizon the backward rays approach the horizon
    asymptotically in ingoing Kerr-Schild coordinates, which the kernel's
    fixed RK4 step crosses (as the reference's Metal kernel does) and Tsit5
    at rtol 1e-10 does not, so there the twin is the reference's result."""
    import numpy as np
    from oracle import oracle as O
    from spacetime_gb300 import workloads
    W, H = w.width, w.height
    sky = workloads.sky()
    if workload == "config4":
        frames = [0]
        crops = [((W - 480) // 2, 480, (H - 270) // 2, 270)] + [
            (c, 160, r, 90) for c in (320, 1840, 3360) for r in (180, 1035, 1890)]
    else:
        frames = [0, len(w.cams) // 2, len(w.cams) - 1]
        crops = [((W - 320) // 2, 320, (H - 180) // 2, 180)]
    out = {"oracle": "Tsit5 rtol 1e-10", "frames": {}}
    for f in frames:
        wf = w.scaled(W, H)
        wf.cam = w.cams[f]
        pd = ctx.params(w.semantics, width=W, height=H, precision=p.precision, r_guard=p.r_guard,
                        crit_band=p.crit_band, crit_r=p.crit_r, renorm_every=p.renorm_every, **w.params)
        d = ctx.render_raw(w.cams[f], w.bh, pd, diag=True).diag
        refs = [O.scene_for(wf, sky, O.INT_TSIT5, rect=rect).render() for rect in crops]
        ref = np.concatenate([x[0].reshape(-1, 3) for x in refs]).astype(np.float64)
        rays = np.concatenate([x[1].reshape(-1) for x in refs])
        img = np.concatenate([track_img[f][r0:r0 + rh, c0:c0 + cw].reshape(-1, 3) for c0, cw, r0, rh in crops])
        dg = np.concatenate([d[r0:r0 + rh, c0:c0 + cw].reshape(-1) for c0, cw, r0, rh in crops])
        e = _errors(img, dg, ref, rays)
        tw = [O.scene_for(wf, sky, O.INT_RK4, rect=rect).render() for rect in crops]
        e["vs_fp64_twin"] = _errors(img, dg, np.concatenate([x[0].reshape(-1, 3) for x in tw]).astype(np.float64),
                                    np.concatenate([x[1].reshape(-1) for x in tw]))
        e["camera_r"] = float(np.linalg.norm(w.cams[f].pos))
        e["crops"] = [list(c) for c in crops]
        out["frames"][str(f)] = e
    return out


def run_training(args):
    """config 3, the learned surrogate's training: FP64 labels generated on the
    GPU (Sobol-sampled rays, the integrator's own rules), then AdamW steps of
    the 6 -> 256x4 -> 6 BF16 network at batch 16384, the hidden-layer GEMMs on
    tcgen05 (default) and on mma.sync (SPACETIME_GB300_TRAIN_MMA=sync), timed
    with CUDA-synchronised wall clock, each path from the same starting
    parameters.  Tensor work per step: three hidden layers x (forward, input
    gradient, weight gradient) x 2 x 16384 x 256 x 256 flops."""
    import numpy as np
    import torch
    from spacetime_gb300.surrogate import Surrogate
    torch.cuda.set_device(0)
    batch, steps, warm = 16384, max(args.steps, 1) * 50, max(args.warmup, 3) * 10
    n_labels = 1 << 21
    out, t_lab = {}, None
    for mode in ("tcgen05", "mma_sync"):
        if mode == "mma_sync":
            os.environ["SPACETIME_GB300_TRAIN_MMA"] = "sync"
        sur = Surrogate(0, seed=1)
        t0 = time.perf_counter()
        sur.generate(n_labels, offset=0, copy=False)
        torch.cuda.synchronize()
        t_lab = t_lab or time.perf_counter() - t0
        sur.train(warm, batch=batch, lr=1e-3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hist = sur.train(steps, batch=batch, lr=1e-3)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        sur.close()
        os.environ.pop("SPACETIME_GB300_TRAIN_MMA", None)
        flops = 3 * 3 * 2.0 * batch * 256 * 256
        out[mode] = {"ms_per_step": dt / steps * 1e3, "samples_per_s": batch * steps / dt,
                     "hidden_gemm_tflops": flops * steps / dt / 1e12, "loss_last": float(np.mean(hist[-50:]))}
    bf16 = measured_peaks().get("bf16_tflops")
    line = {
        "metric": "surrogate training samples/s (config3: batch 16384, BF16 6-256x4-6 MLP, AdamW)",
        "value": out["tcgen05"]["samples_per_s"], "unit": "samples/s", "n_gpus": 1, "steps": steps,
        "warmup": warm, "ms_per_step": out["tcgen05"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": "config3: surrogate training, FP64 labels of Sobol-sampled rays",
                   "labels": n_labels, "label_rate_per_s": n_labels / t_lab, "batch": batch},
        "roofline": {"bound": "tensor", "achieved": out["tcgen05"]["hidden_gemm_tflops"], "peak": bf16,
                     "unit": "TFLOP/s",
                     "frac": out["tcgen05"]["hidden_gemm_tflops"] / bf16 if bf16 else None, "traffic": None,
                     "note": "hidden-layer GEMM flops over the whole step time (edge layers, loss, "
                             "transposes and AdamW included in the time)"},
        "paths": out,
        "tcgen05_vs_mma_sync": out["mma_sync"]["ms_per_step"] / out["tcgen05"]["ms_per_step"],
    }
    print(json.dumps(line))
    return 0


def run_track(args):
    """config2 (240 frames 1280x720 free fall, Schwarzschild, thin disc) or
    config4 (8 frames 3840x2160, Kerr a=0.99, boosted 0.3c, gas 512x128x64):
    one step = the whole track in one launch (st_render_frames), with the
    autotuned schedule and CUDA-graph replay."""
    import numpy as np
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from spacetime_gb300 import _abi, autotune, workloads
    from spacetime_gb300.api import Context
    w = workloads.config2() if args.workload == "config2" else workloads.config4()
    prec = {"fp64": _abi.ST_PREC_FP64, "fp32": _abi.ST_PREC_FP32, "fp32g": _abi.ST_PREC_FP32_GUARDED,
            "fp32gdf": _abi.ST_PREC_FP32_GUARDED_DF}[args.precision]
    ctx = Context(workloads.sky(), disc=w.disc, volume=w.vol, emitter=w.emitter, device=local)
    p = ctx.params(w.semantics, width=w.width, height=w.height, precision=prec, r_guard=args.r_guard,
                   crit_band=args.crit_band, crit_r=args.crit_r, renorm_every=args.renorm, **w.params)
    tuned = autotune.tune(ctx, w.cams, w.bh, p, sample_frames=min(8, len(w.cams)), repeats=1)
    autotune.apply(p, tuned)
    p.graph = 1
    for _ in range(args.warmup):
        ctx.render_frames_raw(w.cams, w.bh, p)
    torch.cuda.synchronize()
    clocks = ClockSampler(local, args.clocks_csv)
    clocks.start()
    kms, tot = [], []
    for _ in range(args.steps):
        r = ctx.render_frames_raw(w.cams, w.bh, p)
        kms.append(r.stats["kernel_ms"])
        tot.append(r.stats["total_ms"])
        st = r.stats
    clk = clocks.stop()
    rays = len(w.cams) * w.width * w.height
    ms = float(np.mean(kms))
    value = rays / (ms * 1e-3) / 1e6
    kerr = getattr(w.bh, "a", 0.0) != 0.0
    variants = {}
    if args.precision == "fp32" and not args.no_variants:
        # the same track on the plain FP64-guarded path (renormalisation every 256
        # steps, FP64 steps inside 3 M and for near-critical rays inside 4 M)
        pg = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32_GUARDED,
                        r_guard=3.0, crit_band=0.05, crit_r=4.0, renorm_every=256, **w.params)
        autotune.apply(pg, tuned)
        pg.graph = 1
        ctx.render_frames_raw(w.cams, w.bh, pg)
        rg = ctx.render_frames_raw(w.cams, w.bh, pg)
        msg = rg.stats["kernel_ms"]
        variants["fp32_fp64_guarded"] = {"value": rays / (msg * 1e-3) / 1e6, "ms_per_step": msg,
                                         "fp64_steps_per_track": rg.stats["fp64_steps"],
                                         "speedup_of_value": (rays / (ms * 1e-3)) / (rays / (msg * 1e-3))}
        # the same guards with the guard steps in double-float on the FP32 pipe
        pd = ctx.params(w.semantics, width=w.width, height=w.height, precision=_abi.ST_PREC_FP32_GUARDED_DF,
                        r_guard=3.0, crit_band=0.05, crit_r=4.0, renorm_every=256, **w.params)
        autotune.apply(pd, tuned)
        pd.graph = 1
        ctx.render_frames_raw(w.cams, w.bh, pd)
        rd = ctx.render_frames_raw(w.cams, w.bh, pd)
        msd = rd.stats["kernel_ms"]
        variants["fp32_df_guarded"] = {"value": rays / (msd * 1e-3) / 1e6, "ms_per_step": msd,
                                       "guard_steps_per_track": rd.stats["fp64_steps"],
                                       "speedup_of_value": msd / ms}
    flops = st["steps"] * flops_per_step(kerr) + st["gas_samples"] * FLOPS_GAS_SAMPLE
    achieved = flops / (ms * 1e-3) / 1e12
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_max = measured_peaks().get("sm_max_mhz", 2070.0)
    fp32_nominal = sms * 128 * 2 * sm_max * 1e6 / 1e12
    fp32_measured, _ = measure_fp32_peak(local)
    fp32_peak = fp32_measured or fp32_nominal
    cpu = None
    accuracy = None
    if not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(workload=args.workload, frame_size=(w.width, w.height))
        except Exception as e:
            cpu = {"value": None, "sample": f"failed: {e}"}
        try:
            accuracy = track_accuracy(ctx, w, p, r.image, args.workload)
        except Exception as e:  # report, do not fail the bench
            accuracy = {"failed": str(e)}
    line = {
        "metric": f"Mrays/s {args.workload} track", "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision != "fp64" else "f64", "data": "synthetic",
        "config": {"workload": w.name, "frames": len(w.cams), "size": f"{w.width}x{w.height}",
                   "schedule": tuned, "graph": True, "steps_per_track": st["steps"],
                   "gas_samples_per_track": st["gas_samples"], "per_frame_ms": ms / len(w.cams),
                   "l2": "inputs stay L2-resident by design; per-step time is kernel time of the whole track"},
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": None,
                     "peak_note": "measured FP32 FMA ceiling (st_measure_fp32_peak)" if fp32_measured else
                     "nominal FP32 FMA rate", "peak_nominal": fp32_nominal},
        "e2e": {"value": rays / (float(np.mean(tot)) * 1e-3) / 1e6, "unit": UNIT,
                "h2d_bytes_per_step": int(st["h2d_bytes"]), "d2h_bytes_per_step": int(rays * 12)},
        "gpu_launches": args.steps * 2, "clocks": clk, "cpu_baseline": cpu,
        "accuracy_vs_oracle": accuracy,
        "variants": variants,
    }
    print(json.dumps(line))
    ctx.close()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp64", "fp32", "fp32g", "fp32gdf"])
    ap.add_argument("--no-variants", action="store_true", help="skip the FP32G / FP64 comparison runs")
    ap.add_argument("--schedule", default="pixel", choices=["pixel", "persistent"])
    ap.add_argument("--size", default="1920x1080", help="frame WxH (profiling uses a smaller case)")
    ap.add_argument("--r-guard", type=float, default=3.0)
    ap.add_argument("--crit-band", type=float, default=0.05)
    ap.add_argument("--crit-r", type=float, default=4.0)
    ap.add_argument("--renorm", type=int, default=256)
    ap.add_argument("--chunk", type=int, default=32)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--clocks-csv", default=None)
    ap.add_argument("--workload", default="config1",
                    choices=["config1", "config1_thin", "config1_nogas", "config2", "config3", "config4"],
                    help="config1 is the headline; the others are the remaining benchmark configurations")
    ap.add_argument("--surrogate", default=None,
                    help="trained surrogate parameters (.npy; 'shipped' = spacetime_gb300/data/surrogate_kerr.npy) "
                         "for config1_thin / config1_nogas")
    ap.add_argument("--sigma", type=float, default=SIGMA_TARGET, help="surrogate gate: max predicted std-dev (rad)")
    ap.add_argument("--fluid-only", action="store_true",
                    help="print only the fluid disc timing (DiscFluidSim / step_sim!) as one JSON line")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.fluid_only:
        import torch
        from spacetime_gb300.api import Context
        torch.cuda.set_device(0)
        print(json.dumps({"fluid_disc": fluid_variant(Context, 0, steps=args.steps)}), flush=True)
        return 0
    if args.workload in ("config2", "config4"):
        return run_track(args)
    if args.workload == "config3":
        return run_training(args)

    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from spacetime_gb300 import _abi, workloads
    from spacetime_gb300.api import Context

    w = {"config1": workloads.config1, "config1_thin": workloads.config1_thin,
         "config1_nogas": workloads.config1_nogas}[args.workload]()
    W, H = (int(x) for x in args.size.lower().split("x"))
    w = w.scaled(W, H)
    prec = {"fp64": _abi.ST_PREC_FP64, "fp32": _abi.ST_PREC_FP32, "fp32g": _abi.ST_PREC_FP32_GUARDED,
            "fp32gdf": _abi.ST_PREC_FP32_GUARDED_DF}[args.precision]
    sched = _abi.ST_SCHED_PERSISTENT if args.schedule == "persistent" else _abi.ST_SCHED_PIXEL
    ctx = Context(workloads.sky(), disc=w.disc, volume=w.vol, emitter=w.emitter, device=local)
    sur = None
    extra = {}
    if args.surrogate:
        from spacetime_gb300.surrogate import Surrogate
        sur = Surrogate(local)
        from spacetime_gb300.surrogate import TRAINED
        sur.set_params(np.load(TRAINED if args.surrogate == "shipped" else args.surrogate))
        ctx.set_surrogate(sur)
        extra = dict(surrogate=1, surrogate_sigma=args.sigma)
    p = ctx.params(w.semantics, width=w.width, height=w.height, precision=prec, schedule=sched,
                   r_guard=args.r_guard, crit_band=args.crit_band, crit_r=args.crit_r,
                   renorm_every=args.renorm, chunk_steps=args.chunk, **w.params, **extra)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        ctx.render_device(w.cam, w.bh, p)
    barrier()
    clocks = ClockSampler(local, args.clocks_csv)
    clocks.start()
    kernel_ms, stats_last = [], None
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        _, st = ctx.render_device(w.cam, w.bh, p)
        kernel_ms.append(st["kernel_ms"])
        stats_last = st
    served = stats_last.get("surrogate_rays", 0)
    barrier()
    wall = time.perf_counter() - t_wall0
    # e2e: through st_render into pinned host memory
    host = torch.empty((w.height, w.width, 3), dtype=torch.float32, pin_memory=True)
    host_np = host.numpy()
    e2e_ms = []
    e2e_stats = {"h2d_bytes": 0}
    barrier()
    for _ in range(0 if args.no_e2e else args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = ctx.render_raw(w.cam, w.bh, p, out=host_np)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_stats = r.stats
    barrier()
    clk = clocks.stop()

    rays = w.width * w.height
    ms_step = float(np.mean(kernel_ms))
    e2e_step = float(np.mean(e2e_ms)) if e2e_ms else float("nan")
    if world > 1:
        t = torch.tensor([ms_step, e2e_step], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_step, e2e_step = float(t[0]), float(t[1])
    value = world * rays / (ms_step * 1e-3) / 1e6
    e2e_value = world * rays / (e2e_step * 1e-3) / 1e6

    steps = stats_last["steps"]
    gas = stats_last["gas_samples"]
    flops = steps * flops_per_step(True) + gas * FLOPS_GAS_SAMPLE
    achieved = flops / (ms_step * 1e-3) / 1e12
    props = torch.cuda.get_device_properties(local)
    sms = props.multi_processor_count
    peaks = measured_peaks()
    sm_max = peaks.get("sm_max_mhz", 2070.0)
    fp32_nominal = sms * 128 * 2 * sm_max * 1e6 / 1e12
    fp32_measured, fp32_ms = measure_fp32_peak(local)
    fp32_peak = fp32_measured or fp32_nominal
    if rank != 0:
        return 0
    variants = {}
    headline = None
    if not args.no_variants and (W, H) == (1920, 1080) and args.workload == "config1":
        # the same frame with FP64 guards (renormalisation every 256 steps, steps
        # inside 3 M, near-critical rays inside 4 M) and all in FP64
        for name, kw, reps in (("fp32_fp64_guarded", dict(precision=_abi.ST_PREC_FP32_GUARDED), 3),
                               ("fp32_df_guarded", dict(precision=_abi.ST_PREC_FP32_GUARDED_DF), 3),
                               ("fp64", dict(precision=_abi.ST_PREC_FP64), 1)):
            pv = ctx.params(w.semantics, width=W, height=H, schedule=sched, r_guard=3.0, crit_band=0.05,
                            crit_r=4.0, renorm_every=256, **w.params, **kw)
            ctx.render_device(w.cam, w.bh, pv)
            ts = []
            for _ in range(reps):
                flush.zero_()
                torch.cuda.synchronize()
                _, stv = ctx.render_device(w.cam, w.bh, pv)
                ts.append(stv["kernel_ms"])
            ms = float(np.mean(ts))
            variants[name] = {"value": rays / (ms * 1e-3) / 1e6, "ms_per_step": ms,
                              "fp64_steps_per_frame": stv["fp64_steps"]}
        for name in variants:
            variants[name]["speedup_of_value"] = value / variants[name]["value"]
        try:
            headline = headline_block(Context, local, flush, args.sigma)
        except Exception as e:  # report, do not fail the bench
            headline = {"failed": str(e)}
        try:
            variants["layered_schwarzschild"] = layered_variant(Context, local, flush)
        except Exception as e:  # report, do not fail the bench
            variants["layered_schwarzschild"] = {"failed": str(e)}
        try:
            variants["fluid_disc"] = fluid_variant(Context, local)
        except Exception as e:  # report, do not fail the bench
            variants["fluid_disc"] = {"failed": str(e)}
        try:
            variants["features"] = features_variant(Context, local, flush)
        except Exception as e:  # report, do not fail the bench
            variants["features"] = {"failed": str(e)}
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        try:
            pd = ctx.params(w.semantics, width=W, height=H, precision=prec, schedule=sched,
                            r_guard=args.r_guard, crit_band=args.crit_band, crit_r=args.crit_r,
                            renorm_every=args.renorm, chunk_steps=args.chunk, **w.params)
            rd = ctx.render_raw(w.cam, w.bh, pd, diag=True)
            cpu = cpu_baseline(gpu_frame=rd.image, gpu_diag=rd.diag, workload=args.workload) \
                if (W, H) == (1920, 1080) else cpu_baseline(workload=args.workload)
        except Exception as e:  # report, do not fail the bench
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}
    # DRAM bytes of one launch, from an ncu capture of this exact frame (the
    # two dram__bytes counters take one pass, so it was captured at full size)
    if args.workload == "config1" and (W, H) == (1920, 1080) and args.precision == "fp32" and args.schedule == "pixel":
        traffic = TRACE_1080P_DRAM_BYTES
        traffic_note = ("dram__bytes_read.sum + dram__bytes_write.sum of one launch, ncu "
                        "(profiles/trace_fp32_kerr_gas_1080p_dram.md): compulsory reads of the gas texture, "
                        "table and sampled sky; the kernel is issue-bound, HBM idle")
    else:
        traffic, traffic_note = None, "captured for the default 1920x1080 FP32 frame only"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision != "fp64" else "f64", "data": "synthetic",
        "config": {
            "workload": config1_workload(W, H)
                        if args.workload == "config1" else
                        f"{w.name}: config1's camera and hole, {W}x{H}, sky 2048x1024, kernel rules, samples=1",
            "precision": {"fp64": "FP64", "fp32": "FP32 (MUFU sqrt/rcp/exp/log)",
                          "fp32g": "FP32 RHS, float-float state, FP64 guards",
                          "fp32gdf": "FP32 RHS, float-float state, double-float guards"}[args.precision],
            "guards": {"r_guard": args.r_guard, "crit_band": args.crit_band, "renorm_every": args.renorm},
            "surrogate": ("not applied to this frame: every ray starts inside the gas slab, and the gas "
                          "line integral needs the integrated path; the surrogate arm on this frame and on "
                          "the same camera and hole with a thin disc and with neither is in `headline`")
                         if args.workload == "config1" else
                         ({"params": os.path.basename(args.surrogate), "sigma_gate_rad": args.sigma,
                           "served_fraction": served / (W * H)} if args.surrogate else False),
            "schedule": args.schedule,
            "parallelism": f"replicas{world}",
            "l2": "flushed between timed steps (256 MiB write)",
            "steps_per_frame": steps, "fp64_steps_per_frame": stats_last["fp64_steps"],
            "gas_samples_per_frame": gas,
            "geodesic_steps_per_s": steps / (ms_step * 1e-3),
            "wall_s": wall,
        },
        "roofline": {
            "bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": achieved / fp32_peak, "traffic": traffic,
            "traffic_note": traffic_note,
            "peak_note": (f"measured FP32 FMA ceiling (st_measure_fp32_peak: FMA-chain kernel at full occupancy, "
                          f"best of 3 launches of {fp32_ms:.1f} ms, CUDA events); MEASURED_PEAKS.json has no FP32 "
                          "figure" if fp32_measured else
                          "nominal FP32 FMA rate (the measurement failed)"),
            "peak_nominal": fp32_nominal,
            "frac_of_nominal": achieved / fp32_nominal,
            "flops_per_step": flops_per_step(True), "flops_per_gas_sample": FLOPS_GAS_SAMPLE,
        },
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(e2e_stats["h2d_bytes"]),
                "d2h_bytes_per_step": int(rays * 3 * 4), "ms_per_step": e2e_step},
        "gpu_launches": args.steps,
        "clocks": clk,
        "cpu_baseline": cpu,
        "headline": headline,
        "variants": variants,
    }
    print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
