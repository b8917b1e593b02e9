"""Build libspacetime_gb300.so in-tree with nvcc for sm_103a.

One translation unit per trace precision plus the host API, compiled in
parallel and linked with the CUDA runtime.  Objects go to _build/ (ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.environ.get("ST_OBJ_DIR", os.path.join(ROOT, "_build", "obj"))
LIB = os.environ.get("SPACETIME_GB300_LIB", os.path.join(HERE, "libspacetime_gb300.so"))
# per-unit flags: the FP32 trace units use the MUFU forms of sqrt, division,
# exp and log (their double arithmetic is unaffected) and ask ptxas for enough
# resident blocks per SM to keep FP32 latency hidden
FAST = os.environ.get("ST_FASTMATH", "1") == "1"
MINB_FP32 = os.environ.get("ST_MINB_FP32", "7")
MINB_FP32G = os.environ.get("ST_MINB_FP32G", "4")
MINB_FP64 = os.environ.get("ST_MINB_FP64", "1")
UNIT_FLAGS = {
    "st_trace_fp32.cu": (["--use_fast_math"] if FAST else []) + [f"-DST_MINB={MINB_FP32}"],
    "st_trace_fp32_guarded.cu": (["--use_fast_math"] if FAST else []) + [f"-DST_MINB={MINB_FP32G}"],
    "st_trace_fp64.cu": [f"-DST_MINB={MINB_FP64}"],
    # the fluid solver rounds every float operation as written (no contraction)
    "st_fluid.cu": ["-fmad=false"],
}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["st_trace_fp64.cu", "st_trace_fp32.cu", "st_trace_fp32_guarded.cu", "st_api.cu", "st_surrogate.cu", "st_noalloc.cu",
           "st_layered.cu", "st_rawio.cpp", "st_fluid.cu", "st_peak.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "spacetime_gb300.h"))
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
    if verbose:
        flags += ["-Xptxas", "-v"]
    exe = nvcc()

    def one(src: str) -> str:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
        stamp = o + ".flags"
        want = " ".join(flags + UNIT_FLAGS.get(src, []))
        same = os.path.exists(stamp) and open(stamp).read() == want
        if not force and same and _newer(o, [s] + headers):
            return o
        r = subprocess.run([exe] + flags + UNIT_FLAGS.get(src, []) + ["-c", s, "-o", o], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr)
        with open(stamp, "w") as f:
            f.write(want)
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    if force or not _newer(LIB, objs):
        r = subprocess.run([exe, "-shared"] + ARCH + ["-o", LIB] + objs + ["-lcudart"], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
