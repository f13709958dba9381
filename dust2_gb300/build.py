"""Build the CUDA engine into dust2_gb300/_lib/libdust2_gb300.so.

Every .cu file under csrc/ is compiled for sm_103a in parallel and linked
into one shared library with a plain C ABI (include/dust2_gb300.h).
Floating-point contraction is disabled on both the device (-fmad=false)
and host (-ffp-contract=off) sides: the kernels and the CPU oracle share
their arithmetic headers and must round identically; fused operations
are written explicitly as fma().
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent
REPO = ROOT.parent
CSRC = ROOT / "csrc"
BUILD_DIR = ROOT / "_build"
LIB_DIR = ROOT / "_lib"
LIB = LIB_DIR / "libdust2_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-strict-aliasing",
    "-I", str(CSRC), "-I", str(CSRC / "compat"), "-I", str(REPO / "include"),
]


def nvcc():
    path = shutil.which("nvcc")
    if path is None:
        cand = Path("/usr/local/cuda/bin/nvcc")
        if cand.exists():
            return str(cand)
        raise RuntimeError("nvcc not found")
    return path


def sources():
    return sorted(CSRC.glob("*.cu"))


def headers():
    out = list(CSRC.rglob("*.hpp")) + list(CSRC.rglob("*.cuh"))
    out.append(REPO / "include" / "dust2_gb300.h")
    return out


def _newest(paths):
    return max((p.stat().st_mtime for p in paths), default=0.0)


def _compile(src, obj, extra):
    cmd = [nvcc()] + NVCC_FLAGS + list(extra) + ["-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(
            f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{res.stdout}\n"
            f"{res.stderr}")
    return res.stderr


def build(force=False, verbose=False, extra_flags=()):
    """Compile and link the engine library if any source changed."""
    srcs = sources()
    if not force and LIB.exists():
        if LIB.stat().st_mtime >= _newest(srcs + headers() + [Path(__file__)]):
            return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    hdr_time = _newest(headers() + [Path(__file__)])
    jobs = []
    for src in srcs:
        obj = BUILD_DIR / (src.stem + ".o")
        if (force or not obj.exists()
                or obj.stat().st_mtime < max(src.stat().st_mtime, hdr_time)):
            jobs.append((src, obj))
    n_workers = max(1, min(len(jobs), os.cpu_count() or 1))
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(n_workers) as ex:
            futs = [ex.submit(_compile, s, o, extra_flags) for s, o in jobs]
            for f in futs:
                msg = f.result()
                if verbose and msg:
                    sys.stderr.write(msg)
    objs = [str(BUILD_DIR / (s.stem + ".o")) for s in srcs]
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + objs + [
        "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


def ptxas_report(src_name):
    """Register / spill report of one translation unit (-Xptxas -v)."""
    src = CSRC / src_name
    cmd = [nvcc()] + NVCC_FLAGS + ["-Xptxas", "-v", "-c", str(src), "-o",
                                   os.devnull]
    res = subprocess.run(cmd, capture_output=True, text=True)
    return res.stdout + res.stderr


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build(force=force, verbose=True))
