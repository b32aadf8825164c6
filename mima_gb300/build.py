"""Builds the sm_103a shared library ``mima_gb300/lib/librrtmg_gpu.so`` in-tree.

Every translation unit is compiled by nvcc in parallel with one
``-gencode arch=compute_103a,code=sm_103a``; the FP64 kernels are compiled with
``--fmad=false`` (separately rounded multiplies and adds, for bit-level
reproducibility of the FP64 path), the FP32-split kernels with contraction and
with the hardware-approximate FP32 division and square root (within 2 ulp;
the SW solver does about nine FP32 divisions per layer and g-point, and the
IEEE-rounded sequences cost it 19 % of its time at T85 x 40 with no change in
its error against the oracle).
The library has a plain C ABI (include/rrtmg_gpu.h) and links the CUDA
runtime statically, so it needs no torch at load time.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "librrtmg_gpu.so"
PEAK_LIB = LIBDIR / "libfp32peak.so"   # FP32 FMA-rate microkernel for the benchmark's roofline
OBJDIR = LIBDIR / "obj"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          f"-I{ROOT / 'include'}", f"-I{CSRC}", "--expt-relaxed-constexpr"]

UNITS = {
    "kernels_fp64.cu": ["--fmad=false"],
    "kernels_split.cu": ["--prec-div=false", "--prec-sqrt=false"],
    "adjoint.cu": [],
    "driver.cu": ["--fmad=false"],
    "tables_host.cu": [],
    "abi.cu": ["-Xcompiler", "-fvisibility=default"],
}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librrtmg_gpu.so")
    return exe


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None, variant: str | None = None) -> Path:
    """Builds the library.  ``variant``: a named build with the ``extra`` nvcc
    flags (e.g. ``-DRRTMG_TABLE_PREFETCH_L2=0``, no L2 prefetch of the band
    tables) into ``lib/variants/<variant>/``, for timing it beside the default
    library (load it with RRTMG_GPU_LIB)."""
    if variant:
        vdir = LIBDIR / "variants" / variant
        return _build_into(vdir / "obj", vdir / "librrtmg_gpu.so", force, verbose, extra)
    return _build_into(OBJDIR, LIB, force, verbose, extra, peak=True)


def _build_into(objdir: Path, lib: Path, force: bool, verbose: bool, extra, peak: bool = False) -> Path:
    OBJDIR.mkdir(parents=True, exist_ok=True)
    objdir.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    peak_src = CSRC / "fp32_peak.cu"
    if peak and (force or not PEAK_LIB.exists() or peak_src.stat().st_mtime > PEAK_LIB.stat().st_mtime):
        cmd = [cc, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", str(peak_src), "-o", str(PEAK_LIB)]
        procs.append(("fp32_peak.cu", subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                                      text=True)))
    for unit, flags in UNITS.items():
        src = CSRC / unit
        obj = objdir / (unit + ".o")
        objs.append(obj)
        if force or _stale(obj, src):
            cmd = [cc, *ARCH, *COMMON, *flags, *(extra or []), "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    errors = []
    for unit, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {unit} ---\n{out}")
        elif verbose and out.strip():
            print(out)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or any(u != "fp32_peak.cu" for u, _ in procs) or not lib.exists():
        tmp = lib.with_suffix(".so.tmp")
        cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
