"""Build of the native library ``_lib/libkurucz_gb300.so`` (sm_103a only).

Eight translation units compiled in parallel with nvcc and linked into one
shared library exporting the C ABI of ``include/kurucz_gb300.h``:

* ``ks_f32.cu``  kernels in single precision (mixed path), ``--fmad=false``
* ``ks_f32_batch.cu`` their batched launches (one per stage over a job table)
* ``ks_f64.cu``  kernels in double precision, ``--fmad=false``
* ``ks_f64_batch.cu`` their batched launches
* ``ks_api.cu``  C ABI, tables, bins, reach-class partition, drivers
* ``ks_pops.cu`` FP64 populations (molecular equilibrium, Saha, Doppler), ``--fmad=false``
* ``ks_hydrogen.cu`` hydrogen line opacity (HPROF4 profiles, FP64), ``--fmad=false``
* ``ks_gfall.cpp`` native gfall reader
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_build"
LIB_NAME = "libkurucz_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build the library")
    return cand


def _units():
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "--expt-relaxed-constexpr"]
    return [
        # no implicit multiply-add contraction in either precision: the FMAs
        # the kernels want are written as fmaf/__fmaf_rn, so a kernel body
        # inlined into the single-synthesis and the batched kernels rounds
        # identically in both (the batch equals single syntheses bit for bit)
        (CSRC / "ks_f32.cu", common + ["--fmad=false"]),
        (CSRC / "ks_f32_batch.cu", common + ["--fmad=false"]),
        (CSRC / "ks_f64.cu", common + ["--fmad=false"]),
        (CSRC / "ks_f64_batch.cu", common + ["--fmad=false"]),
        (CSRC / "ks_api.cu", common),
        # FP64 populations: products and sums rounded one by one, as the reference's
        (CSRC / "ks_pops.cu", common + ["--fmad=false"]),
        (CSRC / "ks_hydrogen.cu", common + ["--fmad=false"]),
        (CSRC / "ks_gfall.cpp", ["-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread"]),
    ]


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def _newest_source_mtime() -> float:
    files = list(CSRC.glob("*")) + [PKG.parent / "include" / "kurucz_gb300.h", Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.exists())


def up_to_date() -> bool:
    lib = lib_path()
    return lib.exists() and lib.stat().st_mtime >= _newest_source_mtime()


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return lib_path()
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(item):
        src, flags = item
        obj = BUILD_DIR / (src.name + ".o")
        cmd = [cc, *flags, "-I", str(CSRC), "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{res.stdout}\n{res.stderr}")
        return obj

    units = _units()
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = OUT_DIR / (LIB_NAME + ".tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True))
