"""Build libgfirst.so (sm_103a) and the `gfirst` command line in-tree.

Every .cu file is compiled with nvcc for sm_103a only, every host .cpp with
g++ -ffp-contract=off (the geometry tables must not be fused differently on
x86 and Arm), in parallel; outputs go to gfirst_gb300/lib/.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "lib"
INC = PKG.parent / "include"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU = ["gf_fp.cu", "gf_bp.cu", "gf_image.cu", "gf_sino.cu", "gf_noalloc.cu"]
CPP = ["gf_plan.cpp", "gf_capi.cpp", "gf_recon.cpp", "gf_io.cpp", "gf_batch.cpp", "gf_tune.cpp", "gf_server.cpp"]
LIB = OUT / "libgfirst.so"
CLI = OUT / "gfirst"


def _nvcc() -> str:
    p = CUDA / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _headers_mtime() -> float:
    hs = list(SRC.glob("*.h")) + list(SRC.glob("*.cuh")) + list(INC.glob("*.h"))
    return max(h.stat().st_mtime for h in hs)


def _stale(obj: Path, src: Path, hdr: float) -> bool:
    return not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr)


def _run(cmd: list) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False, extra_nvcc: list | None = None) -> Path:
    OUT.mkdir(exist_ok=True)
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for f in CU:
        src, obj = SRC / f, OUT / (f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, hdr):
            jobs.append([_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", *(extra_nvcc or []), "-I", str(SRC), "-c", str(src),
                         "-o", str(obj)])
    for f in CPP + ["gf_cli.cpp"]:
        src, obj = SRC / f, OUT / (f + ".o")
        if f != "gf_cli.cpp":
            objs.append(obj)
        if force or _stale(obj, src, hdr):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I", str(CUDA / "include"), "-I", str(SRC), "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for _ in ex.map(_run, jobs):
            pass
    if force or jobs or not LIB.exists():
        _run([_nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(LIB),
              "-L", str(CUDA / "lib64")])
        _run(["g++", str(OUT / "gf_cli.cpp.o"), "-o", str(CLI), "-L", str(OUT), "-lgfirst",
              "-Wl,-rpath,$ORIGIN", "-L", str(CUDA / "lib64"), "-lcudart"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
