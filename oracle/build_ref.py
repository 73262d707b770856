"""Build the host-emulated reference program into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  This recipe reads the GFIRST sources where they
lie ($GFIRST_REFERENCE, else a tree named `reference` beside the repository
checkout), copies the definitions
of the functions listed below verbatim into oracle/_ref/*.inc (git-ignored,
never committed), and compiles them with oracle/ref_shim.h + ref_main.cpp
into one executable per geometry:

    oracle/_ref/gfirst_ref_<geom>         exact FP32 texture weights
    oracle/_ref/gfirst_ref_<geom>_tex8    8-bit texture weights (hardware-like)

Each executable is the reference program itself (its main() and osem3d(),
GFIRST.cu:44-621) with the four positional CLI modes, running its kernels on
the CPU.  tests/golden/make_golden.py runs them to record golden outputs.
The reference tree is absent on the GPU machine; there this script does nothing.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"


def reference_dir() -> Path:
    """The GFIRST source tree: $GFIRST_REFERENCE, else `reference` beside the checkout."""
    env = os.environ.get("GFIRST_REFERENCE")
    return Path(env) if env else HERE.parent.parent / "reference"


REF = reference_dir()

KERNEL_FUNCS = [
    "FORWPROJ_K", "BACKWPROJ_K", "divVxVGPU", "CleanMemoryK", "chequearError",
    "calcGaussianCoefficients", "convolutionXY_GPU", "jointbilateralfilter3D_K",
]
DRIVER_FUNCS = ["osem3d", "main"]
# The reference's GPU build (ref_gpu_main.cu) also takes its host launch
# wrappers and texture set-up, and the CPU routines the driver calls.
GPU_HOST_FUNCS = [
    "FORWPROJ", "BACKWPROJ", "dividirVxVGPU", "CleanMemory", "UpdateImage", "actualizarCorr", "actualizarCalib",
    "crearTexturas", "convolutionXY", "jointbilateralfilter3D",
]
CPU_FUNCS = ["WriteImage", "CreateInitialCylinder", "ReadImage", "ReadSinogram_Type", "gaussian_filterZ"]

# The preclinical geometry the GPU baseline (ref_gpu_main.cu) is built for.
GPU_GEOMS = {
    "preclinical": dict(RES=128, NZS=159, NRAD=128, NANG=160, SPAN=3, NSEG=53, PITCH=1.6, FOV=100.0,
                        DIAM=165.7758),
}

# Geometries the golden fixtures use (name -> GFIRST.h constants).
GEOMS = {
    "tiny": dict(RES=16, NZS=15, NRAD=17, NANG=8, SPAN=3, NSEG=5, PITCH=1.6, FOV=12.5, DIAM=20.7219750, NITER=20),
    "tinyb": dict(RES=20, NZS=18, NRAD=24, NANG=12, SPAN=5, NSEG=3, PITCH=1.63, FOV=15.0, DIAM=24.86637, NITER=20),
    "small": dict(RES=64, NZS=32, NRAD=64, NANG=64, SPAN=3, NSEG=11, PITCH=1.6, FOV=51.2, DIAM=84.8772096, NITER=20),
}


def planes(g: dict) -> int:
    """nz_acum[NSEGMENTS] by GFIRST.cu:133-140."""
    p = 0
    for i in range(g["NSEG"]):
        k = (i + 1) // 2
        zmin = 0 if i == 0 else (k - 1) * g["SPAN"] + (g["SPAN"] // 2 + 1)
        n = g["NZS"] - 2 * zmin
        if n <= 0:
            raise ValueError("segment without planes")
        p += n
    return p


def _skip_literal(src: str, i: int) -> int:
    q = src[i]
    i += 1
    while src[i] != q:
        i += 2 if src[i] == "\\" else 1
    return i + 1


def extract(path: Path, name: str) -> str:
    src = path.read_text(encoding="utf-8", errors="replace")
    m = re.search(r"^[ \t]*(?:__global__[ \t]+)?[A-Za-z_][\w \t\*]*?\b" + re.escape(name) + r"[ \t]*\(", src, re.M)
    if not m:
        raise RuntimeError(f"{name} not found in {path}")
    start = m.start()
    i = src.index("{", m.end())
    depth = 0
    while True:
        c = src[i]
        if src.startswith("//", i):
            i = src.index("\n", i)
            continue
        if src.startswith("/*", i):
            i = src.index("*/", i) + 2
            continue
        if c in "\"'":
            i = _skip_literal(src, i)
            continue
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                break
        i += 1
    line = src.count("\n", 0, start) + 1
    return f'#line {line} "{path}"\n' + src[start:i + 1] + "\n"


def main() -> int:
    if not (REF / "GFIRST.cu").exists():
        print(f"build_ref: no reference tree at {REF}; nothing to build")
        return 0
    OUT.mkdir(exist_ok=True)
    kern = "".join(extract(REF / "GFIRST_GPU_Kernels.cu", f) for f in KERNEL_FUNCS)
    drv = "".join(extract(REF / "GFIRST.cu", f) for f in DRIVER_FUNCS)
    (OUT / "ref_kernels.inc").write_text(kern)
    (OUT / "ref_driver.inc").write_text(drv)
    (OUT / "ref_gpu_host.inc").write_text("".join(extract(REF / "GFIRST_GPU_Kernels.cu", f) for f in GPU_HOST_FUNCS))
    (OUT / "ref_cpu.inc").write_text("".join(extract(REF / "GFIRST_CPU_Kernels.cpp", f) for f in CPU_FUNCS))
    jobs = []
    for name, g in GEOMS.items():
        for tex8 in (False, True):
            exe = OUT / (f"gfirst_ref_{name}" + ("_tex8" if tex8 else ""))
            defs = [f"-DGFR_{k}={v}" for k, v in g.items() if k not in ("PITCH", "FOV", "DIAM")]
            defs += [f"-DGFR_PITCH={g['PITCH']}f", f"-DGFR_FOV={g['FOV']}f", f"-DGFR_DIAM={g['DIAM']}f",
                     f"-DGFR_NSINOGS={planes(g)}"]
            if tex8:
                defs.append("-DGFR_TEX8=1")
            cmd = ["g++", "-std=c++20", "-O2", "-fopenmp", "-ffp-contract=off", "-fpermissive", "-w",
                   f"-I{REF}", f"-I{HERE}", f"-I{OUT}", *defs, str(HERE / "ref_main.cpp"), "-o", str(exe)]
            jobs.append((exe, subprocess.Popen(cmd, stderr=subprocess.PIPE, text=True)))
    rc = 0
    for exe, p in jobs:
        _, err = p.communicate()
        if p.returncode != 0:
            print(f"build_ref: {exe.name} failed:\n{err}", file=sys.stderr)
            rc = 1
    return rc


def gpu_sources_present() -> bool:
    return all((OUT / f).exists() for f in ("ref_kernels.inc", "ref_driver.inc", "ref_gpu_host.inc", "ref_cpu.inc"))


def gpu_build(name: str = "preclinical", niter: int = 2, force: bool = False) -> Path:
    """Compiles the reference's GPU program for geometry `name` with NITER =
    niter, from the sources main() extracted into oracle/_ref/ (they travel
    with the repository copy; the reference tree itself is not needed
    here), with the flags of the reference's compile.sh (-O3
    -use_fast_math) for sm_103a.  Returns the executable's path."""
    if not gpu_sources_present():
        raise FileNotFoundError("oracle/_ref/ holds no extracted reference sources (run build_ref.py beside "
                                "the reference tree)")
    g = GPU_GEOMS[name]
    exe = OUT / f"gfirst_refgpu_{name}_n{niter}"
    if exe.exists() and not force:
        return exe
    defs = [f"-DGFR_{k}={v}" for k, v in g.items() if k not in ("PITCH", "FOV", "DIAM")]
    defs += [f"-DGFR_PITCH={g['PITCH']}f", f"-DGFR_FOV={g['FOV']}f", f"-DGFR_DIAM={g['DIAM']}f",
             f"-DGFR_NSINOGS={planes(g)}", f"-DGFR_NITER={niter}"]
    nvcc = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/bin/nvcc"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-use_fast_math", "-std=c++17", "-w",
           "--expt-extended-lambda", f"-I{HERE}", f"-I{OUT}", *defs, str(HERE / "ref_gpu_main.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference GPU build failed:\n" + r.stderr[-3000:])
    return exe


if __name__ == "__main__":
    sys.exit(main())
