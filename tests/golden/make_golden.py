"""Record golden outputs of the reference program itself.

Runs oracle/_ref/gfirst_ref_<geom> -- GFIRST's own main()/osem3d() and
kernels, compiled from the reference sources by oracle/build_ref.py and run
on the CPU with emulated textures -- in each of its four CLI modes on the
seeded inputs of tests/golden/inputs.py, and stores what it writes
(proj_ref.raw, img_GPU_D/T_ITER20.raw, SINOG_VLOR.raw) in
tests/golden/golden_<geom>.npz.

Needs the reference tree (only present in the development container):
    python oracle/build_ref.py && python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(HERE))
import inputs  # noqa: E402

REFDIR = ROOT / "oracle" / "_ref"


def run_mode(exe: Path, files: dict, mode: int) -> dict:
    args = {0: ["img.raw"], 1: ["sinoD.raw", "norm.raw"], 2: ["sinoD.raw", "sinoT.raw", "norm.raw"],
            3: ["sinoD.raw", "sinoT.raw", "norm.raw", "vlor.raw"]}[mode]
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for k, v in files.items():
            (td / k).write_bytes(v)
        subprocess.run([str(exe), *args], cwd=td, check=True, stdout=subprocess.DEVNULL)
        out = {}
        for f in ["proj_ref.raw", "img_GPU_D_ITER20.raw", "img_GPU_T_ITER20.raw", "SINOG_VLOR.raw"]:
            if (td / f).exists():
                out[f] = np.fromfile(td / f, dtype=np.float32)
        return out


def main() -> int:
    names = sys.argv[1:] or ["tiny", "tinyb", "small"]
    for name in names:
        exe = REFDIR / f"gfirst_ref_{name}"
        if not exe.exists():
            print(f"missing {exe}; run oracle/build_ref.py first")
            return 1
        files = inputs.case_files(name)
        store = {"inputs_sha": np.array(json.dumps({k: inputs.sha(v) for k, v in files.items()}))}
        modes = [0, 1, 2, 3] if name != "small" else [0, 1]
        for mode in modes:
            out = run_mode(exe, files, mode)
            key = {"proj_ref.raw": "proj_ref", "img_GPU_D_ITER20.raw": "img_D",
                   "img_GPU_T_ITER20.raw": "img_T", "SINOG_VLOR.raw": "sinog_vlor"}
            for f, arr in out.items():
                if name == "small" and f == "proj_ref.raw":
                    store[f"m{mode}_proj_ref_sha"] = np.array(inputs.sha(arr.tobytes()))
                    store[f"m{mode}_proj_ref_sample"] = arr[::97].copy()
                else:
                    store[f"m{mode}_{key[f]}"] = arr
            if name == "tiny" and mode in (0, 1):
                out8 = run_mode(REFDIR / f"gfirst_ref_{name}_tex8", files, mode)
                store[f"m{mode}_tex8_proj_ref"] = out8["proj_ref.raw"]
                if mode == 1:
                    store["m1_tex8_img_D"] = out8["img_GPU_D_ITER20.raw"]
            print(f"{name} mode {mode}: {sorted(out)}")
        np.savez_compressed(HERE / f"golden_{name}.npz", **store)
    return 0


if __name__ == "__main__":
    sys.exit(main())
