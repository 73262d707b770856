"""Kernel micro-benchmark: time one projector stage on a named geometry.

    python -m gfirst_gb300.kbench --op bp|fp|subiter [--geometry preclinical] [--subsets 16] [--reps 5]
                                  [--storage f32|f16|bf16] [--tune] [--bp-form view|voxel] [--pairs]

Runs a mode-1 reconstruction's stages on synthetic data and reports the
device time per launch from the library's own stage events.  With --pairs,
two frames of one normalization run as a fused group instead (the paired
back projector), timed per frame and iteration on the host clock.  Small
enough to run under a profiler (one context, a few launches).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

import gfirst_gb300 as gf

GEOMS = {"preclinical": gf.Geometry.preclinical, "reference": gf.Geometry.reference, "small": gf.Geometry.small}


def run(op: str, geometry: str, nsub: int, reps: int, storage: str = "f32", tune: bool = False,
        bp_form: str = "view", pairs: bool = False) -> dict:
    g = GEOMS[geometry]()
    ctx = gf.Context(g, nsub=nsub)
    ctx.set_bp_form(bp_form)
    tuned = ctx.tune() if tune else None
    P, ndata, nvox = gf.sizes(g)
    rs = np.random.RandomState(5)
    dsino = np.concatenate([rs.poisson(20.0, ndata), np.zeros(ndata)]).astype(np.float32)
    norm = rs.uniform(0.85, 1.15, ndata).astype(np.float32)
    r = gf.Recon(ctx, 1, niter=1, storage=storage)
    r.load(dsino=dsino, norm=norm)
    if pairs:
        r2 = gf.Recon(ctx, 1, niter=1, storage=storage)
        r2.load(dsino=np.roll(dsino, 17), norm=norm)
        b = gf.Batch([r, r2])
        b.set_fused(True, pairs=True)
        b.iterate(1, graph=False)  # warm-up
        b.sync()
        t0 = time.perf_counter()
        b.iterate(reps, graph=False)
        b.sync()
        dt = time.perf_counter() - t0
        out = {"geometry": geometry, "subsets": nsub, "reps": reps, "storage": storage, "tuned": tuned,
               "bp_form": bp_form, "groups": b.groups(), "ms_per_frame_iteration": 1000 * dt / (2 * reps)}
        b.close()
        r2.close()
        r.close()
        ctx.close()
        return out
    r.subiteration()  # warm-up
    r.profile(True)
    for _ in range(reps):
        r.subiteration()
    out = {"geometry": geometry, "subsets": nsub, "reps": reps, "storage": storage, "tuned": tuned,
           "bp_form": bp_form}
    for name, sid in gf.STAGES.items():
        tot, n = r.profile_read(sid)
        if n:
            out[name + "_ms"] = tot / n
    r.close()
    ctx.close()
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="subiter", choices=["bp", "fp", "subiter"])
    ap.add_argument("--geometry", default="preclinical", choices=sorted(GEOMS))
    ap.add_argument("--subsets", type=int, default=16)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--storage", default="f32", choices=["f32", "f16", "bf16"])
    ap.add_argument("--tune", action="store_true")
    ap.add_argument("--bp-form", default="view", choices=["voxel", "view"])
    ap.add_argument("--pairs", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run(a.op, a.geometry, a.subsets, a.reps, a.storage, a.tune, a.bp_form, a.pairs)))


if __name__ == "__main__":
    main()
