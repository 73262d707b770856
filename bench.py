#!/usr/bin/env python3
"""OSEM sub-iterations/s of the preclinical 3D OSEM workload on GB300.

Workload (one "step"): a full FP32 reconstruction of the preclinical
configuration -- 128x128x159 image, 128 radial bins x 160 angles x 4319
planes (span 3, 53 segments), 16 subsets x 2 iterations = 32
sub-iterations -- from the initial cylinder, with the sinogram and
normalization resident in HBM.  Inputs: a seeded mouse-like phantom
(ellipsoidal body + 10 organs at 2-20x contrast), forward-projected, times
normalization gains U(0.85, 1.15), Poisson at 5e7 counts.

  python bench.py [--gpus N --steps K --warmup W]    this library on N GPUs (replicas)
  python bench.py --impl reference ...               the CPU restatement of the
                                                     reference path (oracle), all cores
  python bench.py --impl reference-shim              the reference program's own GPU design
                                                     (extracted, shimmed textures) on this GPU
  python bench.py --workload frames                  32 dynamic frames: one after another
                                                     in FP32 vs one CUDA graph, FP16 storage
  python bench.py --workload small                   the small configuration in full: GPU vs the
                                                     CPU oracle, images against FP32/FP64 oracles
  python bench.py --workload cli                     the reference's default job through the
                                                     `gfirst` command line, wall clock
  python bench.py --workload triples                 mode 3 (doubles + VLOR triples), FP32/FP16/BF16
                                                     storage, error against the FP64 oracle
  python bench.py --workload serving [--serve-seconds T]
                                                     Poisson request stream through gf_server:
                                                     serial FP32 vs continuous batching, FP16
Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NSUB, NITER = 16, 2
GEOM = (128, 159, 128, 160, 3, 53, 1.6, 165.7758, 100.0)
COUNTS = 5e7
METRIC = "OSEM subiters/s"
UNIT = "subiter/s"
WORKLOAD = ("preclinical 3D OSEM, FP32: 128x128x159 image (0.78x0.78x0.8 mm), 128 radial x 160 angles x "
            "4319 planes (span 3, 53 segments), 16 subsets x 2 iterations per step")
DATA = ("synthetic: seeded mouse-like phantom (body + 10 organs, 2-20x), forward-projected, "
        "gains U(0.85,1.15), Poisson 5e7 counts")


def phantom(seed: int = 1002) -> np.ndarray:
    """Mouse-like phantom [NZS][RES][RES]: ellipsoidal body (activity 1) and 10 hot organs."""
    res, nzs = GEOM[0], GEOM[1]
    rs = np.random.RandomState(seed)
    z, y, x = np.meshgrid(np.arange(nzs, dtype=np.float32), np.arange(res, dtype=np.float32),
                          np.arange(res, dtype=np.float32), indexing="ij")
    c = (res - 1) / 2.0
    cz = (nzs - 1) / 2.0
    body = ((x - c) / 40.0) ** 2 + ((y - c) / 30.0) ** 2 + ((z - cz) / 70.0) ** 2 <= 1.0
    img = np.where(body, 1.0, 0.0).astype(np.float32)
    for _ in range(10):
        ox, oy, oz = rs.uniform(-25, 25), rs.uniform(-18, 18), rs.uniform(-50, 50)
        sx, sy, sz = rs.uniform(3, 9), rs.uniform(3, 9), rs.uniform(4, 14)
        act = rs.uniform(2.0, 20.0)
        organ = ((x - c - ox) / sx) ** 2 + ((y - c - oy) / sy) ** 2 + ((z - cz - oz) / sz) ** 2 <= 1.0
        img = np.where(organ & body, act, img)
    return img.ravel()


def sinogram_from_projection(proj: np.ndarray, seed: int = 1003):
    rs = np.random.RandomState(seed)
    gains = rs.uniform(0.85, 1.15, proj.size).astype(np.float32)
    lam = proj.astype(np.float64) * gains
    lam *= COUNTS / lam.sum()
    prompts = rs.poisson(lam).astype(np.float32)
    dsino = np.concatenate([prompts, np.zeros_like(prompts)])  # prompts, then background 0
    return dsino, gains


def clocks_start(device: int):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    try:
        return subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "100",
                                 "-i", str(device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except OSError:
        return None


def clocks_stop(p) -> dict:
    if p is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    p.terminate()
    out, _ = p.communicate(timeout=10)
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in out.strip().splitlines():
        f = [t.strip() for t in line.split(",")]
        if len(f) < 9:
            continue
        try:
            sm.append(float(f[1]))
            smax.append(float(f[2]))
        except ValueError:
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower().startswith("active"):
                reasons.add(n)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
            "samples": len(sm), "reasons": sorted(reasons)}


def peaks() -> tuple:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(P: int, ndata: int, nvox: int) -> dict:
    """Compulsory HBM bytes per launch (one sub-iteration of 10 angles).
    FP: image read + per ray (data 4 + background 4 + mask 1 + ratio out 4).
    BP: per bin (ratio 4 + mask 1) + the update ratio NUMER/DENOM written."""
    bins_sub = ndata // NSUB
    return {"fp": nvox * 4 + bins_sub * 13, "bp": bins_sub * 5 + nvox * 4}


def committed_traffic() -> dict:
    p = ROOT / "profiles" / "dram_traffic.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


# ----------------------------------------------------------------- CPU (oracle)
def cpu_subiterations(nsteps: int, warmup: int, dsino=None, norm=None, tag: str = "f32", snapshots=()) -> dict:
    """Times sub-iterations of the CPU oracle (FP32 restatement of the reference
    path, OpenMP over all host cores): psf, projection of one subset, ratio, back
    projection, update.  Test infrastructure, used only as the baseline and as
    the checker: the returned "images" hold the oracle's image after each
    sub-iteration count listed in `snapshots` (tag "f64": the FP64 oracle)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import gfo

    gfo.build()
    o = gfo.Oracle(GEOM, tag)
    if dsino is None:
        proj = np.zeros(o.ndata, o.dt)
        img = phantom()
        for s in range(NSUB):
            o.fp(img, NSUB, s, out=proj)
        dsino, norm = sinogram_from_projection(proj)
    res = np.float32(GEOM[0])
    data, bg = dsino[: o.ndata] * res, dsino[o.ndata:] * res
    proj_blank = np.zeros(o.ndata, o.dt)
    cyl = o.cylinder(1.0)
    for s in range(NSUB):
        o.fp(cyl, NSUB, s, out=proj_blank)
    calib = o.calib(proj_blank, norm)
    img = o.cylinder(1.0)
    proj = np.zeros(o.ndata, o.dt)
    corr = np.zeros(o.ndata, o.dt)

    def step(k: int) -> None:
        nonlocal img
        s = k % NSUB
        psf = o.conv_xy(img, 1.5)
        o.fp(psf, NSUB, s, out=proj)
        o.ratio(proj, data, bg, NSUB, s, corr=corr)
        numer, denom = o.bp(corr, calib, NSUB, s)
        img = o.update(img, numer, denom, 1.5)

    images = {}
    for k in range(warmup):
        step(k)
    t0 = time.perf_counter()
    for k in range(nsteps):
        step(warmup + k)
        if warmup + k + 1 in snapshots:
            images[warmup + k + 1] = np.array(img, copy=True)
    dt = time.perf_counter() - t0
    return {"value": nsteps / dt, "unit": UNIT, "cores": gfo.cores(), "kind": "port", "seconds": dt,
            "sample": f"{nsteps} sub-iteration(s) of the preclinical workload (one subset each: psf, projection, "
                      f"ratio, back projection, update), CPU {tag.upper()} oracle, OpenMP",
            "images": images}


def run_reference(args) -> int:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cpu = cpu_subiterations(args.steps, args.warmup)
    cpu.pop("images", None)
    line = {"metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * cpu["seconds"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA, "impl": "reference",
            "config": {"workload": WORKLOAD, "step": "one sub-iteration (a bounded sample of the reconstruction)",
                       "parallelism": "host cores (OpenMP)"},
            "cpu_baseline": cpu, "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------- reference design on the GPU
def run_reference_shim(args) -> int:
    """The reference program's own GPU design on this GPU: its kernels, host
    wrappers, texture set-up and osem3d()/main(), extracted from the
    reference sources by oracle/build_ref.py (test infrastructure, in the
    git-ignored oracle/_ref/) and built with CUDA 13 for sm_103a through
    oracle/ref_gpu_shim.cuh, which maps the removed texture-reference API on
    texture objects.  Mode 1 (`gfirst sino.raw norm.raw`) on the preclinical
    configuration's data, no subsets (the reference's NSUBSETS = 1): one
    launch of the forward and of the back projector per (segment, angle)
    view with the host scatter/gather between them.  Wall clock of the whole
    program at NITER = 2 and NITER = 20; the difference over 18 gives the
    seconds per iteration.  Beside it, this library on the same data with
    one subset (the same work per iteration) and its image after 20
    iterations against the reference program's."""
    import subprocess
    import tempfile

    import torch

    import gfirst_gb300 as gf

    if int(os.environ.get("RANK", "0")) != 0:
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import build_ref

    base = {"impl": "reference-shim", "label": "reference design, shimmed"}
    if not build_ref.gpu_sources_present():
        print(json.dumps(dict(base, unavailable="the reference's sources were not extracted into oracle/_ref/ "
                                               "(build_ref.py runs where the reference tree is)")))
        return 0
    exes = {n: build_ref.gpu_build("preclinical", n) for n in (2, 20)}
    torch.cuda.set_device(0)
    g = gf.Geometry(*GEOM)
    ctx = gf.Context(g, nsub=NSUB)
    dimg = ctx.put(phantom())
    dproj = ctx.array(ctx.ndata).zero()
    for s_ in range(NSUB):
        ctx.forward_project(dimg, s_, dproj)
    proj = dproj.download()
    dimg.free()
    dproj.free()
    ctx.close()
    dsino, norm = sinogram_from_projection(proj)
    out = {}
    with tempfile.TemporaryDirectory() as d:
        dd = Path(d)
        dsino.astype(np.float32).tofile(dd / "sino.raw")
        norm.astype(np.float32).tofile(dd / "norm.raw")

        def run(n):
            t0 = time.perf_counter()
            r = subprocess.run([str(exes[n]), "sino.raw", "norm.raw"], cwd=d, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference GPU program failed: {r.stderr[-500:]}")
            return time.perf_counter() - t0

        run(2)  # first run: driver and module loading
        clk = clocks_start(0)
        t2 = min(run(2) for _ in range(2))
        t20 = run(20)
        clocks = clocks_stop(clk)
        ref_img = np.fromfile(dd / "img_GPU_D_ITER20.raw", np.float32)
    per_iter = (t20 - t2) / 18.0
    # this library, same data, one subset (one iteration = every view once)
    c1 = gf.Context(g, nsub=1)
    tuned = c1.tune()
    r = gf.Recon(c1, 1, niter=20)
    r.load(dsino=dsino, norm=norm)
    r.iterate(2)
    c1.sync()
    t0 = time.perf_counter()
    gf._ck(gf.lib().gf_recon_restart(r.h))
    r.iterate(20)
    c1.sync()
    lib_per_iter = (time.perf_counter() - t0) / 20.0
    img = r.image(0, scaled=True)
    r.close()
    c1.close()
    rel = float(np.linalg.norm(np.float64(img) - ref_img) / np.linalg.norm(np.float64(ref_img)))
    line = dict(base, metric="OSEM iterations/s (no subsets)", value=1.0 / per_iter, unit="iter/s", n_gpus=1,
                steps=20, warmup=2, ms_per_step=1000.0 * per_iter, higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="f32 (-use_fast_math, hardware texture filtering)", data=DATA,
                config={"workload": "preclinical 3D OSEM, mode 1, 128x128x159 image, 128 radial x 160 angles x "
                                    "4319 planes (span 3, 53 segments), no subsets",
                        "step": "one iteration of the reference program (every view once), wall clock "
                                "difference of NITER = 20 and NITER = 2 runs over 18",
                        "seconds_niter2": t2, "seconds_niter20": t20},
                library={"ms_per_iteration": 1000.0 * lib_per_iter, "iterations_per_s": 1.0 / lib_per_iter,
                         "speedup_vs_reference_design": per_iter / lib_per_iter, "tile_shapes": tuned,
                         "image_rel_l2_vs_reference_gpu_after_20": rel},
                clocks=clocks)
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------- GPU
def max_over_ranks(x: float, dist) -> float:
    """The slowest rank's figure (the job ends when its last replica does)."""
    if dist is None:
        return x
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: float, seconds: float) -> float:
    """Units all replicas processed (each rank the same work) over the slowest rank's time."""
    return world * units_per_rank / seconds


def run_gpu(args) -> int:
    import torch

    import gfirst_gb300 as gf

    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    g = gf.Geometry(*GEOM)
    ctx = gf.Context(g, nsub=NSUB, device=local)
    tuned = ctx.tune()  # tile shapes for this geometry, picked by timing (set-up, not timed)
    # the library queues its kernels on this stream; the CUDA events below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    gf._ck(gf.lib().gf_set_stream(ctx.h, gf.ctypes.c_void_p(stream.cuda_stream)))
    # data: the library's own projector on the phantom, then gains and Poisson on the host
    dimg = ctx.put(phantom())
    dproj = ctx.array(ctx.ndata).zero()
    for s in range(NSUB):
        ctx.forward_project(dimg, s, dproj)
    proj = dproj.download()
    dimg.free()
    dproj.free()
    dsino, norm = sinogram_from_projection(proj)

    r = gf.Recon(ctx, 1, niter=NITER)
    r.load(dsino=dsino, norm=norm)

    def step():
        gf._ck(gf.lib().gf_recon_restart(r.h))
        r.iterate(NITER)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    r.profile(True)
    l0 = ctx.launches()
    clk = clocks_start(local)
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    barrier()
    clocks = clocks_stop(clk)
    launches = ctx.launches() - l0
    ms = max_over_ranks(e0.elapsed_time(e1), dist)
    subiters = NSUB * NITER * args.steps
    value = whole_job_rate(world, subiters, ms / 1000.0)
    stage = {}
    for name, sid in gf.STAGES.items():
        tot, n = r.profile_read(sid)
        if n:
            stage[name] = {"ms_per_launch": tot / n, "launches": n, "share": None, "total_ms": tot}
    total_stage = sum(v["total_ms"] for v in stage.values())
    for v in stage.values():
        v["share"] = v["total_ms"] / total_stage if total_stage else None
    r.profile(False)

    # roofline of the dominant kernel (forward or back projector)
    P, ndata, nvox = gf.sizes(g)
    alg = algorithmic_bytes(P, ndata, nvox)
    peak, peak_src = peaks()
    traffic = committed_traffic()
    dom = max(("fp", "bp"), key=lambda k: stage.get(k, {}).get("total_ms", 0.0))
    roof = {}
    for k in ("fp", "bp"):
        if k not in stage:
            continue
        ach = alg[k] / (stage[k]["ms_per_launch"] / 1000.0) / 1e9
        roof[k] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                   "traffic": traffic.get(k, {}).get("bytes_per_launch"), "algorithmic_bytes": alg[k],
                   "ms_per_launch": stage[k]["ms_per_launch"], "peak_source": f"{peak_src} hbm_gbs"}
    roofline = dict(roof[dom], kernel=dom)
    roofline["other"] = {k: v for k, v in roof.items() if k != dom}
    # the projectors are bound on chip: instruction issue against the SMs'
    # peak (4 warp instructions per SM per cycle at the sampled clock), from
    # the warp-instruction count ncu measured per launch and the live duration
    props = torch.cuda.get_device_properties(local)
    onchip = {}
    for k in ("fp", "bp"):
        ins = traffic.get(k, {}).get("warp_instructions")
        if k in stage and ins:
            rate = ins / (stage[k]["ms_per_launch"] / 1000.0)
            peak_rate = props.multi_processor_count * 4 * (clocks["sm_mhz"] or clocks["sm_max_mhz"] or 0) * 1e6
            onchip[k] = {"bound": "issue", "achieved": rate / 1e12, "peak": peak_rate / 1e12,
                         "unit": "T warp-instr/s", "frac": rate / peak_rate if peak_rate else None,
                         "warp_instructions_per_launch": ins,
                         "ncu_lsu_data_pipe_pct": traffic[k].get("lsu_data_pipe_pct")}
    roofline["onchip"] = onchip

    # end to end through the public API with host buffers: load (host->device of the
    # sinogram and normalization) + 32 sub-iterations + scaled image back to the host
    e2e = None
    if args.e2e_steps > 0:
        # end to end through the public C-ABI with pinned host buffers: every
        # step uploads its sinogram + normalization, runs the 32 sub-iterations
        # and reads the scaled image back.  Three reconstructions of one
        # context take the steps in turn: steps k+1 and k+2 are queued
        # (gf_recon_load_async, their uploads on the context's copy stream,
        # overlapping step k's iterations) before step k's image is read back
        # (also on the copy stream, after step k's own work only), so an
        # upload has two steps' iterations to finish in; the
        # one-reconstruction sequential loop is reported beside it.
        NB = 3  # reconstructions (and host buffer sets) in rotation
        n2 = 2 * ndata
        per = n2 + ndata + nvox
        hp = gf.ctypes.c_void_p()
        gf._ck(gf.lib().gf_host_alloc(gf.ctypes.c_size_t(NB * per * 4), gf.ctypes.byref(hp)))
        buf = np.ctypeslib.as_array(gf.ctypes.cast(hp, gf.ctypes.POINTER(gf.ctypes.c_float)), (NB * per,))
        host = []
        for i in range(NB):
            b = buf[i * per:(i + 1) * per]
            hs, hn, ho = b[:n2], b[n2:n2 + ndata], b[n2 + ndata:]
            hs[:] = dsino
            hn[:] = norm
            host.append((hs, hn, ho))
        recs = [gf.Recon(ctx, 1, niter=NITER) for _ in range(NB)]
        ptr = lambda a: a.ctypes.data_as(gf.ctypes.c_void_p)  # noqa: E731
        lib = gf.lib()

        def issue(k, wait=False):
            r, (hs, hn, _) = recs[k % NB], host[k % NB]
            fn = lib.gf_recon_load if wait else lib.gf_recon_load_async
            gf._ck(fn(r.h, None, ptr(hs), None, ptr(hn), None, gf.ctypes.c_int64(0)))
            r.iterate(NITER)

        def read(k):
            gf._ck(lib.gf_recon_get_image(recs[k % NB].h, 0, 1, ptr(host[k % NB][2])))

        for k in range(NB):  # warm-up: device staging, the geometry projection
            issue(k, wait=True)
            read(k)
        # a long-running host keeps the garbage collector off its set-up's
        # objects: a full collection over the interpreter's and torch's
        # objects stalls the issuing thread for tens of milliseconds
        gc.collect()
        gc.freeze()
        # where a sequential step's time goes (host clock): the synchronous load,
        # queueing the iterations, then waiting for them and reading the image
        phases = {"load_ms": [], "queue_ms": [], "wait_read_ms": []}
        for k in range(3):
            t0 = time.perf_counter()
            gf._ck(lib.gf_recon_load(recs[0].h, None, ptr(host[0][0]), None, ptr(host[0][1]), None,
                                     gf.ctypes.c_int64(0)))
            t1 = time.perf_counter()
            recs[0].iterate(NITER)
            t2 = time.perf_counter()
            read(0)
            t3 = time.perf_counter()
            phases["load_ms"].append(1000 * (t1 - t0))
            phases["queue_ms"].append(1000 * (t2 - t1))
            phases["wait_read_ms"].append(1000 * (t3 - t2))
        phases = {k: statistics.median(v) for k, v in phases.items()}
        barrier()
        t0 = time.perf_counter()
        seq_ms = []
        for k in range(args.e2e_steps):  # one reconstruction at a time
            ts = time.perf_counter()
            issue(0, wait=True)
            read(0)
            seq_ms.append(1000 * (time.perf_counter() - ts))
        dt_seq = max_over_ranks(time.perf_counter() - t0, dist)

        def pipelined(nsteps, times=None):
            ts = time.perf_counter()
            for k in range(min(NB - 1, nsteps)):
                issue(k)
            for k in range(nsteps):
                if k + NB - 1 < nsteps:
                    issue(k + NB - 1)
                read(k)
                if times is not None:
                    t1 = time.perf_counter()
                    times.append(1000 * (t1 - ts))
                    ts = t1

        # warm-up of the pipelined loop itself (3 steps), then the timed loop
        # from an empty pipeline
        pipelined(3)
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        step_ms = []  # host clock from one image's read-back to the next
        pipelined(args.e2e_steps, step_ms)
        torch.cuda.synchronize()
        dt = max_over_ranks(time.perf_counter() - t0, dist)
        e2e = {"value": whole_job_rate(world, NSUB * NITER * args.e2e_steps, dt), "unit": UNIT,
               "h2d_bytes_per_step": (n2 + ndata) * 4, "d2h_bytes_per_step": nvox * 4,
               "steps": args.e2e_steps, "ms_per_step": 1000.0 * dt / args.e2e_steps,
               "step_ms": [round(x, 2) for x in step_ms],
               "median_step_ms": round(statistics.median(step_ms), 2),
               "path": "per step: gf_recon_load_async(pinned host sinogram+normalization) + gf_recon_iterate(2) + "
                       "gf_recon_get_image(scaled); three reconstructions of one context take the steps in turn, "
                       "the next two steps' uploads (copy stream) and iterations queued before this step's "
                       "image is read back",
               "sequential_phases": phases,
               "sequential": {"value": whole_job_rate(world, NSUB * NITER * args.e2e_steps, dt_seq),
                              "ms_per_step": 1000.0 * dt_seq / args.e2e_steps,
                              "step_ms": [round(x, 2) for x in seq_ms],
                              "path": "gf_recon_load + gf_recon_iterate(2) + gf_recon_get_image, one "
                                      "reconstruction, each step after the previous one"}}
        gc.unfreeze()
        for rr in recs:
            rr.close()
        gf.lib().gf_host_free(hp)

    cpu, accuracy = None, None
    if rank == 0 and world == 1 and args.cpu_steps > 0:
        # The CPU oracle's sub-iterations are the baseline and the checker: the
        # GPU image after the same sub-iterations from the same start is
        # compared with the FP32 oracle's, and, on a shorter sample, with the
        # FP64 oracle's (the accuracy bound is stated against FP64).
        n64 = min(args.fp64_steps, args.cpu_steps)
        cpu = cpu_subiterations(args.cpu_steps, 0, dsino, norm, snapshots={args.cpu_steps, n64})
        img32 = cpu.pop("images")

        def gpu_image_after(n):
            gf._ck(gf.lib().gf_recon_restart(r.h))
            for _ in range(n):
                r.subiteration()
            return r.image(0)

        def rel(a, b):
            return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b.astype(np.float64)))

        accuracy = {"subiterations": args.cpu_steps,
                    "rel_l2_vs_fp32_oracle": rel(gpu_image_after(args.cpu_steps), img32[args.cpu_steps]),
                    "tolerance": 1e-3,
                    "sample": f"doubles image after the first {args.cpu_steps} sub-iterations of the headline "
                              f"reconstruction (same inputs, same start); FP64 oracle on the first {n64}"}
        if n64 > 0:
            img64 = cpu_subiterations(n64, 0, dsino, norm, tag="f64", snapshots={n64})["images"][n64]
            g64 = gpu_image_after(n64)
            accuracy["fp64_subiterations"] = n64
            accuracy["rel_l2_vs_fp64_oracle"] = rel(g64, img64)
            accuracy["fp32_oracle_vs_fp64_oracle"] = rel(img32[n64], img64)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA,
                "config": {"workload": WORKLOAD,
                           "step": "one full reconstruction (32 sub-iterations) from the initial cylinder, "
                                   "data resident in HBM",
                           "l2": "inputs larger than L2: each sub-iteration streams a different subset's data "
                                 "and mask (1.1 GB in all, 68 MB per sub-iteration; L2 129 MB)",
                           "parallelism": f"replicas x{world}", "subsets": NSUB, "iterations": NITER,
                           "tile_shapes": tuned},
                "rays_per_s": value * ndata / NSUB, "ray_samples_per_s": value * ndata / NSUB * (g.res + 1),
                "voxel_views_per_s": value * nvox * (g.nang // NSUB) * g.nseg,
                "stages": stage, "roofline": roofline, "accuracy": accuracy,
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
        print(json.dumps(line))
    r.close()
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ----------------------------------------------------------------- other workloads
def ellipsoid_phantom(res: int, nzs: int, seed: int, norgans: int = 6) -> tuple:
    """Body ellipsoid and hot organ ellipsoids scaled to the image, [NZS][RES][RES]:
    returns (body without organs, organs at their contrast)."""
    rs = np.random.RandomState(seed)
    z, y, x = np.meshgrid(np.arange(nzs, dtype=np.float32), np.arange(res, dtype=np.float32),
                          np.arange(res, dtype=np.float32), indexing="ij")
    c, cz = (res - 1) / 2.0, (nzs - 1) / 2.0
    ax, ay, az = 0.31 * res, 0.23 * res, 0.44 * nzs
    body = ((x - c) / ax) ** 2 + ((y - c) / ay) ** 2 + ((z - cz) / az) ** 2 <= 1.0
    organs = np.zeros_like(x)
    for _ in range(norgans):
        ox, oy, oz = rs.uniform(-0.6, 0.6) * ax, rs.uniform(-0.6, 0.6) * ay, rs.uniform(-0.7, 0.7) * az
        sx, sy, sz = rs.uniform(0.07, 0.2) * ax, rs.uniform(0.07, 0.2) * ay, rs.uniform(0.05, 0.15) * az
        o = ((x - c - ox) / sx) ** 2 + ((y - c - oy) / sy) ** 2 + ((z - cz - oz) / sz) ** 2 <= 1.0
        organs = np.where(o & body, rs.uniform(2.0, 20.0), organs)
    bg = np.where(body & (organs == 0), 1.0, 0.0).astype(np.float32)
    return bg.ravel(), organs.astype(np.float32).ravel()


def project(gf, ctx, img: np.ndarray):
    """Full projection of a [NZS][RES][RES] image with the library's projector, left on the device."""
    import torch

    d = ctx.put(img)
    out = torch.zeros(ctx.ndata, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the library's stream does not wait for torch's
    arr = gf.DeviceArray.view(ctx, out.data_ptr(), ctx.ndata)
    for s in range(ctx.nsub):
        ctx.forward_project(d, s, arr)
    ctx.sync()
    d.free()
    return out


def noisy_sinogram(lam, gains, counts: float, seed: int):
    """Prompts ~ Poisson(lam * gains scaled to `counts`), background 0; (dsino, norm) on the host."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    m = lam * gains
    m = m * (counts / float(m.sum()))
    prompts = torch.poisson(m, generator=g)
    dsino = np.zeros(2 * lam.numel(), np.float32)
    dsino[: lam.numel()] = prompts.cpu().numpy()
    return dsino, gains.cpu().numpy()


def gpu_gains(n: int, seed: int):
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    return 0.85 + 0.3 * torch.rand(n, generator=g, device="cuda")


def run_frames(args) -> int:
    """32 dynamic frames at the preclinical geometry (or, with --frames-geometry
    small, the 64x64x32 one, where one frame does not fill the GPU).  Seeded two-compartment
    time-activity curves (blood-like washout in the body, uptake in the organs)
    shape each frame; counts are log-uniform over 1e5-5e7; each frame uses 4, 8
    or 16 subsets and 2 iterations.  Plain: the frames one after another in FP32
    with the default tile shapes.  Batched: FP16 storage of the ratio sinogram,
    autotuned tile shapes, every frame's iteration replayed from one CUDA graph
    (frames run as parallel branches); batched_f32 the same in FP32 storage.
    Fused (and fused_f32): the same graph with the frames fused into groups of
    up to 16 whatever their subset counts (one tuned tile-shape set for every
    frame), each step of a group one launch per stage over the frames that
    have that subset, the back projection two frames per warp for frames of
    one subset count (the frames share the scanner's normalization);
    fused_launch_only: the groups with one frame per warp (gf_batch_set_fused).
    Data resident in HBM in every arm.  The first and last frames of every arm
    are compared with the FP64 oracle (--fp64-oracle 0 skips that)."""
    import torch

    import gfirst_gb300 as gf

    torch.cuda.set_device(0)
    nf, niter = args.frames, 2
    rs = np.random.RandomState(2024)
    nsubs = rs.choice([4, 8, 16], nf)
    counts = np.exp(rs.uniform(np.log(1e5), np.log(5e7), nf))
    t = np.cumsum(np.geomspace(0.5, 6.0, nf))  # frame mid-times, minutes
    blood = 1.0 + 9.0 * np.exp(-t / 1.5)
    uptake = 1.0 - np.exp(-t / 12.0)
    geo = GEOM if args.frames_geometry == "preclinical" else SMALL_GEOM
    g = gf.Geometry(*geo)
    c0 = gf.Context(g, nsub=16)
    bg, organs = ellipsoid_phantom(geo[0], geo[1], 7, norgans=10)
    pb, po = project(gf, c0, bg), project(gf, c0, organs)
    c0.close()
    gains = gpu_gains(pb.numel(), 11)
    data = []
    for k in range(nf):
        data.append(noisy_sinogram(blood[k] * pb + uptake[k] * po, gains, counts[k], 100 + k))
    del pb, po, gains
    torch.cuda.empty_cache()

    def build(storage: str, tune: bool, one_shape: bool = False):
        ctxs, recs, tuned = [], [], []
        # tuned once per subset count (one_shape: once for all frames, so that
        # frames of every count can share a fused launch), then set on the
        # other frames' contexts
        shapes = {}
        for k in range(nf):
            c = gf.Context(g, nsub=int(nsubs[k]))
            key = 0 if one_shape else int(nsubs[k])
            if tune and key not in shapes:
                shapes[key] = c.tune()
            elif tune:
                t = shapes[key]
                c.set_tile_shapes(t["fp_run"], t["fp_chunk"], t["bp_warps"])
            tuned.append(shapes.get(key) if tune else None)
            r = gf.Recon(c, 1, niter=niter, storage=storage)
            r.load(dsino=data[k][0], norm=data[k][1])
            r._keep = None
            ctxs.append(c)
            recs.append(r)
        return ctxs, recs, tuned

    subiters = int(sum(int(s) * niter for s in nsubs))
    out = {}
    check = sorted({0, nf - 1})  # frames whose images are compared with the FP64 oracle
    imgs = {}
    # fused: 0 no, 1 groups with frame pairs back-projected together, 2 groups only
    arms = {"plain": ("f32", False, 0), "batched_f32": ("f32", True, 0), "batched": ("f16", True, 0),
            "fused_launch_only": ("f16", True, 2), "fused_f32": ("f32", True, 1), "fused": ("f16", True, 1)}
    for arm, (storage, batched, fused) in arms.items():
        ctxs, recs, tuned = build(storage, batched, one_shape=fused > 0)
        batch = gf.Batch(recs) if batched else None
        if fused:
            batch.set_fused(True, pairs=fused == 1)

        def once():
            for r in recs:
                r.restart()
            if batch is None:
                for c, r in zip(ctxs, recs):  # one frame at a time
                    r.iterate(niter)
                    c.sync()
            else:
                batch.iterate(niter, graph=True)
                batch.sync()

        for _ in range(args.warmup):
            once()
        gc.collect()
        gc.freeze()  # the issuing thread stays clear of full collections over the set-up's objects
        l0 = sum(c.launches() for c in ctxs)
        clk = clocks_start(0)
        time.sleep(0.3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            once()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / args.steps
        clocks = clocks_stop(clk)
        gc.unfreeze()
        launches = (sum(c.launches() for c in ctxs) - l0) // args.steps
        img0 = recs[0].image()
        for k in check:
            imgs[(arm, k)] = recs[k].image()
        out[arm] = {"ms_per_step": 1000.0 * dt, "subiters_per_s": subiters / dt, "frames_per_s": nf / dt,
                    "storage": storage, "graph": batched, "fused": fused,
                    "units": batch.groups() if batch is not None else (nf, 1, 0),
                    "gpu_launches_per_step": launches, "clocks": clocks,
                    "tuned": sorted({json.dumps(x, sort_keys=True) for x in tuned if x}) or None,
                    "frame0_image_sum": float(img0.astype(np.float64).sum())}
        if batch is not None:
            batch.close()
        for r in recs:
            r.close()
        for c in ctxs:
            c.close()
    rel = abs(out["batched"]["frame0_image_sum"] / out["plain"]["frame0_image_sum"] - 1.0)

    def rl2(a, b):
        return float(np.linalg.norm(np.float64(a) - b) / np.linalg.norm(np.float64(b)))

    # accuracy: the first and last frames of every arm against the FP64 oracle
    # on the same inputs (test infrastructure, used only as the checker)
    accuracy = None
    if args.fp64_oracle:
        sys.path.insert(0, str(ROOT / "oracle"))
        import gfo

        gfo.build()
        accuracy = {"tolerance": 1e-3}
        for k in check:
            t0 = time.perf_counter()
            ref = gfo.Oracle(geo, "f64").recon(1, nsub=int(nsubs[k]), niter=niter, dsino=data[k][0],
                                              norm=data[k][1])["img_d"]
            accuracy[f"frame{k}"] = {"subsets": int(nsubs[k]), "counts": float(counts[k]),
                                     "oracle_seconds": time.perf_counter() - t0,
                                     **{f"{arm}_rel_l2_vs_fp64": rl2(imgs[(arm, k)], ref) for arm in arms}}
    line = {"metric": METRIC, "value": out["fused"]["subiters_per_s"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["fused"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 arithmetic",
            "data": "synthetic: seeded body + 10 organs, two-compartment curves, gains U(0.85,1.15), Poisson",
            "config": {"workload": f"{nf} dynamic frames, " + ("preclinical geometry (128x128x159, 128x160x4319)"
                                   if geo is GEOM else "small geometry (64x64x32, 64x64x192)") +
                                   f", {niter} iterations, subsets per frame in {{4,8,16}}",
                       "subsets": [int(x) for x in nsubs], "counts": [float(x) for x in counts],
                       "subiterations_per_step": subiters,
                       "step": "every frame restarted from the cylinder and reconstructed, data resident"},
            "arms": out, "speedup_fused_vs_plain": out["fused"]["subiters_per_s"] / out["plain"]["subiters_per_s"],
            "speedup_fused_f32_vs_plain": out["fused_f32"]["subiters_per_s"] / out["plain"]["subiters_per_s"],
            "speedup_batched_vs_plain": out["batched"]["subiters_per_s"] / out["plain"]["subiters_per_s"],
            "speedup_batched_f32_vs_plain": out["batched_f32"]["subiters_per_s"] / out["plain"]["subiters_per_s"],
            "frame0_sum_rel_diff_f16_vs_f32": rel, "accuracy": accuracy}
    print(json.dumps(line))
    return 0


SMALL_GEOM = (64, 32, 64, 64, 3, 11, 1.6, 84.8772096, 51.2)


def run_small(args) -> int:
    """The small plain-FP32 configuration, reconstructed in full on the GPU and
    by the CPU oracle (FP32, OpenMP over the host cores) on the same inputs:
    64x64x32 voxels of 0.8 mm, 64 radial x 64 angles x 192 planes (span 3, 11
    segments); a water cylinder (radius 0.9 FOV/2, activity 0.1) with 6 seeded
    ellipsoids (semi-axes 2-8 voxels, activity 0.5-5), forward-projected,
    gains U(0.9, 1.1), Poisson at 1e6 counts; 4 subsets x 3 iterations.  The
    images are compared with the FP32 and FP64 oracles (test infrastructure,
    used only as the checker and the CPU baseline)."""
    import torch

    import gfirst_gb300 as gf

    torch.cuda.set_device(0)
    nsub, niter = 4, 3
    res, nzs = SMALL_GEOM[0], SMALL_GEOM[1]
    rs = np.random.RandomState(1001)
    z, y, x = np.meshgrid(np.arange(nzs, dtype=np.float32), np.arange(res, dtype=np.float32),
                          np.arange(res, dtype=np.float32), indexing="ij")
    c = (res - 1) / 2.0
    cyl = ((x - c) ** 2 + (y - c) ** 2) <= (0.9 * res / 2) ** 2
    img = np.where(cyl, 0.1, 0.0).astype(np.float32)
    for _ in range(6):
        r = rs.uniform(0, 0.6 * res / 2)
        ph = rs.uniform(0, 2 * np.pi)
        ox, oy, oz = r * np.cos(ph), r * np.sin(ph), rs.uniform(-nzs / 2 + 4, nzs / 2 - 4)
        sx, sy, sz = rs.uniform(2, 8, 3)
        e = ((x - c - ox) / sx) ** 2 + ((y - c - oy) / sy) ** 2 + ((z - (nzs - 1) / 2 - oz) / sz) ** 2 <= 1.0
        img = np.where(e & cyl, rs.uniform(0.5, 5.0), img).astype(np.float32)
    g = gf.Geometry(*SMALL_GEOM)
    ctx = gf.Context(g, nsub=nsub)
    lam = project(gf, ctx, img.ravel()).double().cpu().numpy()
    gains = rs.uniform(0.9, 1.1, lam.size)
    lam = lam * gains
    lam *= 1e6 / lam.sum()
    dsino = np.concatenate([rs.poisson(lam), np.zeros(lam.size)]).astype(np.float32)
    norm = gains.astype(np.float32)
    tuned = ctx.tune()

    r = gf.Recon(ctx, 1, niter=niter)
    r.load(dsino=dsino, norm=norm)
    for _ in range(args.warmup):
        r.restart()
        r.iterate(niter)
    ctx.sync()
    steps = max(args.steps, 1)
    t0 = time.perf_counter()
    for _ in range(steps):
        r.restart()
        r.iterate(niter)
    ctx.sync()
    dt = (time.perf_counter() - t0) / steps
    gpu_img = r.image(0)
    # the same reconstruction with the image and the ratio sinogram in FP16
    r16 = gf.Recon(ctx, 1, niter=niter, storage="f16", image_storage="f16")
    r16.load(dsino=dsino, norm=norm)
    for _ in range(args.warmup):
        r16.restart()
        r16.iterate(niter)
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        r16.restart()
        r16.iterate(niter)
    ctx.sync()
    dt16 = (time.perf_counter() - t0) / steps
    img16 = r16.image(0)
    r16.close()
    # end to end: load from host buffers, iterate, read the image back
    t0 = time.perf_counter()
    for _ in range(steps):
        r.load(dsino=dsino, norm=norm)
        r.iterate(niter)
        out_img = r.image(0)
    e2e = (time.perf_counter() - t0) / steps
    r.close()
    ctx.close()

    sys.path.insert(0, str(ROOT / "oracle"))
    import gfo

    gfo.build()
    t0 = time.perf_counter()
    ref32 = gfo.Oracle(SMALL_GEOM, "f32").recon(1, nsub=nsub, niter=niter, dsino=dsino, norm=norm)
    cpu_s = time.perf_counter() - t0
    ref64 = gfo.Oracle(SMALL_GEOM, "f64").recon(1, nsub=nsub, niter=niter, dsino=dsino, norm=norm)

    def rel(a, b):
        return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))

    subiters = nsub * niter
    line = {"metric": METRIC, "value": subiters / dt, "unit": UNIT, "n_gpus": 1, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * dt, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded water cylinder + 6 ellipsoids, "
            "gains U(0.9,1.1), Poisson 1e6 counts",
            "config": {"workload": "small plain FP32 OSEM: 64x64x32 image (0.8 mm), 64 radial x 64 angles x 192 "
                                   "planes (span 3, 11 segments), 4 subsets x 3 iterations",
                       "step": "one full reconstruction from the cylinder, data resident", "tile_shapes": tuned},
            "e2e": {"value": subiters / e2e, "unit": UNIT, "ms_per_step": 1000.0 * e2e,
                    "h2d_bytes_per_step": int(dsino.nbytes + norm.nbytes), "d2h_bytes_per_step": int(out_img.nbytes)},
            "cpu_baseline": {"value": subiters / cpu_s, "unit": UNIT, "cores": gfo.cores(), "kind": "port",
                             "sample": "the full reconstruction (12 sub-iterations), CPU FP32 oracle, OpenMP",
                             "seconds": cpu_s},
            "gpu_vs_cpu_speedup": (subiters / dt) / (subiters / cpu_s),
            "rel_l2_vs_fp32_oracle": rel(gpu_img, ref32["img_d"]), "rel_l2_vs_fp64_oracle": rel(gpu_img, ref64["img_d"]),
            "fp16_image_and_ratio": {"subiters_per_s": subiters / dt16, "ms_per_step": 1000.0 * dt16,
                                     "rel_l2_vs_fp64_oracle": rel(img16, ref64["img_d"])},
            "fp32_oracle_vs_fp64": rel(ref32["img_d"], ref64["img_d"])}
    print(json.dumps(line))
    return 0


def run_cli(args) -> int:
    """The reference's default job through the drop-in command line: `gfirst
    sino.raw norm.raw` on the geometry compiled into the reference (128x128x159,
    147 radial x 168 angles x 1293 planes, span 11, 15 segments), 60 iterations
    without subsets, images written every 20 iterations.  Inputs are seeded
    synthetic raw files (mouse-like phantom projected by the library, gains
    U(0.85, 1.15), Poisson 5e7); the wall clock of the whole process is timed
    (start-up, file reads, set-up, iterations, file writes)."""
    import subprocess
    import tempfile

    import torch

    import gfirst_gb300 as gf

    torch.cuda.set_device(0)
    g = gf.Geometry.reference()
    ctx = gf.Context(g, nsub=1)
    bg, organs = ellipsoid_phantom(g.res, g.nzs, 81, norgans=10)
    lam = project(gf, ctx, bg + organs)
    ctx.close()
    dsino, norm = noisy_sinogram(lam, gpu_gains(lam.numel(), 82), COUNTS, 83)
    del lam
    torch.cuda.empty_cache()
    runs = []
    with tempfile.TemporaryDirectory() as d:
        dd = Path(d)
        dsino.astype(np.float32).tofile(dd / "sino.raw")
        norm.astype(np.float32).tofile(dd / "norm.raw")
        for _ in range(max(args.steps, 1)):
            t0 = time.perf_counter()
            r = subprocess.run([str(gf.CLI_PATH), "sino.raw", "norm.raw"], cwd=d, capture_output=True, text=True)
            runs.append(time.perf_counter() - t0)
            if r.returncode != 0:
                print(json.dumps({"workload": "cli", "error": r.stderr[-500:]}))
                return 1
        outs = sorted(p.name for p in dd.glob("img_GPU_D_ITER*.raw"))
        img = np.fromfile(dd / "img_GPU_D_ITER60.raw", np.float32)
    best = min(runs)
    line = {"metric": "OSEM iterations/s", "value": 60 / best, "unit": "iter/s", "n_gpus": 1, "steps": len(runs),
            "warmup": 0, "ms_per_step": 1000.0 * best, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded body + 10 organs, gains U(0.85,1.15), "
            "Poisson 5e7, float32 raw files",
            "config": {"workload": "`gfirst sino.raw norm.raw`: reference geometry 128x128x159, 147x168x1293 "
                                   "(span 11, 15 segments), 60 iterations, no subsets, writes every 20",
                       "step": "one run of the command line, wall clock of the process"},
            "seconds_per_run": runs, "outputs": outs, "image_finite": bool(np.isfinite(img).all()),
            "image_sum": float(img.astype(np.float64).sum())}
    print(json.dumps(line))
    return 0


def run_triples(args) -> int:
    """Doubles + triples joint reconstruction (mode 3) at the preclinical
    geometry.  Two seeded tracers with different ellipsoid maps; doubles =
    Poisson of the projection of both at 4e7 counts, triples sinogram = Poisson
    of the second tracer's projection at 2e6; 2e6 VLOR events, each a true bin
    drawn in proportion to the second tracer's projection and a partner bin
    drawn uniformly over the masked bins, stored as float32 LOR endpoint pairs
    and converted on the device.  8 subsets x 3 iterations in FP32, FP16 and
    BF16 storage of the ratio sinogram; each image's error against the FP64
    oracle run on the host on the same inputs (test infrastructure, used only
    as the checker)."""
    import torch

    import gfirst_gb300 as gf

    torch.cuda.set_device(0)
    nsub, niter, nev = 8, 3, args.events
    g = gf.Geometry(*GEOM)
    ctx = gf.Context(g, nsub=nsub)
    bg1, org1 = ellipsoid_phantom(GEOM[0], GEOM[1], 61, norgans=10)
    bg2, org2 = ellipsoid_phantom(GEOM[0], GEOM[1], 62, norgans=6)
    t1, t2 = bg1 + org1, 0.3 * bg2 + org2
    p1, p2 = project(gf, ctx, t1), project(gf, ctx, t2)
    res = GEOM[0]
    yy, xx = np.meshgrid(np.arange(res), np.arange(res), indexing="ij")
    cyl = ((xx - res / 2) ** 2 + (yy - res / 2) ** 2 <= (res / 2) ** 2).astype(np.float32)
    pblank = project(gf, ctx, np.broadcast_to(cyl, (GEOM[1], res, res)).ravel())
    gains = gpu_gains(p1.numel(), 71)
    dsino, norm = noisy_sinogram(p1 + p2, gains, 4e7, 72)
    tsino, _ = noisy_sinogram(p2, gains, 2e6, 73)
    # events: true bin ~ second tracer's projection, partner uniform over masked bins
    rs = np.random.RandomState(74)
    lam2 = (p2 * gains).double().cpu().numpy()
    cdf = np.cumsum(lam2)
    true_bins = np.searchsorted(cdf, rs.uniform(0, cdf[-1], nev), side="right")
    masked = np.flatnonzero(pblank.cpu().numpy() > 0.01)
    partner = masked[rs.randint(0, masked.size, nev)]
    swap = rs.rand(nev) < 0.5
    pairs = np.stack([np.where(swap, partner, true_bins), np.where(swap, true_bins, partner)], axis=1)
    del lam2, cdf, p1, p2, pblank, gains
    torch.cuda.empty_cache()
    lors = gf.bins_endpoints(g, pairs.ravel()).reshape(nev, 12)
    dl, de = ctx.put(lors), ctx.array(2 * nev, np.int32)
    ctx.vlor_from_endpoints(dl, nev, de)
    events = de.download().reshape(nev, 2)
    dl.free()
    de.free()
    round_trip = bool(np.array_equal(events, pairs + 1))

    out = {}
    imgs = {}
    for storage in ("f32", "f16", "bf16"):
        r = gf.Recon(ctx, 3, niter=niter, storage=storage)
        r.load(dsino=dsino, tsino=tsino, norm=norm, events=events)
        r.iterate(1)  # warm-up
        ctx.sync()
        gf._ck(gf.lib().gf_recon_restart(r.h))
        ctx.sync()
        t0 = time.perf_counter()
        r.iterate(niter)
        ctx.sync()
        dt = time.perf_counter() - t0
        imgs[storage] = (r.image(0), r.image(1))
        out[storage] = {"seconds": dt, "subiters_per_s": 2 * nsub * niter / dt}
        # stage times of the same reconstruction (library CUDA events), not timed above
        r.restart()
        r.profile(True)
        r.iterate(niter)
        stages = {}
        for name, sid in gf.STAGES.items():
            tot, n = r.profile_read(sid)
            if n:
                stages[name] = {"launches": n, "ms_per_launch": tot / n, "total_ms": tot}
        out[storage]["stages"] = stages
        r.profile(False)
        r.close()
    if not args.fp64_oracle:
        print(json.dumps({"workload": "triples", "arms": out, "config": {"events": nev, "subsets": nsub,
                                                                         "iterations": niter}}))
        ctx.close()
        return 0
    # FP64 oracle on the host (the checker)
    sys.path.insert(0, str(ROOT / "oracle"))
    import gfo

    gfo.build()
    t0 = time.perf_counter()
    ref = gfo.Oracle(GEOM, "f64").recon(3, nsub=nsub, niter=niter, dsino=dsino, tsino=tsino, norm=norm, ev=events)
    oracle_s = time.perf_counter() - t0
    ref32 = None
    if args.fp32_oracle:
        ref32 = gfo.Oracle(GEOM, "f32").recon(3, nsub=nsub, niter=niter, dsino=dsino, tsino=tsino, norm=norm,
                                               ev=events)

    def rel(a, b):
        return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))

    for storage, (d, t) in imgs.items():
        out[storage]["rel_l2_vs_fp64_doubles"] = rel(d, ref["img_d"])
        out[storage]["rel_l2_vs_fp64_triples"] = rel(t, ref["img_t"])
        if ref32 is not None:
            out[storage]["rel_l2_vs_fp32_oracle_doubles"] = rel(d, ref32["img_d"])
            out[storage]["rel_l2_vs_fp32_oracle_triples"] = rel(t, ref32["img_t"])
    if ref32 is not None:  # how far the FP32 reference algorithm itself sits from FP64
        out["fp32_oracle"] = {"rel_l2_vs_fp64_doubles": rel(ref32["img_d"], ref["img_d"]),
                              "rel_l2_vs_fp64_triples": rel(ref32["img_t"], ref["img_t"])}
    line = {"metric": METRIC, "value": out["f32"]["subiters_per_s"], "unit": UNIT, "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": 1000.0 * out["f32"]["seconds"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 arithmetic",
            "data": "synthetic: two seeded ellipsoid tracers, gains U(0.85,1.15), Poisson 4e7 / 2e6, "
                    f"{nev} VLOR events as float32 endpoint pairs",
            "config": {"workload": "doubles + triples joint reconstruction (mode 3), preclinical geometry, "
                                   f"{nsub} subsets x {niter} iterations",
                       "events": nev, "endpoint_round_trip_exact": round_trip,
                       "step": "one reconstruction from the initial images, data resident"},
            "arms": out, "fp64_oracle_seconds": oracle_s, "oracle_cores": gfo.cores()}
    print(json.dumps(line))
    ctx.close()
    return 0


SERVE_SIZES = {
    "64^3": ((64, 64, 64, 64, 3, 21, 1.6, 84.8772096, 51.2), 8),
    "96^3": ((96, 96, 96, 96, 3, 31, 1.6, 127.3158, 76.8), 8),
    "128x128x159": (GEOM, 16),
}


def run_serving(args) -> int:
    """Poisson request stream through gf_server.  Arrivals at 20/s (seeded);
    sizes uniform over 64^3, 96^3 and 128x128x159 voxels; a quarter are bare
    forward projections of seeded ellipsoid phantoms, the rest reconstructions
    of 2 or 3 iterations with counts log-uniform over 1e5-5e7 (drawn from a
    pool of 6 pre-generated noisy sinograms per size).  HBM budget 150 GB.
    Plain: FP32, one request at a time.  Batched: FP16 storage of the ratio
    sinogram, up to 8 requests in flight (continuous batching).  Latency runs
    from submission to the result in host memory.  With --serve-closed C the
    same request mix runs as a closed loop instead (--serve-requests of them,
    C in flight at all times), which measures each arm's capacity rather than
    the offered rate.  Accuracy: sampled reconstructions of the batched arm
    against the same requests in the plain arm, and one 64^3 request of each
    arm against the FP64 oracle (test infrastructure, used as the checker)."""
    import threading

    import torch

    import gfirst_gb300 as gf

    torch.cuda.set_device(0)
    rs = np.random.RandomState(77)
    pool = {}
    for name, (geo, nsub) in SERVE_SIZES.items():
        g = gf.Geometry(*geo)
        c = gf.Context(g, nsub=nsub)
        bg, organs = ellipsoid_phantom(geo[0], geo[1], 31, norgans=6)
        lam = project(gf, c, bg + organs)
        c.close()
        gains = gpu_gains(lam.numel(), 32)
        lv = np.exp(rs.uniform(np.log(1e5), np.log(5e7), 6))
        sinos = [noisy_sinogram(lam, gains, float(x), 40 + i) for i, x in enumerate(lv)]
        if args.serve_pinned:  # clients hand the server page-locked buffers
            sinos = [(gf.host_copy(a), gf.host_copy(b)) for a, b in sinos]
        imgs = []
        for i in range(4):
            b, o = ellipsoid_phantom(geo[0], geo[1], 50 + i)
            imgs.append(gf.host_copy(b + o) if args.serve_pinned else b + o)
        pool[name] = (g, nsub, sinos, imgs, [float(x) for x in lv])
        del lam, gains
    torch.cuda.empty_cache()
    names = list(SERVE_SIZES)
    n = int(rs.poisson(args.serve_rate * args.serve_seconds))
    arrivals = np.sort(rs.uniform(0.0, args.serve_seconds, n))
    reqs = []
    for i in range(n):
        nm = names[rs.randint(3)]
        if rs.rand() < 0.25:
            reqs.append(("project", nm, rs.randint(4), 0))
        else:
            reqs.append(("recon", nm, rs.randint(6), 2 + rs.randint(2)))
    budget = 150 * 10**9
    closed = args.serve_closed > 0
    if closed:  # a fixed list of requests, kept args.serve_closed in flight: the arms' capacity
        n = args.serve_requests
        reqs = reqs[:n] if len(reqs) >= n else (reqs * (n // max(len(reqs), 1) + 1))[:n]
    # outputs kept for the accuracy comparison: every 8th reconstruction request
    sample = [i for i, q in enumerate(reqs) if q[0] == "recon"][::8][:24]
    kept = {}
    out = {}
    for arm, storage, max_active in (("plain", "f32", 1), ("batched", "f16", 8)):
        srv = gf.Server(budget, max_active=max_active)
        lat = {"project": [], "recon": []}
        lock = threading.Lock()

        def submit(i):
            kind, nm, k, it = reqs[i]
            g, nsub, sinos, imgs, _ = pool[nm]
            if kind == "project":
                return srv.submit_project(g, imgs[k], nsub)
            return srv.submit_recon(g, sinos[k][0], sinos[k][1], nsub, it, storage)

        def finish(i, rid):
            res, ms = srv.wait(rid)
            with lock:
                lat[reqs[i][0]].append(ms)
                if i in sample:
                    kept[(arm, i)] = np.array(res, copy=True)

        gc.collect()
        gc.freeze()  # the client threads stay clear of full collections over the set-up's objects
        clk = clocks_start(0)
        t0 = time.perf_counter()
        if closed:
            nxt = [0]

            def worker():
                while True:
                    with lock:
                        i = nxt[0]
                        nxt[0] += 1
                    if i >= n:
                        return
                    finish(i, submit(i))

            ths = [threading.Thread(target=worker) for _ in range(args.serve_closed)]
            for th in ths:
                th.start()
            for th in ths:
                th.join()
        else:
            ids = [None] * n

            def submitter():
                for i in range(n):
                    d = arrivals[i] - (time.perf_counter() - t0)
                    if d > 0:
                        time.sleep(d)
                    ids[i] = submit(i)

            th = threading.Thread(target=submitter)
            th.start()
            for i in range(n):
                while ids[i] is None:
                    time.sleep(0.0005)
                finish(i, ids[i])
            th.join()
        t_end = time.perf_counter()
        clocks = clocks_stop(clk)
        gc.unfreeze()
        st = srv.stats()
        srv.close()
        by_kind = {k: {"n": len(v), "p50_ms": float(np.percentile(v, 50)), "p99_ms": float(np.percentile(v, 99))}
                   for k, v in lat.items() if v}
        out[arm] = {"storage": storage, "max_active": max_active, "completed": st["completed"],
                    "failed": st["failed"], "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                    "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
                    "throughput_per_s": st["completed"] / (t_end - t0),
                    "makespan_s": t_end - t0, "peak_active": st["peak_active"],
                    "mean_queue_ms": st["queue_ms"], "mean_load_ms": st["load_ms"], "mean_run_ms": st["run_ms"],
                    "peak_bytes": st["peak_bytes"], "by_kind": by_kind, "clocks": clocks}

    def rel(a, b):
        return float(np.linalg.norm(np.float64(a) - b) / max(np.linalg.norm(np.float64(b)), 1e-30))

    # accuracy: each sampled reconstruction of the batched (FP16-storage) arm
    # against the same request in the plain FP32 arm, and the first sampled
    # 64^3 request of both arms against the FP64 oracle on its inputs
    diffs = [rel(kept[("batched", i)], kept[("plain", i)]) for i in sample
             if ("batched", i) in kept and ("plain", i) in kept]
    accuracy = {"requests_compared": len(diffs),
                "batched_vs_plain_rel_l2_max": max(diffs) if diffs else None,
                "batched_vs_plain_rel_l2_median": float(np.median(diffs)) if diffs else None}
    small = [i for i in sample if reqs[i][1] == "64^3"]
    if small and args.fp64_oracle:
        i = small[0]
        _, nm, k, it = reqs[i]
        g, nsub, sinos, _, _ = pool[nm]
        sys.path.insert(0, str(ROOT / "oracle"))
        import gfo

        gfo.build()
        ref = gfo.Oracle(g.tuple(), "f64").recon(1, nsub=nsub, niter=it, dsino=sinos[k][0], norm=sinos[k][1])
        accuracy["fp64_request"] = {"size": nm, "subsets": nsub, "iterations": int(it),
                                    "plain_rel_l2_vs_fp64": rel(kept[("plain", i)], ref["img_d"]),
                                    "batched_rel_l2_vs_fp64": rel(kept[("batched", i)], ref["img_d"])}
    wl = (f"closed loop: {n} requests, {args.serve_closed} in flight at all times (capacity)" if closed else
          f"Poisson request stream, {args.serve_rate:g} req/s for {args.serve_seconds:g} s")
    line = {"metric": "requests/s", "value": out["batched"]["throughput_per_s"], "unit": "req/s", "n_gpus": 1,
            "steps": n, "warmup": 0, "ms_per_step": out["batched"]["mean_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 arithmetic",
            "data": "synthetic: seeded ellipsoid phantoms, gains U(0.85,1.15), Poisson",
            "config": {"workload": wl + ", sizes 64^3 / 96^3 / 128x128x159, 25% bare projections, "
                                        "2-3 iterations, HBM budget 150 GB",
                       "requests": n, "subsets": {k: v[1] for k, v in SERVE_SIZES.items()},
                       "count_levels": {k: pool[k][4] for k in names}},
            "arms": out, "speedup_batched_vs_plain": out["batched"]["throughput_per_s"] /
                                                     out["plain"]["throughput_per_s"],
            "accuracy": accuracy}
    print(json.dumps(line))
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference", "reference-shim"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=12)
    ap.add_argument("--fp64-steps", type=int, default=4, help="sub-iterations of the FP64 oracle for the "
                    "headline's accuracy field (0: FP32 oracle only)")
    ap.add_argument("--workload", default="recon", choices=["recon", "frames", "serving", "triples", "small", "cli"])
    ap.add_argument("--events", type=int, default=2_000_000)
    ap.add_argument("--fp32-oracle", type=int, default=1, help="triples: also compare with the FP32 oracle")
    ap.add_argument("--fp64-oracle", type=int, default=1, help="triples: compare with the FP64 oracle (0: GPU only)")
    ap.add_argument("--frames", type=int, default=32)
    ap.add_argument("--frames-geometry", default="preclinical", choices=["preclinical", "small"])
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-closed", type=int, default=0,
                    help="serving: keep this many requests in flight (closed loop, capacity) instead of the stream")
    ap.add_argument("--serve-requests", type=int, default=300, help="serving, closed loop: requests in all")
    ap.add_argument("--serve-pinned", type=int, default=1,
                    help="serving: request inputs in page-locked host memory (0: pageable numpy arrays)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.impl == "reference-shim":
        return run_reference_shim(args)
    if args.workload == "frames":
        return run_frames(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "triples":
        return run_triples(args)
    if args.workload == "small":
        return run_small(args)
    if args.workload == "cli":
        return run_cli(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
