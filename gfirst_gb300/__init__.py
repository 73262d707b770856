"""gfirst_gb300 -- GB300 (sm_103a) implementation of GFIRST's OSEM hot path.

The product is the C-ABI library lib/libgfirst.so (include/gfirst.h) and the
`gfirst` command line (lib/gfirst), a drop-in for the reference program's
four modes.  This module is a thin ctypes front end over that C-ABI; it never
computes anything itself and raises if the library is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libgfirst.so"
CLI_PATH = _HERE / "lib" / "gfirst"

STAGES = {"psf": 0, "fp": 1, "vlor": 2, "bp": 3, "update": 4, "bilateral": 5}
STATUS = {0: "GF_OK", 1: "GF_ERR_ARG", 2: "GF_ERR_GEOMETRY", 3: "GF_ERR_CUDA", 4: "GF_ERR_NOMEM",
          5: "GF_ERR_IO", 6: "GF_ERR_STATE", 7: "GF_ERR_NODEV", 8: "GF_ERR_TIMEOUT"}


class GfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class _CGeom(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("res", "nzs", "nrad", "nang", "span", "nseg")] + \
               [(n, ctypes.c_float) for n in ("pitch_mm", "diam_det_mm", "fov_mm")]


class _CParams(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("niter", ctypes.c_int32), ("psf_fw", ctypes.c_float),
                ("psf_bw", ctypes.c_float), ("scale_d", ctypes.c_float), ("scale_t", ctypes.c_float),
                ("storage", ctypes.c_int32), ("image_storage", ctypes.c_int32)]


STORE = {"f32": 0, "f16": 1, "bf16": 2}


@dataclass(frozen=True)
class Geometry:
    """The compile-time constants of GFIRST.h:4-36, chosen at run time."""
    res: int
    nzs: int
    nrad: int
    nang: int
    span: int
    nseg: int
    pitch: float
    diam: float
    fov: float

    def c(self) -> _CGeom:
        return _CGeom(self.res, self.nzs, self.nrad, self.nang, self.span, self.nseg, self.pitch, self.diam, self.fov)

    def tuple(self) -> tuple:
        return (self.res, self.nzs, self.nrad, self.nang, self.span, self.nseg, self.pitch, self.diam, self.fov)

    @staticmethod
    def reference() -> "Geometry":
        """GFIRST.h as compiled: Inveon, 128x128x159, 147x168, span 11, 15 segments."""
        return Geometry(128, 159, 147, 168, 11, 15, 1.63, 165.7758, 100.0)

    @staticmethod
    def small() -> "Geometry":
        """64x64x32 image of 0.8 mm, 64 radial x 64 angles, span 3, 11 segments (192 planes)."""
        return Geometry(64, 32, 64, 64, 3, 11, 1.6, 84.8772096, 51.2)

    @staticmethod
    def preclinical() -> "Geometry":
        """128x128x159 image (0.78 x 0.78 x 0.8 mm), 128 radial x 160 angles, span 3, 53 segments (4319 planes)."""
        return Geometry(128, 159, 128, 160, 3, 53, 1.6, 165.7758, 100.0)


def _load() -> ctypes.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(str(LIB_PATH))
    lib.gf_last_error.restype = ctypes.c_char_p
    for name in ("gf_create", "gf_destroy", "gf_device_alloc"):
        getattr(lib, name)
    lib.gf_destroy.restype = None
    lib.gf_recon_destroy.restype = None
    lib.gf_batch_destroy.restype = None
    lib.gf_server_destroy.restype = None
    lib.gf_copy_to_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.gf_copy_to_host.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
    lib.gf_device_alloc.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]
    lib.gf_device_free.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    return lib


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = _load()
    return _lib


def _ck(st: int) -> None:
    if st != 0:
        raise GfError(st, lib().gf_last_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def sizes(g: Geometry) -> tuple:
    p, nd, nv = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    _ck(lib().gf_geometry_sizes(ctypes.byref(g.c()), ctypes.byref(p), ctypes.byref(nd), ctypes.byref(nv)))
    return p.value, nd.value, nv.value


def segment_table(g: Geometry):
    idz, zmin, acc = (np.zeros(g.nseg, np.int32), np.zeros(g.nseg, np.int32), np.zeros(g.nseg + 1, np.int32))
    _ck(lib().gf_segment_table(ctypes.byref(g.c()), _ptr(idz), _ptr(zmin), _ptr(acc)))
    return idz, zmin, acc


def bp_staged_rows(g: Geometry) -> dict:
    """The per-view back projector's staged-row buffer (gf_bp_staged_rows)."""
    lo, hi, rb = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    _ck(lib().gf_bp_staged_rows(ctypes.byref(g.c()), ctypes.byref(lo), ctypes.byref(hi), ctypes.byref(rb)))
    return {"pad_lo": lo.value, "pad_hi": hi.value, "rbuf": rb.value}


def lor_index(g: Geometry, seg: int, iz0: int, theta: int, ird: int) -> int:
    out = ctypes.c_int64()
    _ck(lib().gf_lor_index(ctypes.byref(g.c()), seg, iz0, theta, ird, ctypes.byref(out)))
    return out.value


class DeviceArray:
    """A device buffer owned through the C-ABI's allocation helpers."""

    def __init__(self, ctx: "Context", n: int, dtype=np.float32):
        self.ctx, self.n, self.dtype = ctx, int(n), np.dtype(dtype)
        p = ctypes.c_void_p()
        _ck(lib().gf_device_alloc(ctx.h, self.nbytes, ctypes.byref(p)))
        self.p = p
        self._owned = True

    @classmethod
    def view(cls, ctx: "Context", ptr: int, n: int, dtype=np.float32) -> "DeviceArray":
        """Borrow device memory allocated elsewhere (e.g. a torch tensor's data_ptr());
        never freed here."""
        a = cls.__new__(cls)
        a.ctx, a.n, a.dtype = ctx, int(n), np.dtype(dtype)
        a.p = ctypes.c_void_p(int(ptr))
        a._owned = False
        return a

    @property
    def nbytes(self) -> int:
        return self.n * self.dtype.itemsize

    def upload(self, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a, dtype=self.dtype).ravel()
        assert a.size == self.n
        _ck(lib().gf_copy_to_device(self.ctx.h, self.p, _ptr(a), self.nbytes))
        return self

    def download(self) -> np.ndarray:
        out = np.empty(self.n, self.dtype)
        _ck(lib().gf_copy_to_host(self.ctx.h, _ptr(out), self.p, self.nbytes))
        return out

    def zero(self) -> "DeviceArray":
        return self.upload(np.zeros(self.n, self.dtype))

    def free(self) -> None:
        if self.p and self._owned:
            lib().gf_device_free(self.ctx.h, self.p)
        self.p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """gf_ctx: geometry, subsets and a stream on one device."""

    def __init__(self, g: Geometry, nsub: int = 1, device: int = 0):
        self.g, self.nsub = g, nsub
        self.P, self.ndata, self.nvox = sizes(g)
        h = ctypes.c_void_p()
        _ck(lib().gf_create(ctypes.byref(g.c()), nsub, device, ctypes.byref(h)))
        self.h = h

    def close(self) -> None:
        if self.h:
            lib().gf_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def array(self, n: int, dtype=np.float32) -> DeviceArray:
        return DeviceArray(self, n, dtype)

    def put(self, a: np.ndarray, dtype=np.float32) -> DeviceArray:
        a = np.ascontiguousarray(a, dtype=dtype).ravel()
        return DeviceArray(self, a.size, dtype).upload(a)

    def sync(self) -> None:
        _ck(lib().gf_synchronize(self.h))

    def launches(self) -> int:
        n = ctypes.c_int64()
        _ck(lib().gf_kernel_launches(self.h, ctypes.byref(n)))
        return n.value

    def set_bp_form(self, form: str) -> None:
        """Back projector's axial interpolation: "voxel" (GF_BP_PER_VOXEL) or "view" (GF_BP_PER_VIEW)."""
        _ck(lib().gf_set_bp_form(self.h, {"voxel": 0, "view": 1}[form]))

    def set_tile_shapes(self, fp_run: int, fp_chunk: int, bp_warps: int) -> None:
        _ck(lib().gf_set_tile_shapes(self.h, fp_run, fp_chunk, bp_warps))

    def tune(self) -> dict:
        r, lc, w = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _ck(lib().gf_tune(self.h, ctypes.byref(r), ctypes.byref(lc), ctypes.byref(w)))
        return {"fp_run": r.value, "fp_chunk": lc.value, "bp_warps": w.value}

    # operators on device arrays (reference file layouts)
    def forward_project(self, img: DeviceArray, subset: int, proj: DeviceArray) -> None:
        _ck(lib().gf_forward_project(self.h, img.p, subset, proj.p))

    def ratio(self, proj, data, bg, subset, corr) -> None:
        _ck(lib().gf_ratio(self.h, proj.p, data.p, bg.p, subset, corr.p))

    def norm_mask(self, proj_blank, blank, calib) -> None:
        _ck(lib().gf_norm_mask(self.h, proj_blank.p, blank.p, calib.p))

    def back_project(self, corr, calib, subset, numer, denom) -> None:
        _ck(lib().gf_back_project(self.h, corr.p, calib.p, subset, numer.p, denom.p))

    def psf_xy(self, src, psf, dst) -> None:
        _ck(lib().gf_psf_xy(self.h, src.p, ctypes.c_float(psf), dst.p))

    def image_update(self, img, numer, denom, psf_bw=1.5) -> None:
        _ck(lib().gf_image_update(self.h, img.p, numer.p, denom.p, ctypes.c_float(psf_bw)))

    def bilateral(self, src, ref, max_ref, dst, r=4, sigma3d=0.75, sigmai=0.025) -> None:
        _ck(lib().gf_bilateral(self.h, src.p, ref.p, ctypes.c_float(max_ref), r, ctypes.c_float(sigma3d),
                               ctypes.c_float(sigmai), dst.p))

    def vlor_count(self, ev, nev, cnt) -> None:
        _ck(lib().gf_vlor_count(self.h, ev.p, ctypes.c_int64(nev), cnt.p))

    def vlor_from_endpoints(self, lors, nev, events) -> None:
        _ck(lib().gf_vlor_from_endpoints(self.h, lors.p, ctypes.c_int64(nev), events.p))

    def vlor_split(self, ev, nev, proj, blankt, out) -> None:
        _ck(lib().gf_vlor_split(self.h, ev.p, ctypes.c_int64(nev), proj.p, blankt.p, out.p))


def recon_defaults(mode: int) -> _CParams:
    p = _CParams()
    _ck(lib().gf_recon_defaults(mode, ctypes.byref(p)))
    return p


class Recon:
    """gf_recon: one reconstruction of a CLI mode, resident on the device."""

    def __init__(self, ctx: Context, mode: int, niter: int = 60, psf_fw: float = 1.5, psf_bw: float = 1.5,
                 storage: str = "f32", image_storage: str = "f32"):
        self.ctx, self.mode = ctx, mode
        p = recon_defaults(mode)
        p.niter, p.psf_fw, p.psf_bw, p.storage = niter, psf_fw, psf_bw, STORE[storage]
        p.image_storage = STORE[image_storage]
        self.params = p
        h = ctypes.c_void_p()
        _ck(lib().gf_recon_create(ctx.h, ctypes.byref(p), ctypes.byref(h)))
        self.h = h

    def close(self) -> None:
        if self.h:
            # gf_destroy has already destroyed the reconstructions of a closed context
            if self.ctx.h:
                lib().gf_recon_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load(self, image=None, dsino=None, tsino=None, norm=None, events=None, wait: bool = True) -> None:
        """Inputs as the CLI reads them.  wait=False queues the load
        (gf_recon_load_async): the arrays are kept referenced here until the
        next load, and must not be modified until the context's stream has
        passed it."""
        f32 = lambda a: None if a is None else np.ascontiguousarray(a, np.float32).ravel()  # noqa: E731
        image, dsino, tsino, norm = f32(image), f32(dsino), f32(tsino), f32(norm)
        ev = None if events is None else np.ascontiguousarray(events, np.int32)
        nev = 0 if ev is None else ev.size // 2
        self._keep = (image, dsino, tsino, norm, ev)
        p = lambda a: None if a is None else _ptr(a)  # noqa: E731
        fn = lib().gf_recon_load if wait else lib().gf_recon_load_async
        _ck(fn(self.h, p(image), p(dsino), p(tsino), p(norm), p(ev), ctypes.c_int64(nev)))

    def iterate(self, n: int = 1) -> None:
        _ck(lib().gf_recon_iterate(self.h, n))

    def restart(self) -> None:
        _ck(lib().gf_recon_restart(self.h))

    def subiteration(self) -> None:
        _ck(lib().gf_recon_subiteration(self.h))

    def image(self, typ: int = 0, scaled: bool = False) -> np.ndarray:
        out = np.empty(self.ctx.nvox, np.float32)
        _ck(lib().gf_recon_get_image(self.h, typ, int(scaled), _ptr(out)))
        return out

    def proj_ref(self) -> np.ndarray:
        out = np.empty(self.ctx.ndata, np.float32)
        _ck(lib().gf_recon_get_proj_ref(self.h, _ptr(out)))
        return out

    def profile(self, enable: bool = True) -> None:
        _ck(lib().gf_recon_profile(self.h, int(enable)))

    def profile_read(self, stage: int) -> tuple:
        ms, n = ctypes.c_double(), ctypes.c_int64()
        _ck(lib().gf_recon_profile_read(self.h, stage, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def sinog_vlor(self) -> np.ndarray:
        out = np.empty(self.ctx.ndata, np.float32)
        _ck(lib().gf_recon_get_sinog_vlor(self.h, _ptr(out)))
        return out


class Batch:
    """gf_batch: loaded reconstructions advancing together, optionally from a CUDA graph."""

    def __init__(self, recons):
        self.recons = list(recons)
        arr = (ctypes.c_void_p * len(self.recons))(*[r.h.value for r in self.recons])
        h = ctypes.c_void_p()
        _ck(lib().gf_batch_create(len(self.recons), arr, ctypes.byref(h)))
        self.h = h

    def set_fused(self, fused: bool = True, pairs: bool = True) -> None:
        """Fused groups: frames that match (any subset counts) run each stage
        as one launch; with pairs, frames of one subset count and equal
        normalization back-project two per warp (gf_batch_set_fused 1, else 2;
        fused=False: 0)."""
        _ck(lib().gf_batch_set_fused(self.h, 0 if not fused else (1 if pairs else 2)))

    def groups(self) -> tuple:
        """(units, largest group, frame pairs back-projected together) as the batch stands now."""
        n, big, pr = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _ck(lib().gf_batch_groups(self.h, ctypes.byref(n), ctypes.byref(big), ctypes.byref(pr)))
        return n.value, big.value, pr.value

    def iterate(self, n: int = 1, graph: bool = True) -> None:
        _ck(lib().gf_batch_iterate(self.h, n, int(graph)))

    def sync(self) -> None:
        _ck(lib().gf_batch_synchronize(self.h))

    def close(self) -> None:
        if self.h:
            lib().gf_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _CRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("geometry", _CGeom), ("nsubsets", ctypes.c_int32),
                ("niter", ctypes.c_int32), ("storage", ctypes.c_int32), ("h_image", ctypes.c_void_p),
                ("h_dsino", ctypes.c_void_p), ("h_norm", ctypes.c_void_p), ("h_out", ctypes.c_void_p)]


class _CServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("submitted", "completed", "failed", "queued", "active")] + \
               [(n, ctypes.c_double) for n in ("p50_ms", "p99_ms", "mean_ms", "max_ms", "throughput_per_s")] + \
               [(n, ctypes.c_int64) for n in ("bytes_in_use", "peak_bytes", "budget_bytes")] + \
               [("peak_active", ctypes.c_int32)] + \
               [(n, ctypes.c_double) for n in ("queue_ms", "load_ms", "run_ms")]


class Server:
    """gf_server: HBM-budget admission and continuous batching on one device."""

    def __init__(self, budget_bytes: int, max_active: int = 8, device: int = 0):
        h = ctypes.c_void_p()
        _ck(lib().gf_server_create(device, ctypes.c_int64(int(budget_bytes)), max_active, ctypes.byref(h)))
        self.h = h
        self._keep = {}

    def submit_recon(self, g: Geometry, dsino, norm, nsub: int = 1, niter: int = 2, storage: str = "f32"):
        P, ndata, nvox = sizes(g)
        dsino = np.ascontiguousarray(dsino, np.float32)
        norm = np.ascontiguousarray(norm, np.float32)
        out = np.empty(nvox, np.float32)
        q = _CRequest(0, g.c(), nsub, niter, STORE[storage], None, _ptr(dsino), _ptr(norm), _ptr(out))
        rid = ctypes.c_int64()
        _ck(lib().gf_server_submit(self.h, ctypes.byref(q), ctypes.byref(rid)))
        self._keep[rid.value] = (dsino, norm, out)
        return rid.value

    def submit_project(self, g: Geometry, image, nsub: int = 1):
        P, ndata, nvox = sizes(g)
        image = np.ascontiguousarray(image, np.float32)
        out = np.empty(ndata, np.float32)
        q = _CRequest(1, g.c(), nsub, 0, 0, _ptr(image), None, None, _ptr(out))
        rid = ctypes.c_int64()
        _ck(lib().gf_server_submit(self.h, ctypes.byref(q), ctypes.byref(rid)))
        self._keep[rid.value] = (image, out)
        return rid.value

    def wait(self, rid: int):
        """Result and latency (ms) of request rid; each request is waited for once."""
        lat = ctypes.c_double()
        try:
            _ck(lib().gf_server_wait(self.h, ctypes.c_int64(rid), ctypes.byref(lat)))
        finally:
            keep = self._keep.pop(rid, None)
        return keep[-1], lat.value

    def stats(self) -> dict:
        s = _CServerStats()
        _ck(lib().gf_server_get_stats(self.h, ctypes.byref(s)))
        return {n: getattr(s, n) for n, _ in _CServerStats._fields_}

    def close(self) -> None:
        if self.h:
            lib().gf_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Pinned:
    """Page-locked host memory from gf_host_alloc, freed when the last array over it goes."""

    def __init__(self, nbytes: int):
        self.p = ctypes.c_void_p()
        _ck(lib().gf_host_alloc(ctypes.c_size_t(max(int(nbytes), 1)), ctypes.byref(self.p)))
        self.__array_interface__ = {"shape": (int(nbytes),), "typestr": "|u1", "data": (self.p.value, False),
                                    "version": 3}

    def __del__(self):
        try:
            if self.p:
                lib().gf_host_free(self.p)
                self.p = ctypes.c_void_p()
        except Exception:
            pass


def host_empty(n: int, dtype=np.float32) -> np.ndarray:
    """An uninitialised numpy array of n elements in page-locked host memory
    (gf_host_alloc): host<->device copies from it run at the link's speed
    and overlap with kernels."""
    dt = np.dtype(dtype)
    return np.asarray(_Pinned(n * dt.itemsize)).view(dt)


def host_copy(a: np.ndarray, dtype=np.float32) -> np.ndarray:
    """A page-locked copy of array a (flattened)."""
    a = np.asarray(a, dtype=dtype).ravel()
    out = host_empty(a.size, dtype)
    out[:] = a
    return out


def recon_bytes(g: Geometry, nsub: int, mode: int = 1, storage: str = "f32") -> int:
    p = recon_defaults(mode)
    p.storage = STORE[storage]
    b = ctypes.c_int64()
    _ck(lib().gf_recon_bytes(ctypes.byref(g.c()), nsub, ctypes.byref(p), ctypes.c_int64(0), ctypes.byref(b)))
    return b.value


def read_sinogram(path, ndata: int):
    out = np.empty(2 * ndata, np.float32)
    st = lib().gf_read_sinogram(str(path).encode(), ctypes.c_int64(ndata), _ptr(out))
    return out, st


def read_vlor(path) -> np.ndarray:
    n = ctypes.c_int64()
    _ck(lib().gf_read_vlor(str(path).encode(), None, ctypes.byref(n)))
    out = np.zeros(max(1, n.value) * 2, np.int32)
    _ck(lib().gf_read_vlor(str(path).encode(), _ptr(out), ctypes.byref(n)))
    return out[: 2 * n.value].reshape(-1, 2)


def bin_endpoints(g: Geometry, bin_index: int) -> np.ndarray:
    out = np.empty(6, np.float32)
    _ck(lib().gf_bin_endpoints(ctypes.byref(g.c()), ctypes.c_int64(bin_index), _ptr(out)))
    return out


def bins_endpoints(g: Geometry, bins) -> np.ndarray:
    """Endpoints (n, 6) of the lines of response of 0-based bins."""
    b = np.ascontiguousarray(bins, np.int64).ravel()
    out = np.empty((b.size, 6), np.float32)
    _ck(lib().gf_bins_endpoints(ctypes.byref(g.c()), ctypes.c_int64(b.size), _ptr(b), _ptr(out)))
    return out


def read_vlor_endpoints(path) -> np.ndarray:
    n = ctypes.c_int64()
    _ck(lib().gf_read_vlor_endpoints(str(path).encode(), None, ctypes.byref(n)))
    out = np.zeros(max(1, n.value) * 12, np.float32)
    _ck(lib().gf_read_vlor_endpoints(str(path).encode(), _ptr(out), ctypes.byref(n)))
    return out[: 12 * n.value].reshape(-1, 12)


def read_image(path, nvox: int) -> np.ndarray:
    out = np.empty(nvox, np.float32)
    _ck(lib().gf_read_image(str(path).encode(), ctypes.c_int64(nvox), _ptr(out)))
    return out


def gpu_available() -> bool:
    """True when a device of this library's architecture is present."""
    try:
        g = Geometry(16, 15, 17, 8, 3, 5, 1.6, 20.721975, 12.5)
        Context(g).close()
        return True
    except (GfError, ImportError, OSError):
        return False


os.environ.setdefault("CUDA_MODULE_LOADING", "LAZY")
