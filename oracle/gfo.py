"""ctypes binding of the CPU oracle (oracle/liboracle_f32.so / _f64.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker, never by the product.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


class Geom(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in ("res", "nzs", "nrad", "nang", "span", "nseg")] + \
               [(n, ctypes.c_float) for n in ("pitch", "diam", "fov")]


class Params(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("nsub", ctypes.c_int32), ("niter", ctypes.c_int32),
                ("psf_fw", ctypes.c_float), ("psf_bw", ctypes.c_float)]


def build(force: bool = False) -> None:
    """Compile the oracle twice (float and double) with gcc."""
    src = HERE / "gf_oracle.c"
    for tag, real in (("f32", "float"), ("f64", "double")):
        out = HERE / f"liboracle_{tag}.so"
        if out.exists() and not force and out.stat().st_mtime >= src.stat().st_mtime:
            continue
        cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", f"-DGFO_REAL={real}",
               str(src), "-o", str(out), "-lm"]
        subprocess.run(cmd, check=True)


_LIBS: dict = {}


def lib(tag: str = "f32") -> ctypes.CDLL:
    if tag not in _LIBS:
        path = HERE / f"liboracle_{tag}.so"
        if not path.exists():
            build()
        _LIBS[tag] = ctypes.CDLL(str(path))
        _LIBS[tag].gfo_planes.restype = ctypes.c_int64
        _LIBS[tag].gfo_lor.restype = ctypes.c_int64
        _LIBS[tag].gfo_max_ref.restype = ctypes.c_double if tag == "f64" else ctypes.c_float
    return _LIBS[tag]


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """Thin numpy front end; `dt` is float32 for the parity build, float64 for the accuracy build."""

    def __init__(self, geom: tuple, tag: str = "f32"):
        self.g = Geom(*geom[:6], *geom[6:9])
        self.tag = tag
        self.L = lib(tag)
        self.dt = np.float32 if tag == "f32" else np.float64
        self.P = int(self.L.gfo_planes(ctypes.byref(self.g)))
        if self.P < 0:
            raise ValueError("invalid geometry")
        res, nzs, nrad, nang = geom[:4]
        self.ndata = self.P * nang * nrad
        self.nvox = res * res * nzs
        self.geom = geom

    def a(self, x):
        return np.ascontiguousarray(x, dtype=self.dt)

    def _out(self, buf, n):
        """A caller's output buffer, written in place by the C oracle: it must
        hold n elements of this build's real type, contiguous."""
        if buf is None:
            return np.zeros(n, self.dt)
        if buf.dtype != self.dt or buf.size != n or not buf.flags.c_contiguous:
            raise ValueError(f"output buffer must be {n} contiguous {np.dtype(self.dt).name}")
        return buf

    def segments(self):
        n = self.g.nseg
        idz, zmin, acc = (np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n + 1, np.int32))
        self.L.gfo_segments(ctypes.byref(self.g), _p(idz), _p(zmin), _p(acc))
        return idz, zmin, acc

    def fp(self, img, nsub=1, subset=0, out=None):
        img = self.a(img)
        out = self._out(out, self.ndata)
        self.L.gfo_fp(ctypes.byref(self.g), _p(img), nsub, subset, _p(out))
        return out

    def ratio(self, proj, data, bg, nsub=1, subset=0, corr=None):
        corr = self._out(corr, self.ndata)
        self.L.gfo_ratio(ctypes.byref(self.g), _p(self.a(proj)), _p(self.a(data)), _p(self.a(bg)), nsub, subset,
                         _p(corr))
        return corr

    def calib(self, proj_blank, blank):
        out = np.zeros(self.ndata, self.dt)
        self.L.gfo_calib(ctypes.byref(self.g), _p(self.a(proj_blank)), _p(self.a(blank)), _p(out))
        return out

    def bp(self, corr, calib, nsub=1, subset=0):
        numer, denom = np.zeros(self.nvox, self.dt), np.zeros(self.nvox, self.dt)
        self.L.gfo_bp(ctypes.byref(self.g), _p(self.a(corr)), _p(self.a(calib)), nsub, subset, _p(numer),
                      _p(denom))
        return numer, denom

    @staticmethod
    def gauss9(psf: float) -> np.ndarray:
        g = np.zeros(9, np.float32)
        lib("f32").gfo_gauss9(ctypes.c_float(psf), _p(g))
        return g

    def conv_xy(self, img, psf=1.5):
        out = np.zeros(self.nvox, self.dt)
        self.L.gfo_conv_xy(ctypes.byref(self.g), _p(self.a(img)), _p(self.gauss9(psf)), _p(out))
        return out

    def filter_z(self, img, out_init=None):
        out = np.zeros(self.nvox, self.dt) if out_init is None else self.a(out_init).copy()
        self.L.gfo_filter_z(ctypes.byref(self.g), _p(self.a(img)), _p(out))
        return out

    def update(self, img, numer, denom, psf_bw=1.5):
        img = self.a(img).copy()
        self.L.gfo_update(ctypes.byref(self.g), _p(img), _p(self.a(numer)), _p(self.a(denom)),
                          _p(self.gauss9(psf_bw)))
        return img

    def bilateral(self, inp, ref, max_ref=None, r=4, sigma3d=0.75, sigmai=0.025):
        ref = self.a(ref)
        if max_ref is None:
            max_ref = self.L.gfo_max_ref(ctypes.c_int64(self.nvox), _p(ref))
        out = np.zeros(self.nvox, self.dt)
        real = ctypes.c_double if self.tag == "f64" else ctypes.c_float
        self.L.gfo_bilateral(ctypes.byref(self.g), _p(self.a(inp)), _p(ref), real(max_ref), r,
                             ctypes.c_float(sigma3d), ctypes.c_float(sigmai), _p(out))
        return out

    def blend(self, img2, filtered):
        img2 = self.a(img2).copy()
        self.L.gfo_blend(ctypes.c_int64(self.nvox), _p(img2), _p(self.a(filtered)))
        return img2

    def cylinder(self, val=1.0):
        out = np.zeros(self.nvox, self.dt)
        real = ctypes.c_double if self.tag == "f64" else ctypes.c_float
        self.L.gfo_cylinder(ctypes.byref(self.g), real(val), _p(out))
        return out

    def vlor_count(self, ev):
        cnt = np.zeros(self.ndata, self.dt)
        ev = np.ascontiguousarray(ev, np.int32)
        self.L.gfo_vlor_count(ctypes.byref(self.g), _p(ev), ctypes.c_int64(len(ev)), _p(cnt))
        return cnt

    def blankt(self, cnt, datos_t):
        out = np.zeros(self.ndata, self.dt)
        self.L.gfo_blankt(ctypes.byref(self.g), _p(self.a(cnt)), _p(self.a(datos_t)), _p(out))
        return out

    def vlor_split(self, ev, proj, blankt):
        out = np.zeros(self.ndata, self.dt)
        ev = np.ascontiguousarray(ev, np.int32)
        self.L.gfo_vlor_split(ctypes.byref(self.g), _p(ev), ctypes.c_int64(len(ev)), _p(self.a(proj)),
                              _p(self.a(blankt)), _p(out))
        return out

    def output_image(self, img, scale=np.float32(3.70e-4 * 162.0)):
        out = np.zeros(self.nvox, self.dt)
        self.L.gfo_output_image(ctypes.byref(self.g), _p(self.a(img)), ctypes.c_float(scale), _p(out))
        return out

    def recon(self, mode, nsub=1, niter=1, image=None, dsino=None, tsino=None, norm=None, ev=None,
              psf_fw=1.5, psf_bw=1.5):
        p = Params(mode, nsub, niter, psf_fw, psf_bw)
        ev = np.zeros((0, 2), np.int32) if ev is None else np.ascontiguousarray(ev, np.int32)
        outs = {k: np.zeros(n, self.dt) for k, n in
                (("proj_ref", self.ndata), ("img_d", self.nvox), ("img_t", self.nvox), ("sinog_vlor", self.ndata))}
        conv = lambda x: None if x is None else self.a(x)  # noqa: E731
        rc = self.L.gfo_recon(ctypes.byref(self.g), ctypes.byref(p), _p(conv(image)), _p(conv(dsino)),
                              _p(conv(tsino)), _p(conv(norm)), _p(ev), ctypes.c_int64(len(ev)),
                              _p(outs["proj_ref"]), _p(outs["img_d"]), _p(outs["img_t"]), _p(outs["sinog_vlor"]))
        if rc != 0:
            raise ValueError("oracle recon failed")
        return outs


def machine() -> str:
    return platform.machine()


def cores() -> int:
    return int(lib("f32").gfo_threads())


os.environ.setdefault("OMP_PROC_BIND", "false")
