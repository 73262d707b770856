"""Seeded input files for the golden runs and the parity tests.

numpy's legacy RandomState is used on purpose: its streams are stable across
numpy versions, so the same bytes are produced on every machine.  The golden
fixtures store a sha256 of every generated file, which the tests re-check.
"""
from __future__ import annotations

import hashlib

import numpy as np

# name -> (res, nzs, nrad, nang, span, nseg, pitch, diam, fov); must match
# oracle/build_ref.py's GEOMS.
GEOMS = {
    "tiny": (16, 15, 17, 8, 3, 5, 1.6, 20.7219750, 12.5),
    "tinyb": (20, 18, 24, 12, 5, 3, 1.63, 24.86637, 15.0),
    "small": (64, 32, 64, 64, 3, 11, 1.6, 84.8772096, 51.2),
}


def planes(res, nzs, nrad, nang, span, nseg, *rest) -> int:
    p = 0
    for i in range(nseg):
        k = (i + 1) // 2
        zmin = 0 if i == 0 else (k - 1) * span + (span // 2 + 1)
        p += nzs - 2 * zmin
    return p


def sizes(name: str):
    g = GEOMS[name]
    res, nzs, nrad, nang = g[0], g[1], g[2], g[3]
    return planes(*g) * nang * nrad, res * res * nzs


def phantom(name: str, seed: int) -> np.ndarray:
    """Water cylinder (0.1) plus a few uniform ellipsoids, [NZS][RES][RES]."""
    res, nzs = GEOMS[name][0], GEOMS[name][1]
    rs = np.random.RandomState(seed)
    z, y, x = np.meshgrid(np.arange(nzs), np.arange(res), np.arange(res), indexing="ij")
    c = (res - 1) / 2.0
    img = np.where((x - c) ** 2 + (y - c) ** 2 <= (0.9 * res / 2) ** 2, 0.1, 0.0)
    for _ in range(6):
        r = rs.uniform(0, 0.5 * res / 2)
        a = rs.uniform(0, 2 * np.pi)
        cx, cy, cz = c + r * np.cos(a), c + r * np.sin(a), rs.uniform(0.2, 0.8) * (nzs - 1)
        sx, sy, sz = rs.uniform(0.08, 0.2, size=3) * np.array([res, res, nzs])
        act = rs.uniform(0.5, 5.0)
        img = np.where(((x - cx) / sx) ** 2 + ((y - cy) / sy) ** 2 + ((z - cz) / sz) ** 2 <= 1.0, act, img)
    return img.astype(np.float32)


def sinogram_counts(name: str, seed: int, scale: float, bg: float) -> np.ndarray:
    """int32 [2*NDATA]: prompts shaped like a centred cylinder's projection, then background."""
    res, nzs, nrad, nang = GEOMS[name][:4]
    ndata, _ = sizes(name)
    rs = np.random.RandomState(seed)
    r = (np.arange(nrad) - (nrad - 1) / 2.0) / (nrad / 2.0)
    prof = np.clip(1.0 - r ** 2, 0.0, None) ** 0.5
    lam = np.tile(prof, ndata // nrad) * scale * (1.0 + 0.3 * rs.uniform(size=ndata))
    prompts = rs.poisson(lam).astype(np.int32)
    back = rs.poisson(bg, size=ndata).astype(np.int32)
    back[rs.randint(0, ndata, size=max(1, ndata // 500))] = -1  # exercises the bg<0 clamp
    return np.concatenate([prompts, back]).astype(np.int32)


def norm_gains(name: str, seed: int) -> np.ndarray:
    """float32 [NDATA] gains U(0.9, 1.1) with about 2% gaps (0)."""
    ndata, _ = sizes(name)
    rs = np.random.RandomState(seed)
    g = rs.uniform(0.9, 1.1, size=ndata).astype(np.float32)
    g[rs.uniform(size=ndata) < 0.02] = 0.0
    return g


def vlor_events(name: str, seed: int, n: int, tail: int) -> bytes:
    """int32 pairs of 1-based bins, with some rejected indices; `tail` extra
    bytes (0 or 4) make a partial last record."""
    ndata, _ = sizes(name)
    rs = np.random.RandomState(seed)
    ev = rs.randint(1, ndata + 1, size=(n, 2)).astype(np.int32)
    bad = rs.randint(0, n, size=max(4, n // 100))
    choices = np.array([0, 1, ndata + 1, -5, ndata], dtype=np.int32)
    ev[bad, rs.randint(0, 2, size=bad.size)] = choices[rs.randint(0, choices.size, size=bad.size)]
    raw = ev.tobytes()
    if tail:
        raw += np.array([rs.randint(2, ndata)], dtype=np.int32).tobytes()[:tail]
    return raw


def case_files(name: str) -> dict:
    """All input files of one geometry's golden runs, as bytes."""
    ndata, nvox = sizes(name)
    files = {"img.raw": phantom(name, 11).tobytes()}
    files["sinoD.raw"] = sinogram_counts(name, 21, 40.0, 0.5).tobytes()
    norm = norm_gains(name, 31)
    files["norm.raw"] = norm.tobytes()
    t = sinogram_counts(name, 41, 6.0, 0.2)
    if name == "tinyb":
        # doubles stored as float32 (detected by the >1e6 rule), triples file short
        files["sinoD.raw"] = sinogram_counts(name, 21, 40.0, 0.5).astype(np.float32).tobytes()
        t = t[: ndata + ndata // 2]
    files["sinoT.raw"] = t.tobytes()
    files["vlor.raw"] = vlor_events(name, 51, max(200, ndata // 4), 4 if name == "tinyb" else 0)
    return files


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()
