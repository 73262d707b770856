"""Oracle-side readers for GFIRST's raw file formats (numpy restatement).

TEST INFRASTRUCTURE ONLY: these feed oracle/liboracle_*.so in tests, the
smoke check and the CPU-baseline leg of bench.py.  The product has its own
C++ readers (gfirst_gb300/csrc/gf_io.cpp), which the tests check against
these and against the reference's golden runs.
"""
from __future__ import annotations

import numpy as np


def read_sinogram_type(raw: bytes, ndata: int) -> np.ndarray:
    """ReadSinogram_Type, GFIRST_CPU_Kernels.cpp:104-142.

    Reads the file as int32 into a zeroed 2*ndata buffer (the reference reads
    every int of the file into that buffer without a bound; here anything
    past 2*ndata is ignored), converts to float, and if the largest value
    exceeds 1e6 re-reads the file's words as float32 instead (entries past
    the end of the file stay 0).  A missing file gives zeros.
    """
    n = 2 * ndata
    words = len(raw) // 4
    m = min(words, n)
    ints = np.zeros(n, dtype=np.int32)
    ints[:m] = np.frombuffer(raw, dtype="<i4", count=m)
    sino = ints.astype(np.float32)
    mx = np.float32(0.0)
    pos = sino[sino > 0]
    if pos.size:
        mx = pos.max()
    if mx > 1.0e6:
        sino = np.zeros(n, dtype=np.float32)
        sino[:m] = np.frombuffer(raw, dtype="<f4", count=m)
    return sino


def read_vlor(raw: bytes) -> np.ndarray:
    """VLOR list as GFIRST.cu:232-240 / 375-388 consume it.

    Records are int32 pairs (1-based sinogram bins).  The reference loops
    `while (!feof) { fread(VLOR, 4, 2) ... }`, so after the last full record
    it runs the body once more with whatever the failed read left in the
    buffer: the last record again, or, when 4-7 bytes remain, (new first
    word, old second word).  A file shorter than one record yields no events
    here (the reference would use an uninitialised buffer).
    """
    nfull = len(raw) // 8
    rec = np.frombuffer(raw, dtype="<i4", count=2 * nfull).reshape(nfull, 2)
    if nfull == 0:
        return np.zeros((0, 2), dtype=np.int32)
    last = rec[-1].copy()
    if len(raw) % 8 >= 4:
        last[0] = np.frombuffer(raw, dtype="<i4", count=1, offset=8 * nfull)[0]
    return np.ascontiguousarray(np.vstack([rec, last[None, :]]).astype(np.int32))


def read_image(raw: bytes, nvox: int) -> np.ndarray:
    """ReadImage, GFIRST_CPU_Kernels.cpp:58-66 (short files leave zeros here)."""
    out = np.zeros(nvox, dtype=np.float32)
    m = min(len(raw) // 4, nvox)
    out[:m] = np.frombuffer(raw, dtype="<f4", count=m)
    return out
