"""The back projector's lane-chunk window for narrow segments (CPU).

For a segment whose rows fill NCH <= Q - 2 lane chunks (Q = NZP / 32),
`gf_bp.cu` issues the voxel work of a view only for the NCH + 1 lane chunks
starting at chunk min(izlo / 32, Q - NCH - 1), izlo = max(floor((zmin - t) -
1), 0) in float32, where t = yrot * fz is the view's axial shift.  That is
only correct if every voxel the per-voxel test accepts -- z = (iz + t) + 0.5
rounded to float32 at each step, zmin <= z < NZS - zmin, as in
BACKWPROJ_K (GFIRST_GPU_Kernels.cu:148-151) -- lies in the window.  This test
checks that for every zmin of a range of axial sizes and many shifts t,
including shifts that put z within rounding of a range boundary.
"""
import numpy as np

F = np.float32


def window(nzs: int, zmin: int, t: np.ndarray):
    """(lo, W) per shift t, or None when the kernel runs the whole column."""
    q = (nzs + 31) // 32
    nch = (nzs - 2 * zmin + 2 + 31) // 32
    w = nch + 1
    if w >= q:
        return None
    a = ((F(zmin) - t).astype(F) - F(1.0)).astype(F)
    izlo = np.maximum(np.floor(a).astype(np.int64), 0)
    return np.minimum(izlo >> 5, q - w), w


def in_range(nzs: int, zmin: int, t: np.ndarray) -> np.ndarray:
    iz = np.arange(nzs, dtype=F)
    z = ((iz[None, :] + t[:, None]).astype(F) + F(0.5)).astype(F)
    return (z >= F(zmin)) & (z < F(nzs - zmin))


def shifts(rs, n: int) -> np.ndarray:
    wide = rs.uniform(-400.0, 400.0, n)
    near = np.round(rs.uniform(-300.0, 300.0, n)) + rs.choice([-3e-5, -1e-6, 0.0, 1e-6, 3e-5, 0.5, -0.5], n)
    return np.concatenate([wide, near]).astype(F)


def test_window_holds_every_in_range_voxel():
    rs = np.random.RandomState(11)
    checked = 0
    for nzs in (64, 95, 96, 100, 130, 159, 161, 200, 223, 255, 256):
        for zmin in range(0, (nzs + 1) // 2):
            if nzs - 2 * zmin <= 0:
                continue
            t = shifts(rs, 300)
            win = window(nzs, zmin, t)
            if win is None:
                continue
            lo, w = win
            inr = in_range(nzs, zmin, t)
            iz = np.arange(nzs)[None, :]
            outside = (iz < 32 * lo[:, None]) | (iz > 32 * (lo[:, None] + w) - 1)
            bad = np.nonzero((inr & outside).any(axis=1))[0]
            assert bad.size == 0, (nzs, zmin, float(t[bad[0]]))
            checked += t.size
    assert checked > 100_000


def test_window_applies_to_the_narrow_preclinical_segments():
    # span 3 at NZS 159: zmin = 3|k| - 1 (GFIRST.cu:133-140); segments
    # |k| = 12..26 (30 of 53) run a window of 4, 3 or 2 of the 5 lane chunks
    widths = {}
    for k in range(1, 27):
        win = window(159, 3 * k - 1, np.zeros(1, dtype=F))
        if win is not None:
            widths[k] = win[1]
    assert sorted(widths) == list(range(12, 27))
    assert [widths[k] for k in (12, 16, 17, 21, 22, 26)] == [4, 4, 3, 3, 2, 2]


# ------------------------------------------------------------------ per-view form
# GF_BP_PER_VIEW stages a view's rows at offset pad_lo of a buffer of rbuf
# rows per warp (the rest at the gap sentinel) and lets lane chunk q read
# rows j and j + 1, j = iz + floor(t) - (zmin - 1), for every voxel iz of the
# chunks it issues (the window above, or all Q chunks).  Every such read must
# stay inside the buffer: checked here for every column, angle and segment of
# each geometry, with the kernel's float32 arithmetic for yrot, t and izlo.

def _fz(geo):
    res, nzs, nrad, nang, span, nseg, pitch, diam, fov = geo
    vx = F(F(fov) / F(res))
    out = []
    for s in range(nseg):
        k = (s + 1) // 2
        idz = k * (1 - (s % 2) * 2)
        zmin = 0 if idz == 0 else (abs(idz) - 1) * span + (span // 2 + 1)
        sgn = 0 if idz == 0 else (1 if idz > 0 else -1)
        fz = F(float(F(vx * F(sgn * zmin))) / (float(F(diam)) / 2.0))
        out.append((zmin, nzs - 2 * zmin, fz))
    return out


def _reads(geo):
    """(min j, max j + 1, nrow) of every segment over all columns and angles."""
    res, nzs, nrad, nang = geo[:4]
    q = (nzs + 31) // 32
    resm = F(F(res - 1) * F(0.5))
    pi = F(3.1415926)
    th = np.arange(nang, dtype=F)
    ang = ((-th / F(nang)).astype(F) * pi).astype(F) + pi
    sn, cs = np.sin(ang.astype(np.float64)).astype(F), np.cos(ang.astype(np.float64)).astype(F)
    iy, ix = np.meshgrid(np.arange(res, dtype=F), np.arange(res, dtype=F), indexing="ij")
    xv, yv = (ix.ravel() - resm).astype(F), (iy.ravel() - resm).astype(F)
    yrot = ((-xv[:, None] * sn[None, :]).astype(F) + (yv[:, None] * cs[None, :]).astype(F)).astype(F)
    out = []
    for zmin, npl, fz in _fz(geo):
        nrow = npl + 2
        w = (nrow + 31) // 32 + 1
        t = (yrot * fz).astype(F)
        k = np.floor(t).astype(np.int64) - (zmin - 1)
        if w < q:
            izlo = np.maximum(np.floor(((F(zmin) - t).astype(F) - F(1.0)).astype(F)).astype(np.int64), 0)
            c0 = np.minimum(izlo >> 5, q - w)
            c1 = c0 + w - 1
        else:
            c0, c1 = np.zeros_like(k), np.full_like(k, q - 1)
        out.append((int((32 * c0 + k).min()), int((32 * c1 + 32 + k).max()), nrow))
    return out


def _geometries():
    import gfirst_gb300 as gf

    gs = [gf.Geometry.preclinical().tuple(), gf.Geometry.reference().tuple(), gf.Geometry.small().tuple(),
          (16, 15, 17, 8, 3, 5, 1.6, 20.7219750, 12.5), (20, 18, 24, 12, 5, 3, 1.63, 24.86637, 15.0)]
    gs += [(16, nzs, 16, 12, 3, 7, 1.6, 20.7219750, 12.5) for nzs in (33, 64, 96, 130, 200, 256)]
    gs += [(64, 64, 64, 64, 3, 21, 1.6, 84.8772096, 51.2), (96, 96, 96, 96, 3, 31, 1.6, 127.3158, 76.8)]
    # narrow scanners (small detector diameter): the largest axial shifts
    gs += [(64, 100, 40, 32, 1, 41, 2.0, 60.0, 51.2), (32, 200, 20, 16, 2, 61, 2.0, 30.0, 25.6)]
    return gs


def test_per_view_reads_stay_in_the_staged_buffer():
    import __graft_entry__

    __graft_entry__.build()
    import gfirst_gb300 as gf

    for geo in _geometries():
        b = gf.bp_staged_rows(gf.Geometry(*geo))
        assert b["rbuf"] == b["pad_lo"] + geo[1] + 2 + b["pad_hi"]
        for jmin, jmax1, nrow in _reads(geo):
            assert jmin >= -b["pad_lo"], (geo, jmin, b)
            assert jmax1 <= nrow - 1 + b["pad_hi"], (geo, jmax1, nrow, b)
            assert b["pad_lo"] + jmax1 < b["rbuf"], (geo, jmax1, b)
