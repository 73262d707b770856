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
