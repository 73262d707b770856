"""Inputs of bench.py's roofline on CPU: the algorithmic bytes per launch of
the two projectors at the preclinical configuration, and the committed ncu
figures (DRAM bytes and warp instructions per launch) the JSON line quotes.
"""
import importlib.util
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_roof", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_algorithmic_bytes_of_the_preclinical_subiteration():
    import gfirst_gb300 as gf

    b = _bench()
    P, ndata, nvox = gf.sizes(gf.Geometry.preclinical())
    assert (P, ndata, nvox) == (4319, 88_453_120, 2_605_056)
    alg = b.algorithmic_bytes(P, ndata, nvox)
    # 16 subsets: 5.53 M bins; FP reads the image and per bin data, background
    # and mask and writes the ratio; BP reads ratio and mask and writes the
    # update ratio NUMER/DENOM
    assert alg["fp"] == nvox * 4 + (ndata // 16) * 13 == 82_288_384
    assert alg["bp"] == (ndata // 16) * 5 + nvox * 4 == 38_061_824


def test_committed_traffic_covers_both_projectors():
    b = _bench()
    t = b.committed_traffic()
    bins, nvox = 88_453_120 // 16, 2_605_056
    # the inputs as the library stores them in FP32: the FP reads the image
    # and per bin a (data, background) pair and the mask (12 B); the BP reads
    # per bin a (ratio, mask) pair (8 B)
    stored_in = {"fp": nvox * 4 + bins * 12, "bp": bins * 8}
    for k in ("fp", "bp"):
        e = t[k]
        assert e["bytes_per_launch"] == e["read"] + e["write"]
        assert e["warp_instructions"] > 0 and 0 < e["issue_active_pct"] <= 100
        # DRAM reads within 15 % of the stored inputs: each input byte leaves
        # HBM once, nothing is re-read
        assert abs(e["read"] / stored_in[k] - 1) < 0.15
        assert "ncu" in e["command"] and "--clock-control none" in e["command"]
