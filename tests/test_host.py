"""Host-side logic of the library, no GPU needed: the C-ABI loads and exports
every entry point of include/gfirst.h, geometry and LOR indexing agree bit
for bit with the oracle, and the raw-file readers follow the reference."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import gfo
import gfo_io
import inputs

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def gf():
    import __graft_entry__

    from gfirst_gb300 import _build

    _build.build()
    import gfirst_gb300

    gfirst_gb300.lib()
    return gfirst_gb300


def declared_symbols():
    text = (ROOT / "include" / "gfirst.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:gf_status|void|int32_t|const char\*)\s+(gf_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol(gf):
    syms = declared_symbols()
    assert len(syms) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", str(gf.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gf_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        getattr(gf.lib(), s)


def test_abi_version(gf):
    assert gf.lib().gf_abi_version() == 3


GEOS = [inputs.GEOMS["tiny"], inputs.GEOMS["tinyb"], inputs.GEOMS["small"],
        (128, 159, 147, 168, 11, 15, 1.63, 165.7758, 100.0), (128, 159, 128, 160, 3, 53, 1.6, 165.7758, 100.0)]


@pytest.mark.parametrize("geo", GEOS)
def test_segment_table_and_sizes_match_oracle(gf, geo):
    g = gf.Geometry(*geo)
    o = gfo.Oracle(geo)
    P, ndata, nvox = gf.sizes(g)
    assert (P, ndata, nvox) == (o.P, o.ndata, o.nvox)
    idz, zmin, acc = gf.segment_table(g)
    oi, oz, oa = o.segments()
    assert np.array_equal(idz, oi) and np.array_equal(zmin, oz) and np.array_equal(acc, oa)


def test_reference_geometry_constants(gf):
    g = gf.Geometry.reference()
    P, ndata, nvox = gf.sizes(g)
    assert P == 1293 and ndata == 1293 * 168 * 147 and nvox == 128 * 128 * 159   # GFIRST.h:9-16
    assert gf.sizes(gf.Geometry.preclinical())[0] == 4319
    assert gf.sizes(gf.Geometry.small())[0] == 192


@pytest.mark.parametrize("geo", GEOS[:3])
def test_lor_index_bit_exact(gf, geo):
    g = gf.Geometry(*geo)
    o = gfo.Oracle(geo)
    lib = gfo.lib()
    _, zmin, _ = o.segments()
    rs = np.random.RandomState(3)
    for _ in range(200):
        s = rs.randint(0, g.nseg)
        iz0 = rs.randint(zmin[s], g.nzs - zmin[s])
        t, r = rs.randint(0, g.nang), rs.randint(0, g.nrad)
        assert gf.lor_index(g, s, iz0, t, r) == lib.gfo_lor(gfo.ctypes.byref(o.g), s, iz0, t, r)
    # every bin is reached exactly once
    seen = np.zeros(o.ndata, np.int32)
    for s in range(g.nseg):
        for iz0 in range(zmin[s], g.nzs - zmin[s]):
            base = gf.lor_index(g, s, iz0, 0, 0)
            seen[base:base + g.nang * g.nrad] += 1
    assert (seen == 1).all()


def test_invalid_geometry_rejected(gf):
    bad = gf.Geometry(16, 15, 17, 8, 3, 7, 1.6, 20.7, 12.5)  # segment +-3 has no planes
    with pytest.raises(gf.GfError) as e:
        gf.sizes(bad)
    assert e.value.status == 2
    with pytest.raises(gf.GfError):
        gf.lor_index(gf.Geometry(*inputs.GEOMS["tiny"]), 1, 0, 0, 0)  # plane below zmin


def test_no_device_fails_loudly(gf):
    if gf.gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gf.GfError) as e:
        gf.Context(gf.Geometry(*inputs.GEOMS["tiny"]))
    assert e.value.status == 7


@pytest.mark.parametrize("name", ["tiny", "tinyb"])
def test_sinogram_reader_matches_reference_rule(gf, name, tmp_path):
    files = inputs.case_files(name)
    ndata, nvox = inputs.sizes(name)
    for key in ("sinoD.raw", "sinoT.raw", "norm.raw"):
        p = tmp_path / key
        p.write_bytes(files[key])
        got, st = gf.read_sinogram(p, ndata)
        assert st == 0
        assert np.array_equal(got, gfo_io.read_sinogram_type(files[key], ndata)), key
    got, st = gf.read_sinogram(tmp_path / "missing.raw", ndata)
    assert st == 5 and not got.any()


def test_vlor_reader_end_of_file_rule(gf, tmp_path):
    for name in ("tiny", "tinyb"):
        raw = inputs.case_files(name)["vlor.raw"]
        p = tmp_path / f"{name}.raw"
        p.write_bytes(raw)
        assert np.array_equal(gf.read_vlor(p), gfo_io.read_vlor(raw))
    p = tmp_path / "empty.raw"
    p.write_bytes(b"")
    assert gf.read_vlor(p).shape == (0, 2)


def test_image_reader(gf, tmp_path):
    files = inputs.case_files("tiny")
    _, nvox = inputs.sizes("tiny")
    p = tmp_path / "img.raw"
    p.write_bytes(files["img.raw"])
    assert np.array_equal(gf.read_image(p, nvox), gfo_io.read_image(files["img.raw"], nvox))
    p.write_bytes(files["img.raw"][:100])
    short = gf.read_image(p, nvox)
    assert np.array_equal(short[:25], gfo_io.read_image(files["img.raw"], nvox)[:25]) and not short[25:].any()


def test_cli_usage_without_arguments(gf):
    out = subprocess.run([str(gf.CLI_PATH)], capture_output=True, text=True)
    assert out.returncode == 0 and "1 Input  --> Projection" in out.stdout


@pytest.mark.parametrize("geo", [inputs.GEOMS["tiny"], (128, 159, 128, 160, 3, 53, 1.6, 165.7758, 100.0)])
def test_bin_endpoints_lie_on_the_detector_ring(gf, geo):
    g = gf.Geometry(*geo)
    _, ndata, _ = gf.sizes(g)
    rs = np.random.RandomState(0)
    for b in rs.randint(0, ndata, size=200):
        e = gf.bin_endpoints(g, int(b)).astype(np.float64)
        r1, r2 = np.hypot(e[0], e[1]), np.hypot(e[3], e[4])
        assert abs(r1 - g.diam / 2) < 1e-3 and abs(r2 - g.diam / 2) < 1e-3
        assert abs(e[2]) < g.nzs * g.pitch and abs(e[5]) < g.nzs * g.pitch


def test_batched_bin_endpoints_equal_single(gf):
    g = gf.Geometry.preclinical()
    _, ndata, _ = gf.sizes(g)
    bins = np.random.RandomState(3).randint(0, ndata, size=500)
    many = gf.bins_endpoints(g, bins)
    assert np.array_equal(many, np.stack([gf.bin_endpoints(g, int(b)) for b in bins]))
    with pytest.raises(gf.GfError):
        gf.bins_endpoints(g, [0, ndata])  # out of range


def test_vlor_endpoint_reader(gf, tmp_path):
    lors = np.arange(12 * 3, dtype=np.float32).reshape(3, 12)
    p = tmp_path / "v.raw"
    p.write_bytes(lors.tobytes() + b"\x00" * 20)
    assert np.array_equal(gf.read_vlor_endpoints(p), lors)
