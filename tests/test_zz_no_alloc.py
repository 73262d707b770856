"""gf_forward_project_noalloc: forward projection for callers that cannot
allocate device memory (a host that owns the whole device memory map, an
embedding framework with its own pool, code where an allocation would stall
or be refused).  Its scratch is a fixed file-scope device array instead of
context buffers; its output must equal gf_forward_project's, call after call,
and sit within the projection tolerance of the CPU oracle.

This file is collected last on purpose, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes
import ctypes.util

import numpy as np
import pytest

import gfo
import inputs

pytestmark = pytest.mark.gpu

FP_TOL = 1e-4


@pytest.fixture(scope="module")
def gf():
    import __graft_entry__

    __graft_entry__.build()
    import gfirst_gb300

    if not gfirst_gb300.gpu_available():
        pytest.fail("no sm_103 GPU available to the library")
    return gfirst_gb300


def device_sync():
    # the entry point runs on the legacy default stream; wait for the whole device
    name = ctypes.util.find_library("cudart") or "libcudart.so"
    try:
        rt = ctypes.CDLL(name)
    except OSError:
        rt = ctypes.CDLL("/usr/local/cuda/lib64/libcudart.so")
    assert rt.cudaDeviceSynchronize() == 0


def noalloc(gf, g, nsub, subset, dimg, dproj):
    return gf.lib().gf_forward_project_noalloc(ctypes.byref(g.c()), nsub, subset, dimg.p, dproj.p, None)


def rel(a, b):
    return float(np.linalg.norm(np.float64(a) - b) / max(np.linalg.norm(np.float64(b)), 1e-30))


@pytest.mark.parametrize("name", ["tinyb", "small"])
def test_noalloc_matches_forward_project_twice(gf, name):
    geo = inputs.GEOMS[name]
    g = gf.Geometry(*geo)
    nsub = 3
    ctx = gf.Context(g, nsub=nsub)
    rs = np.random.RandomState(12)
    for call, subset in enumerate((1, 2)):
        img = rs.uniform(0.0, 2.0, ctx.nvox).astype(np.float32)
        dimg = ctx.put(img)
        want_d = ctx.array(ctx.ndata).zero()
        ctx.forward_project(dimg, subset, want_d)
        want = want_d.download()
        out = ctx.array(ctx.ndata).zero()
        st = noalloc(gf, g, nsub, subset, dimg, out)
        assert st == 0, gf.lib().gf_last_error().decode()
        device_sync()
        got = out.download()
        oracle = gfo.Oracle(geo).fp(img, nsub, subset)  # bins of other subsets stay 0 in both
        assert rel(got, oracle) < FP_TOL, f"call {call}: against the CPU oracle"
        assert rel(got, want) < FP_TOL, f"call {call}"
        assert np.array_equal(got, want), f"call {call}: same kernels, same inputs"


def test_noalloc_rejects_geometry_beyond_its_scratch(gf):
    g = gf.Geometry(256, 96, 64, 8, 3, 1, 1.6, 165.7758, 100.0)  # 256x256x96 voxels: 25 MB > 16 MiB
    ctx = gf.Context(gf.Geometry(*inputs.GEOMS["tiny"]))
    dimg, dproj = ctx.array(16), ctx.array(16)
    st = noalloc(gf, g, 1, 0, dimg, dproj)
    assert st == 1  # GF_ERR_ARG
    assert "scratch" in gf.lib().gf_last_error().decode()
