"""Index map of the one-launch image update (gf_image.cu update_kernel), on
the CPU: a CTA covers `cs` output slices from z0 = chunk*cs with lanes
l = 0..31 holding slices z0 - 2 + l, outputs on lanes 2..cs+1.  The axial
taps read lanes l-2..l+2 and the edge slices take the neighbour lane's
product, so every output must find its sources on lanes 2..29 of its own
CTA, and the image values it reads (its own slice, or slice 1 / NZS-2 for
the edge copies) must be outputs of the same CTA: the update is in place.
The chunk length is 28, or 27 where slice NZS-1 would start a chunk; the
GPU parity tests check the kernel against the oracle at the sizes where
each rule applies."""
import pytest


def chunk(nzs: int) -> int:
    return 27 if nzs > 1 and (nzs - 1) % 28 == 0 else 28


def cover(nzs: int):
    nzp = (nzs + 31) // 32 * 32
    cs = chunk(nzs)
    owner = {}
    for c in range((nzp + cs - 1) // cs):
        z_of = {lane: c * cs - 2 + lane for lane in range(32)}
        outs = {lane for lane in range(32) if 2 <= lane < cs + 2 and z_of[lane] < nzp}
        for lane in sorted(outs):
            z = z_of[lane]
            assert z not in owner, (nzs, z)
            owner[z] = c
            if z >= nzs:
                continue  # padding slices are written 0
            # the product this output takes: its own, or the neighbour's at the edges
            src = lane + 1 if z == 0 else (lane - 1 if z == nzs - 1 else lane)
            assert src in outs, (nzs, z)        # image value read from the CTA's own outputs
            assert 2 <= src <= 29, (nzs, z)     # taps src-2..src+2 inside the warp
    return owner, nzp


@pytest.mark.parametrize("nzs", range(5, 257))
def test_every_slice_written_once_from_its_own_cta(nzs):
    owner, nzp = cover(nzs)
    assert sorted(owner) == list(range(nzp))


def test_chunk_rule_sizes():
    assert chunk(159) == 28 and chunk(29) == 27 and chunk(57) == 27 and chunk(253) == 27
    # with 28 everywhere, slice NZS-1 would open a chunk and read slice NZS-2 from another CTA
    for nzs in (29, 57, 85, 113, 141, 169, 197, 225, 253):
        assert (nzs - 1) % 28 == 0 and (nzs - 1) % 27 != 0
