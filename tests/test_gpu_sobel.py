"""Sobel 3x3 derivatives (u8 -> s16) on the fused stencil engine: every output
element must equal the CPU oracle (the restatement of
kleidicv/src/filters/sobel_neon.cpp), bytes outside the destination rows must
stay untouched, and both the TMA path (16-byte aligned source) and the plain
load path (unaligned source) are covered, with aligned and unaligned
destinations."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402
from gpu_harness import device_image, device_output, read_output  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()

# (width, height, channels, source offset, source pad elements, dst pad elements, dst offset)
CASES = [(2, 2, 1, 0, 0, 0, 0), (3, 2, 4, 0, 13, 1, 2), (2, 9, 3, 5, 0, 0, 0), (17, 5, 2, 0, 15, 3, 0),
         (64, 48, 1, 0, 0, 0, 0), (257, 33, 3, 0, 16, 0, 0), (640, 480, 4, 0, 0, 0, 0),
         (1000, 37, 1, 3, 7, 1, 6), (1920, 1080, 1, 0, 64, 32, 0), (501, 301, 4, 1, 0, 0, 2),
         (4096, 7, 2, 0, 0, 5, 0), (33, 1000, 1, 0, 15, 0, 0), (3840, 2160, 4, 0, 0, 0, 0)]


def _run(horizontal, w, h, c, soff, spad, dpad, doff, seed):
    rng = np.random.default_rng(seed)
    host = rng.integers(0, 256, (h, w * c + spad), dtype=np.uint8)
    if seed % 3 == 0:  # large flat areas and 0/255 steps: the extreme magnitudes
        host[:, : (w * c) // 2] = 0
        host[: h // 2, (w * c) // 2:] = 255
    sbuf, sptr, sstride = device_image(torch, host, offset=soff)
    dbuf, dptr, dstride = device_output(torch, h, w * c, np.int16, pad_elems=dpad, offset=doff)
    ctx = kcv.Context.for_torch(0)
    fn = kcv.sobel_3x3_horizontal_s16_u8 if horizontal else kcv.sobel_3x3_vertical_s16_u8
    assert fn(sptr, sstride, dptr, dstride, w, h, c, ctx) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    got, pad_ok = read_output(dbuf, h, w * c, np.int16, dstride, offset=doff)
    err, want = oracle.sobel_3x3_s16_u8(host, w, h, c, horizontal, nthreads=8)
    assert err == 0
    ctx.close()
    return got, want[:, : w * c], pad_ok


@pytest.mark.parametrize("horizontal", [True, False], ids=["dx", "dy"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: "x".join(map(str, c[:3])) + f"_o{c[3]}_d{c[6]}")
def test_sobel_matches_oracle(horizontal, case):
    got, want, pad_ok = _run(horizontal, *case, seed=sum(case) + int(horizontal))
    assert pad_ok, "wrote outside the destination rows"
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{len(bad)} elements differ, first at {bad[0].tolist()}"


def test_sobel_extremes_reach_1020():
    w, h, c = 300, 200, 1
    got, want, _ = _run(True, w, h, c, 0, 0, 0, 0, seed=3)
    assert np.array_equal(got, want) and np.abs(got).max() == 1020


def test_sobel_rejections_match_oracle():
    ctx = kcv.Context.for_torch(0)
    buf = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    for (w, h, c, ds, want) in [(1, 5, 1, 64, kcv.NOT_IMPLEMENTED), (5, 5, 5, 64, kcv.NOT_IMPLEMENTED),
                                (5, 5, 1, 63, kcv.ALIGNMENT), (5, 5, 0, 64, kcv.OK)]:
        for fn in (kcv.sobel_3x3_horizontal_s16_u8, kcv.sobel_3x3_vertical_s16_u8):
            assert fn(p, 64, p + 1024, ds, w, h, c, ctx) == want
    assert kcv.sobel_3x3_horizontal_s16_u8(None, 64, p, 64, 5, 5, 1, ctx) == kcv.NULL_POINTER
    assert ctx.synchronize() == kcv.OK
    ctx.close()
