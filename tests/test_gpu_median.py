"""Median blur on the GPU: every element type, window size, border and channel
count of the reference's tests (and larger, padded, unaligned images) must
equal the oracle exactly; u8 windows 9..255 go through the sliding-histogram
kernel."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402
from gpu_harness import device_image, device_output, read_output  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()
DTYPES = ["s8", "u8", "u16", "s16", "u32", "s32", "f32"]


def random_image(rng, dt, h, elems):
    dt = np.dtype(dt)
    if dt.kind == "f":
        return rng.uniform(-1e6, 1e6, (h, elems)).astype(dt)
    info = np.iinfo(dt)
    return rng.integers(info.min, int(info.max) + 1, (h, elems), dtype=dt)


def run(dtype, w, h, c, k, border, seed, pad=0, soff=0, dpad=0, doff=0, ctx=None):
    dt = oracle.MEDIAN_DTYPES[dtype]
    rng = np.random.default_rng(seed)
    host = random_image(rng, dt, h, w * c + pad)
    if seed % 4 == 0:  # few distinct values: many equal keys in a window
        host = (host % 3).astype(dt)
    sbuf, sptr, sstride = device_image(torch, host, offset=soff)
    dbuf, dptr, dstride = device_output(torch, h, w * c, dt, pad_elems=dpad, offset=doff)
    own = ctx is None
    ctx = ctx or kcv.Context.for_torch(0)
    assert kcv.median_blur(dtype, sptr, sstride, dptr, dstride, w, h, c, k, k, border, ctx) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    if own:
        ctx.close()
    got, pad_ok = read_output(dbuf, h, w * c, dt, dstride, offset=doff)
    want = oracle.median_blur(host, w, h, c, k, border)
    return got, want, pad_ok


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [3, 5, 7])
def test_reference_shapes(dtype, k):
    ctx = kcv.Context.for_torch(0)
    for c in (1, 2, 3, 4):
        for border in (kcv.REPLICATE, kcv.REFLECT, kcv.WRAP, kcv.REVERSE):
            got, want, pad_ok = run(dtype, 2 * k + 2, k, c, k, border, seed=k * 7 + c + border, ctx=ctx)
            assert pad_ok and np.array_equal(got, want), (c, border)
    # The reference's padded case: src padding 5, dst padding 13, 3 channels, REPLICATE.
    got, want, pad_ok = run(dtype, 2 * k + 2, k, 3, k, kcv.REPLICATE, seed=1, pad=5, dpad=13, ctx=ctx)
    assert pad_ok and np.array_equal(got, want)
    ctx.close()


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("case", [(333, 77, 3, 5, 2), (640, 480, 1, 7, 4), (101, 203, 4, 3, 3), (7, 300, 2, 7, 1),
                                  (1920, 1080, 1, 3, 1)])
def test_larger_images(dtype, case):
    w, h, c, k, border = case
    got, want, pad_ok = run(dtype, w, h, c, k, border, seed=w + h + k, pad=3,
                            soff=np.dtype(oracle.MEDIAN_DTYPES[dtype]).itemsize, dpad=2)
    assert pad_ok
    bad = np.argwhere(got != want)
    assert bad.size == 0, f"{len(bad)} differ, first {bad[0].tolist()}"


@pytest.mark.parametrize("k", [9, 15, 17, 31, 63])
def test_u8_histogram_sizes(k):
    ctx = kcv.Context.for_torch(0)
    for c, border in ((1, kcv.REPLICATE), (3, kcv.REFLECT), (4, kcv.WRAP), (2, kcv.REVERSE)):
        got, want, pad_ok = run("u8", 2 * k + 2, k, c, k, border, seed=k + c, ctx=ctx)
        assert pad_ok and np.array_equal(got, want), (c, border)
    got, want, pad_ok = run("u8", 500, 130, 3, k, kcv.REVERSE, seed=k, pad=7, dpad=1, ctx=ctx)
    assert pad_ok and np.array_equal(got, want)
    ctx.close()


def test_u8_max_window():
    # MaxFilterSize (:389-396): 512 x 255, K = 255; the oracle checks a subset of rows.
    w, h, k = 2 * 255 + 2, 255, 255
    rng = np.random.default_rng(5)
    host = rng.integers(0, 256, (h, w), dtype=np.uint8)
    sbuf, sptr, sstride = device_image(torch, host)
    dbuf, dptr, dstride = device_output(torch, h, w, np.uint8, pad_elems=3)
    ctx = kcv.Context.for_torch(0)
    assert kcv.median_blur("u8", sptr, sstride, dptr, dstride, w, h, 1, k, k, kcv.REPLICATE, ctx) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    ctx.close()
    got, pad_ok = read_output(dbuf, h, w, np.uint8, dstride)
    rows = [0, 1, 2, 126, 127, 200, 253, 254]
    assert pad_ok and np.array_equal(got[rows], oracle.median_blur(host, w, h, 1, k, kcv.REPLICATE, out_rows=rows))


def test_rejections():
    ctx = kcv.Context.for_torch(0)
    buf = torch.zeros(1 << 16, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    assert kcv.median_blur("u8", p, 64, p, 64, 10, 10, 1, 5, 5, kcv.REPLICATE, ctx) == kcv.NOT_IMPLEMENTED
    assert kcv.median_blur("u16", p, 64, p + 8192, 64, 100, 100, 1, 9, 9, kcv.REPLICATE, ctx) == kcv.NOT_IMPLEMENTED
    assert kcv.median_blur("f32", p, 63, p + 8192, 64, 10, 10, 1, 5, 5, kcv.REPLICATE, ctx) == kcv.ALIGNMENT
    assert kcv.median_blur("u8", p, 64, p + 8192, 64, 10, 10, 1, 5, 5, kcv.CONSTANT, ctx) == kcv.NOT_IMPLEMENTED
    assert ctx.synchronize() == kcv.OK
    ctx.close()


@pytest.mark.parametrize("case", [(4, 270000, 1, 3), (9, 70000, 1, 9)])
def test_tall_narrow_images(case):
    """Heights beyond the grid's 65535-block y limit: the small-window kernel
    (four rows per block) and the sliding-histogram kernel (one row per block)
    both loop over rows."""
    w, h, c, k = case
    got, want, pad_ok = run("u8", w, h, c, k, 1, 21)
    assert pad_ok and np.array_equal(got, want)
