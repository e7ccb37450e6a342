"""GPU parity: every entry point, through the C ABI, against the CPU oracle.

Bit-exact for all integer results (tolerance 0): kernel sizes, sigmas,
channel counts, all border types, minimum sizes (k-1), multi-strip widths,
padded and misaligned layouts, and the reference's own known-answer tests.
"""
import json
import os

import numpy as np
import pytest

from tests.gpu_harness import device_image, device_output, padded, pyr_sizes, read_output

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

BORDERS = [1, 2, 3, 4]  # REPLICATE, REFLECT, WRAP, REVERSE


@pytest.fixture(scope="module")
def ctx(kcv):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = kcv.Context.for_torch(0)
    yield c
    c.close()


def run_gaussian(kcv, ctx, host, w, h, c, k, sigma, border, *, bv=None, offset=0, dst_pad=7,
                 dst_offset=0):
    _keep, src_ptr, src_stride = device_image(torch, host, offset)
    obuf, dptr, dstride = device_output(torch, h, w * c, np.uint8, dst_pad, dst_offset)
    err = kcv.gaussian_blur_u8(src_ptr, src_stride, dptr, dstride, w, h, c, k, k, sigma, sigma, border,
                               ctx, border_value=bv)
    assert err == kcv.OK, kcv.ERROR_NAMES.get(err, err)
    assert ctx.synchronize() == kcv.OK
    return read_output(obuf, h, w * c, np.uint8, dstride, dst_offset)


def check_gaussian(kcv, oracle, ctx, rng, w, h, c, k, sigma, border, bv=None, offset=0, pad=5,
                   high=255, low=0):
    host = padded(rng, h, w * c, np.uint8, pad, low=low, high=high)
    got, pad_ok = run_gaussian(kcv, ctx, host, w, h, c, k, sigma, border, bv=bv, offset=offset)
    err, want = oracle.gaussian_blur_u8(host, w, h, c, k, sigma, border, ext=bv is not None,
                                        border_value=bv or 0, nthreads=8)
    assert err == oracle.OK
    assert pad_ok, "write outside the destination rows"
    if not np.array_equal(got, want):
        bad = np.argwhere(got != want)
        raise AssertionError(f"{len(bad)} mismatches (w={w} h={h} c={c} k={k} s={sigma} b={border}); "
                             f"first {bad[:4].tolist()} got {got[tuple(bad[0])]} want {want[tuple(bad[0])]}")


@pytest.mark.parametrize("k", [3, 5, 7, 9, 15, 21])
@pytest.mark.parametrize("sigma", [0.0, 1.5])
@pytest.mark.parametrize("c", [1, 2, 3, 4])
def test_gaussian_fixed_sizes(kcv, oracle, ctx, k, sigma, c):
    rng = np.random.default_rng(k * 31 + c + int(sigma * 10))
    for border in BORDERS:
        for (w, h) in [(k - 1, k - 1), (k + 4, k + 2), (37, max(23, k - 1)), (603, k + 1),
                       (131, 300)]:
            check_gaussian(kcv, oracle, ctx, rng, w, h, c, k, sigma, border)


@pytest.mark.parametrize("k,sigma", [(7, 1.5), (5, 0.0), (15, 2.5), (21, 4.0), (3, 0.7)])
def test_gaussian_constant_border_extension(kcv, oracle, ctx, k, sigma):
    rng = np.random.default_rng(k)
    for c in (1, 3, 4):
        for bv in (0, 17, 255):
            check_gaussian(kcv, oracle, ctx, rng, 45, k + 3, c, k, sigma, 0, bv=bv)


def test_gaussian_copy_case(kcv, oracle, ctx):
    assert kcv.half_kernel(3, 0.1) is None  # all weight in the centre tap
    rng = np.random.default_rng(1)
    for c in (1, 4):
        check_gaussian(kcv, oracle, ctx, rng, 50, 9, c, 3, 0.1, 2)


@pytest.mark.parametrize("k,sigma", [(11, 0.0), (13, 2.2), (17, 3.0), (31, 5.0), (63, 0.0), (255, 40.0)])
def test_gaussian_arbitrary_sizes(kcv, oracle, ctx, k, sigma):
    rng = np.random.default_rng(k)
    r = k // 2
    wmin = (r + 7) // 8 * 8 + r
    for c in (1, 3, 4):
        for (w, h) in [(wmin, k - 1), (wmin + 9, k + 3), (300, max(12, k - 1))]:
            check_gaussian(kcv, oracle, ctx, rng, w, h, c, k, sigma, 1)


@pytest.mark.parametrize("k,i", [(59, 3103), (123, 3810), (137, 3614), (165, 3464), (131, 1459)])
def test_gaussian_arbitrary_weights_not_summing_to_256(kcv, oracle, ctx, k, i):
    """Kernels whose rounded weights sum to 257 (or 255): the reference's
    vector paths saturate and its border/scalar paths wrap; near-white images
    exercise both."""
    sigma = float(np.float32(i) / np.float32(100))
    hk = kcv.half_kernel(k, sigma)
    assert hk is not None and 2 * sum(hk[:-1]) + hk[-1] != 256
    rng = np.random.default_rng(k)
    r = k // 2
    wmin = (r + 7) // 8 * 8 + r
    for c in (1, 2, 4):
        for (w, h) in [(wmin, k - 1), (wmin + 33, k + 5)]:
            check_gaussian(kcv, oracle, ctx, rng, w, h, c, k, sigma, 1, low=250, high=255)
    # narrow rows (width*channels < 16 is impossible here since width >= 13),
    # so also an image with a mid region narrower than one vector:
    check_gaussian(kcv, oracle, ctx, rng, wmin + 1, k - 1, 1, k, sigma, 1, low=250, high=255)


@pytest.mark.parametrize("k,sigma", [(3, 0.8), (5, 1.1), (7, 1.5), (7, 2.6)])
def test_gaussian_four_channel_streaming(kcv, oracle, ctx, k, sigma):
    """The four-channel streaming Gaussian (16-byte aligned rows): several
    warp strips and bands, ragged widths (edge pixels on both sides, lanes
    past the aligned span), minimum sizes, every border and CONSTANT values,
    aligned and unaligned destinations, and a source 8 bytes off alignment
    (the generic kernel)."""
    rng = np.random.default_rng(k * 10 + int(sigma * 10))
    sizes = [(121, 37), (240, 15), (723, 203), (1999, 64), (k - 1, k - 1), (k + 2, 11), (33, 300)]
    for i, (w, h) in enumerate(sizes):
        for border in BORDERS + [0]:
            pad = (16 - (w * 4) % 16) % 16 + 16  # rows a multiple of 16 bytes
            host = padded(rng, h, w * 4, np.uint8, pad)
            bv = int(rng.integers(0, 256)) if border == 0 else None
            offset = 8 if (i + border) % 4 == 0 else 0
            got, pad_ok = run_gaussian(kcv, ctx, host, w, h, 4, k, sigma, border, bv=bv, offset=offset,
                                       dst_pad=pad if border % 2 else 7)
            err, want = oracle.gaussian_blur_u8(host, w, h, 4, k, sigma, border, ext=bv is not None,
                                                border_value=bv or 0, nthreads=8)
            assert err == oracle.OK and pad_ok
            if not np.array_equal(got, want):
                bad = np.argwhere(got != want)
                raise AssertionError(f"{len(bad)} mismatches (w={w} h={h} k={k} s={sigma} b={border} "
                                     f"off={offset}); first {bad[:4].tolist()}")


@pytest.mark.parametrize("k,sigma", [(3, 0.8), (5, 1.1), (7, 1.5)])
def test_gaussian_four_channel_unaligned_rows(kcv, oracle, ctx, k, sigma):
    """The four-channel streaming Gaussian on rows that are 4-byte but not
    16-byte aligned (every pixel copied on its own): row strides of w * 4
    bytes with w % 4 != 0, base offsets of 4, 8 and 12 bytes, destinations
    4-byte aligned (word stores) and not (bytes), every border; a base 2
    bytes off (not whole pixels) takes the tiled kernel."""
    rng = np.random.default_rng(70 + k)
    cases = [(1366, 77, 0, 0), (723, 41, 4, 0), (1001, 23, 8, 1), (33, 100, 12, 0), (k + 1, k + 2, 4, 3),
             (3841, 19, 0, 2), (517, 9, 2, 0)]
    for i, (w, h, offset, dpad) in enumerate(cases):
        for border in BORDERS + [0]:
            host = padded(rng, h, w * 4, np.uint8, 0)
            bv = int(rng.integers(0, 256)) if border == 0 else None
            got, pad_ok = run_gaussian(kcv, ctx, host, w, h, 4, k, sigma, border, bv=bv, offset=offset,
                                       dst_pad=dpad)
            err, want = oracle.gaussian_blur_u8(host, w, h, 4, k, sigma, border, ext=bv is not None,
                                                border_value=bv or 0, nthreads=8)
            assert err == oracle.OK and pad_ok
            if not np.array_equal(got, want):
                bad = np.argwhere(got != want)
                raise AssertionError(f"{len(bad)} mismatches (w={w} h={h} k={k} b={border} off={offset}); "
                                     f"first {bad[:4].tolist()}")


@pytest.mark.parametrize("offset", [1, 3, 8])
def test_gaussian_misaligned_and_padded(kcv, oracle, ctx, offset):
    rng = np.random.default_rng(offset)
    for (k, sigma, c) in [(5, 0.0, 1), (7, 1.5, 4), (3, 0.0, 3)]:
        for border in BORDERS:
            check_gaussian(kcv, oracle, ctx, rng, 301, 17, c, k, sigma, border, offset=offset, pad=3)


# ---------------------------------------------------------------------------
SEP_DT = {"u8": np.uint8, "u16": np.uint16, "s16": np.int16}


def run_separable(kcv, ctx, dt, host, w, h, c, kx, ky, border, bv=None, offset=0, dst_pad=3):
    dtype = SEP_DT[dt]
    _keep, sp, ss = device_image(torch, host, offset)
    obuf, dp, ds = device_output(torch, h, w * c, dtype, dst_pad)
    err = kcv.separable_filter_2d(dt, sp, ss, dp, ds, w, h, c, kx, 5, ky, 5, border, ctx, border_value=bv)
    assert err == kcv.OK, kcv.ERROR_NAMES.get(err, err)
    assert ctx.synchronize() == kcv.OK
    return read_output(obuf, h, w * c, dtype, ds)


@pytest.mark.parametrize("dt", ["u8", "u16", "s16"])
@pytest.mark.parametrize("c", [1, 2, 3, 4])
def test_separable(kcv, oracle, ctx, dt, c):
    dtype = SEP_DT[dt]
    info = np.iinfo(dtype)
    rng = np.random.default_rng(c * 7 + len(dt))
    borders = BORDERS + ([0] if dt == "s16" else [])
    for border in borders:
        for (w, h) in [(4, 4), (13, 6), (211, 9), (1100, 5)]:
            for trange in ((0, 4), (info.min, info.max)) if dt != "s16" else ((-4, 4), (info.min, info.max)):
                kx = rng.integers(trange[0], trange[1] + 1, 5)
                ky = rng.integers(trange[0], trange[1] + 1, 5)
                host = padded(rng, h, w * c, dtype, 2)
                bv = 17 if border == 0 else None
                got, pad_ok = run_separable(kcv, ctx, dt, host, w, h, c, kx, ky, border, bv)
                err, want = oracle.separable_filter_2d(host, w, h, c, kx.astype(dtype), ky.astype(dtype),
                                                       border, ext=bv is not None, border_value=bv or 0)
                assert err == oracle.OK
                assert pad_ok
                assert np.array_equal(got, want), (dt, c, border, w, h, trange)


@pytest.mark.parametrize("dt", ["u16", "s16"])
def test_separable_16bit_5x5_one_channel(kcv, oracle, ctx, dt):
    """The one-channel 16-bit 5x5 streaming kernel: several warp strips and
    bands (heights not a multiple of its 5-row step), ragged widths, a source
    8 bytes off 16-byte alignment (element gathers), every border, full-range
    taps (u16 saturation), and s16 taps exactly at and just past the limit of
    its fp32 path (32768 * sum|kx| * sum|ky| <= 2^24; past it the generic
    kernel runs)."""
    dtype = SEP_DT[dt]
    info = np.iinfo(dtype)
    rng = np.random.default_rng(91 + len(dt))
    sizes = [(241, 37), (480, 11), (723, 203), (1999, 64), (16, 7), (9, 5)]
    borders = BORDERS + [0]
    taps = [(rng.integers(0, 5, 5), rng.integers(0, 5, 5))] if dt == "u16" else \
        [(rng.integers(-4, 5, 5), rng.integers(-4, 5, 5))]
    if dt == "u16":
        taps.append((rng.integers(0, 65536, 5), rng.integers(0, 65536, 5)))
        taps.append((np.array([0, 0, 65535, 0, 0]), np.array([1, 0, 0, 0, 0])))
    else:
        taps.append((np.array([-8, 4, 0, 2, 2]), np.array([1, -9, 0, 4, 2])))   # 16 * 16 * 32768 = 2^23
        taps.append((np.array([-16, 8, 0, 4, 4]), np.array([1, -9, 0, 4, 2])))  # 32 * 16 = 512: at the limit
        taps.append((np.array([-16, 8, 0, 4, 5]), np.array([1, -9, 0, 4, 2])))  # 33 * 16: generic kernel
        taps.append((rng.integers(-32768, 32768, 5), rng.integers(-32768, 32768, 5)))
    for i, (w, h) in enumerate(sizes):
        for border in borders:
            kx, ky = taps[(i + border) % len(taps)]
            offset = 8 if (i + border) % 3 == 0 else 0
            pad = (8 - w % 8) % 8 + 8  # rows a multiple of 16 bytes
            host = padded(rng, h, w, dtype, pad, low=int(info.min), high=int(info.max))
            bv = 4097 if border == 0 else None
            got, pad_ok = run_separable(kcv, ctx, dt, host, w, h, 1, kx, ky, border, bv, offset=offset,
                                        dst_pad=pad if border % 2 else 3)
            err, want = oracle.separable_filter_2d(host, w, h, 1, kx.astype(dtype), ky.astype(dtype), border,
                                                   ext=bv is not None, border_value=bv or 0)
            assert err == oracle.OK and pad_ok
            assert np.array_equal(got, want), (dt, w, h, border, offset, kx.tolist(), ky.tolist())


@pytest.mark.parametrize("dt", ["u8", "u16"])
def test_separable_constant_extension(kcv, oracle, ctx, dt):
    dtype = SEP_DT[dt]
    rng = np.random.default_rng(3)
    for c in (1, 4):
        kx, ky = rng.integers(0, 5, 5), rng.integers(0, 5, 5)
        host = padded(rng, 9, 40 * c, dtype, 0)
        got, _ = run_separable(kcv, ctx, dt, host, 40, 9, c, kx, ky, 0, 17)
        err, want = oracle.separable_filter_2d(host, 40, 9, c, kx.astype(dtype), ky.astype(dtype), 0,
                                               ext=True, border_value=17)
        assert err == 0 and np.array_equal(got, want)


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("c", [1, 2, 3, 4])
def test_blur_and_downsample(kcv, oracle, ctx, c):
    rng = np.random.default_rng(c)
    for border in BORDERS + [0]:
        for (w, h) in [(4, 4), (5, 5), (161, 7), (9, 12), (777, 33), (1031, 8)]:
            host = padded(rng, h, w * c, np.uint8, 3)
            ow, oh = (w + 1) // 2, (h + 1) // 2
            _k, sp, ss = device_image(torch, host)
            obuf, dp, ds = device_output(torch, oh, ow * c, np.uint8, 5)
            bv = 17 if border == 0 else None
            err = kcv.blur_and_downsample_u8(sp, ss, w, h, dp, ds, c, border, ctx, border_value=bv)
            assert err == kcv.OK
            assert ctx.synchronize() == kcv.OK
            got, pad_ok = read_output(obuf, oh, ow * c, np.uint8, ds)
            e2, want = oracle.blur_and_downsample_u8(host, w, h, c, border, ext=bv is not None,
                                                     border_value=bv or 0)
            assert e2 == 0 and pad_ok
            assert np.array_equal(got, want), (c, border, w, h)


@pytest.mark.parametrize("c", [1, 2, 3, 4])
def test_blur_and_downsample_unaligned_rows(kcv, oracle, ctx, c):
    """Unaligned sources take the staged path: every row misaligned by the
    same amount (aligned stride, base offset 1..15) or by a different amount
    (odd stride), widths over several strips and below one, every border."""
    rng = np.random.default_rng(40 + c)
    for border in BORDERS + [0]:
        for (w, h, offset, pad) in [(1500, 70, 0, 3), (1536, 41, 5, 0), (263, 9, 7, 9), (3001, 23, 15, 1),
                                    (40, 33, 3, 5), (17, 4, 1, 0)]:
            if pad == 0:
                pad = (-(w * c)) % 16  # 16-byte rows: only the base is unaligned
            host = padded(rng, h, w * c, np.uint8, pad)
            ow, oh = (w + 1) // 2, (h + 1) // 2
            _k, sp, ss = device_image(torch, host, offset)
            obuf, dp, ds = device_output(torch, oh, ow * c, np.uint8, 5)
            bv = 17 if border == 0 else None
            err = kcv.blur_and_downsample_u8(sp, ss, w, h, dp, ds, c, border, ctx, border_value=bv)
            assert err == kcv.OK
            assert ctx.synchronize() == kcv.OK
            got, pad_ok = read_output(obuf, oh, ow * c, np.uint8, ds)
            e2, want = oracle.blur_and_downsample_u8(host, w, h, c, border, ext=bv is not None,
                                                     border_value=bv or 0)
            assert e2 == 0 and pad_ok
            assert np.array_equal(got, want), (c, border, w, h, offset, pad)


def test_pyramid_five_levels(kcv, oracle, ctx):
    rng = np.random.default_rng(9)
    for (w, h, c) in [(515, 301, 1), (200, 131, 3), (128, 96, 4)]:
        host = padded(rng, h, w * c, np.uint8, 0)
        _k, sp, ss = device_image(torch, host)
        sizes = pyr_sizes(w, h, 5)
        outs = [device_output(torch, lh, lw * c, np.uint8, 0) for (lw, lh) in sizes]
        err = kcv.build_pyramid_u8(sp, ss, w, h, c, [o[1] for o in outs], [o[2] for o in outs], 4, ctx)
        assert err == kcv.OK
        assert ctx.synchronize() == kcv.OK
        level = host
        lw, lh = w, h
        for (ow, oh), (buf, _p, st) in zip(sizes, outs):
            e2, want = oracle.blur_and_downsample_u8(level, lw, lh, c, 4)
            got, _ = read_output(buf, oh, ow * c, np.uint8, st)
            assert e2 == 0 and np.array_equal(got, want)
            level, lw, lh = want, ow, oh


# ---------------------------------------------------------------------------
def _kats():
    with open(os.path.join(os.path.dirname(__file__), "golden", "kats.json")) as f:
        return json.load(f)["cases"]


@pytest.mark.parametrize("case", _kats(), ids=lambda c: c["name"])
def test_reference_kats_through_c_abi(kcv, oracle, ctx, case):
    dtype = np.dtype(case["dtype"])
    host = np.array(case["src"], dtype=dtype)
    w, h, c = case["width"], case["height"], case["channels"]
    if case["func"] == "gaussian_blur_u8":
        got, _ = run_gaussian(kcv, ctx, host, w, h, c, case["kernel_width"], case["sigma_x"], case["border"])
        err, want = oracle.gaussian_blur_u8(host, w, h, c, case["kernel_width"], case["sigma_x"], case["border"])
    elif case["func"] == "separable_filter_2d":
        dt = "u8" if dtype == np.uint8 else "u16"
        got, _ = run_separable(kcv, ctx, dt, host, w, h, c, case["kernel_x"], case["kernel_y"], case["border"])
        err, want = oracle.separable_filter_2d(host, w, h, c, np.array(case["kernel_x"], dtype),
                                               np.array(case["kernel_y"], dtype), case["border"])
    else:
        _k, sp, ss = device_image(torch, host)
        ow, oh = (w + 1) // 2, (h + 1) // 2
        obuf, dp, ds = device_output(torch, oh, ow * c, np.uint8, 0)
        assert kcv.blur_and_downsample_u8(sp, ss, w, h, dp, ds, c, case["border"], ctx) == kcv.OK
        assert ctx.synchronize() == kcv.OK
        got, _ = read_output(obuf, oh, ow * c, np.uint8, ds)
        err, want = oracle.blur_and_downsample_u8(host, w, h, c, case["border"])
    exp = np.array(case["expected"], dtype=np.int64)
    assert np.abs(got.astype(np.int64) - exp).max() <= case["tolerance"]
    assert np.array_equal(got, want)  # and bit-exact to the oracle


# ---------------------------------------------------------------------------
# Full-size configurations: bit-exact against the (multithreaded) oracle.

def test_config_hd_gray_binomial5(kcv, oracle, ctx):
    rng = np.random.default_rng(0)
    host = padded(rng, 1080, 1920, np.uint8, 64)
    check_host = host
    got, pad_ok = run_gaussian(kcv, ctx, check_host, 1920, 1080, 1, 5, 0.0, 1, dst_pad=64)
    err, want = oracle.gaussian_blur_u8(host, 1920, 1080, 1, 5, 0.0, 1, nthreads=16)
    assert err == 0 and pad_ok and np.array_equal(got, want)


def test_config_4k_rgba_sigma7(kcv, oracle, ctx):
    rng = np.random.default_rng(1)
    host = padded(rng, 2160, 3840 * 4, np.uint8, 0)
    got, pad_ok = run_gaussian(kcv, ctx, host, 3840, 2160, 4, 7, 1.5, 4, dst_pad=0)
    err, want = oracle.gaussian_blur_u8(host, 3840, 2160, 4, 7, 1.5, 4, nthreads=16)
    assert err == 0 and pad_ok and np.array_equal(got, want)


@pytest.mark.parametrize("dt,border", [("u16", 2), ("u16", 3), ("s16", 0)])
def test_config_4k_separable(kcv, oracle, ctx, dt, border):
    dtype = SEP_DT[dt]
    rng = np.random.default_rng(1)
    host = padded(rng, 2160, 3840, dtype, 0)
    kx = rng.integers(0, 5, 5)
    ky = rng.integers(0, 5, 5)
    bv = 17 if border == 0 else None
    got, _ = run_separable(kcv, ctx, dt, host, 3840, 2160, 1, kx, ky, border, bv)
    err, want = oracle.separable_filter_2d(host, 3840, 2160, 1, kx.astype(dtype), ky.astype(dtype), border,
                                           ext=bv is not None, border_value=bv or 0, nthreads=16)
    assert err == 0 and np.array_equal(got, want)


def test_arbitrary_size_tall_narrow_image(kcv, oracle, ctx):
    """A 13x70000 image with an 11x11 generated kernel: more rows than the
    grid's 65535-block y limit in both passes of the two-pass kernel."""
    rng = np.random.default_rng(70000)
    check_gaussian(kcv, oracle, ctx, rng, 13, 70000, 1, 11, 2.0, 1)


@pytest.mark.parametrize("c", [2, 3, 4])
@pytest.mark.parametrize("k,w", [(11, 13), (13, 21), (17, 47), (31, 40), (63, 71), (101, 301)])
def test_arbitrary_size_right_border_lanes(kcv, oracle, ctx, k, w, c):
    """Arbitrary sizes with 2-4 channels: the right-border vectors' replicated
    lanes take the reference's shifted channel pattern."""
    rng = np.random.default_rng(k * 10 + c)
    for sigma in (0.0, 3.0):
        check_gaussian(kcv, oracle, ctx, rng, w, k + 3, c, k, sigma, 1)


def _pyramid_levels(oracle, host, w, h, c, levels, border):
    out, level, lw, lh = [], host, w, h
    for _ in range(levels):
        e, level = oracle.blur_and_downsample_u8(level, lw, lh, c, border)
        assert e == 0
        lw, lh = (lw + 1) // 2, (lh + 1) // 2
        out.append(level)
    return out


@pytest.mark.parametrize("c", [1, 2, 3, 4])
def test_pyramid_one_launch_many_levels(kcv, oracle, ctx, c):
    """Pyramids built in one cooperative launch (more levels than one launch
    carries inline, so also two launches), ragged sizes, every border."""
    rng = np.random.default_rng(40 + c)
    for (w, h, levels, border) in [(2001, 1499, 9, 4), (1030, 777, 7, 1), (133, 67, 4, 2), (4099, 259, 6, 3)]:
        host = padded(rng, h, w * c, np.uint8, 0)
        _k, sp, ss = device_image(torch, host)
        sizes = pyr_sizes(w, h, levels)
        outs = [device_output(torch, lh, lw * c, np.uint8, 3) for (lw, lh) in sizes]
        err = kcv.build_pyramid_u8(sp, ss, w, h, c, [o[1] for o in outs], [o[2] for o in outs], border, ctx)
        assert err == kcv.OK
        assert ctx.synchronize() == kcv.OK
        for lv, ((ow, oh), (buf, _p, st), want) in enumerate(zip(sizes, outs, _pyramid_levels(
                oracle, host, w, h, c, levels, border))):
            got, pad_ok = read_output(buf, oh, ow * c, np.uint8, st)
            assert pad_ok, (c, w, h, lv)
            assert np.array_equal(got, want), (c, w, h, border, lv)


def test_pyramids_batched_one_launch(kcv, oracle, ctx):
    """Many pyramids of mixed channel counts, sizes, borders and level counts
    through kleidicv_gpu_build_pyramids_u8, plus a misaligned source (byte
    loads) and an invalid entry reported per entry."""
    rng = np.random.default_rng(77)
    cases, keep, expect = [], [], []
    for i in range(24):
        c = int(rng.choice([1, 3, 4]))
        w, h = int(rng.integers(40, 700)), int(rng.integers(40, 500))
        levels = int(rng.integers(1, 5))
        border = int(rng.choice([1, 2, 3, 4]))
        host = padded(rng, h, w * c, np.uint8, 1)
        buf, sp, ss = device_image(torch, host, offset=1 if i == 5 else 0)
        sizes = pyr_sizes(w, h, levels)
        outs = [device_output(torch, lh, lw * c, np.uint8, 0) for (lw, lh) in sizes]
        keep += [buf, outs]
        cases.append((sp, ss, w, h, c, [o[1] for o in outs], [o[2] for o in outs], border))
        expect.append((host, w, h, c, levels, border, sizes, outs))
    err, st = kcv.build_pyramids_u8(cases, ctx)
    assert err == kcv.OK and st == [kcv.OK] * len(cases)
    assert ctx.synchronize() == kcv.OK
    for host, w, h, c, levels, border, sizes, outs in expect:
        for (ow, oh), (buf, _p, stv), want in zip(sizes, outs, _pyramid_levels(oracle, host, w, h, c, levels,
                                                                               border)):
            got, _ = read_output(buf, oh, ow * c, np.uint8, stv)
            assert np.array_equal(got, want), (w, h, c, border)
    bad = list(cases[0])
    bad[7] = 0  # CONSTANT: not implemented on the drop-in path
    err, st = kcv.build_pyramids_u8([cases[1], tuple(bad)], ctx)
    assert err == kcv.NOT_IMPLEMENTED and st == [kcv.OK, kcv.NOT_IMPLEMENTED]


def test_pyramids_batched_more_entries_than_the_shared_search(kcv, oracle, ctx):
    """600 small pyramids in one call: a phase with more entries than the
    kernel keeps in shared memory for its entry search (the search then reads
    the table in global memory)."""
    rng = np.random.default_rng(79)
    cases, expect, keep = [], [], []
    for i in range(600):
        w, h = int(rng.integers(8, 40)), int(rng.integers(8, 30))
        levels = int(rng.integers(1, 3))
        host = padded(rng, h, w, np.uint8, 16 - w % 16)
        buf, sp, ss = device_image(torch, host)
        sizes = pyr_sizes(w, h, levels)
        outs = [device_output(torch, lh, lw, np.uint8, 0) for (lw, lh) in sizes]
        keep += [buf, outs]
        cases.append((sp, ss, w, h, 1, [o[1] for o in outs], [o[2] for o in outs], 4))
        expect.append((host, w, h, levels, sizes, outs))
    err, st = kcv.build_pyramids_u8(cases, ctx)
    assert err == kcv.OK and st == [kcv.OK] * len(cases)
    assert ctx.synchronize() == kcv.OK
    for host, w, h, levels, sizes, outs in expect:
        for (ow, oh), (buf, _p, stv), want in zip(sizes, outs, _pyramid_levels(oracle, host, w, h, 1, levels, 4)):
            got, _ = read_output(buf, oh, ow, np.uint8, stv)
            assert np.array_equal(got, want), (w, h)


@pytest.mark.parametrize("dt", ["u16", "s16"])
def test_separable_16bit_tall_image(kcv, oracle, ctx, dt):
    """70001 rows: more bands than a wave of resident warps holds, several
    items per warp."""
    dtype = SEP_DT[dt]
    rng = np.random.default_rng(81)
    w, h = 248, 70001
    host = padded(rng, h, w, dtype, 8)
    kx = rng.integers(0, 5, 5) if dt == "u16" else rng.integers(-4, 5, 5)
    ky = rng.integers(0, 5, 5) if dt == "u16" else rng.integers(-4, 5, 5)
    got, pad_ok = run_separable(kcv, ctx, dt, host, w, h, 1, kx, ky, 3, dst_pad=8)
    err, want = oracle.separable_filter_2d(host, w, h, 1, kx.astype(dtype), ky.astype(dtype), 3, nthreads=8)
    assert err == oracle.OK and pad_ok and np.array_equal(got, want)


def test_gaussian_four_channel_tall_image(kcv, oracle, ctx):
    rng = np.random.default_rng(82)
    w, h = 36, 70001
    host = padded(rng, h, w * 4, np.uint8, 16)
    got, pad_ok = run_gaussian(kcv, ctx, host, w, h, 4, 7, 1.5, 4, dst_pad=16)
    err, want = oracle.gaussian_blur_u8(host, w, h, 4, 7, 1.5, 4, nthreads=8)
    assert err == oracle.OK and pad_ok and np.array_equal(got, want)


def test_blur_and_downsample_tiled_and_pyramid_kernels_agree(kcv, ctx):
    """A forced tile shape selects the tiled stencil; both kernels give the
    same bytes."""
    rng = np.random.default_rng(78)
    w, h, c = 1001, 707, 3
    host = padded(rng, h, w * c, np.uint8, 0)
    _k, sp, ss = device_image(torch, host)
    ow, oh = (w + 1) // 2, (h + 1) // 2
    outs = []
    for tiled in (False, True):
        if tiled:
            assert ctx.set_tile_shape(128, 0, 4, 0) == kcv.OK
        obuf, dp, ds = device_output(torch, oh, ow * c, np.uint8, 0)
        assert kcv.blur_and_downsample_u8(sp, ss, w, h, dp, ds, c, 2, ctx) == kcv.OK
        assert ctx.synchronize() == kcv.OK
        outs.append(read_output(obuf, oh, ow * c, np.uint8, ds)[0])
    assert ctx.set_tile_shape(0) == kcv.OK
    assert np.array_equal(outs[0], outs[1])
