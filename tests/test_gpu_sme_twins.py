"""The `_sme` twins of the drop-in entries (kleidicv.h:2010, 2054, 2097, 2109,
2165, 2220) are the same calls as their base entries: the same bytes as the
CPU oracle on valid calls and the same error codes on rejected ones."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402
from gpu_harness import device_image, device_output, read_output, padded  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()


def _taps(vals, ct):
    return (ct * 5)(*[int(v) for v in vals])


def test_gaussian_twin():
    rng = np.random.default_rng(61)
    ctx = kcv.Context.for_torch(0)
    for (w, h, c, k, sigma, border) in [(301, 77, 4, 7, 1.5, kcv.REVERSE), (64, 40, 1, 5, 0.0, kcv.REFLECT),
                                       (129, 33, 3, 15, 2.5, kcv.REPLICATE)]:
        host = padded(rng, h, w * c, np.uint8, 3)
        _k, sp, ss = device_image(torch, host)
        obuf, dp, ds = device_output(torch, h, w * c, np.uint8, 5)
        e = kcv.lib().kleidicv_gpu_gaussian_blur_u8_sme(sp, ss, dp, ds, w, h, c, k, k, sigma, sigma, border,
                                                        ctx.handle)
        assert e == kcv.OK and ctx.synchronize() == kcv.OK
        got, pad_ok = read_output(obuf, h, w * c, np.uint8, ds)
        err, want = oracle.gaussian_blur_u8(host, w, h, c, k, sigma, border)
        assert err == oracle.OK and pad_ok and np.array_equal(got, want)
    # Rejections match the base entry: even size, CONSTANT border, null pointers.
    lib = kcv.lib()
    for args in [(None, 64, None, 64, 8, 8, 1, 5, 5, 0.0, 0.0, kcv.REFLECT),
                 (1, 64, 1, 64, 8, 8, 1, 4, 4, 0.0, 0.0, kcv.REFLECT),
                 (1, 64, 1, 64, 8, 8, 1, 5, 5, 0.0, 0.0, kcv.CONSTANT)]:
        assert (lib.kleidicv_gpu_gaussian_blur_u8_sme(*args, ctx.handle) ==
                lib.kleidicv_gpu_gaussian_blur_u8(*args, ctx.handle) != kcv.OK)
    ctx.close()


@pytest.mark.parametrize("dt", ["u8", "u16"])
def test_separable_twin(dt):
    rng = np.random.default_rng(62)
    dtype, ct = (np.uint8, ctypes.c_uint8) if dt == "u8" else (np.uint16, ctypes.c_uint16)
    fn = getattr(kcv.lib(), f"kleidicv_gpu_separable_filter_2d_{dt}_sme")
    ctx = kcv.Context.for_torch(0)
    for (w, h, c, border) in [(257, 41, 1, kcv.REFLECT), (90, 23, 3, kcv.WRAP)]:
        host = padded(rng, h, w * c, dtype, 0)
        kx, ky = rng.integers(0, 5, 5), rng.integers(0, 5, 5)
        _k, sp, ss = device_image(torch, host)
        obuf, dp, ds = device_output(torch, h, w * c, dtype, 2)
        e = fn(sp, ss, dp, ds, w, h, c, _taps(kx, ct), 5, _taps(ky, ct), 5, border, ctx.handle)
        assert e == kcv.OK and ctx.synchronize() == kcv.OK
        got, pad_ok = read_output(obuf, h, w * c, dtype, ds)
        err, want = oracle.separable_filter_2d(host, w, h, c, kx.astype(dtype), ky.astype(dtype), border)
        assert err == oracle.OK and pad_ok and np.array_equal(got, want)
    k5 = _taps([1] * 5, ct)
    assert fn(1, 64, 1, 64, 8, 8, 1, k5, 3, k5, 3, kcv.REFLECT, ctx.handle) == kcv.NOT_IMPLEMENTED
    ctx.close()


def test_blur_and_downsample_twin():
    rng = np.random.default_rng(63)
    ctx = kcv.Context.for_torch(0)
    for (w, h, c, border) in [(777, 33, 3, kcv.REFLECT), (1024, 64, 4, kcv.REPLICATE)]:
        host = padded(rng, h, w * c, np.uint8, 0)
        ow, oh = (w + 1) // 2, (h + 1) // 2
        _k, sp, ss = device_image(torch, host)
        obuf, dp, ds = device_output(torch, oh, ow * c, np.uint8, 5)
        e = kcv.lib().kleidicv_gpu_blur_and_downsample_u8_sme(sp, ss, w, h, dp, ds, c, border, ctx.handle)
        assert e == kcv.OK and ctx.synchronize() == kcv.OK
        got, pad_ok = read_output(obuf, oh, ow * c, np.uint8, ds)
        err, want = oracle.blur_and_downsample_u8(host, w, h, c, border)
        assert err == oracle.OK and pad_ok and np.array_equal(got, want)
    ctx.close()


@pytest.mark.parametrize("horizontal", [True, False])
def test_sobel_twin(horizontal):
    rng = np.random.default_rng(64)
    name = "horizontal" if horizontal else "vertical"
    fn = getattr(kcv.lib(), f"kleidicv_gpu_sobel_3x3_{name}_s16_u8_sme")
    ctx = kcv.Context.for_torch(0)
    w, h, c = 501, 37, 2
    host = padded(rng, h, w * c, np.uint8, 7)
    _k, sp, ss = device_image(torch, host)
    obuf, dp, ds = device_output(torch, h, w * c, np.int16, 1)
    assert fn(sp, ss, dp, ds, w, h, c, ctx.handle) == kcv.OK and ctx.synchronize() == kcv.OK
    got, pad_ok = read_output(obuf, h, w * c, np.int16, ds)
    err, want = oracle.sobel_3x3_s16_u8(host, w, h, c, horizontal)
    assert err == 0 and pad_ok and np.array_equal(got, want)
    ctx.close()
