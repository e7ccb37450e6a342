"""Median blur without a GPU: the numpy oracle against a literal restatement of
the reference test's own model (test/api/test_median_blur.cpp:108-186: map the
window through get_physical_index, sort, take the middle) on the reference's
test shapes, the error cases of :206-369, and the C ABI's validation against
the oracle's order of checks."""
import numpy as np
import pytest

MAX_PIXELS = (1 << 48) - 1
DTYPES = ["s8", "u8", "u16", "s16", "u32", "s32", "f32"]
BORDERS = [1, 2, 3, 4]  # REPLICATE, REFLECT, WRAP, REVERSE


def physical_index(i, n, border):  # test_median_blur.cpp:114-155
    if 0 <= i < n:
        return i
    if border == 1:
        return min(max(i, 0), n - 1)
    if border == 2:
        return -i - 1 if i < 0 else 2 * n - i - 1
    if border == 3:
        return (i + n) % n
    if border == 4:
        return -i if i < 0 else 2 * n - i - 2
    return 0


def reference_model(src, w, h, c, k, border):
    r = k // 2
    out = np.zeros((h, w * c), src.dtype)
    for y in range(h):
        for x in range(w):
            for ch in range(c):
                win = sorted(src[physical_index(y + dy, h, border), physical_index(x + dx, w, border) * c + ch]
                             for dy in range(-r, r + 1) for dx in range(-r, r + 1))
                out[y, x * c + ch] = win[len(win) // 2]
    return out


def random_image(rng, dtype, h, elems):
    dt = np.dtype(dtype)
    if dt.kind == "f":
        return rng.uniform(-1e6, 1e6, (h, elems)).astype(dt)
    info = np.iinfo(dt)
    return rng.integers(info.min, int(info.max) + 1, (h, elems), dtype=dt)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [3, 5, 7])
def test_oracle_equals_reference_model(oracle, dtype, k):
    rng = np.random.default_rng(k * 11 + DTYPES.index(dtype))
    w, h = 2 * k + 2, k  # get_test_cases (:67-94)
    for c in (1, 2, 3, 4):
        for border in BORDERS:
            src = random_image(rng, oracle.MEDIAN_DTYPES[dtype], h, w * c + 5)
            got = oracle.median_blur(src, w, h, c, k, border)
            assert np.array_equal(got, reference_model(src, w, h, c, k, border)), (c, border)


@pytest.mark.parametrize("k", [9, 15, 17])
def test_oracle_equals_reference_model_u8_histogram_sizes(oracle, k):
    rng = np.random.default_rng(k)
    w, h = 2 * k + 2, k
    for c, border in ((1, 1), (3, 2), (4, 3), (2, 4)):
        src = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
        assert np.array_equal(oracle.median_blur(src, w, h, c, k, border), reference_model(src, w, h, c, k, border))


def median_cases(dtype):
    """(src_null, src_stride, dst_null, dst_stride, w, h, c, kw, kh, border, same, expected) per
    test_median_blur.cpp; strides are in bytes."""
    es = {"s8": 1, "u8": 1, "u16": 2, "s16": 2, "u32": 4, "s32": 4, "f32": 4}[dtype]
    NI, NP, RG, AL = 1, 2, 3, 5
    s = 128 * es
    cases = [
        (0, s, 0, s, 25, 25, 5, 5, 5, 1, False, NI),                        # ChannelNumber :206-214
        (0, s, 0, s, 25, 25, 1, 5, 5, 5, False, NI),                        # BorderNotImplemented :216-223
        (0, s, 0, s, 100, 3, 1, 7, 7, 1, False, NI),                        # HeightTooSmall :225-232
        (0, s, 0, s, 3, 100, 1, 7, 7, 1, False, NI),                        # WidthTooSmall :234-241
        (1, s, 0, s, 5, 5, 1, 5, 5, 1, False, NP), (0, s, 1, s, 5, 5, 1, 5, 5, 1, False, NP),  # NullPointer
        (0, s, 0, s, MAX_PIXELS, MAX_PIXELS, 1, 5, 5, 1, False, RG),        # OversizeImage :251-274
        (0, s, 0, s, MAX_PIXELS + 1, MAX_PIXELS, 1, 5, 5, 1, False, RG),
        (0, s, 0, s, 10, MAX_PIXELS, 1, 5, 5, 1, False, RG),
        (0, s, 0, s, 1000, 1000, 1, 257, 257, 1, False, NI),                # UnsupportedFilterSizes
        (0, s, 0, s, 1000, 1000, 1, 100, 5, 1, False, NI), (0, s, 0, s, 1000, 1000, 1, 5, 100, 1, False, NI),
        (0, s, 0, s, 1000, 1000, 1, 1, 1, 1, False, NI), (0, s, 0, s, 1000, 1000, 1, 4, 4, 1, False, NI),
        (0, s, 0, s, 1000, 1000, 1, 9, 9, 5, False, NI),
        (0, s, 0, s, 1000, 1000, 1, 9, 9, 1, False, 0 if dtype == "u8" else NI),
        (0, s, 0, s, 10, 10, 1, 5, 5, 1, True, NI),                         # SrcDstChannelCombinations
        (0, s, 0, s, 10, 10, 4, 5, 5, 1, True, NI),
        (0, s, 0, s, 10, 10, 1, 5, 5, 1, False, 0), (0, s, 0, s, 10, 10, 4, 5, 5, 1, False, 0),
        (1, s, 1, s, 1000, 1000, 9, 4, 4, 6, True, NP),                     # pointers come first
    ]
    if es > 1:
        cases += [(0, s + 1, 0, s, 10, 10, 1, 5, 5, 1, False, AL), (0, s, 0, s + 1, 10, 10, 1, 5, 5, 1, False, AL),
                  (0, s + 1, 0, s, 10, 1, 1, 5, 5, 1, False, NI),           # single row: stride unchecked
                  (0, s + 1, 0, s, MAX_PIXELS + 1, 3, 1, 5, 5, 1, False, AL)]
    return cases


@pytest.mark.parametrize("dtype", DTYPES)
def test_oracle_error_codes(oracle, dtype):
    for sn, ss, dn, ds, w, h, c, kw, kh, b, same, want in median_cases(dtype):
        assert oracle.median_blur_check(dtype, sn, ss, dn, ds, w, h, c, kw, kh, b, same) == want, \
            (sn, ss, dn, ds, w, h, c, kw, kh, b, same)


@pytest.mark.parametrize("dtype", DTYPES)
def test_abi_validation_matches_oracle(kcv, oracle, dtype):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("validation parity runs where no GPU can pick the calls up")
    except ImportError:
        pass
    fn = getattr(kcv.lib(), f"kleidicv_gpu_median_blur_{dtype}")
    for sn, ss, dn, ds, w, h, c, kw, kh, b, same, want in median_cases(dtype):
        src = None if sn else 0x1000
        dst = None if dn else (0x1000 if same else 0x2000)
        got = fn(src, ss, dst, ds, w, h, c, kw, kh, b, None)
        assert got == (kcv.ERROR_NO_DEVICE if want == 0 else want), (sn, ss, dn, ds, w, h, c, kw, kh, b, same)
