"""Sobel 3x3 (u8 -> s16) without a GPU: the oracle against the reference's own
tests (kleidicv test/api/test_sobel.cpp) -- the two masks applied as a 2-D
correlation with a replicated border (:87-112), the 2x2 valid-size case
(:178-195) and every error-code case (:120-290) -- and the C ABI's validation
against the oracle's order of checks."""
import ctypes

import numpy as np
import pytest

# The masks of test_sobel.cpp:91-93 and :108-110 (weights as applied).
MASK_X = np.array([[-1, 0, 1], [-2, 0, 2], [-1, 0, 1]])
MASK_Y = np.array([[-1, -2, -1], [0, 0, 0], [1, 2, 1]])
MAX_PIXELS = (1 << 48) - 1  # KLEIDICV_MAX_IMAGE_PIXELS


def mask_correlation(img, w, h, c, mask):
    a = img[:h, : w * c].reshape(h, w, c).astype(np.int64)
    p = np.pad(a, ((1, 1), (1, 1), (0, 0)), mode="edge")
    out = np.zeros((h, w, c), np.int64)
    for dy in range(3):
        for dx in range(3):
            out += mask[dy, dx] * p[dy:dy + h, dx:dx + w, :]
    return out.reshape(h, w * c).astype(np.int16)


@pytest.mark.parametrize("horizontal", [True, False])
@pytest.mark.parametrize("shape", [(2, 2, 1), (3, 5, 2), (17, 9, 3), (64, 33, 4), (5, 2, 1), (2, 7, 4),
                                   (131, 3, 1)])
def test_oracle_equals_mask(oracle, horizontal, shape):
    w, h, c = shape
    rng = np.random.default_rng(w * 31 + h)
    for extreme in (False, True):
        img = rng.integers(0, 256, (h, w * c + 3), dtype=np.uint8)
        if extreme:  # the largest magnitudes: a 0 -> 255 step across the derivative's axis
            axis, split = (1, (w // 2) * c) if horizontal else (0, h // 2)
            img = ((np.indices(img.shape)[axis] >= split) * 255).astype(np.uint8)
        err, got = oracle.sobel_3x3_s16_u8(img, w, h, c, horizontal)
        assert err == 0
        want = mask_correlation(img, w, h, c, MASK_X if horizontal else MASK_Y)
        assert np.array_equal(got[:, : w * c], want)
    if w > 3 and h > 3:
        assert np.abs(want).max() == 1020  # the stripes reach the extreme


def test_oracle_valid_image_size_case(oracle):
    src = np.array([[1, 2], [1, 2]], np.uint8)  # test_sobel.cpp:182-185
    err, gx = oracle.sobel_3x3_s16_u8(src, 2, 2, 1, True)
    assert err == 0 and gx.tolist() == [[4, 4], [4, 4]]
    err, gy = oracle.sobel_3x3_s16_u8(src, 2, 2, 1, False)
    assert err == 0 and gy.tolist() == [[0, 0], [0, 0]]


def _sobel_cases():
    """(src?, src_stride, dst?, dst_stride, w, h, c, expected) from
    test_sobel.cpp, plus the combinations that pin the order of checks."""
    NI, NP, AL, RG = 1, 2, 5, 3
    return [
        (1, 1, 1, 2, 0, 1, 1, NI), (1, 1, 1, 2, 1, 0, 1, NI),      # ZeroImageSize :152-176
        (1, 1, 1, 2, 1, 1, 1, NI), (1, 1, 1, 2, 1, 8, 1, NI),      # UndersizeImage :197-223
        (1, 1, 1, 2, 13, 1, 1, NI),
        (1, 2, 1, 5, 3, 3, 1, AL),                                  # Misalignment :120-150
        (1, 3, 1, 4, 3, 3, 1, 0),                                   # u8 source: any stride
        (1, 1, 1, 2, MAX_PIXELS + 1, 3, 1, RG),                     # OversizeImage :248-274
        (1, 1, 1, 2, MAX_PIXELS, MAX_PIXELS, 1, RG),
        (1, 1, 1, 2, 2, 2, 5, NI),                                  # ChannelNumber :276-290
        (0, 1, 1, 2, 3, 3, 1, NP), (1, 1, 0, 2, 3, 3, 1, NP),      # test_null_args :98-100
        (0, 1, 1, 2, 1, 1, 1, NI),                                  # size check comes first
        (0, 1, 0, 3, 3, 3, 9, NP), (1, 1, 0, 3, 3, 3, 9, NP),      # null before alignment
        (1, 1, 1, 3, 3, 3, 9, AL), (1, 1, 1, 3, 3, 1, 9, NI),      # height 1 fails the size check
        (1, 1, 1, 3, MAX_PIXELS + 1, 3, 9, AL),                     # alignment before range
        (1, 1, 1, 2, MAX_PIXELS + 1, 3, 9, RG),                     # range before channels
        (1, 1, 1, 2, 2, 2, 0, 0),                                   # no channels: nothing to do
    ]


@pytest.mark.parametrize("horizontal", [True, False])
def test_oracle_error_codes(oracle, horizontal):
    fn = oracle.lib().ko_sobel_3x3_horizontal_s16_u8 if horizontal else oracle.lib().ko_sobel_3x3_vertical_s16_u8
    src = np.zeros(64, np.uint8)
    dst = np.zeros(64, np.int16)
    for sp, ss, dp, ds, w, h, c, want in _sobel_cases():
        # Buffers hold every accepted call's few pixels (w, h <= 3, c <= 9 when OK).
        got = fn(src.ctypes.data if sp else None, ss, dst.ctypes.data if dp else None, ds, w, h, c, 1)
        assert got == want, (sp, ss, dp, ds, w, h, c, got, want)


@pytest.mark.parametrize("horizontal", [True, False])
def test_abi_validation_matches_oracle(kcv, oracle, horizontal):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("validation parity runs where no GPU can pick the calls up")
    except ImportError:
        pass
    lib = kcv.lib()
    name = "sobel_3x3_horizontal_s16_u8" if horizontal else "sobel_3x3_vertical_s16_u8"
    fn = getattr(lib, "kleidicv_gpu_" + name)
    ofn = getattr(oracle.lib(), "ko_" + name)
    FAKE = 0x1000  # never dereferenced: every call fails validation or finds no device
    for sp, ss, dp, ds, w, h, c, want in _sobel_cases():
        src = FAKE if sp else None
        dst = FAKE if dp else None
        got = fn(src, ss, dst, ds, w, h, c, None)
        if want != 0:
            assert got == want, (sp, ss, dp, ds, w, h, c, got)
            assert ofn(src, ss, dst, ds, w, h, c, 1) == want
        elif c == 0:
            assert got == 0  # nothing to enqueue
        else:
            assert got == kcv.ERROR_NO_DEVICE
