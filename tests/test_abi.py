"""The C ABI without a GPU: the library loads, exports every function that
include/kleidicv_gpu.h declares (with the binding's argument table), rejects
invalid calls with the reference's error codes in the reference's order of
checks (the oracle restates that order), and fails loudly with
KLEIDICV_GPU_ERROR_NO_DEVICE, instead of computing anything on the CPU, when
a valid call finds no sm_103 device."""
import ctypes
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "kleidicv_gpu.h")


HAL_HEADER = os.path.join(REPO, "include", "kleidicv_gpu_hal.h")
THREAD_HEADER = os.path.join(REPO, "include", "kleidicv_gpu_thread.h")


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(kleidicv_gpu_\w+)\s*\(", text))
    # The HAL header's exported shim functions (its inline OpenCV wiring is not exported).
    hal = re.sub(r"/\*.*?\*/", "", open(HAL_HEADER).read(), flags=re.S)
    names |= set(re.findall(r"\b(kleidicv_gpu_hal_\w+)\s*\(", hal))
    thr = re.sub(r"/\*.*?\*/", "", open(THREAD_HEADER).read(), flags=re.S)
    names |= set(re.findall(r"\b(kleidicv_gpu_thread_\w+)\s*\(", thr))
    return sorted(names)


@pytest.fixture(scope="module")
def lib(kcv):
    if not os.path.exists(kcv.LIB_PATH):
        kcv.build()
    return kcv.lib()


@pytest.fixture(scope="module")
def no_gpu():
    try:
        import torch

        return not torch.cuda.is_available()
    except ImportError:
        return True


def test_header_declares_functions():
    names = _declared_functions()
    assert "kleidicv_gpu_gaussian_blur_u8" in names and len(names) >= 30


def test_every_declared_function_is_exported_and_bound(lib, kcv):
    for name in _declared_functions():
        assert hasattr(lib, name), f"{name} declared in the header but not exported"
        assert name in kcv.SIGNATURES, f"{name} has no entry in the binding's argument table"


def test_half_kernel_matches_reference_generator(kcv):
    """The library's weight generator (host side of every Gaussian call)
    against the reference's own generator outputs (golden subset)."""
    import json

    golden = json.load(open(os.path.join(REPO, "tests", "golden", "sigma.json")))["subset"]
    for key, want in golden.items():
        k, i = map(int, key.split(":"))
        got = kcv.half_kernel(k, float(np.float32(i) / np.float32(100)))
        assert got == want, (key, got, want)
    assert len(golden) > 100


# --- validation parity ------------------------------------------------------

FAKE = 0x1000  # never dereferenced: the calls below fail validation or find no device


def _buffers(w, h, c, es, fake=False):
    if fake or w * h * max(c, 1) > (1 << 20):
        return FAKE, max(w * max(c, 1) * es, 1), None
    a = np.zeros((max(h, 1), max(w * max(c, 1), 1) * es), np.uint8)
    return a.ctypes.data, a.strides[0], a


def _gauss_cases():
    rng = np.random.default_rng(3)
    cases = []
    for k in (1, 2, 3, 4, 5, 7, 9, 11, 13, 15, 21, 23, 255, 257):
        for border in range(7):
            for (w, h) in ((64, 48), (k - 2 if k > 2 else 1, 40), (40, k - 2 if k > 2 else 1), (9, 9)):
                c = int(rng.integers(0, 6))
                cases.append(dict(w=max(w, 0), h=max(h, 0), c=c, kw=k, kh=k, sx=0.0, sy=0.0, border=border))
    cases += [dict(w=64, h=64, c=1, kw=5, kh=7, sx=0.0, sy=0.0, border=2),
              dict(w=64, h=64, c=1, kw=5, kh=5, sx=1.0, sy=2.0, border=2),
              dict(w=64, h=64, c=1, kw=5, kh=5, sx=1.0, sy=1.0, border=2, src_null=True),
              dict(w=64, h=64, c=1, kw=5, kh=5, sx=1.0, sy=1.0, border=2, dst_null=True),
              dict(w=1 << 30, h=1 << 30, c=1, kw=5, kh=5, sx=0.0, sy=0.0, border=2, fake=True),
              dict(w=20, h=64, c=1, kw=15, kh=15, sx=0.0, sy=0.0, border=1),
              dict(w=20, h=64, c=1, kw=13, kh=13, sx=0.0, sy=0.0, border=1),
              dict(w=13, h=64, c=1, kw=13, kh=13, sx=0.0, sy=0.0, border=1)]
    return cases


def _expect(oracle_code, kcv, no_gpu, lib_code):
    if oracle_code != 0:
        assert lib_code == oracle_code
    elif no_gpu:
        assert lib_code in (0, kcv.ERROR_NO_DEVICE)


@pytest.mark.parametrize("ext", [False, True])
def test_gaussian_validation_matches_oracle(lib, kcv, oracle, no_gpu, ext):
    if not no_gpu:
        pytest.skip("validation parity runs where no GPU can pick the calls up")
    n = 0
    for cs in _gauss_cases():
        fake = cs.get("fake", False)
        sp, ss, sa = _buffers(cs["w"], cs["h"], cs["c"], 1, fake)
        dp, ds, da = _buffers(cs["w"], cs["h"], cs["c"], 1, fake)
        if cs.get("src_null"):
            sp = None
        if cs.get("dst_null"):
            dp = None
        if ext:
            got = lib.kleidicv_gpu_gaussian_blur_u8_ex(sp, ss, dp, ds, cs["w"], cs["h"], cs["c"], cs["kw"], cs["kh"],
                                                       cs["sx"], cs["sy"], cs["border"], 17, None)
        else:
            got = lib.kleidicv_gpu_gaussian_blur_u8(sp, ss, dp, ds, cs["w"], cs["h"], cs["c"], cs["kw"], cs["kh"],
                                                    cs["sx"], cs["sy"], cs["border"], None)
        ref = oracle.lib().ko_gaussian_blur_u8(sp, ss, dp, ds, cs["w"], cs["h"], cs["c"], cs["kw"], cs["kh"],
                                               cs["sx"], cs["sy"], cs["border"], int(ext), 17, 1)
        _expect(ref, kcv, no_gpu, got)
        n += 1
    assert n > 200


@pytest.mark.parametrize("dtype", ["u8", "u16"])
def test_separable_validation_matches_oracle(lib, kcv, oracle, no_gpu, dtype):
    if not no_gpu:
        pytest.skip("validation parity runs where no GPU can pick the calls up")
    es = 1 if dtype == "u8" else 2
    ct = ctypes.c_uint8 if dtype == "u8" else ctypes.c_uint16
    fn = getattr(lib, f"kleidicv_gpu_separable_filter_2d_{dtype}")
    ofn = getattr(oracle.lib(), f"ko_separable_filter_2d_{dtype}")
    taps = (ct * 7)(*([1] * 7))
    tp = ctypes.cast(taps, ctypes.c_void_p).value
    n = 0
    for kw in (3, 5, 7):
        for kh in (3, 5):
            for border in range(7):
                for (w, h, c) in ((32, 16, 1), (3, 16, 2), (32, 3, 3), (32, 16, 5), (32, 16, 0)):
                    for odd_stride in (False, True):
                        for null in (None, "src", "dst", "kx", "ky"):
                            sp, ss, sa = _buffers(w, h, c, es)
                            dp, ds, da = _buffers(w, h, c, es)
                            if odd_stride and es == 2:
                                ss += 1
                            kx = ky = tp
                            if null == "src":
                                sp = None
                            if null == "dst":
                                dp = None
                            if null == "kx":
                                kx = None
                            if null == "ky":
                                ky = None
                            got = fn(sp, ss, dp, ds, w, h, c, kx, kw, ky, kh, border, None)
                            # Safe on the host: the oracle reads through the pointers only
                            # after every check passed, and then they are real buffers.
                            ref = ofn(sp, ss, dp, ds, w, h, c, kx, kw, ky, kh, border, 0, 0, 1)
                            _expect(ref, kcv, no_gpu, got)
                            n += 1
    assert n > 500


def test_blur_and_downsample_validation_matches_oracle(lib, kcv, oracle, no_gpu):
    if not no_gpu:
        pytest.skip("validation parity runs where no GPU can pick the calls up")
    n = 0
    for (w, h, c) in ((16, 16, 1), (3, 16, 1), (16, 3, 2), (16, 16, 0), (16, 16, 5), (4, 4, 4), (1 << 30, 1 << 30, 1)):
        fake = w * h > (1 << 20)
        for border in range(7):
            for null in (None, "src", "dst"):
                sp, ss, sa = _buffers(w, h, c, 1, fake)
                dp, ds, da = _buffers((w + 1) // 2, (h + 1) // 2, c, 1, fake)
                if null == "src":
                    sp = None
                if null == "dst":
                    dp = None
                got = lib.kleidicv_gpu_blur_and_downsample_u8(sp, ss, w, h, dp, ds, c, border, None)
                ref = oracle.lib().ko_blur_and_downsample_u8(sp, ss, w, h, dp, ds, c, border, 0, 0, 1)
                _expect(ref, kcv, no_gpu, got)
                n += 1
    assert n > 100


def test_no_cpu_fallback(lib, kcv, no_gpu):
    if not no_gpu:
        pytest.skip("checks the behaviour on a host without a GPU")
    a = np.zeros((64, 64), np.uint8)
    b = np.zeros((64, 64), np.uint8)
    got = lib.kleidicv_gpu_gaussian_blur_u8(a.ctypes.data, 64, b.ctypes.data, 64, 64, 64, 1, 5, 5, 0.0, 0.0, 1, None)
    assert got == kcv.ERROR_NO_DEVICE
    assert not b.any()  # nothing was computed on the host
    h = ctypes.c_void_p()
    assert lib.kleidicv_gpu_context_create(ctypes.byref(h), 0, None, 0) == kcv.ERROR_NO_DEVICE
    cfg = kcv.ServerConfig(0, 0, 0, 0)
    assert lib.kleidicv_gpu_server_create(ctypes.byref(cfg), 0, ctypes.byref(h)) == kcv.ERROR_NO_DEVICE
    st = (ctypes.c_int * 1)()
    assert lib.kleidicv_gpu_batch_plan_create(None, 0, st, ctypes.byref(h), None) == kcv.ERROR_NO_DEVICE
    got = lib.kleidicv_gpu_gaussian_blur_u8_noalloc(a.ctypes.data, 64, b.ctypes.data, 64, 64, 64, 1, 31, 31, 0.0,
                                                    0.0, 1, None)
    assert got == kcv.ERROR_NO_DEVICE


def test_rows_beyond_32_bit_device_indexing_are_refused(lib, kcv):
    """Valid for the reference (< 2^48 pixels) but rows over 2^30 bytes or more
    than 2^30 rows: RANGE before any device work (no pointer is dereferenced)."""
    big, tall = (1 << 30) + 16, (1 << 30) + 1
    taps8 = (ctypes.c_uint8 * 5)(1, 1, 1, 1, 1)
    taps16 = (ctypes.c_uint16 * 5)(1, 1, 1, 1, 1)
    assert lib.kleidicv_gpu_gaussian_blur_u8(FAKE, big, FAKE, big, big, 8, 1, 5, 5, 0.0, 0.0, 1, None) == kcv.RANGE
    assert lib.kleidicv_gpu_gaussian_blur_u8(FAKE, 64, FAKE, 64, 64, tall, 1, 5, 5, 0.0, 0.0, 1, None) == kcv.RANGE
    assert lib.kleidicv_gpu_separable_filter_2d_u8(FAKE, big, FAKE, big, big, 8, 1, taps8, 5, taps8, 5, 2,
                                                   None) == kcv.RANGE
    assert lib.kleidicv_gpu_separable_filter_2d_u16(FAKE, 2 * big, FAKE, 2 * big, big // 2 + 8, 8, 1, taps16, 5,
                                                    taps16, 5, 2, None) == kcv.RANGE
    assert lib.kleidicv_gpu_blur_and_downsample_u8(FAKE, big, big, 8, FAKE, big, 1, 2, None) == kcv.RANGE
    assert lib.kleidicv_gpu_sobel_3x3_horizontal_s16_u8(FAKE, big, FAKE, 2 * big, big // 2 + 8, 8, 1,
                                                        None) == kcv.RANGE
    assert lib.kleidicv_gpu_median_blur_u8(FAKE, big, FAKE + 16, big, big, 8, 1, 3, 3, 1, None) == kcv.RANGE


def test_sme_twins_validate_like_their_base_entries(lib, kcv, no_gpu):
    """The `_sme` twins (kleidicv.h:2010, 2054, 2097, 2109, 2165, 2220) return
    exactly what their base entries return for calls that fail validation
    (null pointers, unsupported sizes, borders and channel counts, sizes out
    of range); validation runs before any device work."""
    if not no_gpu:
        pytest.skip("runs where no GPU can pick the calls up (the GPU twin tests cover the rest)")
    t8 = (ctypes.c_uint8 * 5)(1, 2, 3, 2, 1)
    t16 = (ctypes.c_uint16 * 5)(1, 2, 3, 2, 1)
    big = 1 << 30
    cases = {
        "kleidicv_gpu_gaussian_blur_u8": [
            (None, 64, FAKE, 64, 64, 8, 1, 5, 5, 0.0, 0.0, 2, None),
            (FAKE, 64, FAKE, 64, 64, 8, 1, 4, 4, 0.0, 0.0, 2, None),
            (FAKE, 64, FAKE, 64, 64, 8, 1, 5, 5, 0.0, 0.0, 0, None),
            (FAKE, 64, FAKE, 64, 64, 8, 5, 5, 5, 0.0, 0.0, 2, None),
            (FAKE, big, FAKE, big, big, big, 1, 5, 5, 0.0, 0.0, 2, None),
        ],
        "kleidicv_gpu_separable_filter_2d_u8": [
            (None, 64, FAKE, 64, 64, 8, 1, t8, 5, t8, 5, 2, None),
            (FAKE, 64, FAKE, 64, 64, 8, 1, t8, 3, t8, 3, 2, None),
            (FAKE, 64, FAKE, 64, 64, 8, 1, None, 5, t8, 5, 2, None),
            (FAKE, 64, FAKE, 64, 64, 8, 1, t8, 5, t8, 5, 0, None),
        ],
        "kleidicv_gpu_separable_filter_2d_u16": [
            (None, 128, FAKE, 128, 64, 8, 1, t16, 5, t16, 5, 2, None),
            (FAKE, 128, FAKE, 128, 64, 8, 1, t16, 5, None, 5, 2, None),
            (FAKE, 128, FAKE, 128, 64, 8, 5, t16, 5, t16, 5, 2, None),
        ],
        "kleidicv_gpu_blur_and_downsample_u8": [
            (FAKE, 64, 64, 8, None, 32, 1, 2, None),
            (FAKE, 64, 64, 8, FAKE, 32, 5, 2, None),
            (FAKE, 64, 64, 8, FAKE, 32, 1, 0, None),
        ],
        "kleidicv_gpu_sobel_3x3_horizontal_s16_u8": [
            (None, 64, FAKE, 128, 64, 8, 1, None),
            (FAKE, 64, FAKE, 128, 64, 8, 5, None),
        ],
        "kleidicv_gpu_sobel_3x3_vertical_s16_u8": [
            (FAKE, 64, None, 128, 64, 8, 1, None),
            (FAKE, 64, FAKE, 128, 64, 8, 5, None),
        ],
    }
    n = 0
    for name, calls in cases.items():
        base, twin = getattr(lib, name), getattr(lib, name + "_sme")
        for args in calls:
            want = base(*args)
            assert want not in (kcv.OK, kcv.ERROR_NO_DEVICE), (name, args, want)
            assert twin(*args) == want, (name, args)
            n += 1
    assert n == 19
