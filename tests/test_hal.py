"""OpenCV custom-HAL shim without a GPU: every acceptance rule of KleidiCV's
OpenCV adapter (adapters/opencv/kleidicv_hal.cpp) answers
CV_HAL_ERROR_NOT_IMPLEMENTED before any CUDA call, the library's own
rejections map through the adapter's convert_error (:78-91), and a valid call
on a host without an sm_103 device fails with CV_HAL_ERROR_UNKNOWN (OpenCV
raises) instead of computing anything on the CPU."""
import numpy as np
import pytest

OK, NI, UNKNOWN = 0, 1, -1
CV_8U, CV_8S, CV_16U, CV_16S, CV_32F = 0, 1, 2, 3, 5
REPLICATE, REFLECT, WRAP, REFLECT_101, CONSTANT, TRANSPARENT, ISOLATED = 1, 2, 3, 4, 0, 5, 16
FAKE_SRC, FAKE_DST = 0x1000, 0x2000  # never dereferenced by a rejected call


def cv_type(depth, cn):
    return depth + ((cn - 1) << 3)


@pytest.fixture(scope="module")
def lib(kcv):
    return kcv.lib()


@pytest.fixture(scope="module")
def no_gpu():
    try:
        import torch

        return not torch.cuda.is_available()
    except ImportError:
        return True


def sep(lib, **kw):
    a = dict(src=FAKE_SRC, src_step=64, src_type=cv_type(CV_8U, 1), dst=FAKE_DST, dst_step=64,
             dst_type=cv_type(CV_8U, 1), w=32, h=16, fw=32, fh=16, ox=0, oy=0, kx=0x3000, kxl=5, ky=0x3000,
             kyl=5, ktype=CV_8U, ax=-1, ay=-1, delta=0.0, border=REFLECT)
    a.update(kw)
    return lib.kleidicv_gpu_hal_separable_filter_2d(
        a["src"], a["src_step"], a["src_type"], a["dst"], a["dst_step"], a["dst_type"], a["w"], a["h"], a["fw"],
        a["fh"], a["ox"], a["oy"], a["kx"], a["kxl"], a["ky"], a["kyl"], a["ktype"], a["ax"], a["ay"], a["delta"],
        a["border"])


def gauss(lib, **kw):
    a = dict(src=FAKE_SRC, src_step=64, dst=FAKE_DST, dst_step=64, w=32, h=16, depth=CV_8U, cn=1, ml=0, mt=0,
             mr=0, mb=0, kw=5, kh=5, sx=0.0, sy=0.0, border=REFLECT)
    a.update(kw)
    return lib.kleidicv_gpu_hal_gaussian_blur(a["src"], a["src_step"], a["dst"], a["dst_step"], a["w"], a["h"],
                                              a["depth"], a["cn"], a["ml"], a["mt"], a["mr"], a["mb"], a["kw"],
                                              a["kh"], a["sx"], a["sy"], a["border"])


def pyr(lib, **kw):
    a = dict(src=FAKE_SRC, src_step=64, sw=32, sh=16, dst=FAKE_DST, dst_step=64, dw=16, dh=8, depth=CV_8U, cn=1,
             border=REFLECT_101)
    a.update(kw)
    return lib.kleidicv_gpu_hal_pyrdown(a["src"], a["src_step"], a["sw"], a["sh"], a["dst"], a["dst_step"],
                                        a["dw"], a["dh"], a["depth"], a["cn"], a["border"])


def sobel(lib, **kw):
    a = dict(src=FAKE_SRC, src_step=64, dst=FAKE_DST, dst_step=128, w=32, h=16, sd=CV_8U, dd=CV_16S, cn=1,
             ml=0, mt=0, mr=0, mb=0, dx=1, dy=0, ksize=3, scale=1.0, delta=0.0, border=REPLICATE)
    a.update(kw)
    return lib.kleidicv_gpu_hal_sobel(a["src"], a["src_step"], a["dst"], a["dst_step"], a["w"], a["h"], a["sd"],
                                      a["dd"], a["cn"], a["ml"], a["mt"], a["mr"], a["mb"], a["dx"], a["dy"],
                                      a["ksize"], a["scale"], a["delta"], a["border"])


def test_separable_acceptance_rules(lib):
    # kleidicv_hal.cpp:459-515, one rule at a time.
    assert sep(lib, ox=1, fw=33) == NI and sep(lib, oy=1, fh=17) == NI
    assert sep(lib, fw=40) == NI and sep(lib, fh=20) == NI            # sub-matrix margins
    assert sep(lib, dst=FAKE_SRC) == NI                                # in place
    assert sep(lib, dst_type=cv_type(CV_8U, 3)) == NI                  # src type != dst type
    assert sep(lib, ktype=CV_16U) == NI                                # kernel depth != src depth
    assert sep(lib, ktype=cv_type(CV_8U, 2)) == NI                     # kernel with 2 channels
    for d in (CV_8S, CV_16S, CV_32F):
        assert sep(lib, src_type=d, dst_type=d, ktype=d) == NI         # only 8U / 16U
    for b in (CONSTANT, TRANSPARENT, ISOLATED, REFLECT | ISOLATED, 7):
        assert sep(lib, border=b) == NI                                # border subset
    assert sep(lib, ax=0) == NI and sep(lib, ay=4) == NI               # anchor off centre
    assert sep(lib, delta=0.5) == NI
    assert sep(lib, kxl=3, kyl=3) == NI                                # library: 5x5 only
    assert sep(lib, src_type=CV_16U, dst_type=CV_16U, ktype=CV_16U, src_step=63) == NI  # ALIGNMENT
    assert sep(lib, src=0) == UNKNOWN                                  # NULL_POINTER
    assert sep(lib, kx=0) == UNKNOWN


def test_gaussian_acceptance_rules(lib):
    assert gauss(lib, dst=FAKE_SRC) == NI
    for m in ("ml", "mt", "mr", "mb"):
        assert gauss(lib, **{m: 1}) == NI
    assert gauss(lib, depth=CV_16U) == NI
    for b in (CONSTANT, TRANSPARENT, ISOLATED, REPLICATE | ISOLATED):
        assert gauss(lib, border=b) == NI
    assert gauss(lib, kw=4, kh=4) == NI and gauss(lib, kw=5, kh=7) == NI
    assert gauss(lib, sx=1.0, sy=2.0) == NI and gauss(lib, cn=5) == NI
    assert gauss(lib, src=0) == UNKNOWN
    assert lib.kleidicv_gpu_hal_gaussian_blur_binomial(FAKE_SRC, 64, FAKE_SRC, 64, 32, 16, CV_8U, 1, 0, 0, 0, 0, 5,
                                                       REFLECT) == NI


def test_pyrdown_and_sobel_acceptance_rules(lib):
    assert pyr(lib, dst=FAKE_SRC) == NI and pyr(lib, depth=CV_16U) == NI
    assert pyr(lib, dw=15) == NI and pyr(lib, dh=9) == NI
    assert pyr(lib, border=CONSTANT) == NI and pyr(lib, border=REFLECT_101 | ISOLATED) == NI
    assert pyr(lib, sw=3, dw=2) == NI  # library: width >= 4
    assert sobel(lib, dst=FAKE_SRC) == NI and sobel(lib, sd=CV_16U) == NI and sobel(lib, dd=CV_16U) == NI
    assert sobel(lib, ksize=5) == NI and sobel(lib, w=2) == NI and sobel(lib, h=2) == NI
    assert sobel(lib, scale=2.0) == NI and sobel(lib, delta=1.0) == NI
    assert sobel(lib, border=REFLECT) == NI and sobel(lib, mb=1) == NI
    assert sobel(lib, dx=1, dy=1) == NI and sobel(lib, dx=2, dy=0) == NI
    assert sobel(lib, dst_step=127) == NI  # ALIGNMENT of the s16 destination


def test_valid_calls_fail_loudly_without_a_gpu(lib, no_gpu):
    if not no_gpu:
        pytest.skip("checks the behaviour on a host without a GPU")
    src = np.arange(32 * 16, dtype=np.uint8).reshape(16, 32)
    dst = np.zeros_like(src)
    dst16 = np.zeros((16, 32), np.int16)
    taps = np.array([1, 2, 3, 2, 1], np.uint8)
    assert gauss(lib, src=src.ctypes.data, dst=dst.ctypes.data) == UNKNOWN
    assert sep(lib, src=src.ctypes.data, dst=dst.ctypes.data, kx=taps.ctypes.data, ky=taps.ctypes.data) == UNKNOWN
    assert pyr(lib, src=src.ctypes.data, src_step=32, dst=dst.ctypes.data, dst_step=32) == UNKNOWN
    assert sobel(lib, src=src.ctypes.data, src_step=32, dst=dst16.ctypes.data, dst_step=64) == UNKNOWN
    assert not dst.any() and not dst16.any()
