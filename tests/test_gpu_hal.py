"""OpenCV custom-HAL shim on the GPU: cv::GaussianBlur / sepFilter2D / pyrDown /
Sobel hooks with host images (pageable numpy and pinned), device images and a
mix of the two must return CV_HAL_ERROR_OK with exactly the CPU oracle's
output, synchronously, leaving bytes outside the destination rows alone."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()
CV_8U, CV_16U, CV_16S = 0, 2, 3
REPLICATE, REFLECT, WRAP, REFLECT_101 = 1, 2, 3, 4
TO_KCV = {REPLICATE: kcv.REPLICATE, REFLECT: kcv.REFLECT, WRAP: kcv.WRAP, REFLECT_101: kcv.REVERSE}
MODES = ["host", "pinned", "device", "host_to_device"]


def cv_type(depth, cn):
    return depth + ((cn - 1) << 3)


class Buf:
    """A 2-D image (rows x bytes, padded) in the memory kind a test asks for."""

    def __init__(self, arr, kind):
        self.host = np.ascontiguousarray(arr)
        self.kind = kind
        raw = self.host.view(np.uint8)
        if kind == "host":
            self.ptr = self.host.ctypes.data
        elif kind == "pinned":
            self.t = torch.from_numpy(raw.copy()).pin_memory()
            self.ptr = self.t.data_ptr()
        else:
            self.t = torch.from_numpy(raw.copy()).cuda()
            self.ptr = self.t.data_ptr()

    def read(self):
        if self.kind == "host":
            return self.host
        return self.t.cpu().numpy().view(self.host.dtype)


def kinds(mode):
    return {"host": ("host", "host"), "pinned": ("pinned", "pinned"), "device": ("device", "device"),
            "host_to_device": ("host", "device")}[mode]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("case", [(640, 480, 3, 5, 0.0, REFLECT_101), (333, 101, 1, 7, 1.5, REPLICATE),
                                  (64, 64, 4, 15, 2.5, WRAP), (200, 90, 2, 31, 4.0, REPLICATE)])
def test_gaussian_hooks(mode, case):
    w, h, c, k, sigma, border = case
    rng = np.random.default_rng(w + k)
    pad = 7
    host = rng.integers(0, 256, (h, w * c + pad), dtype=np.uint8)
    sk, dk = kinds(mode)
    src = Buf(host, sk)
    dst = Buf(np.full((h, w * c + pad), 0xA5, np.uint8), dk)
    lib = kcv.lib()
    if sigma == 0.0:
        r = lib.kleidicv_gpu_hal_gaussian_blur_binomial(src.ptr, w * c + pad, dst.ptr, w * c + pad, w, h, CV_8U, c,
                                                        0, 0, 0, 0, k, border)
    else:
        r = lib.kleidicv_gpu_hal_gaussian_blur(src.ptr, w * c + pad, dst.ptr, w * c + pad, w, h, CV_8U, c, 0, 0, 0,
                                               0, k, k, sigma, sigma, border)
    assert r == 0
    got = dst.read()  # synchronous: no extra wait
    err, want = oracle.gaussian_blur_u8(host, w, h, c, k, np.float32(sigma), TO_KCV[border])
    assert err == 0
    assert np.array_equal(got[:, : w * c], want[:, : w * c])
    assert (got[:, w * c:] == 0xA5).all()


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("depth", [CV_8U, CV_16U])
def test_separable_hook(mode, depth):
    w, h, c = 501, 77, 3
    dt = np.uint8 if depth == CV_8U else np.uint16
    rng = np.random.default_rng(9 + depth)
    host = rng.integers(0, np.iinfo(dt).max + 1, (h, w * c), dtype=dt)
    kx = np.array([1, 2, 0, 3, 1], dt)
    ky = np.array([2, 1, 4, 0, 1], dt)
    sk, dk = kinds(mode)
    src = Buf(host, sk)
    dst = Buf(np.zeros((h, w * c), dt), dk)
    step = w * c * host.itemsize
    t = cv_type(depth, c)
    r = kcv.lib().kleidicv_gpu_hal_separable_filter_2d(src.ptr, step, t, dst.ptr, step, t, w, h, w, h, 0, 0,
                                                       kx.ctypes.data, 5, ky.ctypes.data, 5, depth, -1, 2, 0.0,
                                                       WRAP)
    assert r == 0
    err, want = oracle.separable_filter_2d(host, w, h, c, kx, ky, kcv.WRAP)
    assert err == 0
    assert np.array_equal(dst.read(), want)


@pytest.mark.parametrize("mode", MODES)
def test_pyrdown_hook(mode):
    w, h, c = 1023, 517, 4
    rng = np.random.default_rng(4)
    host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    dw, dh = (w + 1) // 2, (h + 1) // 2
    sk, dk = kinds(mode)
    src = Buf(host, sk)
    dst = Buf(np.zeros((dh, dw * c), np.uint8), dk)
    r = kcv.lib().kleidicv_gpu_hal_pyrdown(src.ptr, w * c, w, h, dst.ptr, dw * c, dw, dh, CV_8U, c, REFLECT_101)
    assert r == 0
    err, want = oracle.blur_and_downsample_u8(host, w, h, c, kcv.REVERSE)
    assert err == 0
    assert np.array_equal(dst.read(), want)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("dxdy", [(1, 0), (0, 1)])
def test_sobel_hook(mode, dxdy):
    w, h, c = 730, 411, 2
    rng = np.random.default_rng(11)
    host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    sk, dk = kinds(mode)
    src = Buf(host, sk)
    dst = Buf(np.zeros((h, w * c), np.int16), dk)
    r = kcv.lib().kleidicv_gpu_hal_sobel(src.ptr, w * c, dst.ptr, 2 * w * c, w, h, CV_8U, CV_16S, c, 0, 0, 0, 0,
                                         dxdy[0], dxdy[1], 3, 1.0, 0.0, REPLICATE)
    assert r == 0
    err, want = oracle.sobel_3x3_s16_u8(host, w, h, c, dxdy == (1, 0))
    assert err == 0
    assert np.array_equal(dst.read(), want)


def test_rejected_call_touches_nothing():
    host = np.zeros((16, 32), np.uint8)
    dst = np.full((16, 32), 7, np.uint8)
    r = kcv.lib().kleidicv_gpu_hal_gaussian_blur(host.ctypes.data, 32, dst.ctypes.data, 32, 32, 16, CV_8U, 1, 0, 0,
                                                 0, 0, 5, 5, 0.0, 0.0, 0)  # CONSTANT: not the reference's
    assert r == 1 and (dst == 7).all()
