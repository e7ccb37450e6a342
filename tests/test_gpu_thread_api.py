"""Threaded-API entries on the GPU: host images (pageable and pinned), device
images and mixes, with the library's worker pool and with a serial scheduler
written in Python, must give exactly the oracle's output; a scheduler that
fails makes the call fail, and the next call is unaffected."""
import ctypes
import threading

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()
LIB = kcv.lib()
POOL = None


def setup_module():
    global POOL
    POOL = kcv.ThreadPool(8)


def teardown_module():
    POOL.close()


class Img:
    def __init__(self, arr, kind):
        self.host = np.ascontiguousarray(arr)
        self.kind = kind
        raw = self.host.view(np.uint8)
        if kind == "host":
            self.ptr = self.host.ctypes.data
        else:
            self.t = torch.from_numpy(raw.copy())
            self.t = self.t.pin_memory() if kind == "pinned" else self.t.cuda()
            self.ptr = self.t.data_ptr()

    def read(self):
        if self.kind == "host":
            return self.host
        return self.t.cpu().numpy().view(self.host.dtype)


COMBOS = [("host", "host"), ("pinned", "pinned"), ("device", "host"), ("host", "device"), ("pinned", "host")]


def schedulers():
    mt, keep = kcv.serial_scheduler()
    return {"pool": (POOL.mt, None), "serial": (mt, keep)}


@pytest.mark.parametrize("combo", COMBOS, ids=lambda c: f"{c[0]}-{c[1]}")
@pytest.mark.parametrize("sched", ["pool", "serial"])
def test_gaussian_threaded(combo, sched):
    w, h, c = 3840, 2160, 4
    rng = np.random.default_rng(1)
    host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    src, dst = Img(host, combo[0]), Img(np.zeros_like(host), combo[1])
    mt, keep = schedulers()[sched]
    e = LIB.kleidicv_gpu_thread_gaussian_blur_u8(src.ptr, w * c, dst.ptr, w * c, w, h, c, 7, 7, 1.5, 1.5,
                                                 kcv.REVERSE, mt)
    assert e == kcv.OK
    err, want = oracle.gaussian_blur_u8(host, w, h, c, 7, np.float32(1.5), kcv.REVERSE, nthreads=8)
    assert np.array_equal(dst.read(), want)


@pytest.mark.parametrize("combo", COMBOS, ids=lambda c: f"{c[0]}-{c[1]}")
def test_other_ops_threaded(combo):
    rng = np.random.default_rng(2)
    w, h, c = 1001, 333, 3
    h8 = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    h16 = rng.integers(0, 65536, (h, w), dtype=np.uint16)
    # separable u16 (1 channel)
    kx = np.array([1, 2, 3, 2, 1], np.uint16)
    ky = np.array([0, 1, 4, 1, 0], np.uint16)
    src, dst = Img(h16, combo[0]), Img(np.zeros_like(h16), combo[1])
    assert LIB.kleidicv_gpu_thread_separable_filter_2d_u16(src.ptr, 2 * w, dst.ptr, 2 * w, w, h, 1, kx.ctypes.data,
                                                           5, ky.ctypes.data, 5, kcv.WRAP, POOL.mt) == kcv.OK
    assert np.array_equal(dst.read(), oracle.separable_filter_2d(h16, w, h, 1, kx, ky, kcv.WRAP)[1])
    # separable u8
    k8 = np.array([1, 1, 2, 1, 1], np.uint8)
    src, dst = Img(h8, combo[0]), Img(np.zeros_like(h8), combo[1])
    assert LIB.kleidicv_gpu_thread_separable_filter_2d_u8(src.ptr, w * c, dst.ptr, w * c, w, h, c, k8.ctypes.data,
                                                          5, k8.ctypes.data, 5, kcv.REFLECT, POOL.mt) == kcv.OK
    assert np.array_equal(dst.read(), oracle.separable_filter_2d(h8, w, h, c, k8, k8, kcv.REFLECT)[1])
    # blur and downsample
    dw, dh = (w + 1) // 2, (h + 1) // 2
    src, dst = Img(h8, combo[0]), Img(np.zeros((dh, dw * c), np.uint8), combo[1])
    assert LIB.kleidicv_gpu_thread_blur_and_downsample_u8(src.ptr, w * c, w, h, dst.ptr, dw * c, c, kcv.REVERSE,
                                                          POOL.mt) == kcv.OK
    assert np.array_equal(dst.read(), oracle.blur_and_downsample_u8(h8, w, h, c, kcv.REVERSE)[1])
    # sobel x and y
    for horizontal, fn in ((True, LIB.kleidicv_gpu_thread_sobel_3x3_horizontal_s16_u8),
                           (False, LIB.kleidicv_gpu_thread_sobel_3x3_vertical_s16_u8)):
        src, dst = Img(h8, combo[0]), Img(np.zeros((h, w * c), np.int16), combo[1])
        assert fn(src.ptr, w * c, dst.ptr, 2 * w * c, w, h, c, POOL.mt) == kcv.OK
        assert np.array_equal(dst.read(), oracle.sobel_3x3_s16_u8(h8, w, h, c, horizontal)[1])


def test_failing_scheduler_fails_the_call():
    @kcv.THREAD_PARALLEL
    def refuses(callback, callback_data, parallel_data, task_count):
        return 4  # ALLOCATION: the scheduler could not run the tasks

    mt = kcv.ThreadMT(ctypes.cast(refuses, ctypes.c_void_p).value, None)
    host = np.random.default_rng(3).integers(0, 256, (200, 300), dtype=np.uint8)
    dst = np.zeros_like(host)
    assert LIB.kleidicv_gpu_thread_gaussian_blur_u8(host.ctypes.data, 300, dst.ctypes.data, 300, 300, 200, 1, 5, 5,
                                                    0.0, 0.0, kcv.REFLECT, mt) == kcv.ALLOCATION
    assert LIB.kleidicv_gpu_thread_gaussian_blur_u8(host.ctypes.data, 300, dst.ctypes.data, 300, 300, 200, 1, 5, 5,
                                                    0.0, 0.0, kcv.REFLECT, POOL.mt) == kcv.OK
    assert np.array_equal(dst, oracle.gaussian_blur_u8(host, 300, 200, 1, 5, 0.0, kcv.REFLECT)[1])


@pytest.mark.parametrize("combo", COMBOS, ids=lambda c: f"{c[0]}-{c[1]}")
@pytest.mark.parametrize("dtype,k", [("u8", 5), ("f32", 3), ("s16", 7), ("u8", 15)])
def test_median_threaded(combo, dtype, k):
    rng = np.random.default_rng(k)
    w, h, c = 301, 97, 2
    dt = oracle.MEDIAN_DTYPES[dtype]
    if np.dtype(dt).kind == "f":
        host = rng.uniform(-100, 100, (h, w * c)).astype(dt)
    else:
        info = np.iinfo(dt)
        host = rng.integers(info.min, int(info.max) + 1, (h, w * c), dtype=dt)
    src, dst = Img(host, combo[0]), Img(np.zeros_like(host), combo[1])
    fn = getattr(LIB, f"kleidicv_gpu_thread_median_blur_{dtype}")
    stride = w * c * host.itemsize
    assert fn(src.ptr, stride, dst.ptr, stride, w, h, c, k, k, kcv.REFLECT, POOL.mt) == kcv.OK
    assert np.array_equal(dst.read(), oracle.median_blur(host, w, h, c, k, kcv.REFLECT))


# ---------------------------------------------------------------------------
# Asynchronous variants: same results; the call returns before completion.

@pytest.mark.parametrize("combo", COMBOS, ids=lambda c: f"{c[0]}-{c[1]}")
@pytest.mark.parametrize("sched", ["pool", "serial"])
def test_async_calls_in_flight_together(combo, sched):
    """Four calls of different operations are submitted back to back, then
    waited on; each result equals the oracle's, every callback runs exactly
    once with OK, in submission order."""
    rng = np.random.default_rng(11)
    w, h, c = 1203, 611, 4
    h8 = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    h16 = rng.integers(0, 65536, (h, w), dtype=np.uint16)
    kx = np.array([1, 2, 3, 2, 1], np.uint16)
    ky = np.array([0, 1, 4, 1, 0], np.uint16)
    k8 = np.array([1, 1, 2, 1, 1], np.uint8)
    dw, dh = (w + 1) // 2, (h + 1) // 2
    mt, keep = schedulers()[sched]
    order = []

    @kcv.ASYNC_CALLBACK
    def done(status, user):
        order.append((int(user or 0), status))

    cb = ctypes.cast(done, ctypes.c_void_p)
    jobs = []
    s1, d1 = Img(h8, combo[0]), Img(np.zeros_like(h8), combo[1])
    s2, d2 = Img(h16, combo[0]), Img(np.zeros_like(h16), combo[1])
    s3, d3 = Img(h8, combo[0]), Img(np.zeros_like(h8), combo[1])
    s4, d4 = Img(h8, combo[0]), Img(np.zeros((dh, dw * c), np.uint8), combo[1])
    hs = [ctypes.c_void_p() for _ in range(4)]
    assert LIB.kleidicv_gpu_thread_gaussian_blur_u8_async(s1.ptr, w * c, d1.ptr, w * c, w, h, c, 7, 7, 1.5, 1.5,
                                                          kcv.REVERSE, mt, cb, 1, ctypes.byref(hs[0])) == kcv.OK
    assert LIB.kleidicv_gpu_thread_separable_filter_2d_u16_async(s2.ptr, 2 * w, d2.ptr, 2 * w, w, h, 1,
                                                                 kx.ctypes.data, 5, ky.ctypes.data, 5, kcv.WRAP,
                                                                 mt, cb, 2, ctypes.byref(hs[1])) == kcv.OK
    assert LIB.kleidicv_gpu_thread_separable_filter_2d_u8_async(s3.ptr, w * c, d3.ptr, w * c, w, h, c,
                                                                k8.ctypes.data, 5, k8.ctypes.data, 5, kcv.REFLECT,
                                                                mt, cb, 3, ctypes.byref(hs[2])) == kcv.OK
    assert LIB.kleidicv_gpu_thread_blur_and_downsample_u8_async(s4.ptr, w * c, w, h, d4.ptr, dw * c, c,
                                                                kcv.REVERSE, mt, cb, 4, ctypes.byref(hs[3])) == kcv.OK
    for hd in hs:
        assert hd.value
        assert LIB.kleidicv_gpu_async_wait(hd) == kcv.OK
        assert LIB.kleidicv_gpu_async_query(hd) == kcv.OK
    assert order == [(1, 0), (2, 0), (3, 0), (4, 0)]
    assert np.array_equal(d1.read(), oracle.gaussian_blur_u8(h8, w, h, c, 7, 1.5, kcv.REVERSE, nthreads=8)[1])
    assert np.array_equal(d2.read(), oracle.separable_filter_2d(h16, w, h, 1, kx, ky, kcv.WRAP)[1])
    assert np.array_equal(d3.read(), oracle.separable_filter_2d(h8, w, h, c, k8, k8, kcv.REFLECT)[1])
    assert np.array_equal(d4.read(), oracle.blur_and_downsample_u8(h8, w, h, c, kcv.REVERSE)[1])
    for hd in hs:
        assert LIB.kleidicv_gpu_async_release(hd) == kcv.OK
    jobs.clear()


def test_async_returns_before_completion_and_self_releases():
    """A 4K RGBA call returns while its work is still running (the query says
    NOT_READY right after a large submission at least once over several tries);
    a call without a handle signals through its callback only."""
    rng = np.random.default_rng(12)
    w, h, c = 3840, 2160, 4
    host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    want = oracle.gaussian_blur_u8(host, w, h, c, 7, 1.5, kcv.REVERSE, nthreads=8)[1]
    seen_running = False
    for _ in range(4):
        dst = np.zeros_like(host)
        hd = ctypes.c_void_p()
        assert LIB.kleidicv_gpu_thread_gaussian_blur_u8_async(host.ctypes.data, w * c, dst.ctypes.data, w * c, w, h,
                                                              c, 7, 7, 1.5, 1.5, kcv.REVERSE, POOL.mt, None, None,
                                                              ctypes.byref(hd)) == kcv.OK
        seen_running |= LIB.kleidicv_gpu_async_query(hd) == kcv.ERROR_NOT_READY
        assert LIB.kleidicv_gpu_async_release(hd) == kcv.OK
        assert np.array_equal(dst, want)
    assert seen_running
    flag = threading.Event()
    got = []

    @kcv.ASYNC_CALLBACK
    def done(status, user):
        got.append(status)
        flag.set()

    dst = np.zeros_like(host)
    assert LIB.kleidicv_gpu_thread_gaussian_blur_u8_async(host.ctypes.data, w * c, dst.ctypes.data, w * c, w, h, c,
                                                          7, 7, 1.5, 1.5, kcv.REVERSE, POOL.mt,
                                                          ctypes.cast(done, ctypes.c_void_p), None, None) == kcv.OK
    assert flag.wait(30)
    assert got == [kcv.OK]
    assert np.array_equal(dst, want)


def test_async_failing_scheduler_reports_through_the_handle():
    """A scheduler that fails in the download phase (on the completion worker)
    makes the call's final status that failure."""
    calls = [0]

    @kcv.THREAD_PARALLEL
    def second_fails(callback, callback_data, parallel_data, task_count):
        calls[0] += 1
        if calls[0] == 2:
            return 4
        return callback(0, task_count, callback_data)

    mt = kcv.ThreadMT(ctypes.cast(second_fails, ctypes.c_void_p).value, None)
    host = np.random.default_rng(3).integers(0, 256, (200, 300), dtype=np.uint8)
    dst = np.zeros_like(host)
    hd = ctypes.c_void_p()
    assert LIB.kleidicv_gpu_thread_gaussian_blur_u8_async(host.ctypes.data, 300, dst.ctypes.data, 300, 300, 200, 1,
                                                          5, 5, 0.0, 0.0, kcv.REFLECT, mt, None, None,
                                                          ctypes.byref(hd)) == kcv.OK
    assert LIB.kleidicv_gpu_async_wait(hd) == kcv.ALLOCATION
    assert LIB.kleidicv_gpu_async_release(hd) == kcv.OK
