"""The threaded-API layer without a GPU: the library's worker pool fulfils
KleidiCV's scheduler contract (kleidicv_thread.h:42-97: every task index run
exactly once, the first failure reported, nothing run after the call
returns), and the kleidicv_gpu_thread_* entries validate like the reference,
reject a missing scheduler, and fail loudly without a device."""
import ctypes
import threading

import numpy as np
import pytest

CB = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p)


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


@pytest.mark.parametrize("threads", [1, 2, 4, 8])
def test_pool_runs_every_task_once(lib, kcv, threads):
    pool = kcv.ThreadPool(threads)
    try:
        for count in (1, 3, 64, 1000):
            seen = []
            lock = threading.Lock()
            tids = set()

            @CB
            def cb(begin, end, data):
                with lock:
                    seen.extend(range(begin, end))
                    tids.add(threading.get_ident())
                return 0

            assert lib.kleidicv_gpu_thread_pool_parallel(cb, None, pool.handle, count) == 0
            assert sorted(seen) == list(range(count))
        assert lib.kleidicv_gpu_thread_pool_parallel(cb, None, pool.handle, 0) == 0
    finally:
        pool.close()


def test_pool_reports_first_failure_and_stays_usable(lib, kcv):
    pool = kcv.ThreadPool(4)
    try:
        @CB
        def failing(begin, end, data):
            return 3 if begin == 17 else 0  # RANGE from one task

        @CB
        def fine(begin, end, data):
            return 0

        for _ in range(20):
            assert lib.kleidicv_gpu_thread_pool_parallel(failing, None, pool.handle, 40) == 3
            assert lib.kleidicv_gpu_thread_pool_parallel(fine, None, pool.handle, 40) == 0
        assert lib.kleidicv_gpu_thread_pool_parallel(None, None, pool.handle, 4) == 2
        assert lib.kleidicv_gpu_thread_pool_parallel(fine, None, None, 4) == 2
    finally:
        pool.close()


def test_pool_stress_many_small_calls(lib, kcv):
    pool = kcv.ThreadPool(6)
    total = [0]
    lock = threading.Lock()

    @CB
    def cb(begin, end, data):
        with lock:
            total[0] += end - begin
        return 0

    try:
        for i in range(300):
            assert lib.kleidicv_gpu_thread_pool_parallel(cb, None, pool.handle, 1 + i % 7) == 0
        assert total[0] == sum(1 + i % 7 for i in range(300))
    finally:
        pool.close()


def test_entries_validate_then_need_a_scheduler(lib, kcv, oracle, no_gpu):
    pool = kcv.ThreadPool(2)
    none = kcv.ThreadMT(None, None)
    a = np.zeros((16, 64), np.uint8)
    b = np.zeros((16, 64), np.uint8)
    g = lib.kleidicv_gpu_thread_gaussian_blur_u8
    try:
        # Validation first, whatever the scheduler (gaussian_blur_api.cpp order).
        for mt in (none, pool.mt):
            assert g(a.ctypes.data, 64, b.ctypes.data, 64, 64, 16, 1, 4, 4, 0.0, 0.0, kcv.REFLECT, mt) == \
                kcv.NOT_IMPLEMENTED
            assert g(None, 64, b.ctypes.data, 64, 64, 16, 1, 5, 5, 0.0, 0.0, kcv.REFLECT, mt) == kcv.NULL_POINTER
            assert g(a.ctypes.data, 64, b.ctypes.data, 64, 64, 16, 1, 5, 5, 0.0, 0.0, kcv.CONSTANT, mt) == \
                kcv.NOT_IMPLEMENTED
        assert lib.kleidicv_gpu_thread_sobel_3x3_vertical_s16_u8(a.ctypes.data, 64, b.ctypes.data, 63, 32, 16, 1,
                                                                 pool.mt) == kcv.ALIGNMENT
        # A valid call with no scheduler.
        assert g(a.ctypes.data, 64, b.ctypes.data, 64, 64, 16, 1, 5, 5, 0.0, 0.0, kcv.REFLECT, none) == \
            kcv.NULL_POINTER
        if no_gpu:
            assert g(a.ctypes.data, 64, b.ctypes.data, 64, 64, 16, 1, 5, 5, 0.0, 0.0, kcv.REFLECT, pool.mt) == \
                kcv.ERROR_NO_DEVICE
            assert not b.any()
    finally:
        pool.close()


@pytest.mark.parametrize("dtype", ["s8", "u8", "u16", "s16", "u32", "s32", "f32"])
def test_threaded_median_validates_like_the_reference(lib, kcv, oracle, no_gpu, dtype):
    pool = kcv.ThreadPool(2)
    fn = getattr(lib, f"kleidicv_gpu_thread_median_blur_{dtype}")
    es = {"s8": 1, "u8": 1, "u16": 2, "s16": 2, "u32": 4, "s32": 4, "f32": 4}[dtype]
    a = np.zeros(4096, np.uint8)
    b = np.zeros(4096, np.uint8)
    try:
        for (w, h, c, k, border, sstride) in [(10, 10, 1, 5, 1, 64), (10, 10, 5, 5, 1, 64), (10, 10, 1, 4, 1, 64),
                                              (10, 10, 1, 9, 1, 64), (10, 10, 1, 5, 0, 64), (3, 10, 1, 7, 1, 64),
                                              (10, 10, 1, 5, 1, 63), (10, 10, 0, 5, 1, 64)]:
            want = oracle.median_blur_check(dtype, False, sstride, False, 64, w, h, c, k, k, border)
            got = fn(a.ctypes.data, sstride, b.ctypes.data, 64, w, h, c, k, k, border, pool.mt)
            if want != 0:
                assert got == want, (w, h, c, k, border, sstride, got, want)
            elif c == 0:
                assert got == kcv.OK
            elif no_gpu:
                assert got == kcv.ERROR_NO_DEVICE and not b.any()
        assert fn(None, 64, b.ctypes.data, 64, 10, 10, 1, 5, 5, 1, pool.mt) == kcv.NULL_POINTER
        assert fn(a.ctypes.data, 64, b.ctypes.data, 64, 10, 10, 1, 5, 5, 1, kcv.ThreadMT(None, None)) == \
            kcv.NULL_POINTER
        if es > 1:  # median validation checks the source stride's alignment first
            assert fn(a.ctypes.data, 64 + 1, b.ctypes.data, 64, 10, 10, 1, 5, 5, 1, pool.mt) == kcv.ALIGNMENT
    finally:
        pool.close()


def test_async_entries_validate_synchronously(lib, kcv, no_gpu):
    """The asynchronous variants: validation errors come back from the call,
    with no handle and no callback; without a device the call fails loudly;
    the handle functions reject NULL."""
    pool = kcv.ThreadPool(2)
    calls = []

    @kcv.ASYNC_CALLBACK
    def done(status, user):
        calls.append(status)

    a = np.zeros((16, 64), np.uint8)
    b = np.zeros((16, 64), np.uint8)
    g = lib.kleidicv_gpu_thread_gaussian_blur_u8_async
    h = ctypes.c_void_p(12345)
    cb = ctypes.cast(done, ctypes.c_void_p)
    try:
        assert g(a.ctypes.data, 64, b.ctypes.data, 64, 64, 16, 1, 4, 4, 0.0, 0.0, kcv.REFLECT, pool.mt, cb, None,
                 ctypes.byref(h)) == kcv.NOT_IMPLEMENTED
        assert h.value is None
        assert g(None, 64, b.ctypes.data, 64, 64, 16, 1, 5, 5, 0.0, 0.0, kcv.REFLECT, pool.mt, cb, None,
                 ctypes.byref(h)) == kcv.NULL_POINTER
        assert g(a.ctypes.data, 64, b.ctypes.data, 64, 64, 16, 1, 5, 5, 0.0, 0.0, kcv.REFLECT,
                 kcv.ThreadMT(None, None), cb, None, ctypes.byref(h)) == kcv.NULL_POINTER
        assert lib.kleidicv_gpu_thread_separable_filter_2d_u16_async(
            a.ctypes.data, 63, b.ctypes.data, 64, 32, 16, 1, a.ctypes.data, 5, a.ctypes.data, 5, kcv.REFLECT,
            pool.mt, cb, None, ctypes.byref(h)) == kcv.ALIGNMENT
        assert lib.kleidicv_gpu_thread_blur_and_downsample_u8_async(
            a.ctypes.data, 64, 64, 16, b.ctypes.data, 64, 1, kcv.CONSTANT, pool.mt, cb, None,
            ctypes.byref(h)) == kcv.NOT_IMPLEMENTED
        if no_gpu:
            assert g(a.ctypes.data, 64, b.ctypes.data, 64, 64, 16, 1, 5, 5, 0.0, 0.0, kcv.REFLECT, pool.mt, cb,
                     None, ctypes.byref(h)) == kcv.ERROR_NO_DEVICE
            assert h.value is None and not b.any()
        assert calls == []
        for fn in ("kleidicv_gpu_async_query", "kleidicv_gpu_async_wait", "kleidicv_gpu_async_release"):
            assert getattr(lib, fn)(None) == kcv.NULL_POINTER
    finally:
        pool.close()
