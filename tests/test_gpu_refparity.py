"""Parity against the reference itself: KleidiCV and kleidicv_thread built
natively on the AArch64 host (oracle/refimpl.py, ``make -C oracle refnative``).

Two layers, both bit-exact (tolerance 0):
* the C restatement (oracle/kcv_oracle.c) against the reference on a grid of
  kernel sizes, sigmas, channel counts, borders and minimum sizes, so that the
  restatement every other GPU test checks against is pinned byte for byte;
* the GPU entry points (through the C ABI) against the reference on the
  workload shapes: the 3840x2160 RGBA 7x7 sigma-1.5 Gaussian and the u16 5x5
  separable filters of the drop-in sweep, the 1920x1080 5x5 binomial call, a
  sample of the 512-image uneven batch that includes k = 15 (plain calls and
  one batched plan), pyramids, Sobel, median and the LK pyramid.

The reference only builds on AArch64.  Elsewhere these tests skip; on an
AArch64 host with the reference sources staged, a failed reference build is a
test failure (the reason is in oracle/_ref/refnative.log).
"""
import numpy as np
import pytest

from oracle import refimpl
from tests.gpu_harness import device_image, device_output, padded, read_output, read_strided

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

BORDERS = [1, 2, 3, 4]  # REPLICATE, REFLECT, WRAP, REVERSE


@pytest.fixture(scope="module")
def ref():
    if not refimpl.native_host():
        pytest.skip("the reference builds only on AArch64 hosts")
    if not refimpl.staged():
        pytest.skip("reference sources are not staged in oracle/_ref/src")
    why = refimpl.status()
    assert why is None, f"reference library unavailable: {why}"
    return refimpl


@pytest.fixture(scope="module")
def pool(ref):
    p = ref.Pool(16)
    yield p
    p.close()


@pytest.fixture(scope="module")
def ctx(kcv):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = kcv.Context.for_torch(0)
    yield c
    c.close()


def _same(got, want, what):
    if not np.array_equal(got, want):
        bad = np.argwhere(got != want)
        raise AssertionError(f"{what}: {len(bad)} mismatches, first {bad[:4].tolist()} "
                             f"got {got[tuple(bad[0])]} want {want[tuple(bad[0])]}")


# ---------------------------------------------------------------------------
# The C restatement against the reference (CPU only, runs where the reference does).

@pytest.mark.parametrize("k", [3, 5, 7, 9, 15, 21])
@pytest.mark.parametrize("sigma", [0.0, 0.5, 1.0, 1.5, 2.25, 3.7])
def test_oracle_gaussian_fixed_vs_reference(ref, oracle, k, sigma):
    rng = np.random.default_rng(k * 100 + int(sigma * 10))
    for c in (1, 2, 3, 4):
        for w, h in ((k - 1, k - 1), (k + 3, k), (67, 41)):
            host = padded(rng, h, w * c, np.uint8, 3)
            for border in BORDERS:
                e1, want = ref.gaussian_blur_u8(host, w, h, c, k, sigma, border)
                e2, got = oracle.gaussian_blur_u8(host, w, h, c, k, sigma, border)
                assert e1 == e2
                if e1 == 0:
                    _same(got, want, f"oracle k={k} s={sigma} c={c} {w}x{h} b={border}")


@pytest.mark.parametrize("k", [11, 13, 17, 23, 31, 63])
def test_oracle_gaussian_arbitrary_vs_reference(ref, oracle, k):
    rng = np.random.default_rng(k)
    for c in (1, 2, 3, 4):
        for sigma in (0.0, 1.3, 4.0, 11.0):
            for w, h in ((k + 8, k), (97, 71)):
                host = padded(rng, h, w * c, np.uint8, 5)
                for border in BORDERS:
                    e1, want = ref.gaussian_blur_u8(host, w, h, c, k, sigma, border)
                    e2, got = oracle.gaussian_blur_u8(host, w, h, c, k, sigma, border)
                    assert e1 == e2, (k, sigma, c, w, h, border, e1, e2)
                    if e1 == 0:
                        _same(got, want, f"oracle arbitrary k={k} s={sigma} c={c} {w}x{h} b={border}")


def test_oracle_gaussian_errors_vs_reference(ref, oracle):
    """Validation outcomes for unsupported sizes, sigmas, borders and shapes."""
    host = np.zeros((40, 400), np.uint8)
    cases = [(50, 40, 4, 4, 1.0, 1), (50, 40, 4, 5, 1.0, 0), (50, 40, 4, 5, 1.0, 5), (50, 40, 5, 5, 1.0, 1),
             (3, 3, 1, 5, 0.0, 1), (4, 4, 1, 5, 0.0, 1), (50, 40, 1, 257, 1.0, 1), (50, 40, 1, 11, 1.0, 2),
             (10, 40, 1, 11, 1.0, 1), (50, 40, 1, 1, 1.0, 1), (50, 40, 1, 6, 1.0, 1)]
    for w, h, c, k, s, b in cases:
        e1, _ = ref.gaussian_blur_u8(host, w, h, c, k, s, b)
        e2, _ = oracle.gaussian_blur_u8(host, w, h, c, k, s, b)
        assert e1 == e2, (w, h, c, k, s, b, e1, e2)


@pytest.mark.parametrize("dt", ["u8", "u16"])
def test_oracle_separable_vs_reference(ref, oracle, dt):
    dtype = np.uint8 if dt == "u8" else np.uint16
    top = np.iinfo(dtype).max
    rng = np.random.default_rng(5 if dt == "u8" else 6)
    taps = [([1, 2, 3, 2, 1], [0, 1, 4, 1, 0]), ([0, 0, 1, 0, 0], [0, 0, 1, 0, 0]),
            (list(rng.integers(0, top + 1, 5)), list(rng.integers(0, top + 1, 5))),
            (list(rng.integers(0, 5, 5)), list(rng.integers(0, 5, 5)))]
    for kx, ky in taps:
        for c in (1, 2, 3, 4):
            for w, h in ((4, 4), (33, 9), (130, 17)):
                host = padded(rng, h, w * c, dtype, 3)
                for border in BORDERS:
                    e1, want = ref.separable_filter_2d(host, w, h, c, np.array(kx, dtype), np.array(ky, dtype),
                                                       border)
                    e2, got = oracle.separable_filter_2d(host, w, h, c, np.array(kx, dtype), np.array(ky, dtype),
                                                         border)
                    assert e1 == e2 == 0, (e1, e2)
                    _same(got, want, f"oracle separable {dt} {kx}/{ky} c={c} {w}x{h} b={border}")


def test_oracle_blur_and_downsample_vs_reference(ref, oracle):
    rng = np.random.default_rng(7)
    for c in (1, 2, 3, 4):
        for w, h in ((4, 4), (5, 7), (33, 18), (131, 97)):
            host = padded(rng, h, w * c, np.uint8, 2)
            for border in BORDERS:
                e1, want = ref.blur_and_downsample_u8(host, w, h, c, border)
                e2, got = oracle.blur_and_downsample_u8(host, w, h, c, border)
                assert e1 == e2 == 0
                _same(got, want, f"oracle blur_and_downsample c={c} {w}x{h} b={border}")


def test_oracle_sobel_vs_reference(ref, oracle):
    rng = np.random.default_rng(8)
    for c in (1, 3, 4):
        for w, h in ((2, 2), (17, 9), (130, 33)):
            host = padded(rng, h, w * c, np.uint8, 3)
            for horizontal in (True, False):
                e1, want = ref.sobel_3x3_s16_u8(host, w, h, c, horizontal)
                e2, got = oracle.sobel_3x3_s16_u8(host, w, h, c, horizontal)
                assert e1 == e2 == 0
                _same(got, want, f"oracle sobel h={horizontal} c={c} {w}x{h}")


@pytest.mark.parametrize("dtype", [np.int8, np.uint8, np.uint16, np.int16, np.uint32, np.int32, np.float32])
def test_oracle_median_vs_reference(ref, oracle, dtype):
    rng = np.random.default_rng(9)
    ks = (3, 5, 7, 9, 15) if dtype == np.uint8 else (3, 5, 7)
    for k in ks:
        for c in (1, 3):
            w, h = max(k + 5, 23), max(k + 2, 13)
            if dtype == np.float32:
                host = rng.normal(0, 100, (h, w * c)).astype(np.float32)
            else:
                host = padded(rng, h, w * c, dtype, 0)
            for border in BORDERS:
                e1, want = ref.median_blur(host, w, h, c, k, border)
                assert e1 == 0
                got = oracle.median_blur(host, w, h, c, k, border)
                _same(got, want, f"oracle median {np.dtype(dtype).name} k={k} c={c} b={border}")


# ---------------------------------------------------------------------------
# The GPU path against the reference.

def _gpu_gaussian(kcv, ctx, host, w, h, c, k, sigma, border):
    _keep, sp, ss = device_image(torch, host)
    obuf, dp, ds = device_output(torch, h, w * c, np.uint8, 0)
    assert kcv.gaussian_blur_u8(sp, ss, dp, ds, w, h, c, k, k, sigma, sigma, border, ctx) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    got, pad_ok = read_output(obuf, h, w * c, np.uint8, ds)
    assert pad_ok
    return got


def _sweep_inputs():
    import bench

    return bench.make_calls()[0]


def test_gpu_sweep_gaussian_4k_rgba_vs_reference(ref, pool, kcv, ctx):
    """3840x2160x4, 7x7, sigma 1.5, REVERSE: the sweep's Gaussian, byte for byte."""
    call = _sweep_inputs()[0]
    src = call["src"]
    e, want = ref.gaussian_blur_u8(src, 3840, 2160, 4, 7, 1.5, 4, pool=pool)
    assert e == 0
    _same(_gpu_gaussian(kcv, ctx, src, 3840, 2160, 4, 7, 1.5, 4), want, "gpu 4K RGBA 7x7 s1.5")


def test_gpu_sweep_separable_vs_reference(ref, pool, kcv, ctx):
    """The sweep's u16 5x5 calls (REFLECT, WRAP) equal the reference; for the
    u16 CONSTANT call the drop-in answer is NOT_IMPLEMENTED on both sides.  The
    s16 calls have no reference counterpart (an extension of this library)."""
    for call in _sweep_inputs()[1:]:
        src, dt, border = call["src"], call["dtype"], call["border"]
        if dt == "s16":
            continue
        dtype = src.dtype
        kx, ky = np.array(call["kx"], dtype), np.array(call["ky"], dtype)
        _keep, sp, ss = device_image(torch, src)
        obuf, dp, ds = device_output(torch, 2160, 3840, dtype, 0)
        e_gpu = kcv.separable_filter_2d(dt, sp, ss, dp, ds, 3840, 2160, 1, kx, 5, ky, 5, border, ctx)
        if border == 0:
            assert e_gpu == kcv.NOT_IMPLEMENTED, (call["name"], e_gpu)
            e_ref, _ = ref.separable_filter_2d(src, 3840, 2160, 1, kx, ky, border, pool=pool)
            assert e_ref == kcv.NOT_IMPLEMENTED
            continue
        assert e_gpu == kcv.OK
        assert ctx.synchronize() == kcv.OK
        got, _ = read_output(obuf, 2160, 3840, dtype, ds)
        e_ref, want = ref.separable_filter_2d(src, 3840, 2160, 1, kx, ky, border, pool=pool)
        assert e_ref == 0
        _same(got, want, call["name"])


def test_gpu_hd_binomial_vs_reference(ref, kcv, ctx):
    """1920x1080x1, 5x5 binomial, REPLICATE, strides width+64 (seed 0)."""
    rng = np.random.default_rng(0)
    host = padded(rng, 1080, 1920, np.uint8, 64)
    e, want = ref.gaussian_blur_u8(host, 1920, 1080, 1, 5, 0.0, 1)
    assert e == 0
    _same(_gpu_gaussian(kcv, ctx, host, 1920, 1080, 1, 5, 0.0, 1), want, "gpu 1080p binomial 5x5")


def _uneven_batch(n):
    """The first n images of the 512-image uneven batch (seed 2)."""
    rng = np.random.default_rng(2)
    out = []
    for _ in range(n):
        w = int(round(float(np.exp(rng.uniform(np.log(64), np.log(4096))))))
        h = int(round(float(np.exp(rng.uniform(np.log(64), np.log(2160))))))
        c = int(rng.choice([1, 3, 4]))
        k = int(rng.choice([3, 5, 7, 15]))
        sigma = float(rng.uniform(0.5, 4.0))
        border = int(rng.choice([1, 2, 3, 4]))
        out.append((rng.integers(0, 256, (h, w * c), dtype=np.uint8), w, h, c, k, sigma, border))
    return out


def test_gpu_uneven_batch_sample_vs_reference(ref, pool, kcv, ctx):
    """48 images of the uneven batch, through plain calls and one batched plan
    (CUDA graph), against the reference."""
    items = _uneven_batch(48)
    assert any(it[4] == 15 for it in items)
    srcs, dsts, reqs, wants = [], [], [], []
    for host, w, h, c, k, sigma, border in items:
        e, want = ref.gaussian_blur_u8(host, w, h, c, k, sigma, border, pool=pool)
        assert e == 0
        wants.append(want)
        _same(_gpu_gaussian(kcv, ctx, host, w, h, c, k, sigma, border), want,
              f"gpu plain {w}x{h}x{c} k={k} s={sigma:.3f} b={border}")
        s = torch.from_numpy(host).cuda()
        d = torch.zeros_like(s)
        srcs.append(s)
        dsts.append(d)
        reqs.append(kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, s.data_ptr(), w * c, d.data_ptr(), w * c, w, h, c,
                                     k, k, sigma, sigma, border_type=border))
    plan = kcv.BatchPlan(reqs, ctx)
    assert all(st == kcv.OK for st in plan.statuses)
    assert plan.launch(True) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    for d, want, it in zip(dsts, wants, items):
        _same(d.cpu().numpy(), want, f"gpu batched {it[1]}x{it[2]}x{it[3]} k={it[4]}")
    plan.close()


@pytest.mark.parametrize("k", [3, 5, 7, 9, 15, 21])
def test_gpu_sigma_grid_min_sizes_vs_reference(ref, kcv, ctx, k):
    """Sigma grid at the smallest accepted image (k-1 square) and a ragged one."""
    rng = np.random.default_rng(1000 + k)
    for sigma in (0.0, 0.3, 0.8, 1.5, 2.25, 4.0, 9.0):
        for c in (1, 3, 4):
            for w, h in ((k - 1, k - 1), (k + 29, k + 2)):
                host = padded(rng, h, w * c, np.uint8, 0)
                for border in BORDERS:
                    e, want = ref.gaussian_blur_u8(host, w, h, c, k, sigma, border)
                    assert e == 0
                    _same(_gpu_gaussian(kcv, ctx, host, w, h, c, k, sigma, border), want,
                          f"gpu k={k} s={sigma} c={c} {w}x{h} b={border}")


def test_gpu_arbitrary_sizes_vs_reference(ref, kcv, ctx):
    """Arbitrary odd sizes (REPLICATE), every channel count, including the
    right-border lanes whose channel the reference's index pattern shifts."""
    rng = np.random.default_rng(77)
    cases = [(11, 0.0, 1, 300, 200), (17, 3.0, 3, 257, 61), (31, 6.5, 4, 129, 90), (63, 0.0, 1, 640, 70),
             (255, 40.0, 1, 400, 300), (13, 0.0, 2, 21, 13), (13, 2.0, 3, 21, 13), (23, 0.0, 4, 31, 23),
             (29, 5.0, 2, 1001, 40), (41, 0.0, 3, 2000, 44), (99, 9.0, 4, 555, 120), (11, 0.0, 3, 4099, 3000)]
    for k, sigma, c, w, h in cases:
        host = padded(rng, h, w * c, np.uint8, 0)
        e, want = ref.gaussian_blur_u8(host, w, h, c, k, sigma, 1)
        assert e == 0
        _same(_gpu_gaussian(kcv, ctx, host, w, h, c, k, sigma, 1), want, f"gpu arbitrary k={k}")


def test_gpu_pyramid_vs_reference(ref, pool, kcv, ctx):
    """Five REVERSE blur-and-downsample levels of seeded sin+noise images."""
    rng = np.random.default_rng(3)
    for w, h, c in ((2048, 2048, 1), (1024, 768, 4), (1001, 677, 3)):
        y, x = np.mgrid[0:h, 0:w]
        base = 128 + 60 * np.sin(x / 17.0 + y / 29.0)
        img = np.repeat(base[:, :, None], c, axis=2) + rng.uniform(-40, 40, (h, w, c))
        host = np.clip(np.rint(img), 0, 255).astype(np.uint8).reshape(h, w * c)
        cur, cw, ch = host, w, h
        src = torch.from_numpy(host).cuda()
        sp, ss = src.data_ptr(), w * c
        keep = []
        for level in range(5):
            ow, oh = (cw + 1) // 2, (ch + 1) // 2
            e, want = ref.blur_and_downsample_u8(cur, cw, ch, c, 4, pool=pool)
            assert e == 0
            d = torch.zeros((oh, ow * c), dtype=torch.uint8, device="cuda")
            assert kcv.blur_and_downsample_u8(sp, ss, cw, ch, d.data_ptr(), ow * c, c, 4, ctx) == kcv.OK
            assert ctx.synchronize() == kcv.OK
            _same(d.cpu().numpy(), want, f"gpu pyramid {w}x{h}x{c} level {level + 1}")
            keep.append(d)
            cur, cw, ch, sp, ss = want, ow, oh, d.data_ptr(), ow * c


def test_gpu_sobel_vs_reference(ref, kcv, ctx):
    rng = np.random.default_rng(5)
    for w, h, c in ((3840, 2160, 4), (1001, 333, 1), (2, 2, 3)):
        host = padded(rng, h, w * c, np.uint8, 0)
        _keep, sp, ss = device_image(torch, host)
        for horizontal in (True, False):
            obuf, dp, ds = device_output(torch, h, w * c, np.int16, 0)
            fn = kcv.sobel_3x3_horizontal_s16_u8 if horizontal else kcv.sobel_3x3_vertical_s16_u8
            assert fn(sp, ss, dp, ds, w, h, c, ctx) == kcv.OK
            assert ctx.synchronize() == kcv.OK
            got, _ = read_output(obuf, h, w * c, np.int16, ds)
            e, want = ref.sobel_3x3_s16_u8(host, w, h, c, horizontal)
            assert e == 0
            _same(got, want, f"gpu sobel {w}x{h}x{c} h={horizontal}")


@pytest.mark.parametrize("dt,dtype,ks", [("u8", np.uint8, (3, 5, 7, 9, 15)), ("s16", np.int16, (3, 5, 7)),
                                         ("f32", np.float32, (3, 5))])
def test_gpu_median_vs_reference(ref, kcv, ctx, dt, dtype, ks):
    rng = np.random.default_rng(11)
    for k in ks:
        for w, h, c in ((320, 240, 1), (97, 61, 3)):
            if dtype == np.float32:
                host = rng.normal(0, 50, (h, w * c)).astype(np.float32)
            else:
                host = padded(rng, h, w * c, dtype, 0)
            _keep, sp, ss = device_image(torch, host)
            for border in BORDERS:
                obuf, dp, ds = device_output(torch, h, w * c, dtype, 0)
                assert kcv.median_blur(dt, sp, ss, dp, ds, w, h, c, k, k, border, ctx) == kcv.OK
                assert ctx.synchronize() == kcv.OK
                got, _ = read_output(obuf, h, w * c, dtype, ds)
                e, want = ref.median_blur(host, w, h, c, k, border)
                assert e == 0
                _same(got, want, f"gpu median {dt} k={k} {w}x{h}x{c} b={border}")


def test_gpu_lk_pyramid_vs_reference(ref, kcv, ctx):
    """Every level's image and Scharr pairs (interiors) of the LK pyramid."""
    rng = np.random.default_rng(12)
    for w, h, c, levels, ww, wh in ((640, 480, 1, 4, 21, 21), (333, 250, 3, 3, 7, 5)):
        host = padded(rng, h, w * c, np.uint8, 0)
        src = torch.from_numpy(host).cuda()
        pyr = kcv.LKPyramid(src.data_ptr(), w * c, w, h, c, levels, ww, wh, ctx)
        assert pyr.error == kcv.OK
        assert ctx.synchronize() == kcv.OK
        e, want = ref.lk_pyramid(host, w, h, c, levels, ww, wh)
        assert e == 0
        assert pyr.level_count() == len(want)
        for li, (img_want, sch_want) in enumerate(want):
            lw, lh, img, istride, sch, sstride, bw, bh = pyr.level(li)
            assert img_want.shape == (lh, lw * c)
            _same(read_strided(img, lh, lw * c, istride), img_want, f"lk image level {li}")
            got_s = read_strided(sch, lh, lw * c * 4, sstride).copy().view(np.int16)
            _same(got_s, sch_want, f"lk scharr level {li}")
        pyr.close()
