"""Lucas-Kanade pyramid on the GPU: every level's bordered image (reflect-101
border of the window size) and interleaved Scharr pairs must equal the CPU
restatement of kleidicv_build_optical_flow_pyr_lk_pyramid; the Scharr halo is
zero; validation follows the reference's order and level-count rule."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402
from gpu_harness import read_strided  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()

CASES = [(64, 48, 1, 3, 5, 5), (101, 77, 3, 4, 7, 5), (640, 480, 4, 5, 21, 21), (37, 29, 2, 3, 3, 3),
         (1, 1, 1, 1, 3, 3), (2, 5, 1, 2, 3, 4), (1000, 700, 1, 8, 9, 13), (333, 250, 3, 6, 3, 3)]


@pytest.mark.parametrize("case", CASES)
def test_lk_pyramid_matches_oracle(case):
    w, h, c, levels, ww, wh = case
    rng = np.random.default_rng(w * 7 + h)
    pad = 9
    host = rng.integers(0, 256, (h, w * c + pad), dtype=np.uint8)
    src = torch.from_numpy(host).cuda()
    ctx = kcv.Context.for_torch(0)
    pyr = kcv.LKPyramid(src.data_ptr(), w * c + pad, w, h, c, levels, ww, wh, ctx)
    assert pyr.error == kcv.OK
    assert ctx.synchronize() == kcv.OK
    err, want = oracle.lk_pyramid(host, w, h, c, levels, ww, wh)
    assert err == kcv.OK
    assert pyr.level_count() == len(want)
    for li, lv in enumerate(want):
        lw, lh, img, istride, sch, sstride, bw, bh = pyr.level(li)
        assert (lw, lh, bw, bh) == (lv["width"], lv["height"], ww, wh)
        got_img = read_strided(img - bh * istride - bw * c, lh + 2 * bh, (lw + 2 * bw) * c, istride)
        assert np.array_equal(got_img, lv["image"]), f"level {li}: image differs"
        full = read_strided(sch - bh * sstride - bw * c * 4, lh + 2 * bh, (lw + 2 * bw) * c * 4, sstride)
        inner = full[bh:bh + lh, bw * c * 4:(bw + lw) * c * 4].copy().view(np.int16)
        assert np.array_equal(inner, lv["scharr"]), f"level {li}: scharr differs"
        halo = full.copy()
        halo[bh:bh + lh, bw * c * 4:(bw + lw) * c * 4] = 0
        assert not halo.any(), f"level {li}: scharr halo not zero"
    pyr.close()
    ctx.close()


def test_lk_pyramid_validation():
    ctx = kcv.Context.for_torch(0)
    buf = torch.zeros(4096, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    cases = [  # (src, stride, w, h, c, levels, ww, wh)
        (p, 64, 0, 8, 1, 2, 3, 3), (p, 64, 8, 0, 1, 2, 3, 3), (p, 64, 8, 8, 0, 2, 3, 3), (p, 64, 8, 8, 5, 2, 3, 3),
        (p, 64, 8, 8, 1, 0, 3, 3), (p, 64, 8, 8, 1, 2, 2, 3), (p, 64, 8, 8, 1, 2, 3, 2), (p, 64, 8, 8, 1, 2, 2048, 3),
        (p, 7, 8, 8, 1, 2, 3, 3), (None, 64, 8, 8, 1, 2, 3, 3), (p, 64, 1 << 30, 1 << 30, 1, 2, 3, 3)]
    for src, stride, w, h, c, lv, ww, wh in cases:
        pyr = kcv.LKPyramid(src, stride, w, h, c, lv, ww, wh, ctx)
        if src is None:
            want = kcv.NULL_POINTER
        elif w * h > (1 << 48) - 1:
            want = kcv.RANGE
        else:
            want, _ = oracle.lk_level_count(stride, w, h, c, lv, ww, wh)
        assert pyr.error == want, (src, stride, w, h, c, lv, ww, wh, pyr.error)
    assert kcv.lib().kleidicv_gpu_optical_flow_pyr_lk_pyramid_release(None) == kcv.NULL_POINTER
    ctx.close()
