"""Pins the CPU oracle against the reference (CPU only, no GPU).

Fixtures in tests/golden/ were produced by tests/golden/make_golden.py from the
reference tree: its GoogleTest known-answer arrays, and the reference's own
sigma generator and border offset tables compiled from its headers.
"""
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


KATS = _load("kats.json")["cases"]


@pytest.mark.parametrize("case", KATS, ids=[c["name"] for c in KATS])
def test_oracle_matches_reference_kats(oracle, case):
    src = np.array(case["src"], dtype=case["dtype"])
    if case["func"] == "gaussian_blur_u8":
        err, dst = oracle.gaussian_blur_u8(src, case["width"], case["height"], case["channels"],
                                           case["kernel_width"], case["sigma_x"], case["border"],
                                           ksize_y=case["kernel_height"], sigma_y=case["sigma_y"])
    elif case["func"] == "separable_filter_2d":
        err, dst = oracle.separable_filter_2d(src, case["width"], case["height"], case["channels"],
                                              np.array(case["kernel_x"], case["dtype"]),
                                              np.array(case["kernel_y"], case["dtype"]), case["border"])
    else:
        err, dst = oracle.blur_and_downsample_u8(src, case["width"], case["height"], case["channels"],
                                                 case["border"])
    assert err == oracle.OK
    exp = np.array(case["expected"], dtype=np.int64)
    got = dst[: exp.shape[0], : exp.shape[1]].astype(np.int64)
    assert np.abs(got - exp).max() <= case["tolerance"], (case["source"], got, exp)


def test_sigma_generator_matches_reference_grid(oracle):
    """Byte-identical half kernels over k = 3..255 x sigma = i/100, i <= 4000."""
    fx = _load("sigma.json")
    for k in range(3, 256, 2):
        h = hashlib.sha256()
        half = k // 2 + 1
        for i in range(4001):
            sigma = float(np.float32(i) / np.float32(100))
            hk = oracle.half_kernel(k, sigma)
            ok = hk is not None
            vals = hk if ok else [0] * half
            h.update((f"{k} {i} {int(ok)} " + " ".join(map(str, vals)) + "\n").encode())
        assert h.hexdigest() == fx["sha256_per_k"][str(k)], k


def test_sigma_subset_readable(oracle):
    fx = _load("sigma.json")
    for key, want in fx["subset"].items():
        k, i = map(int, key.split(":"))
        assert oracle.half_kernel(k, float(np.float32(i) / np.float32(100))) == want, key


def test_sigma_fixed_sizes_sum_to_256(oracle):
    """Fixed sizes (<= 21) never leave the 16-bit lane range on the grid; the
    arbitrary sizes have a handful of 255/257 sums (handled explicitly)."""
    for k in (3, 5, 7, 9, 15, 21):
        for i in range(0, 4001, 7):
            hk = oracle.half_kernel(k, float(np.float32(i) / np.float32(100)))
            if hk is not None:
                assert 2 * sum(hk[:-1]) + hk[-1] == 256, (k, i)


def test_border_map_matches_reference_tables(oracle):
    fx = _load("border.json")
    for key, digest in fx["sha256_per_k_border"].items():
        k, b = map(int, key.split(":"))
        h = hashlib.sha256()
        for n in range(k - 1, k + 41):
            tab = oracle.border_table(k, n, b)
            for i in range(n):
                h.update((f"{k} {b} {n} {i} " + " ".join(map(str, tab[i])) + "\n").encode())
        assert h.hexdigest() == digest, key
    for key, rows in fx["tables"].items():
        k, b, n = map(int, key.split(":"))
        assert oracle.border_table(k, n, b).tolist() == rows, key


# --------------------------------------------------------------------------
# Independent second formulation, in the style of the reference's KernelTest
# (test/framework/kernel.h:184-201): pad the input explicitly per border type
# (test/framework/border.cpp:319-612), apply the full 2-D mask in wide integer
# arithmetic, then scale.  Binomial and separable results must be identical;
# sigma kernels round the intermediate to u8 so they may differ by 1
# (test/api/test_gaussian_blur.cpp:288-384 uses tolerance 1 for the same reason).

def _pad(img, width, channels, r, border, value=0):
    h = img.shape[0]
    px = img[:, : width * channels].reshape(h, width, channels).astype(np.int64)
    if border == 0:
        return np.pad(px, ((r, r), (r, r), (0, 0)), constant_values=value)
    mode = {1: "edge", 2: "symmetric", 3: "wrap", 4: "reflect"}[border]
    return np.pad(px, ((r, r), (r, r), (0, 0)), mode=mode)


def _mask_conv(img, width, channels, wy, wx, border, value=0):
    r = len(wy) // 2
    p = _pad(img, width, channels, r, border, value)
    h = img.shape[0]
    out = np.zeros((h, width, channels), np.int64)
    for i, a in enumerate(wy):
        for j, b in enumerate(wx):
            out += a * b * p[i:i + h, j:j + width]
    return out.reshape(h, width * channels)


BINOMIAL = {3: ([1, 2, 1], 4), 5: ([1, 4, 6, 4, 1], 8), 7: ([2, 7, 14, 18, 14, 7, 2], 12),
            9: ([4, 13, 30, 51, 60, 51, 30, 13, 4], 16)}


@pytest.mark.parametrize("k", [3, 5, 7, 9])
@pytest.mark.parametrize("border", [1, 2, 3, 4])
@pytest.mark.parametrize("channels", [1, 2, 3, 4])
def test_oracle_binomial_equals_mask_product(oracle, k, border, channels):
    rng = np.random.default_rng(k * 100 + border * 10 + channels)
    for w, h in [(k - 1, k - 1), (k, k + 1), (2 * k + 3, k + 5)]:
        img = rng.integers(0, 256, (h, w * channels + 3), dtype=np.uint8)
        err, dst = oracle.gaussian_blur_u8(img, w, h, channels, k, 0.0, border)
        assert err == 0
        c, s = BINOMIAL[k]
        want = (_mask_conv(img, w, channels, c, c, border) + (1 << (s - 1))) >> s
        assert np.array_equal(dst.astype(np.int64), want)


@pytest.mark.parametrize("k,sigma", [(3, 0.8), (5, 1.1), (7, 1.5), (9, 2.0), (15, 0.0), (21, 3.3),
                                     (11, 0.0), (13, 2.2), (31, 5.0)])
def test_oracle_sigma_within_one_of_mask_product(oracle, k, sigma):
    rng = np.random.default_rng(k)
    hk = oracle.half_kernel(k, sigma)
    full = hk + hk[-2::-1]
    for channels in (1, 3, 4):
        w = k + 9 if k <= 21 else (((k // 2) + 7) // 8 * 8 + k // 2 + 5)
        h = k + 2
        img = rng.integers(0, 256, (h, w * channels), dtype=np.uint8)
        fixed = k in (3, 5, 7, 9, 15, 21)
        borders = [1, 2, 3, 4] if fixed else [1]
        # The arbitrary-size path's right-border vectors take some replicated
        # lanes from another channel of the last pixel when channels > 1
        # (pinned separately below): compare only the columns before them.
        cols = w * channels if fixed or channels == 1 else w * channels - ((channels * (k // 2) + 7) // 8 * 8)
        for border in borders:
            err, dst = oracle.gaussian_blur_u8(img, w, h, channels, k, sigma, border)
            assert err == 0
            want = (_mask_conv(img, w, channels, full, full, border) + 32768) >> 16
            assert np.abs(dst.astype(np.int64) - want)[:, :cols].max() <= 1


def _right_lane_sources(c, w, k):
    """Element index each right-border vector lane of the reference's
    arbitrary-size horizontal pass reads, per (output element, tap distance),
    restated from the index vectors of its GenericBorderHorizontal
    (kleidicv/src/filters/border_generic_neon.h:22-98) and the lane loop of
    horizontal_right_border_vector_path (gaussian_blur_arbitrary_neon.cpp:346-377)."""
    mask = (1 << 64) - 1
    data_idx = sum(i << (8 * i) for i in range(8))
    right = 0
    for i in range(8):
        right = ((right << 8) | (((7 - i) % c) + 8 - c)) & mask
    wc, r = w * c, k // 2
    border_len = (c * r + 7) // 8 * 8
    out = {}
    for xv in range(wc - border_len, wc, 8):
        for i in range(r):  # pair i: right tap at distance r - i columns
            start = xv + c * (r - i)
            if start <= wc - 8:
                continue
            shift = 8 * (start - (wc - 8))
            if shift < 64:
                idx = ((data_idx >> shift) | (right << (64 - shift))) & mask
            else:
                shift = ((start - wc) % c) * 8
                idx = right if shift == 0 else \
                    ((((right >> (8 * c - shift)) << (64 - shift)) | (right >> shift)) & mask)
            for lane in range(8):
                out[(xv + lane, r - i)] = wc - 8 + ((idx >> (8 * lane)) & 0xFF)
    return out


@pytest.mark.parametrize("c", [2, 3, 4])
@pytest.mark.parametrize("k,sigma", [(11, 0.0), (13, 2.2), (23, 4.0), (31, 0.0)])
def test_oracle_arbitrary_right_border_lanes(oracle, c, k, sigma):
    """The arbitrary-size Gaussian's last elements of every row, against a
    direct model of the reference's vector lanes: the horizontal pass over the
    vertical result, with each right-hand tap read where the reference's index
    vector points."""
    rng = np.random.default_rng(k * 10 + c)
    r = k // 2
    w = (r + 7) // 8 * 8 + r + 5
    h = k + 1
    img = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    err, dst = oracle.gaussian_blur_u8(img, w, h, c, k, sigma, 1)
    assert err == 0
    hk = oracle.half_kernel(k, sigma)
    g = np.array(hk + hk[-2::-1], np.int64)
    # vertical pass (u8 intermediate, REPLICATE rows), as the reference computes it
    rows = np.clip(np.arange(h)[:, None] + np.arange(-r, r + 1)[None, :], 0, h - 1)
    vert = ((img.astype(np.int64)[rows] * g[None, :, None]).sum(axis=1) + 128) >> 8
    src = _right_lane_sources(c, w, k)
    wc = w * c
    border_len = (c * r + 7) // 8 * 8
    for x in range(wc - border_len, wc):
        col, ch = divmod(x, c)
        acc = g[r] * vert[:, x]
        for d in range(1, r + 1):
            left = vert[:, max(col - d, 0) * c + ch]
            rgt = vert[:, src[(x, d)]] if (x, d) in src else vert[:, min(col + d, w - 1) * c + ch]
            acc = acc + g[r - d] * (left + rgt)
        want = (acc + 128) >> 8
        assert np.array_equal(dst[:, x], want & 0xFF), f"element {x}"


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("border", [1, 2, 3, 4])
def test_oracle_separable_equals_saturated_mask_product(oracle, dtype, border):
    rng = np.random.default_rng(border)
    hi = np.iinfo(dtype).max
    for channels in (1, 2, 3, 4):
        for kmax in (5, hi):
            kx = rng.integers(0, kmax + 1, 5).astype(dtype)
            ky = rng.integers(0, kmax + 1, 5).astype(dtype)
            w, h = 11, 7
            img = rng.integers(0, hi + 1, (h, w * channels), dtype=dtype)
            err, dst = oracle.separable_filter_2d(img, w, h, channels, kx, ky, border)
            assert err == 0
            want = np.minimum(_mask_conv(img, w, channels, ky.astype(np.int64), kx.astype(np.int64),
                                         border), hi)
            assert np.array_equal(dst.astype(np.int64), want)


@pytest.mark.parametrize("border", [1, 2, 3, 4])
@pytest.mark.parametrize("channels", [1, 2, 3, 4])
def test_oracle_blur_and_downsample_equals_mask_at_even_positions(oracle, border, channels):
    rng = np.random.default_rng(border * 7 + channels)
    for w, h in [(4, 4), (5, 5), (161, 7), (9, 12)]:
        img = rng.integers(0, 256, (h, w * channels), dtype=np.uint8)
        err, dst = oracle.blur_and_downsample_u8(img, w, h, channels, border)
        assert err == 0
        c = [1, 4, 6, 4, 1]
        full = (_mask_conv(img, w, channels, c, c, border) + 128) >> 8
        full = full.reshape(h, w, channels)[::2, ::2].reshape((h + 1) // 2, -1)
        assert np.array_equal(dst.astype(np.int64), full)


def test_oracle_constant_border_extension_is_padding(oracle):
    rng = np.random.default_rng(5)
    w, h, ch = 9, 6, 3
    img = rng.integers(0, 256, (h, w * ch), dtype=np.uint8)
    err, dst = oracle.gaussian_blur_u8(img, w, h, ch, 5, 0.0, 0, ext=True, border_value=17)
    assert err == 0
    want = (_mask_conv(img, w, ch, [1, 4, 6, 4, 1], [1, 4, 6, 4, 1], 0, 17) + 128) >> 8
    assert np.array_equal(dst.astype(np.int64), want)
    assert oracle.gaussian_blur_u8(img, w, h, ch, 5, 0.0, 0)[0] == oracle.NOT_IMPLEMENTED
