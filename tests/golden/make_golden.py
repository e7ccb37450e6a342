"""Generates the committed golden fixtures in tests/golden/ from the reference.

Run in a container that has the reference tree (default /root/reference):

    python tests/golden/make_golden.py [--ref /root/reference]

It writes:
  kats.json    known-answer tests extracted, by parsing the C++ source text,
               from the reference's own GoogleTest files:
                 test/api/test_gaussian_blur.cpp        (ValidImageSize3x3..9x9)
                 test/api/test_separable_filter_2d.cpp  (5x5_U8Overflow*, 5x5_U16Overflow*)
                 test/api/test_blur_and_downsample.cpp  (Minimal_u8)
  sigma.json   digests (and a readable subset) of the reference's Gaussian
               half-kernel generator, kleidicv/include/kleidicv/filters/sigma.h,
               compiled here from the reference tree by `make -C oracle ref`
               and run over k = 3..255 (odd) x sigma = i/100, i = 0..4000.
  border.json  digests (and the n = K-1 / K tables) of the reference's fixed
               border offset tables kleidicv/include/kleidicv/workspace/border_*.h,
               compiled the same way, for K in {3,5,7,9,15,21}, all four fixed
               border types and extents n in [K-1, K+40].

Nothing at test time reads the reference tree: tests compare the oracle with
these fixtures only.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(REPO, "oracle")

BORDERS = {
    "KLEIDICV_BORDER_TYPE_CONSTANT": 0,
    "KLEIDICV_BORDER_TYPE_REPLICATE": 1,
    "KLEIDICV_BORDER_TYPE_REFLECT": 2,
    "KLEIDICV_BORDER_TYPE_WRAP": 3,
    "KLEIDICV_BORDER_TYPE_REVERSE": 4,
    "KLEIDICV_BORDER_TYPE_TRANSPARENT": 5,
    "KLEIDICV_BORDER_TYPE_NONE": 6,
}


# --------------------------------------------------------------------------
# C++ test-source parsing (only the narrow statement forms the KATs use).

def _blocks(text):
    """Yields (test_name, first_line, body) for every TEST/TYPED_TEST block."""
    for m in re.finditer(r"^(?:TYPED_)?TEST\((\w+),\s*(\w+)\)\s*\{", text, re.M):
        start = m.end()
        depth, i = 1, start
        while depth:
            ch = text[i]
            depth += ch == "{"
            depth -= ch == "}"
            i += 1
        yield m.group(2), text.count("\n", 0, m.start()) + 1, text[start:i - 1]


def _split_args(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _statements(body):
    """Splits a block body into top-level statements (comments removed)."""
    body = re.sub(r"//[^\n]*", "", body)
    out, depth, cur = [], 0, ""
    for ch in body:
        if ch in "([{":
            depth += 1
        elif ch in ")]}":
            depth -= 1
        cur += ch
        if ch == ";" and depth == 0:
            out.append(" ".join(cur.split()))
            cur = ""
    return out


def _matching_paren(s, open_idx):
    depth = 0
    for i in range(open_idx, len(s)):
        depth += s[i] == "("
        depth -= s[i] == ")"
        if depth == 0:
            return i
    raise ValueError(s)


class KatParser:
    def __init__(self, kernel_size=None):
        self.arrays = {}
        self.kernel_size = kernel_size
        self.last_call = None
        self.cases = []

    def value(self, tok):
        tok = tok.strip()
        if tok in BORDERS:
            return BORDERS[tok]
        if tok == "validSize":
            return self.kernel_size - 1
        m = re.fullmatch(r"(\w+)\.width\(\)\s*/\s*\w+\.channels\(\)", tok)
        if m:
            return self.arrays[m.group(1)]["width"]
        m = re.fullmatch(r"(\w+)\.(height|channels)\(\)", tok)
        if m:
            return self.arrays[m.group(1)][m.group(2)]
        m = re.fullmatch(r"(\w+)\.(data|stride)\(\)", tok)
        if m:
            return ("array", m.group(1)) if m.group(2) == "data" else ("stride", m.group(1))
        return float(tok) if "." in tok else int(tok)

    def statement(self, st, line_hint):
        m = re.match(r"test::Array2D<\w+> (\w+)\{(.*?)\};", st)
        if m:
            args = _split_args(m.group(2))
            w, h = self.value(args[0]), self.value(args[1])
            self.arrays[m.group(1)] = {"width": w, "height": h, "channels": 1,
                                       "rows": [[None] * w for _ in range(h)]}
            return
        m = re.match(r"(\w+)\.set\((\d+), (\d+), \{(.*)\}\);", st)
        if m and m.group(1) in self.arrays:
            row, col = int(m.group(2)), int(m.group(3))
            vals = [int(v) for v in m.group(4).replace(" ", "").split(",") if v]
            self.arrays[m.group(1)]["rows"][row][col:col + len(vals)] = vals
            return
        if st.startswith("EXPECT_EQ(KLEIDICV_OK,"):
            inner = st[len("EXPECT_EQ(KLEIDICV_OK,"):]
            fn = re.match(r"\s*(\w+)<\w+>\(\)\(", inner)
            open_idx = inner.index("(", inner.index("()") + 2)
            args = [self.value(a) for a in _split_args(inner[open_idx + 1:_matching_paren(inner, open_idx)])]
            self.last_call = (fn.group(1), args, line_hint)
            return
        m = re.match(r"EXPECT_EQ_ARRAY2D(?:_WITH_TOLERANCE)?\((?:(\d+), )?(\w+), (\w+)\);", st)
        if m and self.last_call:
            tol = int(m.group(1) or 0)
            self.cases.append(self.make_case(self.last_call, self.arrays[m.group(2)], tol))

    def snapshot(self, name):
        rows = self.arrays[name]["rows"]
        assert all(v is not None for r in rows for v in r), f"array {name} not fully set"
        return [list(r) for r in rows]

    def make_case(self, call, expected, tol):
        fn, a, line = call
        exp_rows = [list(r) for r in expected["rows"]]
        assert all(v is not None for r in exp_rows for v in r)
        if fn == "gaussian_blur":
            src = self.snapshot(a[0][1])
            return {"func": "gaussian_blur_u8", "src": src, "width": a[4], "height": a[5],
                    "channels": a[6], "kernel_width": a[7], "kernel_height": a[8],
                    "sigma_x": a[9], "sigma_y": a[10], "border": a[11], "expected": exp_rows,
                    "tolerance": tol, "line": line}
        if fn == "separable_filter_2d":
            src = self.snapshot(a[0][1])
            kx = self.snapshot(a[7][1])[0]
            ky = self.snapshot(a[9][1])[0]
            return {"func": "separable_filter_2d", "src": src, "width": a[4], "height": a[5],
                    "channels": a[6], "kernel_x": kx, "kernel_width": a[8], "kernel_y": ky,
                    "kernel_height": a[10], "border": a[11], "expected": exp_rows,
                    "tolerance": tol, "line": line}
        if fn == "blur_and_downsample":
            src = self.snapshot(a[0][1])
            return {"func": "blur_and_downsample_u8", "src": src, "width": a[2], "height": a[3],
                    "channels": a[6], "border": a[7], "expected": exp_rows, "tolerance": tol,
                    "line": line}
        raise ValueError(fn)


def extract_kats(ref):
    kats = []
    specs = [
        ("test/api/test_gaussian_blur.cpp", re.compile(r"ValidImageSize(\d+)x\d+$"), "uint8"),
        ("test/api/test_separable_filter_2d.cpp", re.compile(r"5x5_U(8|16)Overflow\w+$"), None),
        ("test/api/test_blur_and_downsample.cpp", re.compile(r"Minimal_u8$"), "uint8"),
    ]
    for rel, pattern, dtype in specs:
        text = open(os.path.join(ref, rel)).read()
        for name, line, body in _blocks(text):
            m = pattern.match(name)
            if not m:
                continue
            ksize = int(m.group(1)) if rel.endswith("gaussian_blur.cpp") else None
            p = KatParser(ksize)
            for st in _statements(body):
                p.statement(st, line)
            assert p.cases, name
            elem = dtype or ("uint8" if m.group(1) == "8" else "uint16")
            for i, c in enumerate(p.cases):
                c["name"] = f"{name}#{i}"
                c["dtype"] = elem
                c["source"] = f"{rel}:{line}"
                kats.append(c)
    return kats


# --------------------------------------------------------------------------

def sigma_fixture():
    out = subprocess.run([os.path.join(ORACLE, "_ref", "sigma_probe")], check=True,
                         capture_output=True, text=True).stdout
    per_k, subset, all_256, copies = {}, {}, True, 0
    keep_k = {3, 5, 7, 9, 11, 15, 21, 31, 63, 127, 255}
    keep_i = {0, 1, 10, 50, 100, 150, 200, 225, 300, 400, 1000, 4000}
    for line in out.splitlines():
        f = [int(v) for v in line.split()]
        k, i, ok, half = f[0], f[1], f[2], f[3:]
        per_k.setdefault(k, hashlib.sha256())
        per_k[k].update((line + "\n").encode())
        if ok:
            all_256 &= 2 * sum(half[:-1]) + half[-1] == 256
        else:
            copies += 1
        if k in keep_k and i in keep_i:
            subset[f"{k}:{i}"] = half if ok else None
    return {"grid": "k = 3..255 odd; sigma = float32(i) / 100, i = 0..4000",
            "line_format": "<k> <i> <ok> <w0> ... <w_half-1> (weights 0 when !ok)",
            "sha256_per_k": {str(k): h.hexdigest() for k, h in per_k.items()},
            "all_weights_sum_to_256": all_256, "copy_cases": copies, "subset": subset}


def border_fixture():
    out = subprocess.run([os.path.join(ORACLE, "_ref", "border_probe")], check=True,
                         capture_output=True, text=True).stdout
    digests, tables = {}, {}
    for line in out.splitlines():
        f = [int(v) for v in line.split()]
        k, b, n = f[0], f[1], f[2]
        key = f"{k}:{b}"
        digests.setdefault(key, hashlib.sha256()).update((line + "\n").encode())
        if n in (k - 1, k):
            tables.setdefault(f"{k}:{b}:{n}", []).append(f[4:])
    return {"extents": "n = K-1 .. K+40, all indices 0..n-1",
            "line_format": "<K> <border> <n> <i> <m_0> ... <m_K-1>",
            "sha256_per_k_border": {k: h.hexdigest() for k, h in digests.items()},
            "tables": tables}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", ORACLE, "ref", f"REF_ROOT={args.ref}"], check=True)
    kats = extract_kats(args.ref)
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": kats}, f)
    with open(os.path.join(HERE, "sigma.json"), "w") as f:
        json.dump(sigma_fixture(), f, indent=0)
    with open(os.path.join(HERE, "border.json"), "w") as f:
        json.dump(border_fixture(), f)
    print(f"{len(kats)} KATs written", file=sys.stderr)


if __name__ == "__main__":
    main()
