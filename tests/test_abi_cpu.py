"""CPU checks of the C-ABI library: it loads, exports every declared entry
point, and its struct layouts match MDZ's own headers."""
import ctypes as C
import json
import re
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MpVal, native
from mdz_gb300 import abi
from oracle.build import ref_root

ROOT = Path(__file__).resolve().parents[1]
GOLD = ROOT / "tests" / "golden"
_REF_ROOT = ref_root()
REF_SRC = _REF_ROOT / "src" if _REF_ROOT else ROOT / "oracle" / "_absent"


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;]*\)\s*;", text, flags=re.M):
            names.append(m.group(1))
    return names


def test_library_builds_and_exports_every_declared_symbol():
    lib = native.load()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers exactly the declared functions
    assert sorted(set(names)) == sorted(set(native.declared_symbols()))


def test_abi_layout_matches_python_mirror():
    lib = native.load()
    out = (C.c_int64 * 128)()
    n = lib.mdzgpu_abi_layout(out, 128)
    assert list(out[:n]) == abi.layout()


def test_abi_layout_matches_reference_fixture():
    """Offsets of MDZ's image_info / rthdata as gcc lays them out from the
    reference headers (tests/golden/abi_layout.json, made by
    make_abi_layout below where the reference is present)."""
    ref = json.loads((GOLD / "abi_layout.json").read_text())
    assert ref["offsets"] == abi.layout()


LAYOUT_C = r"""
#include <stddef.h>
#include <stdio.h>
#include "image_info.h"
#include "render_threads.h"
#define O(f) printf("%ld\n", (long)offsetof(image_info, f));
int main(void) {
  O(xmin) O(xmax) O(ymax) O(width) O(gxmin) O(gxmax) O(gymax) O(gwidth)
  O(old_cx) O(old_cy) O(old_size) O(pcoords) O(depth) O(thread_count) O(draw_lines)
  O(raw_data) O(rgb_data) O(j_pre) O(drawing_area) O(rnd_pal) O(real_width) O(real_height)
  O(user_width) O(user_height) O(aspect) O(aa_factor) O(family) O(fractal) O(colour_scale)
  O(u.julia.c_re) O(u.julia.c_im) O(palette_ip) O(zoom_new_win) O(use_multi_prec)
  O(use_rounding) O(precision) O(multi_prec_init_done) O(rth_ptr) O(lines_drawn)
  O(ui_ref_center)
  printf("%ld\n", (long)sizeof(image_info));
#define R(f) printf("%ld\n", (long)offsetof(rthdata, f));
  R(img) R(lines_drawn) R(min_line_drawn) R(line_draw_count) R(thread_count) R(check_stop_px)
  R(data)
  printf("%ld\n", (long)sizeof(rthdata));
  return 0;
}
"""


def reference_layout(tmp: Path) -> list[int]:
    src = tmp / "layout.c"
    src.write_text(LAYOUT_C)
    exe = tmp / "layout"
    subprocess.run(["gcc", "-std=gnu99", "-w", "-I", str(ROOT / "oracle" / "shim"), "-I",
                    str(REF_SRC), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return [int(x) for x in out.split()]


@pytest.mark.skipif(not (REF_SRC / "image_info.h").exists(), reason="reference sources absent")
def test_abi_layout_matches_reference_headers(tmp_path):
    assert reference_layout(tmp_path) == abi.layout()


def exact_fixed(v: Fraction, words: int) -> int:
    F = 32 * words - 8
    x = v * (1 << F)
    q = x.numerator // x.denominator if x >= 0 else -((-x.numerator) // x.denominator)
    return q % (1 << (32 * words))


@pytest.mark.parametrize("words", [4, 10, 34])
def test_fixed_point_conversion_is_exact_truncation(words):
    lib = native.load()
    rng = np.random.default_rng(5)
    for _ in range(40):
        e = int(rng.integers(-700, 2))
        mant = int(rng.integers(1, 1 << 62)) | (1 << 62)
        sign = 1 if rng.random() < 0.5 else -1
        val = Fraction(sign * mant, 1) * Fraction(2) ** (e - 63)
        if abs(val) >= 4:
            continue
        mv = MpVal.from_fraction(val, 200)
        s, keep = mv.struct()
        out = (C.c_uint32 * words)()
        assert lib.mdzgpu_fx_from_mpval(C.byref(s), words, out) == 0
        got = sum(int(out[i]) << (32 * i) for i in range(words))
        # magnitude truncated toward zero, then negated
        F = 32 * words - 8
        mag = abs(mv.to_fraction()) * (1 << F)
        q = mag.numerator // mag.denominator
        want = q if sign > 0 else (-q) % (1 << (32 * words))
        assert got == want


def test_fixed_point_rejects_out_of_range():
    lib = native.load()
    s, keep = MpVal.from_fraction(300, 64).struct()
    out = (C.c_uint32 * 4)()
    assert lib.mdzgpu_fx_from_mpval(C.byref(s), 4, out) == -4  # MDZGPU_ERR_RANGE


def test_perturb_spacing_is_40_bits():
    from mdz_gb300 import perturb_spacing
    w = MpVal.from_fraction(Fraction(1, 2 ** 1000), 1088)
    m, e = perturb_spacing(w, 1920)
    assert 1.0 <= m < 2.0
    assert (Fraction(m) * 2 ** 39).denominator == 1
    hs = Fraction(m) * Fraction(2) ** e
    exact = Fraction(1, 2 ** 1000) / 3840
    assert abs(hs - exact) / exact < Fraction(1, 2 ** 39)


def mpfr_pixel_c(rect, W, prec, ix, line):
    """fractal_mpfr_calculate_line's c (src/fractal.c:167-186), each MPFR
    call an exact operation rounded to nearest at `prec` bits."""
    def rn(x):
        return MpVal.from_fraction(x, prec).to_fraction()
    width, xmin, ymax = (rn(v.to_fraction()) for v in (rect.width, rect.xmin, rect.ymax))
    y = rn(ymax - rn(rn(width / W) * line))
    x = rn(rn(rn(Fraction(ix, W)) * width) + xmin)
    return x, y


@pytest.mark.parametrize("prec,cx,cy,size,W,H", [
    (80, "-1.7495931476527795538", "5.79e-8", "2.3e-17", 40, 30),
    (128, "-0.7436447860", "0.1318252536", "1e-30", 33, 17),
    (256, "0.3750001", "-0.44", "0x1p-200", 64, 48),
    (1088, "-0.1592", "1.0317", "0x1p-1000", 24, 12),
])
def test_mp_coordinates_equal_mpfr_roundings(prec, cx, cy, size, W, H):
    from mdz_gb300.views import mdz_rect
    lib = native.load()
    words = max(4, -(-(prec + 40) // 32))
    words += words & 1
    r = mdz_rect(W, H, prec, cx, cy, size)
    xs = (C.c_uint32 * (W * words))()
    ys = (C.c_uint32 * (H * words))()
    args = [v.struct() for v in (r.xmin, r.ymax, r.width)]
    assert lib.mdzgpu_mp_coordinates(*[C.byref(a) for a, _ in args], W, 0, H, prec, words,
                                      xs, ys) == 0
    F = 32 * words - 8

    def fixed(arr, k):
        v = sum(int(arr[k * words + i]) << (32 * i) for i in range(words))
        if v >> (32 * words - 1):
            v -= 1 << (32 * words)
        return Fraction(v, 1 << F)
    for ix in range(W):
        x, _ = mpfr_pixel_c(r, W, prec, ix, 0)
        assert fixed(xs, ix) == x
    for ln in range(H):
        _, y = mpfr_pixel_c(r, W, prec, 0, ln)
        assert fixed(ys, ln) == y


def test_python_half_spacing_equals_library():
    """The perturbation geometry's 40-bit half spacing, computed in Python
    (used where the library must not be loaded: the CPU baseline), equals
    mdzgpu_perturb_spacing on seeded widths and frame sizes."""
    from mdz_gb300 import perturb_spacing
    from mdz_gb300.views import perturb_half_spacing
    rng = np.random.default_rng(17)
    cases = [(MpVal.from_fraction(Fraction(2) ** -1000, 1088), 1920),
             (MpVal.from_fraction(Fraction(3), 80), 240)]
    for _ in range(300):
        e = int(rng.integers(-1100, 3))
        num = int(rng.integers(1, 1 << 62))
        prec = int(rng.choice([64, 80, 256, 1088, 2176]))
        W = int(rng.integers(1, 8000))
        cases.append((MpVal.from_fraction(Fraction(num, 1 << 62) * Fraction(2) ** e, prec), W))
    for w, W in cases:
        assert perturb_half_spacing(w, W) == perturb_spacing(w, W), (w, W)


# the explicit C API's structs: the ctypes mirrors in mdz_gb300/native.py
# against the header, field by field (offsets and sizes from gcc)
NATIVE_STRUCTS = [("Frame", "mdzgpu_frame"), ("Stats", "mdzgpu_stats"),
                  ("MpValStruct", "mdzgpu_mpval"), ("Palette", "mdzgpu_palette"),
                  ("ServeConfig", "mdzgpu_serve_config"), ("Request", "mdzgpu_request"),
                  ("RequestStatus", "mdzgpu_request_status"),
                  ("ServeStats", "mdzgpu_serve_stats")]


def test_native_structs_match_header(tmp_path):
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "mdzgpu.h"', "int main(void) {"]
    want = []
    for py, cname in NATIVE_STRUCTS:
        cls = getattr(native, py)
        lines.append(f'  printf("%ld\\n", (long)sizeof({cname}));')
        want.append((cname, "sizeof", C.sizeof(cls)))
        for f, _ in cls._fields_:
            lines.append(f'  printf("%ld\\n", (long)offsetof({cname}, {f}));')
            want.append((cname, f, getattr(cls, f).offset))
    lines += ["  return 0;", "}"]
    src = tmp_path / "native_layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "native_layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    bad = [(c, f, g, w) for (c, f, w), g in zip(want, got) if g != w]
    assert len(got) == len(want) and not bad, bad
