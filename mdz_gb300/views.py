"""MDZ view geometry: centre/size -> the rectangle the line functions read.

The drop-in layer receives img->xmin/xmax/ymax/width already computed by
MDZ's own coords.c.  The explicit API and bench.py need the same values, so
this module restates that computation exactly, each MPFR call being an exact
rational operation rounded to nearest at the destination precision:
  coords precision  src/coords.c:204-231 (GMP limb rounding of max(p, 80))
  centre -> rect    src/coords.c:265-302 (coords_center_to_rect)
  img-> precision   src/image_info.c:252-280 (max(p, 80))
  aspect            src/image_info.c:118 ((double) w / h)
  size parsing      src/setting.c:179-200 (mpfr_set_str at p bits)
A CPU test checks every value against the reference's own coords.c.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from fractions import Fraction

from .mpval import MpVal, parse_number


def coords_precision(p: int) -> int:
    """Bits of the coords struct's MPFR values for a requested precision."""
    n = max(p, 80)
    return 64 * ((n + 63) // 64)


def img_precision(p: int) -> int:
    return max(p, 80)


def _r(x: Fraction, prec: int) -> Fraction:
    return MpVal.from_fraction(x, prec).to_fraction()


@dataclass
class Rect:
    xmin: MpVal
    xmax: MpVal
    ymax: MpVal
    width: MpVal

    def doubles(self) -> tuple[float, float, float]:
        """mpfr_get_ld(..., GMP_RNDN) with long double = IEEE double."""
        return (float(self.xmin.to_fraction()), float(self.xmax.to_fraction()),
                float(self.ymax.to_fraction()))


def mdz_rect(user_w: int, user_h: int, precision: int, cx: str | Fraction,
             cy: str | Fraction, size: str | Fraction, input_prec: int | None = None) -> Rect:
    """xmin, xmax, ymax, width of image_info after render.c:34-35.  cx, cy,
    size are first rounded to `input_prec` bits (default: the view's
    precision, as mpfr_set_str into a p-bit variable does); values that
    already sit in the coords struct (e.g. a centre computed from a
    rectangle) pass input_prec = coords_precision(precision)."""
    P = coords_precision(precision)
    Pi = img_precision(precision)
    ip = precision if input_prec is None else input_prec
    cxv = _r(parse_number(cx) if isinstance(cx, str) else Fraction(cx), ip)
    cyv = _r(parse_number(cy) if isinstance(cy, str) else Fraction(cy), ip)
    sz = _r(parse_number(size) if isinstance(size, str) else Fraction(size), ip)
    aspect = Fraction(user_w / user_h)  # a double, exactly
    if aspect > 1:
        width = _r(sz, P)
        height = _r(width / aspect, P)
        tmp = _r(width / 2, P)
        xmin = _r(cxv - tmp, P)
        xmax = _r(xmin + width, P)
        tmp = _r(tmp / aspect, P)
        ymin = _r(cyv - tmp, P)
        ymax = _r(ymin + height, P)
    else:
        height = _r(sz, P)
        width = _r(height * aspect, P)
        tmp = _r(height / 2, P)
        ymin = _r(cyv - tmp, P)
        ymax = _r(ymin + height, P)
        tmp = _r(tmp * aspect, P)
        xmin = _r(cxv - tmp, P)
        xmax = _r(xmin + width, P)
    return Rect(MpVal.from_fraction(xmin, Pi), MpVal.from_fraction(xmax, Pi),
                MpVal.from_fraction(ymax, Pi), MpVal.from_fraction(width, Pi))


@dataclass
class View:
    """One MDZ render request (the settings a .mdz file carries)."""
    name: str
    width: int                 # user (output) pixels
    height: int
    depth: int
    cx: str
    cy: str
    size: str                  # real-axis width when width > height
    precision: int = 80
    aa: int = 1
    family: int = 0
    fractal: int = 0
    multi_prec: bool = False
    rounding: bool = True
    julia_re: str = "0"
    julia_im: str = "0"
    extra: dict = field(default_factory=dict)

    @property
    def real_width(self) -> int:
        return self.width * self.aa

    @property
    def real_height(self) -> int:
        return self.height * self.aa

    def rect(self) -> Rect:
        return mdz_rect(self.width, self.height, self.precision, self.cx, self.cy, self.size,
                        self.extra.get("coords_input_prec"))

    def julia(self) -> tuple[MpVal, MpVal]:
        """u.julia.c_re / c_im as image_info holds them: c_re at max(p, 80)
        bits, c_im left at 80 bits (image_info_set_precision changes c_re
        twice, src/image_info.c:270-271)."""
        re_ = _r(parse_number(self.julia_re), self.precision)
        im_ = _r(parse_number(self.julia_im), self.precision)
        return (MpVal.from_fraction(re_, img_precision(self.precision)),
                MpVal.from_fraction(im_, 80))

    @staticmethod
    def from_dict(d: dict) -> "View":
        keys = {f for f in View.__dataclass_fields__} - {"extra"}
        extra = dict(d.get("extra") or {})
        extra.update({k: v for k, v in d.items() if k not in keys and k != "extra"})
        return View(**{k: v for k, v in d.items() if k in keys}, extra=extra)


def perturb_half_spacing(width: MpVal, W: int) -> tuple[float, int]:
    """Half pixel spacing of the perturbation geometry, (hs_m, hs_e) with
    hs = hs_m * 2^hs_e: the top 53 bits of `width` (truncated), divided by
    2 W in double (round to nearest), then rounded to 40 significant bits
    (ties to even), so that (2 ix - W) * hs is exact in FP64 for every pixel.
    Pure Python; the library's mdzgpu_perturb_spacing computes the same."""
    import math
    if width.mant <= 0 or W <= 0:
        raise ValueError("perturbation needs a positive width")
    n = width.nlimbs
    top = width.mant >> (64 * (n - 1))
    mant = float(top >> 11)                   # exact: 53 bits
    e0 = width.exp - 53
    q = mant / (2.0 * W)
    k = math.frexp(q)[1] - 1                  # ilogb
    m = math.ldexp(q, -k)                     # [1, 2)
    m = math.ldexp(float(round(math.ldexp(m, 39))), -39)
    return m, e0 + k
