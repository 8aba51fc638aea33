"""MDZ settings files (.mdz): reading them exactly as MDZ's headless render does.

Restates, line for line in behaviour:
  mdzfile_read_open / mdzfile_read / mdzfile_test_for_name /
  mdzfile_skip_to / mdzfile_get_*      src/mdzfileio.c
  setting_get_index / _long / _double / _mpfr_t / _version   src/setting.c
  image_info_load_settings             src/image_info.c:456-721
  image_info_load_palette, _load_all   src/image_info.c:724-788
  palette_read (RGB packing)           src/palette.c:142-167, src/palette.h
  init_misc's output size              src/main.c (width / height / aa)
The resulting view is what MDZ's line callbacks read: `MdzSettings.view()`
gives an mdz_gb300.View whose rect() equals img->xmin/xmax/ymax/width after
coords_get_rect (checked against the reference's own loader on every file of
its gallery).  One property of MDZ is kept on purpose: a file that gives the
rectangle form (xmin/xmax/ymax) is rendered around the rectangle's centre at
the *default* size 4.0, because coords_set (called when the image size is
set) restores the size from coords->_size, which the rectangle form never
sets (src/coords.c:255-262, :327-333); `intended_view()` gives the
rectangle the file describes instead.

Settings written by MDZ 0.1.x (header "mdz fractal settings 0.1.2") and the
older 0.0.x form (no version; "fractal <family>", "mpfr yes|no") are read.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from fractions import Fraction
from pathlib import Path

from .mpval import MpVal, hexfloat
from .views import View, coords_precision

HEADER = "mdz fractal settings"
FBUFLEN = 4096
FAMILY_STR = ["mandelbrot", "julia"]                       # src/fractal.c:11-16
FRACTAL_STR = ["mandelbrot", "burning ship", "generalized celtic",
               "mandel-celtic hybrid"]                      # src/fractal.c:19-26
NO_YES = ["no", "yes"]                                      # src/setting.c:12
COORDS_STR = ["cx", "xmin"]                                 # src/image_info.c:24
PALOFF_STR = "palette-offset"                               # src/image_info.c:25
MIN_DEPTH, MAX_DEPTH = 1, 2 ** 31 - 1                      # src/image_info.h:19-20
DEFAULT_WIDTH = 480                                         # src/image_info.h:22
DEFAULT_SIZE = Fraction(4)                                  # src/image_info.c:33


class MdzFileError(ValueError):
    pass


def rgb(r: int, g: int, b: int) -> int:
    """RGB() of src/palette.h on a little-endian host, on C ints."""
    return ((r | (g << 8) | (b << 16)) & 0xFFFFFFFF)


class _Reader:
    """mdzfile: sequential line reader with one line of push-back."""

    def __init__(self, text: str, name: str):
        self.name = name
        # fgets(buf, FBUFLEN): pieces of at most FBUFLEN - 1 characters
        self.chunks = []
        for line in text.splitlines(keepends=True):
            while len(line) > FBUFLEN - 1:
                self.chunks.append(line[:FBUFLEN - 1])
                line = line[FBUFLEN - 1:]
            self.chunks.append(line)
        self.pos = 0
        self.line = ""
        self.test = None
        self.eof = False

    @staticmethod
    def _tidy(s: str) -> str:
        out = []
        for ch in s:
            if ch == "\t":
                ch = " "
            elif ch < " ":
                break
            out.append(ch)
        return "".join(out)

    def fgets(self, n: int = FBUFLEN):
        if self.pos >= len(self.chunks):
            return None
        s = self.chunks[self.pos]
        self.pos += 1
        return s

    def read(self) -> bool:
        if self.eof:
            return False
        while True:
            if self.test is not None:
                buf, self.test = self.test, None
            else:
                buf = self.fgets()
                if buf is None:
                    self.eof = True
                    return False
            self.line = self._tidy(buf)
            if not self.line.startswith("#"):
                return True

    def test_for_name(self, name: str) -> bool:
        if not self.read():
            return False
        self.test = self.line
        return len(self.line) >= len(name) + 2 and self.line.startswith(name)

    def skip_to(self, line: str) -> bool:
        while self.read():
            if self.line == line:
                return True
        return False

    # mdzfile_get_*: each reads the next line first
    def get_index(self, name, options):
        if not self.read():
            return 0
        return setting_get_index(self.line, name, options)

    def get_long(self, name, lo, hi):
        if not self.read():
            return None
        return setting_get_long(self.line, name, lo, hi)

    def get_double(self, name, lo, hi):
        if not self.read():
            return None
        return setting_get_double(self.line, name, lo, hi)

    def get_mpfr(self, name, prec):
        if not self.read():
            return None
        return setting_get_mpfr(self.line, name, prec)

    def get_name_index(self, names):
        if not self.read():
            return -1
        s = self.line
        i = 0
        while i < len(s) and s[i] == " ":
            i += 1
        while i < len(s) and s[i] != " ":
            i += 1
        return setting_get_index(s[:i], None, names)


def setting_get_index(buf: str, name, options) -> int:
    if name is not None:
        if len(buf) < len(name) + 2 or not buf.startswith(name):
            return 0   # the reference returns `false` here
        buf = buf[len(name):]
    opt = buf.lstrip(" ")
    for i, o in enumerate(options):
        if opt == o:
            return i
    return -1


_LONG = re.compile(r"\s*([+-]?\d+)")
_DOUBLE = re.compile(r"\s*([+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan))",
                     re.IGNORECASE)
_MPFR10 = re.compile(r"\s*([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE@][+-]?\d+)?)")


def setting_get_long(buf: str, name: str, lo: int, hi: int):
    if len(buf) < len(name) + 1 or not buf.startswith(name):
        return None
    m = _LONG.match(buf[len(name):])
    if not m:
        return None
    v = int(m.group(1))
    if (lo or hi) and not lo <= v <= hi:
        return None
    return v


def setting_get_double(buf: str, name: str, lo: float, hi: float):
    if len(buf) < len(name) + 1 or not buf.startswith(name):
        return None
    m = _DOUBLE.match(buf[len(name):])
    if not m:
        return None
    v = float(m.group(1))   # strtod: correctly rounded
    if (lo or hi) and not lo <= v <= hi:
        return None
    return v


def setting_get_mpfr(buf: str, name: str, prec: int):
    """mpfr_set_str(val, buf + len(name), 10, RNDN) into a prec-bit value:
    the whole rest of the line must be one base-10 number."""
    if len(buf) < len(name) + 1 or not buf.startswith(name):
        return None
    rest = buf[len(name):]
    m = _MPFR10.fullmatch(rest)
    if not m:
        return None
    s = m.group(1).replace("@", "e")
    return MpVal.from_fraction(Fraction(s), prec).to_fraction()


def setting_get_version(buf: str):
    m = re.match(r"\s*([+-]?\d+)\.([+-]?\d+)\.([+-]?\d+)", buf)
    if not m:
        return None
    return tuple(int(x) for x in m.groups())


def _r(x: Fraction, prec: int) -> Fraction:
    return MpVal.from_fraction(x, prec).to_fraction()


@dataclass
class MdzSettings:
    """What MDZ's headless render takes from a settings file."""
    name: str
    version: tuple
    family: int
    fractal: int
    depth: int
    aspect: float
    colour_scale: float
    palette_ip: bool
    multi_prec: bool
    rounding: bool
    precision: int
    centre_form: bool
    cx: Fraction | None = None
    cy: Fraction | None = None
    size: Fraction | None = None
    xmin: Fraction | None = None
    xmax: Fraction | None = None
    ymax: Fraction | None = None
    julia_re: Fraction = Fraction(0)
    julia_im: Fraction = Fraction(0)
    palette_offset: int = 0
    random_palette: dict | None = None
    palette: list = field(default_factory=list)   # guint32 colours (pal_indexes)
    palette_file: str | None = None

    def output_size(self, width: int = 0, height: int = 0, aa: int = 0) -> tuple[int, int, int]:
        """init_misc (src/main.c): the -W / -H / -a options (0 = unset)
        against the size the loader set (w = 480, h = (int)(480 / aspect))."""
        w0 = DEFAULT_WIDTH
        h0 = int(w0 / self.aspect)
        img_aspect = w0 / h0
        w, h = width, height
        if not w and not h:
            w, h = w0, h0
        elif not w:
            w = int(h * img_aspect)
        elif not h:
            h = int(w / img_aspect)
        return w, h, (aa or 1)

    def _centre(self) -> tuple[Fraction, Fraction, Fraction]:
        """coords cx, cy and _size after loading."""
        if self.centre_form:
            return self.cx, self.cy, self.size
        # coords_set_rect + coords_rect_to_center at coords precision, with
        # the aspect the loader set (480 / (int)(480 / aspect))
        P = coords_precision(self.precision)
        w0 = DEFAULT_WIDTH
        aspect0 = Fraction(w0 / int(w0 / self.aspect))
        width = _r(self.xmax - self.xmin, P)
        height = _r(width / aspect0, P)
        ymin = _r(self.ymax - height, P)
        cx = _r(self.xmin + self.xmax, P) / 2
        cy = _r(ymin + self.ymax, P) / 2
        return cx, cy, DEFAULT_SIZE

    def view(self, width: int = 0, height: int = 0, aa: int = 0, name: str | None = None) -> View:
        """The view MDZ renders (`mdz -s file.mdz [-W w -H h -a aa]`)."""
        w, h, a = self.output_size(width, height, aa)
        cx, cy, size = self._centre()
        v = View(name or self.name, w, h, self.depth, hexfloat(cx), hexfloat(cy),
                 hexfloat(size), precision=self.precision, aa=a, family=self.family,
                 fractal=self.fractal, multi_prec=self.multi_prec, rounding=self.rounding,
                 julia_re=hexfloat(self.julia_re), julia_im=hexfloat(self.julia_im))
        if not self.centre_form:
            # the centre was computed in the coords struct at its precision
            v.extra["coords_input_prec"] = coords_precision(self.precision)
        return v

    def intended_view(self, width: int = 0, height: int = 0, aa: int = 0) -> View:
        """The rectangle-form file's own rectangle as a centre/size view
        (same as view() for centre-form files)."""
        if self.centre_form:
            return self.view(width, height, aa)
        v = self.view(width, height, aa)
        v.extra.pop("coords_input_prec", None)
        v.cx = hexfloat((self.xmin + self.xmax) / 2)
        v.size = hexfloat(self.xmax - self.xmin)
        v.cy = hexfloat(self.ymax - (self.xmax - self.xmin) * v.height / v.width / 2)
        return v


def loads(text: str, name: str = "settings", base_dir: Path | None = None) -> MdzSettings:
    """Parse the text of a .mdz file (image_info_load_all with the
    settings and palette sections)."""
    mf = _Reader(text, name)
    if not mf.read() or not mf.line.startswith(HEADER):
        raise MdzFileError(f"{name}: not a recognisable mdz file")
    ver = mf.line[len(HEADER):].lstrip(" ") or "0.0.8"
    version = setting_get_version(ver)
    if version is None:
        raise MdzFileError(f"{name}: error in mdz file header/version")
    old = version[0] == 0 and version[1] == 0

    def err(msg):
        raise MdzFileError(f"{name}: {msg}")

    if not mf.read():
        err("expected settings section")
    if old:
        family = mf.get_index("fractal", FAMILY_STR)
        if family == -1:
            err("error in fractal setting")
        fractal = 0
    else:
        family = mf.get_index("family", FAMILY_STR)
        if family == -1:
            err("error in family setting")
        fractal = mf.get_index("fractal", FRACTAL_STR)
        if fractal == -1:
            err("error in fractal setting")
    depth = mf.get_long("depth", MIN_DEPTH, MAX_DEPTH)
    if depth is None:
        err("Error in depth setting")
    # (double)1e-20f and (double)1e20f: the bounds are float constants
    lo, hi = float(__import__("numpy").float32(1e-20)), float(__import__("numpy").float32(1e20))
    aspect = mf.get_double("aspect", lo, hi)
    if aspect is None:
        err("Error in aspect setting")
    colsc = mf.get_double("colour-scale", lo, hi)
    if colsc is None:
        err("Error in colour-scale setting")
    colip = mf.get_index("colour-interpolate", NO_YES)
    if colip == -1:
        err("Error in colour-interpolate setting")
    if old:
        mp = mf.get_index("mpfr", NO_YES)
        if mp == -1:
            err("Error in mpfr setting")
        rounding = 1
    else:
        mp = mf.get_index("multi-precision", NO_YES)
        if mp == -1:
            err("Error in multi-precision setting")
        rounding = mf.get_index("multi-rounding", NO_YES)
        if rounding == -1:
            err("Error in multi-rounding setting")
    precision = mf.get_long("precision", 80, 99999999)
    if precision is None:
        err("Error in precision setting")
    ctype = mf.get_name_index(COORDS_STR)
    if ctype == -1:
        err("Error in coordinates setting")
    s = MdzSettings(name, version, family, fractal, depth, aspect, colsc, bool(colip),
                    bool(mp), bool(rounding), precision, ctype == 0)
    if s.centre_form:
        s.cx = setting_get_mpfr(mf.line, "cx", precision)
        if s.cx is None:
            err("Error in cx setting")
        s.cy = mf.get_mpfr("cy", precision)
        if s.cy is None:
            err("Error in cy setting")
        s.size = mf.get_mpfr("size", precision)
        if s.size is None:
            err("Error in size setting")
    else:
        s.xmin = setting_get_mpfr(mf.line, "xmin", precision)
        if s.xmin is None:
            err("Error in xmin setting")
        s.xmax = mf.get_mpfr("xmax", precision)
        if s.xmax is None:
            err("Error in xmax setting")
        s.ymax = mf.get_mpfr("ymax", precision)
        if s.ymax is None:
            err("Error in ymax setting")
    if family == 1:
        s.julia_re = mf.get_mpfr("julia-real", precision)
        if s.julia_re is None:
            err("Error in julia-real setting")
        s.julia_im = mf.get_mpfr("julia-imag", precision)
        if s.julia_im is None:
            err("Error in julia-imag setting")
    if mf.test_for_name(PALOFF_STR):
        off = mf.get_long(PALOFF_STR, 0, 255)
        if off is None:
            err("Error in palette offset setting")
        s.palette_offset = off
    if mf.test_for_name("r-strength"):
        rp = {}
        for key in ("r-strength", "r-bands", "g-strength", "g-bands", "b-strength",
                    "b-bands"):
            v = mf.get_double(key, 0.0, 1.0)
            if v is None:
                err(f"Error in {key} setting")
            rp[key] = v
        for key in ("rnd-offset", "rnd-stripe", "rnd-spread"):
            v = mf.get_long(key, 0, 255)
            if v is None:
                err(f"Error in {key} setting")
            rp[key] = v
        s.random_palette = rp
    # palette section
    if not mf.skip_to("palette"):
        err("expected palette section")
    if not mf.read():
        err("palette missing data")
    if mf.line == "data":
        s.palette = _palette_read(mf.fgets)
    elif mf.line.startswith("file") and len(mf.line) >= len("file") + 2:
        fn = mf.line[len("file"):].lstrip(" ")
        s.palette_file = fn
        p = Path(fn)
        if not p.is_absolute() and base_dir is not None:
            p = base_dir / p
        try:
            text = p.read_text()
        except OSError:
            # palette_load fails, and with it the whole load
            err(f"palette file {fn} can not be read")
        s.palette = _palette_read(_Reader(text, str(p)).fgets)
    else:
        err("palette data error")
    if not s.palette:
        err("failed to read the palette")
    return s


def _palette_read(fgets) -> list[int]:
    """palette_read (src/palette.c:142-167): up to 256 ' r g b' lines."""
    out = []
    pat = re.compile(r"\s*([+-]?\d+)\s*([+-]?\d+)\s*([+-]?\d+)")
    while True:
        buf = fgets(256)
        if buf is None or len(out) >= 256:
            break
        m = pat.match(buf)
        if not m:
            break
        out.append(rgb(*(int(x) & 0xFFFFFFFF if int(x) >= 0 else int(x) for x in m.groups())))
    return out


def load(path: str | Path) -> MdzSettings:
    p = Path(path)
    return loads(p.read_text(), p.stem, base_dir=p.parent)


def dumps(s: MdzSettings) -> str:
    """A settings file in MDZ 0.1.2's layout (image_info_save_settings,
    src/image_info.c:335-420) with decimal coordinates that round back to
    the same values, and the palette embedded as data."""
    def dec(x: Fraction) -> str:
        # enough significant digits to round-trip at the precision
        digits = int(math.ceil(s.precision * math.log10(2))) + 2
        if x == 0:
            return "0"
        sign = "-" if x < 0 else ""
        a = abs(x)
        e = math.floor(math.log10(a.numerator) - math.log10(a.denominator))
        q = a / Fraction(10) ** (e - digits + 1)
        n = round(q)
        return f"{sign}{n}e{e - digits + 1}"
    lines = [f"{HEADER} 0.1.2", "settings",
             f"family {FAMILY_STR[s.family]}", f"fractal {FRACTAL_STR[s.fractal]}",
             f"depth {s.depth}", f"aspect {s.aspect:.20f}", f"colour-scale {s.colour_scale:.20f}",
             f"colour-interpolate {NO_YES[int(s.palette_ip)]}",
             f"multi-precision {NO_YES[int(s.multi_prec)]}",
             f"multi-rounding {NO_YES[int(s.rounding)]}", f"precision {s.precision}"]
    if s.centre_form:
        lines += [f"cx {dec(s.cx)}", f"cy {dec(s.cy)}", f"size {dec(s.size)}"]
    else:
        lines += [f"xmin {dec(s.xmin)}", f"xmax {dec(s.xmax)}", f"ymax {dec(s.ymax)}"]
    if s.family == 1:
        lines += [f"julia-real {dec(s.julia_re)}", f"julia-imag {dec(s.julia_im)}"]
    lines += [f"{PALOFF_STR} {s.palette_offset}", "palette", "data"]
    lines += [f" {c & 0xff} {(c >> 8) & 0xff} {(c >> 16) & 0xff}" for c in s.palette]
    return "\n".join(lines) + "\n"
