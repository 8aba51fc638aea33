"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It exposes
  * the restatement in oracle/mdz_oracle.c (libmdzoracle.so), and
  * the unmodified reference compiled by oracle/build_ref.sh
    (oracle/_ref/libmdzref_{d,ld}.so), present only where the reference
    sources are (this container, x86-64).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_D = HERE / "_ref" / "libmdzref_d.so"
REF_LD = HERE / "_ref" / "libmdzref_ld.so"

_orc = None
_refs: dict[str, C.CDLL] = {}


def lib() -> C.CDLL:
    global _orc
    if _orc is None:
        from . import build as _b
        path = _b.build(reference=False)
        L = C.CDLL(str(path))
        L.mdzo_render_fp64.restype = C.c_int64
        L.mdzo_render_fp64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int,
                                       C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_int, C.c_void_p]
        L.mdzo_render_fp64_rows.restype = C.c_int64
        L.mdzo_render_fp64_rows.argtypes = [C.c_int] * 4 + [C.c_int64, C.c_int, C.c_int] + \
            [C.c_double] * 5 + [C.c_int, C.c_void_p]
        L.mdzo_point_fp64.restype = C.c_int64
        L.mdzo_point_fp64.argtypes = [C.c_int, C.c_int64, C.c_double, C.c_double]
        L.mdzo_colour.restype = C.c_int
        L.mdzo_colour.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.mdzo_has_mpfr.restype = C.c_int
        if L.mdzo_has_mpfr():
            L.mdzo_render_mpfr.restype = C.c_int64
            L.mdzo_render_mpfr.argtypes = ([C.c_int] * 4 + [C.c_int64, C.c_int, C.c_int, C.c_long]
                                           + [C.c_char_p, C.c_long] * 5 + [C.c_int, C.c_void_p])
            L.mdzo_points_mpfr.restype = C.c_int
            L.mdzo_points_mpfr.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_long,
                                           C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                           C.c_int, C.c_void_p, C.c_void_p]
            L.mdzo_points_julia_mpfr.restype = C.c_int
            L.mdzo_points_julia_mpfr.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_long,
                                                 C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                                 C.c_char_p, C.c_char_p, C.c_int, C.c_void_p,
                                                 C.c_void_p]
        _orc = L
    return _orc


def has_mpfr() -> bool:
    return bool(lib().mdzo_has_mpfr())


def render_fp64(W, H, depth, xmin, xmax, ymax, family=0, fractal=0, julia=(0.0, 0.0),
                aa=1, threads=1):
    out = np.empty((H, W), np.int32)
    its = lib().mdzo_render_fp64(W, H, aa, depth, family, fractal, xmin, xmax, ymax, julia[0],
                                 julia[1], threads, out.ctypes.data)
    return out, int(its)


def render_fp64_rows(W, H, row0, nrows, depth, xmin, xmax, ymax, family=0, fractal=0,
                     julia=(0.0, 0.0), threads=1):
    out = np.empty((nrows, W), np.int32)
    lib().mdzo_render_fp64_rows(W, H, row0, nrows, depth, family, fractal, xmin, xmax, ymax,
                                julia[0], julia[1], threads, out.ctypes.data)
    return out


def render_mpfr(W, H, depth, prec, xmin, ymax, width, family=0, fractal=0, julia=None,
                row0=0, nrows=None, threads=1):
    """Values are mdz_gb300.MpVal; each is parsed at its own precision."""
    from mdz_gb300.mpval import MpVal
    if nrows is None:
        nrows = H - row0
    jre, jim = julia if julia is not None else (MpVal.zero(80), MpVal.zero(80))
    out = np.empty((nrows, W), np.int32)
    args = []
    for v in (xmin, ymax, width, jre, jim):
        args += [v.hex().encode(), max(v.prec, 2)]
    its = lib().mdzo_render_mpfr(W, H, row0, nrows, depth, family, fractal, prec, *args,
                                 threads, out.ctypes.data)
    return out, int(its)


def colour(raw: np.ndarray, aa: int, interpolate: bool, scale: float, palette, offset: int = 0):
    """MDZ's colouring of raw counts (palette_apply for aa = 1,
    do_anti_aliasing for aa > 1): uint32 [H/aa][W/aa], r | g << 8 | b << 16."""
    raw = np.ascontiguousarray(raw, dtype=np.int32)
    H, W = raw.shape
    pal = np.ascontiguousarray(palette, dtype=np.uint32)
    out = np.zeros((H // aa, W // aa), np.uint32)
    if not lib().mdzo_colour(raw.ctypes.data, W, H, aa, int(interpolate), float(scale),
                             pal.ctypes.data, len(pal), offset, out.ctypes.data):
        raise ValueError("bad colouring arguments")
    return out


def points_mpfr(cre: list[str], cim: list[str], depth: int, prec: int, fractal=0, threads=1):
    n = len(cre)
    a = (C.c_char_p * n)(*[s.encode() for s in cre])
    b = (C.c_char_p * n)(*[s.encode() for s in cim])
    counts = np.empty(n, np.int64)
    mag = np.empty(n, np.float64)
    lib().mdzo_points_mpfr(n, fractal, depth, prec, a, b, threads, counts.ctypes.data,
                           mag.ctypes.data)
    return counts, mag


def points_julia_mpfr(zre, zim, jre: str, jim: str, depth, prec, fractal=0, threads=1):
    """Julia family: z0 = the listed points, c = (jre, jim)."""
    n = len(zre)
    a = (C.c_char_p * n)(*[s.encode() for s in zre])
    b = (C.c_char_p * n)(*[s.encode() for s in zim])
    counts = np.empty(n, np.int64)
    lib().mdzo_points_julia_mpfr(n, fractal, depth, prec, a, b, jre.encode(), jim.encode(),
                                 threads, counts.ctypes.data, None)
    return counts


# ---- the unmodified reference (only where it was compiled) ----

def ref_available(variant: str = "d") -> bool:
    return (REF_D if variant == "d" else REF_LD).exists()


def ref(variant: str = "d") -> C.CDLL:
    if variant not in _refs:
        L = C.CDLL(str(REF_D if variant == "d" else REF_LD))
        L.mdzref_render.restype = C.c_int
        L.mdzref_render.argtypes = ([C.c_int] * 3 + [C.c_long] + [C.c_int] * 4 + [C.c_long]
                                    + [C.c_char_p] * 5 + [C.c_int, C.c_void_p,
                                                          C.POINTER(C.c_double),
                                                          C.POINTER(C.c_double)])
        L.mdzref_view_dump.restype = C.c_int
        L.mdzref_view_dump.argtypes = ([C.c_int] * 3 + [C.c_long] + [C.c_int] * 4 + [C.c_long]
                                       + [C.c_char_p] * 5 + [C.c_char_p, C.c_long])
        L.mdzref_point_mpfr.restype = C.c_long
        L.mdzref_point_mpfr.argtypes = [C.c_int, C.c_long, C.c_long, C.c_char_p, C.c_char_p]
        L.mdzref_point_hw.restype = C.c_long
        L.mdzref_point_hw.argtypes = [C.c_int, C.c_long, C.c_double, C.c_double]
        _refs[variant] = L
    return _refs[variant]


def _view_args(v):
    return (v.width, v.height, v.aa, v.depth, v.family, v.fractal, int(v.multi_prec),
            int(v.rounding), v.precision, v.cx.encode(), v.cy.encode(), v.size.encode(),
            v.julia_re.encode(), v.julia_im.encode())


def ref_render(v, threads=8, variant="d"):
    """Render a View through the reference's own rth_* + fractal.c."""
    out = np.empty((v.real_height, v.real_width), np.int32)
    t = C.c_double()
    t2 = C.c_double()
    ok = ref(variant).mdzref_render(*_view_args(v), threads, out.ctypes.data, C.byref(t),
                                    C.byref(t2))
    if not ok:
        raise RuntimeError("reference render failed")
    return out, t.value


def ref_view_dump(v) -> dict:
    buf = C.create_string_buffer(1 << 16)
    n = ref().mdzref_view_dump(*_view_args(v), buf, 1 << 16)
    if n < 0:
        raise RuntimeError("reference view dump failed")
    from mdz_gb300.mpval import MpVal
    out = {}
    for line in buf.value.decode().splitlines():
        parts = line.split()
        name, kind = parts[0], parts[1]
        if kind == "mpfr":
            prec, sign, exp = int(parts[2]), int(parts[3]), int(parts[4])
            limbs = [int(x, 16) for x in parts[5:]]
            if exp == -(1 << 63) + 1:        # MPFR zero
                out[name] = MpVal.zero(prec)
            elif exp < -(1 << 62):           # NaN / infinity
                out[name] = None
            else:
                out[name] = MpVal.from_limbs(prec, sign, exp, limbs)
        else:
            out[name] = ("mpf", int(parts[2]), int(parts[3]), int(parts[4]),
                         [int(x, 16) for x in parts[5:]])
    return out
