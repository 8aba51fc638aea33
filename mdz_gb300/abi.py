"""ctypes mirror of include/mdz_abi.h: MDZ's image_info / rthdata layouts.

Lets Python callers (and the tests) build the same image_info MDZ's
image_info_set + render_to_file would hand to the drop-in layer
(src/image_info.c:104-144, src/render.c:34-37) and drive rth_* exactly as
render.c does.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import native
from .mpval import MpVal
from .views import View

MPFR_EXP_ZERO = -(1 << 63) + 1


class MdzMpfr(C.Structure):
    _fields_ = [("prec", C.c_long), ("sign", C.c_int), ("exp", C.c_long),
                ("d", C.POINTER(C.c_uint64))]


class MdzMpf(C.Structure):
    _fields_ = [("prec", C.c_int), ("size", C.c_int), ("exp", C.c_long),
                ("d", C.POINTER(C.c_uint64))]


class JuliaInfo(C.Structure):
    _fields_ = [("c_re", MdzMpfr), ("c_im", MdzMpfr)]


class ImageInfo(C.Structure):
    _fields_ = [
        ("xmin", MdzMpfr), ("xmax", MdzMpfr), ("ymax", MdzMpfr), ("width", MdzMpfr),
        ("gxmin", MdzMpf), ("gxmax", MdzMpf), ("gymax", MdzMpf), ("gwidth", MdzMpf),
        ("old_cx", MdzMpfr), ("old_cy", MdzMpfr), ("old_size", MdzMpfr),
        ("pcoords", C.c_void_p), ("depth", C.c_int64), ("thread_count", C.c_int),
        ("draw_lines", C.c_int), ("raw_data", C.POINTER(C.c_int)),
        ("rgb_data", C.POINTER(C.c_uint32)), ("j_pre", C.c_int), ("drawing_area", C.c_void_p),
        ("rnd_pal", C.c_void_p), ("real_width", C.c_int), ("real_height", C.c_int),
        ("user_width", C.c_int), ("user_height", C.c_int), ("aspect", C.c_double),
        ("aa_factor", C.c_int), ("family", C.c_int), ("fractal", C.c_int),
        ("colour_scale", C.c_double), ("julia", JuliaInfo), ("palette_ip", C.c_bool),
        ("zoom_new_win", C.c_bool), ("use_multi_prec", C.c_bool), ("use_rounding", C.c_bool),
        ("precision", C.c_long), ("multi_prec_init_done", C.c_bool), ("rth_ptr", C.c_void_p),
        ("lines_drawn", C.c_int), ("ui_ref_center", C.c_bool),
    ]


class RthData(C.Structure):
    _fields_ = [("img", C.POINTER(ImageInfo)), ("lines_drawn", C.POINTER(C.c_char)),
                ("min_line_drawn", C.c_int), ("line_draw_count", C.c_int),
                ("thread_count", C.c_int), ("check_stop_px", C.c_int), ("data", C.c_void_p)]


def layout() -> list[int]:
    """Offsets in the order mdzgpu_abi_layout reports them."""
    names = [f for f, _ in ImageInfo._fields_]
    offs = []
    for n in names:
        if n == "julia":
            offs += [ImageInfo.julia.offset, ImageInfo.julia.offset + C.sizeof(MdzMpfr)]
        else:
            offs.append(getattr(ImageInfo, n).offset)
    offs.append(C.sizeof(ImageInfo))
    offs += [getattr(RthData, f).offset for f, _ in RthData._fields_]
    offs.append(C.sizeof(RthData))
    return offs


def _set_mpfr(dst: MdzMpfr, v: MpVal, keep: list) -> None:
    arr = (C.c_uint64 * v.nlimbs)(*v.limbs())
    keep.append(arr)
    dst.prec = v.prec
    dst.sign = v.sign
    dst.exp = MPFR_EXP_ZERO if v.mant == 0 else v.exp
    dst.d = C.cast(arr, C.POINTER(C.c_uint64))


def _set_mpf(dst: MdzMpf, v: MpVal, keep: list) -> None:
    """GMP layout of the same value: limb exponent, |size| significant limbs."""
    if v.mant == 0:
        arr = (C.c_uint64 * 1)(0)
        keep.append(arr)
        dst.prec, dst.size, dst.exp = 1, 0, 0
        dst.d = C.cast(arr, C.POINTER(C.c_uint64))
        return
    # value = M * 2^(exp - 64 n); shift M so that the weight of its lowest
    # limb is a whole number of limbs, as GMP's limb exponent requires
    n = v.nlimbs
    shift = v.exp % 64
    mant = v.mant << shift
    w0 = v.exp - 64 * n - shift               # weight (bits) of limbs[0]
    limbs = []
    m = mant
    while m:
        limbs.append(m & ((1 << 64) - 1))
        m >>= 64
    while limbs and limbs[0] == 0:
        limbs.pop(0)
        w0 += 64
    size = len(limbs)
    arr = (C.c_uint64 * size)(*limbs)
    keep.append(arr)
    dst.prec = size
    dst.size = v.sign * size
    dst.exp = w0 // 64 + size
    dst.d = C.cast(arr, C.POINTER(C.c_uint64))


class DropIn:
    """An image_info + rthdata pair driven through the drop-in entry points
    the way render_to_file drives MDZ's own (src/render.c:39-94)."""

    def __init__(self, v: View, gmp_values: dict | None = None):
        self.lib = native.load()
        self.view = v
        self.keep: list = []
        img = ImageInfo()
        r = v.rect()
        _set_mpfr(img.xmin, r.xmin, self.keep)
        _set_mpfr(img.xmax, r.xmax, self.keep)
        _set_mpfr(img.ymax, r.ymax, self.keep)
        _set_mpfr(img.width, r.width, self.keep)
        jre, jim = v.julia()
        _set_mpfr(img.julia.c_re, jre, self.keep)
        _set_mpfr(img.julia.c_im, jim, self.keep)
        for name, val in (("gxmin", r.xmin), ("gxmax", r.xmax), ("gymax", r.ymax),
                          ("gwidth", r.width)):
            _set_mpf(getattr(img, name), (gmp_values or {}).get(name, val), self.keep)
        img.depth = v.depth
        img.real_width, img.real_height = v.real_width, v.real_height
        img.user_width, img.user_height = v.width, v.height
        img.aspect = v.width / v.height
        img.aa_factor = v.aa
        img.family, img.fractal = v.family, v.fractal
        img.use_multi_prec, img.use_rounding = v.multi_prec, v.rounding
        img.precision = v.precision
        img.draw_lines = 64
        self.raw = np.full((v.real_height, v.real_width), -1, np.int32)  # UINT_MAX as int
        img.raw_data = self.raw.ctypes.data_as(C.POINTER(C.c_int))
        self.img = img
        self.rth_ptr = self.lib.rth_create()
        if not self.rth_ptr:
            raise RuntimeError("rth_create failed")
        img.rth_ptr = self.rth_ptr
        if not self.lib.rth_init(self.rth_ptr, 1, 64, C.byref(img)):
            raise RuntimeError("rth_init failed")
        self.rth = RthData.from_address(self.rth_ptr)
        cb = {(False, True): "fractal_calculate_line", (False, False): "fractal_calculate_line",
              (True, True): "fractal_mpfr_calculate_line",
              (True, False): "fractal_gmp_calculate_line"}[(bool(v.multi_prec), bool(v.rounding))]
        self.lib.rth_set_next_line_cb(self.rth_ptr, C.cast(getattr(self.lib, cb), C.c_void_p))
        if not self.lib.rth_ui_init(self.rth_ptr):
            raise RuntimeError("rth_ui_init failed")

    def render(self, timeout_s: float = 600.0) -> dict:
        """render_to_file's loop: start, wait per line, process, until done."""
        lib, rth = self.lib, self.rth_ptr
        lib.rth_ui_start_render(rth)
        lib.rth_ui_wait_until_started(rth)   # as gui_start_rendering does
        drawn_order = []
        t0 = time.time()
        y = 0
        while y < self.view.height:
            if time.time() - t0 > timeout_s:
                raise TimeoutError("drop-in render did not finish")
            lib.rth_ui_wait_for_line_done(rth)
            linesdone = lib.rth_process_lines_rendered(rth)
            if linesdone:
                undrawn = 0
                miny = self.rth.min_line_drawn
                maxy = miny + self.rth.line_draw_count + 1
                if maxy >= self.view.height:
                    maxy = self.view.height
                if linesdone > 0 and maxy > linesdone:
                    maxy = linesdone
                for y in range(miny, maxy):
                    ld = self.rth.lines_drawn[y]
                    if ld == b"\x01":
                        self.rth.lines_drawn[y] = b"\x02"
                        if not undrawn:
                            self.rth.min_line_drawn = y
                        drawn_order.append(y)
                    elif ld == b"\x00":
                        undrawn = 1
                y = maxy
        return {"seconds": time.time() - t0, "render_time": lib.rth_ui_get_render_time(rth),
                "drawn": drawn_order}

    def close(self) -> None:
        if self.rth_ptr:
            self.lib.rth_ui_quit(self.rth_ptr)
            self.rth_ptr = None
