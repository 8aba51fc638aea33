"""mdz_gb300: GB300-native escape-time renderer for MDZ (Mandelbrot Deep Zoom).

The product is libmdzgpu.so (C ABI, include/mdzgpu.h): hand-written sm_103a
kernels behind MDZ's own render_threads.h / fractal.h entry points plus an
explicit mdzgpu_* layer.  This package builds it (mdz_gb300.build), binds it
with ctypes (mdz_gb300.native) and offers a thin Python front end used by the
tests and bench.py.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .mpval import MpVal, hexfloat, parse_number
from .native import Frame, NativeUnavailable, Stats
from .views import Rect, View, mdz_rect, perturb_half_spacing

__all__ = ["Renderer", "MpVal", "View", "Rect", "mdz_rect", "NativeUnavailable", "hexfloat",
           "parse_number", "MDZ_FAMILY", "MDZ_FRACTAL"]

# src/fractal.c:11-26
MDZ_FAMILY = {"mandelbrot": 0, "julia": 1}
MDZ_FRACTAL = {"mandelbrot": 0, "burning ship": 1, "generalized celtic": 2,
               "mandel-celtic hybrid": 3}


class MdzGpuError(RuntimeError):
    pass


def _check(rc: int) -> None:
    if rc != 0:
        raise MdzGpuError(f"mdzgpu error {rc}: {native.last_error()}")


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Renderer:
    """One GPU context (device, stream, reusable buffers)."""

    def __init__(self, device: int = 0):
        self.lib = native.load()
        self.ctx = self.lib.mdzgpu_create(device)
        if not self.ctx:
            raise MdzGpuError(f"mdzgpu_create({device}) failed: {native.last_error()}")

    def close(self) -> None:
        if self.ctx:
            self.lib.mdzgpu_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- FP64 -------------------------------------------------------------
    def render_fp64(self, W: int, H: int, depth: int, xmin: float, xmax: float, ymax: float,
                    family: int = 0, fractal: int = 0, julia=(0.0, 0.0),
                    out: np.ndarray | None = None):
        f = Frame(W, H, family, fractal, depth)
        if out is None:
            out = np.empty((H, W), np.int32)
        st = Stats()
        _check(self.lib.mdzgpu_render_fp64(self.ctx, C.byref(f), xmin, xmax, ymax, julia[0],
                                           julia[1], _ptr(out), C.byref(st)))
        return out, st.as_dict()

    def render_fp64_device(self, W, H, depth, xmin, xmax, ymax, d_out_ptr: int, family=0,
                           fractal=0, julia=(0.0, 0.0)):
        f = Frame(W, H, family, fractal, depth)
        st = Stats()
        _check(self.lib.mdzgpu_render_fp64_device(self.ctx, C.byref(f), xmin, xmax, ymax,
                                                  julia[0], julia[1], C.c_void_p(d_out_ptr),
                                                  C.byref(st)))
        return st.as_dict()

    # -- multi-limb ---------------------------------------------------------
    def _mp_args(self, xmin: MpVal, ymax: MpVal, width: MpVal, julia):
        jre, jim = julia if julia is not None else (MpVal.zero(), MpVal.zero())
        items = [v.struct() for v in (xmin, ymax, width, jre, jim)]
        return [C.byref(s) for s, _ in items], items

    def render_mp(self, W: int, H: int, depth: int, xmin: MpVal, ymax: MpVal, width: MpVal,
                  precision: int, words: int = 0, family: int = 0, fractal: int = 0,
                  julia=None, out: np.ndarray | None = None):
        f = Frame(W, H, family, fractal, depth)
        if out is None:
            out = np.empty((H, W), np.int32)
        st = Stats()
        args, keep = self._mp_args(xmin, ymax, width, julia)
        _check(self.lib.mdzgpu_render_mp(self.ctx, C.byref(f), *args, precision, words,
                                         _ptr(out), C.byref(st)))
        del keep
        return out, st.as_dict()

    def render_mp_device(self, W, H, depth, xmin, ymax, width, precision, d_out_ptr: int,
                         words=0, family=0, fractal=0, julia=None):
        f = Frame(W, H, family, fractal, depth)
        st = Stats()
        args, keep = self._mp_args(xmin, ymax, width, julia)
        _check(self.lib.mdzgpu_render_mp_device(self.ctx, C.byref(f), *args, precision, words,
                                                C.c_void_p(d_out_ptr), C.byref(st)))
        del keep
        return st.as_dict()

    # -- colouring -------------------------------------------------------------
    def colour(self, counts: np.ndarray, aa: int, palette, colour_scale: float = 1.0,
               interpolate: bool = False, offset: int = 0) -> np.ndarray:
        """MDZ's colouring on the GPU: uint32 [H/aa][W/aa], r | g << 8 | b << 16."""
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        H, W = counts.shape
        pal_arr = np.ascontiguousarray(palette, dtype=np.uint32)
        pal = native.Palette(pal_arr.ctypes.data, len(pal_arr), offset, colour_scale,
                             int(interpolate), 0)
        out = np.empty((H // aa, W // aa), np.uint32)
        _check(self.lib.mdzgpu_colour(self.ctx, _ptr(counts), W, H, aa, C.byref(pal),
                                      _ptr(out)))
        return out

    def colour_device(self, d_counts: int, W: int, H: int, aa: int, palette, d_rgb: int,
                      colour_scale: float = 1.0, interpolate: bool = False, offset: int = 0):
        pal_arr = np.ascontiguousarray(palette, dtype=np.uint32)
        pal = native.Palette(pal_arr.ctypes.data, len(pal_arr), offset, colour_scale,
                             int(interpolate), 0)
        _check(self.lib.mdzgpu_colour_device(self.ctx, C.c_void_p(d_counts), W, H, aa,
                                             C.byref(pal), C.c_void_p(d_rgb)))

    # -- perturbation ---------------------------------------------------------
    def render_perturb(self, W: int, H: int, depth: int, cx: MpVal, cy: MpVal, width: MpVal,
                       precision: int, limbs: int = 0, want_mag: bool = False,
                       out: np.ndarray | None = None, mag: np.ndarray | None = None,
                       fractal: int = 0, julia: tuple | None = None):
        """julia = (re, im) as MpVal: the Julia family (z0 = pixel)."""
        f = Frame(W, H, 1 if julia else 0, fractal, depth)
        if out is None:
            out = np.empty((H, W), np.int32)
        if want_mag and mag is None:
            mag = np.empty((H, W), np.float32)
        st = Stats()
        items = [v.struct() for v in (cx, cy, width) + (tuple(julia) if julia else ())]
        refs = [C.byref(s) for s, _ in items]
        if julia:
            _check(self.lib.mdzgpu_render_perturb_julia(
                self.ctx, C.byref(f), *refs, precision, limbs, _ptr(out),
                _ptr(mag if want_mag else None), C.byref(st)))
        else:
            _check(self.lib.mdzgpu_render_perturb(self.ctx, C.byref(f), *refs, precision, limbs,
                                                  _ptr(out), _ptr(mag if want_mag else None),
                                                  C.byref(st)))
        return out, (mag if want_mag else None), st.as_dict()

    def last_escalations(self) -> tuple[np.ndarray, np.ndarray]:
        """Pixel indices (line * W + ix) the last render_perturb re-ran in
        FP64 and in the multi-limb kernel (mdzgpu_last_escalations)."""
        n1, n2 = C.c_int64(), C.c_int64()
        _check(self.lib.mdzgpu_last_escalations(self.ctx, None, 0, C.byref(n1), None, 0,
                                                C.byref(n2)))
        a = np.zeros(max(n1.value, 1), np.uint32)
        b = np.zeros(max(n2.value, 1), np.uint32)
        _check(self.lib.mdzgpu_last_escalations(self.ctx, a.ctypes.data, n1.value, C.byref(n1),
                                                b.ctypes.data, n2.value, C.byref(n2)))
        return a[:n1.value], b[:n2.value]

    def render_perturb_device(self, W, H, depth, cx, cy, width, precision, d_out_ptr: int,
                              d_mag_ptr: int | None = None, limbs: int = 0):
        f = Frame(W, H, 0, 0, depth)
        st = Stats()
        items = [v.struct() for v in (cx, cy, width)]
        _check(self.lib.mdzgpu_render_perturb_device(
            self.ctx, C.byref(f), *[C.byref(s) for s, _ in items], precision, limbs,
            C.c_void_p(d_out_ptr), C.c_void_p(d_mag_ptr) if d_mag_ptr else None, C.byref(st)))
        return st.as_dict()


def perturb_spacing(width: MpVal, W: int) -> tuple[float, int]:
    """(hs_m, hs_e) of the perturbation path's half pixel spacing as the
    library computes it (mdzgpu_perturb_spacing): width / (2 W) rounded to 40
    significant bits."""
    lib = native.load()
    s, keep = width.struct()
    m = C.c_double()
    e = C.c_int32()
    _check(lib.mdzgpu_perturb_spacing(C.byref(s), W, C.byref(m), C.byref(e)))
    del keep
    return m.value, e.value


def perturb_pixel_c(cx: MpVal, cy: MpVal, width: MpVal, W: int, H: int, ix: int, line: int):
    """Exact c of pixel (ix, line) in the perturbation path's geometry
    (computed in Python: the library is not loaded)."""
    from fractions import Fraction
    hs_m, hs_e = perturb_half_spacing(width, W)
    hs = Fraction(hs_m) * Fraction(2) ** hs_e
    return (cx.to_fraction() + (2 * ix - W) * hs, cy.to_fraction() + (H - 2 * line) * hs)
