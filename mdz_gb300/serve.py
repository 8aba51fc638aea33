"""Python front end of the serving engine (mdzgpu_serve_* in include/mdzgpu.h).

A Server owns one GPU.  submit() queues a render request and returns at
once; the engine admits requests while slots and memory allow, runs all
admitted requests together (continuous batching: one work queue per method,
every step advances every queued pixel by a bounded number of iterations)
and writes each result into the request's own numpy buffers.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import native
from .mpval import MpVal

METHOD = {"auto": 0, "perturbation": 1, "multi_limb": 2}
STATE = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "cancelled", 5: "timeout"}
FORMULA = {"mandelbrot": 0, "burning_ship": 1, "generalized_celtic": 2, "variant": 3}


class ServeError(RuntimeError):
    pass


@dataclass
class RenderRequest:
    """One render: centre (cx, cy) and real-axis span as MpVal, square pixels
    (the perturbation geometry, c = centre + ((2 ix - W) hs, (H - 2 line) hs),
    hs = span / (2 W) rounded to 40 bits)."""
    width: int
    height: int
    depth: int
    cx: MpVal
    cy: MpVal
    span: MpVal
    precision: int
    fractal: int = 0
    method: str = "auto"
    want_mag: bool = False
    family: int = 0                              # 1: Julia (z0 = pixel, c = julia)
    julia: tuple[MpVal, MpVal] | None = None
    timeout_ms: float = 0.0
    counts: np.ndarray | None = None
    mag: np.ndarray | None = None
    _keep: list = field(default_factory=list, repr=False)

    def c_struct(self) -> native.Request:
        if self.counts is None:
            self.counts = np.zeros((self.height, self.width), np.int32)
        if self.want_mag and self.mag is None:
            self.mag = np.zeros((self.height, self.width), np.float32)
        vals = [self.cx, self.cy, self.span] + (list(self.julia) if self.julia else [])
        mp = [v.struct() for v in vals]
        self._keep = [k for _, k in mp]
        r = native.Request()
        r.width, r.height = self.width, self.height
        r.family, r.fractal = self.family, self.fractal
        if self.julia:
            r.julia_re, r.julia_im = mp[3][0], mp[4][0]
        r.depth, r.precision = self.depth, self.precision
        r.cx, r.cy, r.span = mp[0][0], mp[1][0], mp[2][0]
        r.method = METHOD[self.method]
        r.timeout_ms = self.timeout_ms
        r.counts = self.counts.ctypes.data
        r.mag2 = self.mag.ctypes.data if self.want_mag else None
        return r


def request_from_view(v, method: str = "auto", want_mag: bool = False,
                      timeout_ms: float = 0.0) -> RenderRequest:
    """A serving request for an MDZ view (mdz_gb300.View, e.g. from a
    settings file): its centre, depth, precision, formula, family and Julia
    constant, over its real (supersampled) pixels.  MDZ's `size` is the
    real-axis width of a wide frame and the imaginary-axis height of a tall
    one (src/coords.c:265-302); the request takes the real-axis span."""
    from fractions import Fraction

    from .mpval import parse_number
    prec = max(int(v.precision), 64)
    W, H = v.real_width, v.real_height
    size = parse_number(v.size)
    aspect = Fraction(v.width / v.height)        # a double, as MDZ computes it
    span = size if aspect > 1 else size * aspect
    julia = None
    if v.family == 1:
        julia = (MpVal.from_fraction(parse_number(v.julia_re), prec),
                 MpVal.from_fraction(parse_number(v.julia_im), prec))
    return RenderRequest(W, H, int(v.depth), MpVal.from_fraction(parse_number(v.cx), prec),
                         MpVal.from_fraction(parse_number(v.cy), prec),
                         MpVal.from_fraction(span, prec), prec, fractal=int(v.fractal),
                         method=method, want_mag=want_mag, family=int(v.family), julia=julia,
                         timeout_ms=timeout_ms)


def request_from_mdz(path, width: int = 0, height: int = 0, aa: int = 0,
                     intended: bool = False, **kw) -> RenderRequest:
    """A serving request for an MDZ settings file (.mdz): the view MDZ's
    headless render takes from it (image_info_load_settings,
    src/image_info.c:456-721; `mdz -s file -W w -H h -a aa`).  MDZ renders a
    rectangle-form file around the rectangle's centre at size 4.0;
    `intended=True` takes the file's own rectangle instead."""
    from . import mdzfile
    s = mdzfile.load(path)
    v = s.intended_view(width, height, aa) if intended else s.view(width, height, aa)
    return request_from_view(v, **kw)


def footprint(req: RenderRequest) -> tuple[int, int]:
    """(device bytes, pinned host bytes) the request holds while admitted."""
    lib = native.load()
    d = C.c_int64()
    h = C.c_int64()
    rc = lib.mdzgpu_serve_footprint(C.byref(req.c_struct()), C.byref(d), C.byref(h))
    if rc:
        raise ServeError(f"footprint: {rc}: {native.last_error()}")
    return d.value, h.value


class Server:
    def __init__(self, device: int = 0, max_requests: int = 0, arena_bytes: int = 0,
                 staging_bytes: int = 0, queue_pixels: int = 0, step_ms: float = 0.0,
                 log_path: str | None = None):
        self.lib = native.load()
        cfg = native.ServeConfig(device, max_requests, arena_bytes, staging_bytes,
                                 queue_pixels, step_ms,
                                 log_path.encode() if log_path else None)
        self.srv = self.lib.mdzgpu_serve_create(C.byref(cfg))
        if not self.srv:
            raise ServeError(f"mdzgpu_serve_create failed: {native.last_error()}")
        self.requests: dict[int, RenderRequest] = {}

    def close(self) -> None:
        if self.srv:
            self.lib.mdzgpu_serve_destroy(self.srv)
            self.srv = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, req: RenderRequest) -> int:
        rid = C.c_int64()
        rc = self.lib.mdzgpu_serve_submit(self.srv, C.byref(req.c_struct()), C.byref(rid))
        if rc:
            raise ServeError(f"submit: {rc}: {native.last_error()}")
        self.requests[rid.value] = req   # keeps the output buffers alive
        return rid.value

    def poll(self, rid: int) -> dict:
        st = native.RequestStatus()
        rc = self.lib.mdzgpu_serve_poll(self.srv, rid, C.byref(st))
        if rc:
            raise ServeError(f"poll: {rc}: {native.last_error()}")
        d = st.as_dict()
        d["state"] = STATE[d["state"]]
        return d

    def wait(self, rid: int, timeout_ms: float = -1.0) -> dict:
        st = native.RequestStatus()
        rc = self.lib.mdzgpu_serve_wait(self.srv, rid, timeout_ms, C.byref(st))
        if rc and rc != -6:
            raise ServeError(f"wait: {rc}: {native.last_error()}")
        d = st.as_dict()
        d["state"] = STATE[d["state"]]
        return d

    def cancel(self, rid: int) -> None:
        rc = self.lib.mdzgpu_serve_cancel(self.srv, rid)
        if rc:
            raise ServeError(f"cancel: {rc}: {native.last_error()}")

    def release(self, rid: int) -> None:
        rc = self.lib.mdzgpu_serve_release(self.srv, rid)
        if rc:
            raise ServeError(f"release: {rc}: {native.last_error()}")
        self.requests.pop(rid, None)

    def stats(self) -> dict:
        st = native.ServeStats()
        rc = self.lib.mdzgpu_serve_get_stats(self.srv, C.byref(st))
        if rc:
            raise ServeError(f"stats: {rc}: {native.last_error()}")
        return st.as_dict()
