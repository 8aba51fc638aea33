"""ctypes binding of libmdzgpu.so (the C ABI declared in include/mdzgpu.h).

The library is built in-tree by mdz_gb300.build; importing this module never
falls back to anything else: if the shared object is missing or fails to
load, NativeUnavailable is raised.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

LIB_PATH = _build.LIB


class NativeUnavailable(RuntimeError):
    pass


class Frame(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("family", C.c_int32),
                ("fractal", C.c_int32), ("depth", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("wall_ms", C.c_double),
                ("pixel_iters", C.c_int64), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64), ("launches", C.c_int32), ("words", C.c_int32),
                ("orbit_ms", C.c_double), ("rebases", C.c_int64), ("orbit_len", C.c_int64),
                ("escalated_fp64", C.c_int64), ("escalated_mp", C.c_int64),
                ("pixel_ms", C.c_double), ("pixel_launches", C.c_int64),
                ("esc_fp64_ms", C.c_double), ("esc_mp_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class MpValStruct(C.Structure):
    _fields_ = [("sign", C.c_int32), ("nlimbs", C.c_int32), ("exp", C.c_int64),
                ("d", C.POINTER(C.c_uint64))]


class Palette(C.Structure):
    _fields_ = [("colours", C.c_void_p), ("indexes", C.c_int32), ("offset", C.c_int32),
                ("colour_scale", C.c_double), ("interpolate", C.c_int32), ("pad", C.c_int32)]


class ServeConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_requests", C.c_int32),
                ("arena_bytes", C.c_int64), ("staging_bytes", C.c_int64),
                ("queue_pixels", C.c_int64), ("step_ms", C.c_double),
                ("log_path", C.c_char_p)]


class Request(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("family", C.c_int32),
                ("fractal", C.c_int32), ("depth", C.c_int64), ("precision", C.c_int64),
                ("cx", MpValStruct), ("cy", MpValStruct), ("span", MpValStruct),
                ("method", C.c_int32), ("pad", C.c_int32), ("timeout_ms", C.c_double),
                ("counts", C.c_void_p), ("mag2", C.c_void_p),
                ("julia_re", MpValStruct), ("julia_im", MpValStruct)]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("error", C.c_int32), ("method", C.c_int32),
                ("words", C.c_int32), ("queue_ms", C.c_double), ("latency_ms", C.c_double),
                ("pixel_iters", C.c_int64), ("escalated_fp64", C.c_int64),
                ("escalated_mp", C.c_int64), ("rebases", C.c_int64), ("steps", C.c_int64),
                ("main_ms", C.c_double), ("esc_wait_ms", C.c_double), ("esc_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("cancelled", C.c_int64), ("timed_out", C.c_int64), ("steps", C.c_int64),
                ("launches", C.c_int64), ("pixel_iters", C.c_int64), ("busy_ms", C.c_double),
                ("latency_p50_ms", C.c_double), ("latency_p99_ms", C.c_double),
                ("latency_max_ms", C.c_double), ("device_bytes_in_use", C.c_int64),
                ("device_bytes_peak", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


P = C.c_void_p
_SIGS = {
    "mdzgpu_create": (P, [C.c_int]),
    "mdzgpu_destroy": (None, [P]),
    "mdzgpu_last_error": (C.c_char_p, []),
    "mdzgpu_version": (C.c_char_p, []),
    "mdzgpu_render_fp64": (C.c_int, [P, C.POINTER(Frame), C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, P, C.POINTER(Stats)]),
    "mdzgpu_render_fp64_device": (C.c_int, [P, C.POINTER(Frame), C.c_double, C.c_double,
                                            C.c_double, C.c_double, C.c_double, P,
                                            C.POINTER(Stats)]),
    "mdzgpu_render_mp": (C.c_int, [P, C.POINTER(Frame)] + [C.POINTER(MpValStruct)] * 5
                         + [C.c_int64, C.c_int32, P, C.POINTER(Stats)]),
    "mdzgpu_render_mp_device": (C.c_int, [P, C.POINTER(Frame)] + [C.POINTER(MpValStruct)] * 5
                                + [C.c_int64, C.c_int32, P, C.POINTER(Stats)]),
    "mdzgpu_render_perturb": (C.c_int, [P, C.POINTER(Frame)] + [C.POINTER(MpValStruct)] * 3
                              + [C.c_int64, C.c_int32, P, P, C.POINTER(Stats)]),
    "mdzgpu_render_perturb_julia": (C.c_int, [P, C.POINTER(Frame)] + [C.POINTER(MpValStruct)] * 5
                                    + [C.c_int64, C.c_int32, P, P, C.POINTER(Stats)]),
    "mdzgpu_render_perturb_device": (C.c_int, [P, C.POINTER(Frame)]
                                     + [C.POINTER(MpValStruct)] * 3
                                     + [C.c_int64, C.c_int32, P, P, C.POINTER(Stats)]),
    "mdzgpu_perturb_spacing": (C.c_int, [C.POINTER(MpValStruct), C.c_int32,
                                         C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "mdzgpu_perturb_limbs": (C.c_int32, [C.c_int64]),
    "mdzgpu_set_wait_limit": (C.c_int, [P, C.c_int32]),
    "mdzgpu_last_escalations": (C.c_int, [P, P, C.c_int64, P, P, C.c_int64, P]),
    "mdzgpu_reference_orbit_formula": (C.c_int, [P, C.c_int32, C.POINTER(MpValStruct),
                                                 C.POINTER(MpValStruct), C.c_int64, C.c_int32,
                                                 C.c_int64, P, P, P, P,
                                                 C.POINTER(C.c_int64)]),
    "mdzgpu_reference_orbit": (C.c_int, [P, C.POINTER(MpValStruct), C.POINTER(MpValStruct),
                                         C.c_int64, C.c_int32, C.c_int64, P, P, P, P,
                                         C.POINTER(C.c_int64)]),
    "mdzgpu_mp_max_words": (C.c_int32, []),
    "mdzgpu_colour": (C.c_int, [P, P, C.c_int32, C.c_int32, C.c_int32, C.POINTER(Palette), P]),
    "mdzgpu_colour_device": (C.c_int, [P, P, C.c_int32, C.c_int32, C.c_int32,
                                       C.POINTER(Palette), P]),
    "mdzgpu_fx_from_mpval": (C.c_int, [C.POINTER(MpValStruct), C.c_int32, P]),
    "mdzgpu_render_mp_noalloc": (C.c_int, [C.POINTER(Frame)] + [C.POINTER(MpValStruct)] * 5
                                 + [C.c_int64, C.c_int32, P, P]),
    "mdzgpu_mp_coordinates": (C.c_int, [C.POINTER(MpValStruct)] * 3
                              + [C.c_int32, C.c_int32, C.c_int32, C.c_int64, C.c_int32, P, P]),
    "mdzgpu_abi_layout": (C.c_int, [P, C.c_int]),
    "mdzgpu_measure_peak": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double)]),
    # serving engine
    "mdzgpu_serve_create": (P, [C.POINTER(ServeConfig)]),
    "mdzgpu_serve_destroy": (None, [P]),
    "mdzgpu_serve_submit": (C.c_int, [P, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "mdzgpu_serve_poll": (C.c_int, [P, C.c_int64, C.POINTER(RequestStatus)]),
    "mdzgpu_serve_wait": (C.c_int, [P, C.c_int64, C.c_double, C.POINTER(RequestStatus)]),
    "mdzgpu_serve_cancel": (C.c_int, [P, C.c_int64]),
    "mdzgpu_serve_release": (C.c_int, [P, C.c_int64]),
    "mdzgpu_serve_get_stats": (C.c_int, [P, C.POINTER(ServeStats)]),
    "mdzgpu_serve_footprint": (C.c_int, [C.POINTER(Request), C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int64)]),
    # drop-in layer
    "rth_create": (P, []),
    "rth_init": (C.c_int, [P, C.c_int, C.c_int, P]),
    "rth_ui_init": (C.c_int, [P]),
    "rth_ui_start_render": (None, [P]),
    "rth_ui_stop_render": (None, [P]),
    "rth_ui_stop_render_and_wait": (None, [P]),
    "rth_ui_quit": (None, [P]),
    "rth_ui_stop_timer": (None, [P]),
    "rth_ui_wait_until_started": (None, [P]),
    "rth_ui_get_render_time": (C.c_double, [P]),
    "rth_set_next_line_cb": (None, [P, P]),
    "rth_process_lines_rendered": (C.c_int, [P]),
    "rth_render_should_stop": (C.c_int, [P]),
    "rth_ui_wait_for_line_done": (C.c_int, [P]),
    "fractal_calculate_line": (C.c_int, [P, C.c_int]),
    "fractal_mpfr_calculate_line": (C.c_int, [P, C.c_int]),
    "fractal_gmp_calculate_line": (C.c_int, [P, C.c_int]),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libmdzgpu.so (built by mdz_gb300.build); raise if unavailable."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path or LIB_PATH)
    if not p.exists():
        raise NativeUnavailable(f"{p} not built: run `python -m mdz_gb300.build`")
    try:
        lib = C.CDLL(str(p))
    except OSError as e:  # pragma: no cover - loader message passes through
        raise NativeUnavailable(f"cannot load {p}: {e}") from e
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def declared_symbols() -> list[str]:
    """Names every include/*.h prototype declares (for export checks)."""
    return list(_SIGS)


def last_error() -> str:
    return (load().mdzgpu_last_error() or b"").decode()
