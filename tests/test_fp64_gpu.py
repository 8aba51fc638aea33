"""FP64 path on the GPU: bit-exact against the reference's double build
(counts from the unmodified MDZ rth_* + fractal.c, tests/golden)."""
import hashlib
import json
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import View, parse_number
from mdz_gb300.abi import DropIn

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "fp64_views.json").read_text())
COUNTS = np.load(GOLD / "fp64_counts.npz")

pytestmark = pytest.mark.gpu


def view_of(name):
    return View.from_dict({k: v for k, v in META[name].items()
                           if k not in ("rect", "sha256", "pixel_iters")})


def julia_doubles(v):
    if not v.family:
        return (0.0, 0.0)
    re_, im_ = v.julia()
    return (float(re_.to_fraction()), float(im_.to_fraction()))


@pytest.mark.parametrize("name", sorted(META))
def test_fp64_explicit_bit_exact(renderer, name):
    v = view_of(name)
    xmin, xmax, ymax = (float(parse_number(s)) for s in META[name]["rect"])
    got, st = renderer.render_fp64(v.real_width, v.real_height, v.depth, xmin, xmax, ymax,
                                   v.family, v.fractal, julia_doubles(v))
    want = COUNTS[name]
    assert got.shape == want.shape
    diff = int((got != want).sum())
    assert diff == 0, f"{diff} pixels differ"
    assert st["pixel_iters"] == META[name]["pixel_iters"]
    assert st["launches"] == 1


@pytest.mark.parametrize("name", ["c1", "aa3", "f1_julia", "odd"])
def test_fp64_dropin_rth_bit_exact(name):
    """Through MDZ's own entry points: rth_init / rth_ui_init /
    rth_ui_start_render / wait / process_lines_rendered / quit."""
    v = view_of(name)
    d = DropIn(v)
    try:
        info = d.render(timeout_s=120)
        assert np.array_equal(d.raw, COUNTS[name])
        assert sorted(info["drawn"]) == list(range(v.height))
        assert info["render_time"] > 0
        # a second render on the same rthdata reuses the watch thread
        d.raw[:] = -1
        d.render(timeout_s=120)
        assert np.array_equal(d.raw, COUNTS[name])
    finally:
        d.close()


def test_fp64_line_entry_point():
    """fractal_calculate_line(img, line) renders one real row."""
    import ctypes as C
    v = view_of("c1")
    d = DropIn(v)
    try:
        for line in (0, 17, 179):
            assert d.lib.fractal_calculate_line(C.byref(d.img), line) == 1
            assert np.array_equal(d.raw[line], COUNTS["c1"][line])
    finally:
        d.close()


def test_fp64_device_output(renderer):
    torch = pytest.importorskip("torch")
    v = view_of("deep")
    xmin, xmax, ymax = (float(parse_number(s)) for s in META["deep"]["rect"])
    buf = torch.empty((v.real_height, v.real_width), dtype=torch.int32, device="cuda")
    st = renderer.render_fp64_device(v.real_width, v.real_height, v.depth, xmin, xmax, ymax,
                                     buf.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(buf.cpu().numpy(), COUNTS["deep"])
    assert st["d2h_bytes"] <= 64


def _c2():
    path = GOLD / "c2_frame.json"
    if not path.exists():
        pytest.skip("c2 fixture not generated")
    meta = json.loads(path.read_text())
    v = View.from_dict({k: x for k, x in meta["view"].items() if k != "seed"})
    return v, meta, np.load(GOLD / "c2_rows.npz")["rows"]


def test_c2_full_frame_explicit_bit_exact(renderer):
    """The seeded 1920x1080, 3x3-supersampled frame (5760x3240 counts, width
    1e-11, maxiter 20000) in full against the unmodified reference's double
    build without FMA (src/fractal.c:29-117, src/frac_mandel.c:5-21): the
    frame's sha256, its iteration total and every 27th row."""
    v, meta, rows = _c2()
    xmin, xmax, ymax = (float(parse_number(s)) for s in meta["rect"])
    got, st = renderer.render_fp64(v.real_width, v.real_height, v.depth, xmin, xmax, ymax)
    assert list(got.shape) == meta["shape"]
    step = meta["row_step"]
    bad = [i * step for i in range(len(rows)) if not np.array_equal(got[i * step], rows[i])]
    assert not bad, f"rows differ: {bad[:10]}"
    assert st["pixel_iters"] == meta["pixel_iters"]
    assert hashlib.sha256(got.tobytes()).hexdigest() == meta["sha256"]


def test_c2_full_frame_dropin_bit_exact():
    """The same frame through MDZ's own entry points (rth_ui_start_render
    with fractal_calculate_line installed, as image_info_set_multi_prec
    does for the hardware-float path)."""
    v, meta, rows = _c2()
    d = DropIn(v)
    try:
        info = d.render(timeout_s=600)
        assert sorted(info["drawn"]) == list(range(v.height))
        step = meta["row_step"]
        bad = [i * step for i in range(len(rows)) if not np.array_equal(d.raw[i * step], rows[i])]
        assert not bad, f"rows differ: {bad[:10]}"
        assert hashlib.sha256(d.raw.tobytes()).hexdigest() == meta["sha256"]
    finally:
        d.close()
