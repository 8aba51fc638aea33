"""Failure paths on the GPU, made without a fault.

* Bounded device waits: with a wait limit of one poll
  (mdzgpu_set_wait_limit), the orbit finisher of the streamed schedule and
  the pixels of the fused schedule give up at once; the kernels return, the
  call reports MDZGPU_ERR_TIMEOUT, and the same context then renders the
  frame bit-identically to a fresh one.
* Stop through MDZ's own entry points (src/render_threads.c:409-440):
  rth_ui_stop_render_and_wait during a long frame returns promptly, the
  rows published before the stop are the reference's, no row is published
  after it, rth_ui_wait_for_line_done returns (bounded) instead of blocking,
  and the next full render is bit-exact.  As in the reference, a stopped
  frame stays incomplete: rth_process_lines_rendered keeps reporting the
  rows done (< height), never -1.
"""
import hashlib
import json
import time
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MdzGpuError, MpVal, Renderer, View
from mdz_gb300.abi import DropIn

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def _deep_view():
    cx = MpVal.from_fraction(-1.7497856353511106, 256)
    cy = MpVal.from_fraction(0.0000153218, 256)
    w = MpVal.from_fraction(2.0 ** -100, 256)
    return cx, cy, w


@pytest.mark.parametrize("schedule", ["steps", "fused"])
def test_bounded_wait_gives_up_and_context_stays_usable(schedule, monkeypatch):
    cx, cy, w = _deep_view()
    W, H, depth, prec = 96, 64, 20000, 192
    with Renderer(0) as ref:
        want, _, _ = ref.render_perturb(W, H, depth, cx, cy, w, prec)
    monkeypatch.setenv("MDZGPU_PERTURB", schedule)
    with Renderer(0) as r:
        assert r.lib.mdzgpu_set_wait_limit(r.ctx, 1) == 0
        t0 = time.time()
        with pytest.raises(MdzGpuError, match="error -6"):
            r.render_perturb(W, H, depth, cx, cy, w, prec)
        assert time.time() - t0 < 60
        # default limit again: the same context renders the frame exactly
        assert r.lib.mdzgpu_set_wait_limit(r.ctx, 0) == 0
        got, _, _ = r.render_perturb(W, H, depth, cx, cy, w, prec)
        assert np.array_equal(got, want)
        assert r.lib.mdzgpu_set_wait_limit(None, 5) == -1
        assert r.lib.mdzgpu_set_wait_limit(r.ctx, -2) == -1


def _c2_view():
    meta = json.loads((GOLD / "c2_frame.json").read_text())
    v = View.from_dict({k: x for k, x in meta["view"].items() if k != "seed"})
    return v, meta


def test_dropin_stop_mid_frame_then_full_render_bit_exact():
    if not (GOLD / "c2_frame.json").exists():
        pytest.skip("c2 fixture not generated")
    v, meta = _c2_view()
    rows = np.load(GOLD / "c2_rows.npz")["rows"]
    step = meta["row_step"]
    d = DropIn(v)
    lib, rth = d.lib, d.rth_ptr
    try:
        lib.rth_ui_start_render(rth)
        lib.rth_ui_wait_until_started(rth)
        t0 = time.time()
        while True:
            n = lib.rth_process_lines_rendered(rth)
            if n < 0 or n >= 40 or time.time() - t0 > 60:
                break
            lib.rth_ui_wait_for_line_done(rth)
        done_before = lib.rth_process_lines_rendered(rth)
        assert 0 < done_before < v.height, "stop must land inside the frame"
        t0 = time.time()
        lib.rth_ui_stop_render_and_wait(rth)
        stop_s = time.time() - t0
        assert stop_s < 5.0, f"stop took {stop_s:.2f}s"
        assert lib.rth_render_should_stop(rth) == 1
        # bounded: returns instead of blocking on a frame that will not finish
        t0 = time.time()
        lib.rth_ui_wait_for_line_done(rth)
        assert time.time() - t0 < 2.0
        after = lib.rth_process_lines_rendered(rth)
        time.sleep(0.5)
        assert lib.rth_process_lines_rendered(rth) == after
        assert 0 < after < v.height          # incomplete, as the reference leaves it
        # every published row equals the reference's
        published = [y for y in range(v.height) if d.rth.lines_drawn[y] != b"\x00"]
        assert published
        checked = 0
        for y in published:
            for r_ in range(y * v.aa, y * v.aa + v.aa):
                if r_ % step == 0:
                    assert np.array_equal(d.raw[r_], rows[r_ // step]), f"row {r_}"
                    checked += 1
        assert checked > 0
        # restart: the whole frame, bit-exact
        d.raw[:] = -1
        d.render(timeout_s=600)
        assert hashlib.sha256(d.raw.tobytes()).hexdigest() == meta["sha256"]
    finally:
        d.close()
