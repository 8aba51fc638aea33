"""The Julia family under perturbation (z0 = the pixel, c fixed; MDZ's
Julia loop, src/fractal.c:55-59 and :78-88) on the GPU: frames at 2^-40 ..
2^-600 around points of the Julia sets' boundaries (basilica, rabbit,
burning-ship and celtic Julia sets) against MPFR at twice the precision
(tests/golden/perturb_julia.npz, made by make_golden.py perturb_julia).
Every view here is resolved by MPFR at its precision (p, 2p and 3p agree),
so the bar is the Mandelbrot one: at most 0.1% of the pixels (at least 2)
differ."""
import json
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MpVal, parse_number

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "perturb_julia_views.json").read_text())
DATA = np.load(GOLD / "perturb_julia.npz")


def render(renderer, name, **kw):
    m = META[name]
    prec = m["prec"]
    vals = [MpVal.from_fraction(parse_number(m[k]), prec)
            for k in ("cx", "cy", "width", "julia_re", "julia_im")]
    return renderer.render_perturb(m["W"], m["H"], m["depth"], vals[0], vals[1], vals[2], prec,
                                   want_mag=True, fractal=m["fractal"],
                                   julia=(vals[3], vals[4]), **kw)


@pytest.mark.parametrize("name", sorted(META))
def test_julia_frame_vs_mpfr_2x(renderer, name):
    counts, mag, st = render(renderer, name)
    want = DATA[name]
    diff = counts != want
    n_diff = int(diff.sum())
    print(f"{name} [{META[name]['kind']}]: differ {n_diff}/{diff.size} (MPFR at p: "
          f"{int((DATA[name + '__p'] != want).sum())}); escalated fp64 "
          f"{st['escalated_fp64']} mp {st['escalated_mp']}; rebases {st['rebases']}")
    assert META[name]["kind"] == "resolved"
    assert n_diff <= max(2, 0.001 * diff.size), f"{name}: {n_diff} differ"
    assert st["pixel_iters"] > 0


def test_julia_needs_its_constant(renderer):
    import ctypes as C
    from mdz_gb300.native import Frame, Stats
    m = META["j_basilica_40"]
    prec = m["prec"]
    vals = [MpVal.from_fraction(parse_number(m[k]), prec).struct()
            for k in ("cx", "cy", "width")]
    out = np.empty((m["H"], m["W"]), np.int32)
    st = Stats()
    # the Julia family through the Mandelbrot-family call: refused
    f = Frame(m["W"], m["H"], 1, 0, m["depth"])
    rc = renderer.lib.mdzgpu_render_perturb(renderer.ctx, C.byref(f),
                                            *[C.byref(s) for s, _ in vals], prec, 0,
                                            out.ctypes.data, None, C.byref(st))
    assert rc != 0
