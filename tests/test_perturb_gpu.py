"""Perturbation method on the GPU, scored against MPFR at twice the
precision (fixtures from the oracle's MPFR loop, tests/golden/perturb.npz).

Bar: at most 0.1% of pixels differ in iteration count from the 2x-precision
MPFR oracle; the smooth-colour error nu = n + 1 - log2(log2|z_n|^2 / 2) is
reported and bounded for pixels whose count matches."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MpVal, parse_number

GOLD = Path(__file__).resolve().parent / "golden"
pytestmark = pytest.mark.gpu

if (GOLD / "perturb_views.json").exists():
    META = json.loads((GOLD / "perturb_views.json").read_text())
    DATA = np.load(GOLD / "perturb.npz")
else:  # pragma: no cover
    META, DATA = {}, {}

FRAMES = sorted(k for k in META if k != "c4")
VIEWS = json.loads((GOLD / "views.json").read_text())


def smooth(n, mag2):
    with np.errstate(all="ignore"):
        return n + 1 - np.log2(np.log2(mag2) / 2)


@pytest.mark.parametrize("name", FRAMES)
def test_perturb_frame_vs_mpfr_2x(renderer, name):
    m = META[name]
    prec = m["prec"]
    cx = MpVal.from_fraction(parse_number(m["cx"]), prec)
    cy = MpVal.from_fraction(parse_number(m["cy"]), prec)
    w = MpVal.from_fraction(parse_number(m["width"]), prec)
    counts, mag, st = renderer.render_perturb(m["W"], m["H"], m["depth"], cx, cy, w, prec,
                                              want_mag=True)
    want = DATA[name]
    diff = counts != want
    frac = float(diff.mean())
    assert frac <= 0.001 or int(diff.sum()) <= 2, f"{name}: {int(diff.sum())} pixels differ"
    ok = (~diff) & (want > 0)
    if ok.any():
        err = np.abs(smooth(counts[ok], mag[ok].astype(np.float64))
                     - smooth(want[ok], DATA[name + "__mag"][ok]))
        assert float(np.nanmax(err)) < 0.05, f"smooth-colour error {np.nanmax(err)}"
    assert st["pixel_iters"] > 0


def test_perturb_config4_samples(renderer):
    """Config 4 (1920x1080, 2^-1000, maxiter 200000): the full frame,
    scored on 4096 seeded pixels against MPFR at 2176 bits."""
    if "c4" not in META:
        pytest.skip("fixture not generated")
    v = VIEWS["c4"]
    prec = v["precision"]
    cx = MpVal.from_fraction(parse_number(v["cx"]), prec)
    cy = MpVal.from_fraction(parse_number(v["cy"]), prec)
    w = MpVal.from_fraction(parse_number(v["size"]), prec)
    counts, mag, st = renderer.render_perturb(v["width"], v["height"], v["depth"], cx, cy, w,
                                              prec, want_mag=True)
    ix, ln = DATA["c4_ix"], DATA["c4_line"]
    got = counts[ln, ix].astype(np.int64)
    want = DATA["c4_counts"]
    frac = float((got != want).mean())
    assert frac <= 0.001, f"{frac:.5f} of the 4096 samples differ"
