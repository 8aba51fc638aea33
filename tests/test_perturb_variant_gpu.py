"""MDZ's variant formula (the mandel/celtic hybrid of src/frac_variant.c:
Re = |Re^2 - Im^2| + Cr on odd iterations, Mandelbrot's on even ones) under
perturbation on the GPU: two reference orbits (folding at odd and at even
steps), rebases onto the one whose parity matches the pixel's iteration.
Frames at 2^-50 .. 2^-500 around boundary points of the formula's set
against MPFR at twice the precision (tests/golden/perturb_variant.npz, made
by make_golden.py perturb_variant): pixel-level parity on the views MPFR
resolves at their precision, the reference's own rate of disagreement
(within three standard deviations of two binomial rates) on the chaotic
ones."""
import json
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MpVal, parse_number

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "perturb_variant_views.json").read_text())
DATA = np.load(GOLD / "perturb_variant.npz")


@pytest.mark.parametrize("name", sorted(META))
def test_variant_frame_vs_mpfr_2x(renderer, name):
    m = META[name]
    prec = m["prec"]
    vals = [MpVal.from_fraction(parse_number(m[k]), prec) for k in ("cx", "cy", "width")]
    counts, _, st = renderer.render_perturb(m["W"], m["H"], m["depth"], *vals, prec,
                                            fractal=3)
    want = DATA[name]
    diff = counts != want
    n_diff, n_ref = int(diff.sum()), int((DATA[name + "__p"] != want).sum())
    print(f"{name} [{m['kind']}]: differ {n_diff}/{diff.size} (MPFR at p: {n_ref}); escalated "
          f"fp64 {st['escalated_fp64']} mp {st['escalated_mp']}; rebases {st['rebases']}")
    if m["kind"] == "resolved":
        assert n_diff <= max(2, 0.001 * diff.size), f"{name}: {n_diff} differ"
    else:
        n = diff.size
        r = n_ref / n
        assert n_diff / n <= r + 3.0 * np.sqrt(2.0 * r * (1.0 - r) / n), name
    assert st["pixel_iters"] > 0
