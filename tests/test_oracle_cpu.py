"""The CPU oracle is pinned to the reference: restatement == unmodified MDZ
(where the reference is compiled) and == the committed golden counts."""
import json
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import View, parse_number
from oracle import oracle as O

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "fp64_views.json").read_text())
COUNTS = np.load(GOLD / "fp64_counts.npz")


def view_of(name):
    return View.from_dict({k: v for k, v in META[name].items()
                           if k not in ("rect", "sha256", "pixel_iters")})


@pytest.mark.parametrize("name", sorted(META))
def test_fp64_restatement_matches_golden(name):
    v = view_of(name)
    rect = v.rect().doubles()
    assert rect == tuple(float(parse_number(s)) for s in META[name]["rect"])
    jre, jim = ((float(v.julia()[0].to_fraction()), float(v.julia()[1].to_fraction()))
                if v.family else (0.0, 0.0))
    got, its = O.render_fp64(v.real_width, v.real_height, v.depth, *rect, v.family, v.fractal,
                             (jre, jim), aa=v.aa, threads=4)
    assert np.array_equal(got, COUNTS[name])
    assert its == META[name]["pixel_iters"]


needs_ref = pytest.mark.skipif(not O.ref_available(), reason="reference not compiled here")


@needs_ref
@pytest.mark.parametrize("view", [
    View("w", 50, 40, 300, "-0.5", "0.3", "2.9"),
    View("tall", 30, 50, 300, "-0.5", "0.1", "2.5"),
    View("deep256", 40, 30, 400, "-1.25066", "0.02012", "1e-40", precision=256),
    View("deep1088", 24, 20, 300, "-0.1592", "1.0317", "0x1p-900", precision=1088),
    View("jul", 40, 30, 400, "0.1", "0", "3", family=1, julia_re="-0.8", julia_im="0.156",
         precision=160),
])
def test_view_geometry_matches_reference(view):
    d = O.ref_view_dump(view)
    r = view.rect()
    assert (d["xmin"], d["xmax"], d["ymax"], d["width"]) == (r.xmin, r.xmax, r.ymax, r.width)
    if view.family:
        assert (d["julia_re"], d["julia_im"]) == view.julia()


@needs_ref
@pytest.mark.parametrize("fractal", [0, 1, 2, 3])
@pytest.mark.parametrize("family", [0, 1])
def test_fp64_restatement_matches_reference(fractal, family):
    v = View("x", 48, 36, 700, "-0.6", "0.2", "3.1", fractal=fractal, family=family,
             julia_re="-0.75", julia_im="0.11", aa=2)
    ref, _ = O.ref_render(v, threads=4)
    rect = v.rect().doubles()
    jre, jim = ((float(v.julia()[0].to_fraction()), float(v.julia()[1].to_fraction()))
                if family else (0.0, 0.0))
    got, _ = O.render_fp64(v.real_width, v.real_height, v.depth, *rect, family, fractal,
                           (jre, jim), aa=2, threads=4)
    assert np.array_equal(got, ref)


@needs_ref
@pytest.mark.skipif(not O.has_mpfr(), reason="libmpfr.so.6 absent")
@pytest.mark.parametrize("fractal", [0, 1, 2, 3])
def test_mpfr_restatement_matches_reference(fractal):
    v = View("m", 24, 18, 400, "-0.7436447860", "0.1318252536", "0x1p-60", precision=192,
             multi_prec=True, rounding=True, fractal=fractal)
    ref, _ = O.ref_render(v, threads=4)
    r = v.rect()
    got, _ = O.render_mpfr(v.real_width, v.real_height, v.depth, v.precision, r.xmin, r.ymax,
                           r.width, fractal=fractal, threads=4)
    assert np.array_equal(got, ref)
