"""Multi-limb fixed-point path on the GPU against the reference's MPFR path.

The bar (fixed point is not MPFR arithmetic): counts equal MPFR at the same
precision p on every pixel where MPFR at 2p -- iterating the same p-bit pixel
c -- agrees with it ("confirmed"), and on at least 99.9% of all pixels.  On
views at the edge of their precision (some gallery views, where MPFR at p
and at 2p disagree on more than 0.1% of the pixels) the second bar is the
confirmed fraction: on unconfirmed pixels the fixed point, carrying 32+ more
bits than p, follows MPFR at 2p instead."""
import ctypes as C
import json
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MpVal, View
from mdz_gb300.abi import DropIn

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "mp_views.json").read_text())
COUNTS = np.load(GOLD / "mp_counts.npz")

pytestmark = pytest.mark.gpu

FRAME_VIEWS = sorted(k for k in META if k not in ("c3_sub", "gmp_small"))


def view_of(name):
    d = {k: v for k, v in META[name].items() if k not in ("gmp", "step")}
    return View.from_dict(d)


def check(got, p, p2, name):
    confirmed = p == p2
    bad_confirmed = int(((got != p) & confirmed).sum())
    agree = float((got == p).mean())
    assert bad_confirmed == 0, f"{name}: {bad_confirmed} confirmed pixels differ"
    assert agree >= min(0.999, float(confirmed.mean())), f"{name}: only {agree:.5f} agree"


@pytest.mark.parametrize("name", FRAME_VIEWS)
def test_mp_explicit_matches_mpfr(renderer, name):
    v = view_of(name)
    r = v.rect()
    julia = v.julia() if v.family else None
    got, st = renderer.render_mp(v.real_width, v.real_height, v.depth, r.xmin, r.ymax, r.width,
                                 v.precision, family=v.family, fractal=v.fractal, julia=julia)
    check(got, COUNTS[name], COUNTS[name + "__2p"], name)
    assert st["words"] * 32 - 8 >= v.precision


@pytest.mark.parametrize("words", [4, 6, 8, 10, 12, 16])
def test_mp_word_counts_agree_on_shallow_view(renderer, words):
    """Every compiled width gives the same counts where 96-bit MPFR is
    confirmed by 192-bit MPFR (a view that needs ~40 bits)."""
    name = "mp96_shallow_f2"
    v = view_of(name)
    r = v.rect()
    got, st = renderer.render_mp(v.real_width, v.real_height, v.depth, r.xmin, r.ymax, r.width,
                                 v.precision, words=words, fractal=v.fractal)
    assert st["words"] == words
    check(got, COUNTS[name], COUNTS[name + "__2p"], name)


def test_mp_config3_subsampled(renderer):
    """Config 3 (640x480, 256 bits, width 2^-200, maxiter 50000) rendered in
    full; scored on every 8th pixel against MPFR-256 / MPFR-512."""
    m = META["c3_sub"]
    v = view_of("c3_sub")
    r = v.rect()
    got, st = renderer.render_mp(v.real_width, v.real_height, v.depth, r.xmin, r.ymax, r.width,
                                 v.precision)
    step = m["step"]
    sub = got[::step, ::step]
    check(sub, COUNTS["c3_sub"], COUNTS["c3_sub__2p"], "c3_sub")
    assert st["words"] == 10


@pytest.mark.parametrize("name", ["gal_honeytrace", "mp_julia", "gal_floral"])
def test_mp_dropin_mpfr_callback(name):
    v = view_of(name)
    d = DropIn(v)
    try:
        d.render(timeout_s=300)
        check(d.raw, COUNTS[name], COUNTS[name + "__2p"], name)
    finally:
        d.close()


def test_mp_dropin_gmp_callback():
    """fractal_gmp_calculate_line reads img->gxmin/gymax/gwidth (GMP layout),
    here the values MDZ's own string conversion leaves in them."""
    m = META["gmp_small"]
    v = view_of("gmp_small")
    g = {}
    for key in ("gxmin", "gymax", "gwidth"):
        _, prec, size, exp, limbs = m["gmp"][key]
        n = abs(size)
        val = sum(Fraction(l) * Fraction(2) ** (64 * (i - n + exp)) for i, l in enumerate(limbs))
        g[key] = MpVal.from_fraction(-val if size < 0 else val, 64 * max(n, 1))
    d = DropIn(v, gmp_values=g)
    try:
        d.render(timeout_s=300)
        want = COUNTS["gmp_small"]
        assert float((d.raw == want).mean()) >= 0.999
    finally:
        d.close()


GMP4 = json.loads((GOLD / "gmp4_views.json").read_text())
GMP4_COUNTS = np.load(GOLD / "gmp4_counts.npz")


def gmp_values(m):
    """The mpf_t values (precision, signed size, exponent, limbs) MDZ's
    string conversion left in img->gxmin/gymax/gwidth, as exact values."""
    g = {}
    for key in ("gxmin", "gymax", "gwidth"):
        _, prec, size, exp, limbs = m["gmp"][key]
        n = abs(size)
        val = sum(Fraction(l) * Fraction(2) ** (64 * (i - n + exp)) for i, l in enumerate(limbs))
        g[key] = MpVal.from_fraction(-val if size < 0 else val, 64 * max(n, 1))
    return g


@pytest.mark.parametrize("name", sorted(GMP4))
def test_mp_dropin_gmp_callback_each_formula(name):
    """fractal_gmp_calculate_line for every formula (frac_mandel_gmp,
    frac_burning_ship_gmp, frac_generalised_celtic_gmp, frac_variant_gmp),
    fed the GMP values MDZ itself left in the image, against the reference's
    own GMP render at 128 bits through rth_* (counts for the whole 48x32
    view): equal on every pixel the 256-bit render confirms, and on at least
    99.9% of them all (or the confirmed fraction, where lower)."""
    m = GMP4[name]
    v = View.from_dict({k: x for k, x in m.items() if k != "gmp"})
    d = DropIn(v, gmp_values=gmp_values(m))
    try:
        d.render(timeout_s=300)
        want, want2 = GMP4_COUNTS[name], GMP4_COUNTS[name + "__2p"]
        for ln, ix in np.argwhere(d.raw != want)[:10]:
            print(f"{name} ({ix},{ln}): gpu {d.raw[ln, ix]} reference {want[ln, ix]} "
                  f"at 256 bits {want2[ln, ix]}")
        check(d.raw, want, want2, name)
        assert len(np.unique(want)) > 20
    finally:
        d.close()


def test_mp_line_entry_point():
    v = view_of("gal_polyp")
    d = DropIn(v)
    try:
        for line in (0, v.real_height // 2, v.real_height - 1):
            assert d.lib.fractal_mpfr_calculate_line(C.byref(d.img), line) == 1
            want = COUNTS["gal_polyp"][line]
            conf = want == COUNTS["gal_polyp__2p"][line]
            assert np.array_equal(d.raw[line][conf], want[conf])
    finally:
        d.close()


def test_mp_rejects_out_of_range(renderer):
    from mdz_gb300 import MdzGpuError
    big = MpVal.from_fraction(-5, 128)
    w = MpVal.from_fraction(1, 128)
    with pytest.raises(Exception):
        renderer.render_mp(8, 8, 10, big, MpVal.from_fraction(1, 128), w, 128)
