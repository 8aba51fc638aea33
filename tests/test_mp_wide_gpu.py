"""The multi-limb path beyond one thread's registers: precisions above 1112
bits run on the warp-cooperative kernel (8, 16 or 32 lanes per pixel,
64-bit limbs, carries resolved across lanes), through the explicit call,
MDZ's own MPFR callback (rth_* with fractal_mpfr_calculate_line) and the
line function.  Scored against MPFR with the bar of the multi-limb tests:
equal to MPFR at p on every pixel MPFR at 2p confirms, and on >= 99.9% of
all pixels.  The views sit around the Misiurewicz point c = i, where counts
vary at every scale; MPFR runs on the host's cores at test time."""
import ctypes as C

import numpy as np
import pytest

from mdz_gb300 import View
from mdz_gb300.abi import DropIn
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (precision, words the kernel takes, log2 of the view width, W, H, depth)
CASES = [(1200, 48, -1130, 48, 32, 2500), (2176, 80, -2100, 48, 32, 4000),
         (4000, 128, -3920, 32, 24, 6000)]


def view_of(prec, wexp, W, H, depth, name="wide"):
    return View(name, W, H, depth, "0", "1", f"0x1p{wexp}", precision=prec, multi_prec=True,
                rounding=True)


def mpfr_counts(v, prec):
    r = v.rect()
    got, _ = O.render_mpfr(v.real_width, v.real_height, v.depth, prec, r.xmin, r.ymax,
                           r.width, threads=16)
    return got


def check(got, p, p2, name):
    confirmed = p == p2
    bad = int(((got != p) & confirmed).sum())
    agree = float((got == p).mean())
    print(f"{name}: {bad} confirmed pixels differ; agree {agree:.5f}; "
          f"confirmed {confirmed.mean():.5f}; {len(np.unique(p))} distinct counts")
    assert bad == 0, f"{name}: {bad} confirmed pixels differ"
    assert agree >= min(0.999, float(confirmed.mean())), f"{name}: only {agree:.5f} agree"


@pytest.fixture(scope="module")
def mpfr_refs():
    if not O.has_mpfr():
        pytest.skip("libmpfr not on this host")
    out = {}
    for prec, words, wexp, W, H, depth in CASES:
        v = view_of(prec, wexp, W, H, depth)
        out[prec] = (mpfr_counts(v, prec), mpfr_counts(v, 2 * prec))
    return out


@pytest.mark.parametrize("prec,words,wexp,W,H,depth", CASES)
def test_wide_explicit_matches_mpfr(renderer, mpfr_refs, prec, words, wexp, W, H, depth):
    v = view_of(prec, wexp, W, H, depth)
    r = v.rect()
    got, st = renderer.render_mp(W, H, depth, r.xmin, r.ymax, r.width, prec)
    assert st["words"] == words
    p, p2 = mpfr_refs[prec]
    assert len(np.unique(p)) > 10
    check(got, p, p2, f"{prec} bits")


@pytest.mark.parametrize("prec,words,wexp,W,H,depth", CASES[:2])
def test_wide_dropin_mpfr_callback(renderer, mpfr_refs, prec, words, wexp, W, H, depth):
    """MDZ's MPFR callback at a precision the one-thread kernel can not hold
    (the reference takes any img->precision, src/coords.c:204-231)."""
    v = view_of(prec, wexp, W, H, depth)
    r = v.rect()
    want, _ = renderer.render_mp(W, H, depth, r.xmin, r.ymax, r.width, prec)
    # one row through the line function (before any render: once a render
    # has ended the status says stop, and the line functions return 0, as
    # the reference's do)
    d = DropIn(v)
    try:
        assert d.lib.fractal_mpfr_calculate_line(C.byref(d.img), 5) == 1
        assert np.array_equal(d.raw[5], want[5])
        info = d.render(timeout_s=300)
        assert sorted(info["drawn"]) == list(range(H))
        assert np.array_equal(d.raw, want)
    finally:
        d.close()
    p, p2 = mpfr_refs[prec]
    check(want, p, p2, f"drop-in {prec} bits")


def test_wide_word_counts_agree_on_shallow_view(renderer):
    """Every warp-cooperative width gives the same counts on a view that
    needs ~60 bits (where 192-bit MPFR confirms 96-bit MPFR), and the same
    as the one-thread kernel."""
    v = View("wide_shallow", 32, 24, 800, "-0.7436447860", "0.1318252536", "0.00002",
             precision=96, multi_prec=True, rounding=True)
    r = v.rect()
    base, _ = renderer.render_mp(32, 24, 800, r.xmin, r.ymax, r.width, 96, words=8)
    for words in (48, 64, 80, 96, 128, 160, 192, 256):
        got, st = renderer.render_mp(32, 24, 800, r.xmin, r.ymax, r.width, 96, words=words)
        assert st["words"] == words
        assert (got != base).mean() <= 0.002, words
