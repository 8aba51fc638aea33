"""CPU checks of the serving engine's host side: request validation and
memory footprints (mdzgpu_serve_footprint needs no GPU), the seeded request
stream, and that a server cannot start without a GPU (no silent fallback)."""
import math
from fractions import Fraction

import numpy as np
import pytest

from mdz_gb300 import MpVal, native, perturb_spacing
from mdz_gb300.serve import RenderRequest, Server, ServeError, footprint
from mdz_gb300.stream import FORMULAS, SIZES, load_pool, make_stream


def req(W=64, H=48, depth=1000, prec=128, fractal=0, method="auto", span="1e-20",
        want_mag=False):
    return RenderRequest(W, H, depth, MpVal.from_fraction(Fraction("-0.75"), prec),
                         MpVal.from_fraction(Fraction("0.1"), prec),
                         MpVal.from_fraction(Fraction(span), prec), prec, fractal=fractal,
                         method=method, want_mag=want_mag)


def al(b):
    return (b + 255) // 256 * 256


def test_footprint_perturbation_layout():
    r = req(W=100, H=60, depth=5000, prec=300, want_mag=True)
    dev, host = footprint(r)
    n = 100 * 60
    L = native.load().mdzgpu_perturb_limbs(300)
    entries = 5002
    orbit = (al(entries * 16) + al(entries * 16) + al(entries * 4) + al(entries * 8)
             + al(entries * 4) + al((entries // 32 + 40) * 4) + al(entries * 8)
             + al(entries * 4) + al((entries // 32 + 40) * 4) + al((entries // 32 + 40) * 4)
             + 256 + al(2 * L * 4) + 256 + al(entries * 2 * L * 4))
    # counts, |z|^2, 32-byte pixel state, two escalation lists, sync, orbit
    # (zq, zd, ze, dd, de, tiny-|Z| bit mask, fold value fm / fe, fold-axis
    # bit mask, attention bit mask, progress, centre, rebases, raw digits),
    # escalation-pass
    # coordinates
    words = 12   # 300 + 40 bits -> 11 words -> even
    expect = (al(4 * n) + al(4 * n) + al(32 * n) + al(256 + 8 * n) + 256 + al(orbit)
              + al((100 + 60) * words * 4))
    assert dev == expect
    assert host >= 8 * n


def test_footprint_multi_limb_scales_with_words():
    d1, _ = footprint(req(fractal=3, prec=128))
    d2, _ = footprint(req(fractal=3, prec=1000))
    assert d2 > 3 * d1
    d3, _ = footprint(req(fractal=1, method="multi_limb", prec=128))
    assert d3 == d1


def julia_req(method="auto", jre="-0.8", prec=128, W=64, H=48):
    r = req(W=W, H=H, prec=prec, method=method, span="1.5")
    r.family = 1
    r.julia = (MpVal.from_fraction(Fraction(jre), prec), MpVal.from_fraction(Fraction("0.156"),
                                                                              prec))
    return r


def test_footprint_julia_adds_the_constant():
    # the Julia family runs on the multi-limb kernel: its coordinate tables
    # carry the constant's two numbers after the pixel rows
    dj, _ = footprint(julia_req())
    dm, _ = footprint(req(W=64, H=48, prec=128, method="multi_limb", span="1.5"))
    words = 6   # 128 + 40 bits -> 6 words
    assert dj - dm == al((64 + 48 + 2) * words * 4) - al((64 + 48) * words * 4)


@pytest.mark.parametrize("kw", [
    dict(method="perturbation"),   # perturbation serves the Mandelbrot family
    dict(jre="4.5"),               # constant out of range
])
def test_footprint_rejects_julia(kw):
    with pytest.raises(ServeError):
        footprint(julia_req(**kw))


@pytest.mark.parametrize("kw", [
    dict(fractal=3, method="perturbation"),   # no perturbation for the hybrid
    dict(prec=4000, fractal=1),               # beyond the multi-limb words
    dict(W=0),
    dict(depth=0),
])
def test_footprint_rejects(kw):
    with pytest.raises(ServeError):
        footprint(req(**kw))


def test_server_needs_a_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(ServeError):
        Server(0)


def test_stream_is_seeded_and_follows_the_distributions():
    pool = load_pool()
    assert {c["fractal"] for c in pool} == set(FORMULAS)
    a = make_stream(400, pool)
    b = make_stream(400, pool)
    assert a == b
    assert make_stream(400, pool, seed=1) != a
    sizes = {(i.width, i.height) for i in a}
    assert sizes == set(SIZES)
    frac = np.array([i.fractal for i in a])
    assert abs((frac == 0).mean() - 0.7) < 0.08
    assert all(1000 <= i.depth <= 100000 for i in a)
    assert all(i.precision == math.ceil(-i.log2_span) + 64 for i in a)
    assert all(-1000 <= i.log2_span <= -10 for i in a)
    assert all(pool[i.centre]["fractal"] == i.fractal for i in a)
    assert abs(np.mean([i.gap for i in a]) - 1.0) < 0.15


def test_stream_request_geometry():
    pool = load_pool()
    it = make_stream(3, pool)[0]
    r = it.request(pool)
    assert r.precision == it.precision
    span = r.span.to_fraction()
    assert abs(math.log2(span) - it.log2_span) < 1e-9
    hs_m, hs_e = perturb_spacing(r.span, it.width)
    # half pixel spacing = span / (2 W), to 40 bits
    assert abs(math.log2(hs_m) + hs_e - (it.log2_span - math.log2(2 * it.width))) < 1e-9
    dev, host = footprint(r)
    assert dev > 4 * it.width * it.height
