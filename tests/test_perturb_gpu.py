"""Perturbation method on the GPU, scored against MPFR at twice the
precision (fixtures from the oracle's MPFR loop, tests/golden/perturb.npz).

Bar: at most 0.1% of pixels (at least 2 on these small frames) differ in
iteration count from the 2x-precision MPFR oracle; the smooth-colour error
nu = n + 1 - log2(log2|z_n|^2 / 2) against the oracle's is reported (printed)
and its 99th percentile over count-matching pixels bounded by 0.01."""
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
    ok = (~diff) & (want > 0)
    err = np.zeros(1)
    if ok.any():
        err = np.abs(smooth(counts[ok], mag[ok].astype(np.float64))
                     - smooth(want[ok], DATA[name + "__mag"][ok]))
    print(f"{name}: count error {int(diff.sum())}/{diff.size} pixels; smooth-colour error "
          f"p99 {np.nanpercentile(err, 99):.2e} max {np.nanmax(err):.2e}; escalated "
          f"fp64 {st['escalated_fp64']} mp {st['escalated_mp']}")
    assert frac <= 0.001 or int(diff.sum()) <= 2, f"{name}: {int(diff.sum())} pixels differ"
    assert float(np.nanpercentile(err, 99)) < 0.01
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
    ok = (got == want) & (want > 0)
    err = np.abs(smooth(got[ok], mag[ln, ix][ok].astype(np.float64))
                 - smooth(want[ok], DATA["c4_mag"][ok])) if ok.any() else np.zeros(1)
    print(f"config 4: {int((got != want).sum())}/4096 samples differ; smooth-colour error "
          f"max {np.nanmax(err):.2e}")
    assert frac <= 0.001, f"{frac:.5f} of the 4096 samples differ"


def test_perturb_rebase_view_samples(renderer):
    """A 2^-1000 frame (1920x1080, maxiter 200000) centred on the nucleus of
    a minibrot whose cardioid spans the frame: the reference orbit passes
    through zero once a period, so pixels rebase there again and again
    (Zhuoran's rebasing, |Z_m + dz| < |dz|) while the ones near the
    cardioid's edge orbit for up to ~2*10^5 iterations before escaping.
    FP32 deltas can not resolve those counts (rounding a step moves c by
    ~2^-24 of its offset; 1.1% of the pixels came out wrong when the FP32
    pass kept them), so the pass hands every pixel stepping from the
    reference's zero to the FP64 pass.  Scored on 4096 seeded pixels against
    MPFR at 2176 bits."""
    path = GOLD / "perturb_rebase.json"
    if not path.exists():
        pytest.skip("fixture not generated")
    m = json.loads(path.read_text())
    data = np.load(GOLD / "perturb_rebase.npz")
    prec = m["prec"]
    cx = MpVal.from_fraction(parse_number(m["cx"]), prec)
    cy = MpVal.from_fraction(parse_number(m["cy"]), prec)
    w = MpVal.from_fraction(parse_number(m["width"]), prec)
    counts, mag, st = renderer.render_perturb(m["W"], m["H"], m["depth"], cx, cy, w, prec,
                                              want_mag=True)
    ix, ln = data["ix"], data["line"]
    got = counts[ln, ix].astype(np.int64)
    want = data["counts"]
    diff = got != want
    ok = (~diff) & (want > 0)
    err = np.abs(smooth(got[ok], mag[ln, ix][ok].astype(np.float64))
                 - smooth(want[ok], data["mag"][ok]))
    print(f"rebase view: {int(diff.sum())}/4096 samples differ "
          f"(max count error {int(np.abs(got - want).max())}); smooth-colour error p99 "
          f"{np.nanpercentile(err, 99):.2e} max {np.nanmax(err):.2e}; rebases {st['rebases']}; "
          f"escalated fp64 {st['escalated_fp64']} mp {st['escalated_mp']}; "
          f"{st['kernel_ms']:.0f} ms")
    # the reference passes through zero once a period: the FP32 pass hands
    # every pixel that steps from such an entry to the FP64 pass
    esc64, esc_mp = renderer.last_escalations()
    assert len(esc64) == st["escalated_fp64"] and len(esc_mp) == st["escalated_mp"]
    assert np.isin(ln.astype(np.int64) * m["W"] + ix, esc64).mean() > 0.9
    assert st["rebases"] > 0
    assert int(want.max()) > 100000
    assert float(diff.mean()) <= 0.001, f"{int(diff.sum())} of the 4096 samples differ"
    assert float(np.nanpercentile(err, 99)) < 0.01


@pytest.mark.parametrize("cx,cy,prec,n", [("-0.75", "0.1", 128, 60),
                                          ("0x1p-40", "1", 320, 100),
                                          ("-1.7497856353511106873", "0.0000153218", 1088, 200)])
def test_reference_orbit_matches_exact(renderer, cx, cy, prec, n):
    """The GPU's multi-limb orbit against exact rational iteration (Python
    big integers at the same digit precision, rounded to double)."""
    import ctypes as C
    from fractions import Fraction
    lib = renderer.lib
    cxv = MpVal.from_fraction(parse_number(cx), prec)
    cyv = MpVal.from_fraction(parse_number(cy), prec)
    L = int(lib.mdzgpu_perturb_limbs(prec))
    F = 28 * (L - 1)
    zr = np.zeros(n + 1)
    zi = np.zeros(n + 1)
    dm = np.zeros(n + 1)
    de = np.zeros(n + 1, np.int32)
    ln = C.c_int64()
    a, ka = cxv.struct()
    b, kb = cyv.struct()
    assert lib.mdzgpu_reference_orbit(renderer.ctx, C.byref(a), C.byref(b), prec, 0, n,
                                      zr.ctypes.data, zi.ctypes.data, dm.ctypes.data,
                                      de.ctypes.data, C.byref(ln)) == 0
    # exact orbit with truncation to F fractional bits (floor), as digits hold it
    CR = int(cxv.to_fraction() * 2 ** F)
    CI = int(cyv.to_fraction() * 2 ** F)
    xr, xi = CR, CI
    for k in range(1, int(ln.value)):
        want_r, want_i = float(Fraction(xr, 2 ** F)), float(Fraction(xi, 2 ** F))
        tol = 2.0 ** -45 * max(1.0, abs(want_r) + abs(want_i))
        assert abs(zr[k] - want_r) <= tol and abs(zi[k] - want_i) <= tol, k
        d = float(Fraction(xr * xr + xi * xi, 2 ** (2 * F)) - 4)
        got_d = float(Fraction(dm[k]) * Fraction(2) ** int(de[k]))
        assert abs(got_d - d) <= 1e-9 * max(1e-300, abs(d)) + 2.0 ** -40, k
        xr, xi = (xr * xr - xi * xi) // 2 ** F + CR, (2 * xr * xi) // 2 ** F + CI


@pytest.mark.parametrize("name", ["p_gal_polyp", "p_mis_b_1000", "p_gal_honeytrace",
                                  "p_gal_spiralblues"])
def test_perturb_schedules_agree(renderer, name, monkeypatch):
    """The three pass-0 schedules (streamed orbit with compacting steps, the
    orbit then one frame launch, the fused cooperative grid) give the same
    counts and |z|^2 bit for bit: the pixel loop is one function whose state
    can be saved and resumed at any iteration."""
    m = META[name]
    prec = m["prec"]
    args = (m["W"] * 2, m["H"] * 2, m["depth"],
            MpVal.from_fraction(parse_number(m["cx"]), prec),
            MpVal.from_fraction(parse_number(m["cy"]), prec),
            MpVal.from_fraction(parse_number(m["width"]) * 2, prec), prec)
    out = {}
    for mode in ("steps", "frame", "fused"):
        monkeypatch.setenv("MDZGPU_PERTURB", mode)
        counts, mag, st = renderer.render_perturb(*args, want_mag=True)
        out[mode] = (counts, mag.view(np.uint32), st)
    for mode in ("frame", "fused"):
        assert np.array_equal(out[mode][0], out["steps"][0]), mode
        assert np.array_equal(out[mode][1], out["steps"][1]), mode
        assert out[mode][2]["pixel_iters"] == out["steps"][2]["pixel_iters"], mode
