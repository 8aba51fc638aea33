"""Generates the committed golden fixtures and seeded views (run where the
reference sources exist; the GPU tests only read the committed outputs).

  python tests/golden/make_golden.py fp64      # fp64_*.npz  (reference double build)
  python tests/golden/make_golden.py views     # views.json  (seeded ray bisection)
  python tests/golden/make_golden.py mp        # mp_*.npz    (reference MPFR path, p and 2p)
  python tests/golden/make_golden.py perturb   # perturb_c4.npz (MPFR at 2176 bits)
  python tests/golden/make_golden.py abi       # abi_layout.json (reference struct offsets)
  python tests/golden/make_golden.py centres   # serve_centres.json (serving stream centres)
  python tests/golden/make_golden.py colour    # colour.npz (reference palette_apply / AA)
  python tests/golden/make_golden.py perturb_fold  # perturb_fold.npz (ship / celtic, MPFR 2p)
  python tests/golden/make_golden.py perturb_julia # perturb_julia.npz (Julia family, MPFR 2p)
  python tests/golden/make_golden.py perturb_variant  # perturb_variant.npz (hybrid, MPFR 2p)
  python tests/golden/make_golden.py c2        # c2_frame.json + c2_rows.npz (full config-2 frame)
  python tests/golden/make_golden.py serve_mdz # mdz/*.mdz + serve_mdz.npz (settings files served)
  python tests/golden/make_golden.py perturb_rebase  # perturb_rebase.npz (2^-1000, rebases at depth)
  python tests/golden/make_golden.py gmp4      # gmp4_counts.npz (GMP callback, four formulas)

Counts come from the UNMODIFIED reference compiled by oracle/build_ref.sh
(oracle/_ref/libmdzref_d.so: long double = double, no FMA) driven through its
own rth_* thread pool, or, for explicit pixel lists, from its frac_*_mpfr
loop through the oracle restatement (checked identical to the reference on
every fixture here).  Seeds: numpy PCG64 with the seeds written below.
"""
from __future__ import annotations

import hashlib
import json
import math
import sys
import time
from fractions import Fraction
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mdz_gb300.mpval import MpVal, hexfloat  # noqa: E402
from mdz_gb300.views import View  # noqa: E402
from oracle import oracle as O  # noqa: E402

GOLD = Path(__file__).resolve().parent
THREADS = 8
JULIA_C = ("-0.8", "0.156")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.int32).tobytes()).hexdigest()


def pixel_iters(a: np.ndarray, depth: int) -> int:
    a = a.astype(np.int64)
    return int(np.where(a == 0, depth, a).sum())


# --------------------------------------------------------------------------
# FP64 fixtures
# --------------------------------------------------------------------------

def fp64_views() -> list[View]:
    vs = [View("c1", 240, 180, 1000, "-0.75", "0", "3.0")]
    # every formula x family on small frames
    centres = {0: ("-0.75", "0.1", "3.0"), 1: ("-0.45", "-0.5", "3.4"),
               2: ("-0.5", "0.2", "3.2"), 3: ("-0.6", "0.15", "3.2")}
    for fr, (cx, cy, sz) in centres.items():
        vs.append(View(f"f{fr}_mandel", 96, 64, 600, cx, cy, sz, fractal=fr))
        vs.append(View(f"f{fr}_julia", 96, 64, 600, "0", "0", "3.2", fractal=fr, family=1,
                       julia_re=JULIA_C[0], julia_im=JULIA_C[1]))
    # anti-aliased, odd sizes, a zoomed view with deep counts, depth 1
    vs.append(View("aa3", 40, 30, 800, "-0.7436447860", "0.1318252536", "0.00003", aa=3))
    vs.append(View("odd", 37, 23, 300, "-0.5", "0", "3.5"))
    vs.append(View("depth1", 33, 17, 1, "-0.5", "0", "4.0"))
    vs.append(View("deep", 128, 96, 20000, "-0.74364478", "0.13182525", "1e-6"))
    return vs


def make_fp64() -> None:
    out = {}
    for v in fp64_views():
        t0 = time.time()
        ref, _ = O.ref_render(v, threads=THREADS, variant="d")
        ld, _ = O.ref_render(v, threads=THREADS, variant="ld")
        r = v.rect()
        xmin, xmax, ymax = r.doubles()
        jre = float(v.julia()[0].to_fraction()) if v.family else 0.0
        jim = float(v.julia()[1].to_fraction()) if v.family else 0.0
        mine, _ = O.render_fp64(v.real_width, v.real_height, v.depth, xmin, xmax, ymax,
                                v.family, v.fractal, (jre, jim), aa=v.aa, threads=THREADS)
        assert np.array_equal(ref, mine), f"oracle restatement differs from reference on {v.name}"
        out[v.name] = ref
        print(f"{v.name}: {ref.shape} iters={pixel_iters(ref, v.depth)} "
              f"ld-differs={int((ld != ref).sum())} ({time.time() - t0:.1f}s)")
    meta = {v.name: dict(v.__dict__, rect=[hexfloat(Fraction(x)) for x in v.rect().doubles()],
                         sha256=sha(out[v.name]), pixel_iters=pixel_iters(out[v.name], v.depth))
            for v in fp64_views()}
    np.savez_compressed(GOLD / "fp64_counts.npz", **out)
    (GOLD / "fp64_views.json").write_text(json.dumps(meta, indent=1, default=str))


C2_ROW_STEP = 27


def make_c2() -> None:
    """The seeded 1920x1080 view with 3x3 supersampling (5760x3240 counts),
    width 1e-11, maxiter 20000, rendered in full by the unmodified reference
    (double build without FMA, rth_* thread pool): the frame's sha256 and
    iteration total, and every 27th row (rows 0, 27, ..., 3213) as the
    committed comparison data."""
    views = json.loads((GOLD / "views.json").read_text())
    v = View.from_dict({k: x for k, x in views["c2"].items() if k != "seed"})
    t0 = time.time()
    ref, t_ref = O.ref_render(v, threads=THREADS, variant="d")
    rows = ref[::C2_ROW_STEP]
    meta = {"view": views["c2"], "shape": list(ref.shape), "sha256": sha(ref),
            "pixel_iters": pixel_iters(ref, v.depth), "row_step": C2_ROW_STEP,
            "rows": len(rows), "rect": [hexfloat(Fraction(x)) for x in v.rect().doubles()],
            "source": "oracle/_ref/libmdzref_d.so (unmodified MDZ, long double = double, "
                      f"no FMA), rth_* with {THREADS} threads",
            "reference_render_s": round(t_ref, 1)}
    np.savez_compressed(GOLD / "c2_rows.npz", rows=rows)
    (GOLD / "c2_frame.json").write_text(json.dumps(meta, indent=1))
    print(f"c2: {ref.shape} iters={meta['pixel_iters']} ({time.time() - t0:.1f}s)")


GMP4_VIEWS = {0: ("-0.6", "0.5", "0.3"), 1: ("-1.5", "0", "0.4"), 2: ("-1.3", "0.2", "0.2"),
              3: ("-0.9", "0.2", "0.4")}


def make_gmp4() -> None:
    """MDZ's GMP callback (fractal_gmp_calculate_line, frac_*_gmp) for all
    four formulas: a 48x32 view each, rendered by the unmodified reference
    through rth_* at 128 bits and, to confirm the counts, at 256 bits; the
    GMP values MDZ's own string conversion leaves in img->gxmin / gymax /
    gwidth at 128 bits (src/my_mpfr_to_str.c:68) are recorded for the
    drop-in test to hand to the same callback.  A pixel whose count changes
    with the precision (the burning ship's real axis, where the row's y is
    a rounding residue that the fold doubles each step) is unconfirmed."""
    out, meta = {}, {}
    for f, (cx, cy, sz) in GMP4_VIEWS.items():
        key = f"gmp_f{f}"
        v = View(key, 48, 32, 1200, cx, cy, sz, precision=128, fractal=f, multi_prec=True,
                 rounding=False)
        v2 = View(key, 48, 32, 1200, cx, cy, sz, precision=256, fractal=f, multi_prec=True,
                  rounding=False)
        c1, _ = O.ref_render(v, threads=THREADS)
        c2, _ = O.ref_render(v2, threads=THREADS)
        d1 = O.ref_view_dump(v)
        out[key] = c1
        out[key + "__2p"] = c2
        meta[key] = dict(v.__dict__, gmp={k: d1[k] for k in ("gxmin", "gymax", "gwidth")})
        print(f"{key}: {len(np.unique(c1))} distinct counts, {(c1 == 0).mean():.3f} inside, "
              f"{int((c1 != c2).sum())} unconfirmed")
    np.savez_compressed(GOLD / "gmp4_counts.npz", **out)
    (GOLD / "gmp4_views.json").write_text(json.dumps(meta, indent=1, default=str))


def _mpf_value(g) -> Fraction:
    _, prec, size, exp, limbs = g
    n = abs(size)
    val = sum(Fraction(l) * Fraction(2) ** (64 * (i - n + exp)) for i, l in enumerate(limbs))
    return -val if size < 0 else val


def make_serve_mdz() -> None:
    """The reference's gallery settings files, written out again by
    mdz_gb300.mdzfile.dumps into tests/golden/mdz/ (the loader reads them
    back to the same settings), and for each the serving request the
    settings-file path builds (64 pixels across, the file's own rectangle)
    with MPFR at p and 2p bits on every pixel of the serving geometry."""
    from mdz_gb300 import mdzfile, perturb_pixel_c
    from mdz_gb300.serve import request_from_mdz
    dst = GOLD / "mdz"
    dst.mkdir(exist_ok=True)
    out, meta = {}, {}
    for f in sorted(_gallery().glob("*.mdz")):
        try:
            s = mdzfile.load(f)
        except mdzfile.MdzFileError as e:
            print(f"{f.name}: skipped ({e})")
            continue
        path = dst / f.name
        path.write_text(mdzfile.dumps(s))
        back = mdzfile.load(path)
        assert back.intended_view(64).__dict__ == s.intended_view(64).__dict__, f.name
        req = request_from_mdz(path, width=64, intended=True)
        W, H, prec = req.width, req.height, req.precision
        t0 = time.time()
        cre, cim = [], []
        for ln in range(H):
            for ix in range(W):
                x, y = perturb_pixel_c(req.cx, req.cy, req.span, W, H, ix, ln)
                cre.append(hexfloat(x))
                cim.append(hexfloat(y))
        c1, _ = O.points_mpfr(cre, cim, req.depth, prec, fractal=req.fractal, threads=THREADS)
        c2, _ = O.points_mpfr(cre, cim, req.depth, 2 * prec, fractal=req.fractal,
                              threads=THREADS)
        key = f.stem
        out[key] = c2.reshape(H, W).astype(np.int32)
        out[key + "__p"] = c1.reshape(H, W).astype(np.int32)
        meta[key] = dict(file=f"mdz/{f.name}", W=W, H=H, depth=req.depth, prec=prec,
                         fractal=req.fractal, oracle_prec=2 * prec)
        print(f"{key}: {W}x{H} depth {req.depth} prec {prec} fractal {req.fractal} "
              f"confirmed {(c1 == c2).mean():.4f} ({time.time() - t0:.1f}s)")
    np.savez_compressed(GOLD / "serve_mdz.npz", **out)
    (GOLD / "serve_mdz.json").write_text(json.dumps(meta, indent=1))


# --------------------------------------------------------------------------
# Seeded views (ray bisection on the reference's own escape loops)
# --------------------------------------------------------------------------

def ray_dir(seed: int) -> tuple[float, float]:
    rng = np.random.Generator(np.random.PCG64(seed))
    theta = float(rng.uniform(0.0, 2.0 * math.pi))
    return math.cos(theta), math.sin(theta)


def bisect_fp64(seed: int, depth: int, fractal: int = 0) -> tuple[float, float]:
    """Ray from 0 at a seeded angle; bisect r in [0, 2] on 'count == 0 at
    depth' (reference double loop) to 53-bit precision."""
    ct, st = ray_dir(seed)
    lo, hi = 0.0, 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if mid == lo or mid == hi:
            break
        if O.lib().mdzo_point_fp64(fractal, depth, mid * ct, mid * st) == 0:
            lo = mid
        else:
            hi = mid
    return lo * ct, lo * st


def bisect_mpfr(seed: int, depth: int, prec: int, start_bits: int = 50,
                fractal: int = 0) -> tuple[Fraction, Fraction]:
    """The same ray bisection continued in MPFR at `prec` bits; 7 points per
    round on THREADS cores (an 8-ary search, 3 bits per round)."""
    ct, st = (Fraction(x) for x in ray_dir(seed))
    lo, hi = Fraction(0), Fraction(2)
    # coarse stage in FP64 (identical predicate where doubles suffice)
    for _ in range(start_bits):
        mid = (lo + hi) / 2
        if O.lib().mdzo_point_fp64(fractal, depth, float(mid * ct), float(mid * st)) == 0:
            lo = mid
        else:
            hi = mid
    k = 8
    while hi - lo > Fraction(2) ** (-prec):
        pts = [lo + (hi - lo) * i / k for i in range(1, k)]
        cre = [MpVal.from_fraction(p * ct, prec).hex() for p in pts]
        cim = [MpVal.from_fraction(p * st, prec).hex() for p in pts]
        counts, _ = O.points_mpfr(cre, cim, depth, prec, fractal=fractal, threads=THREADS)
        inside = [c == 0 for c in counts]
        # last inside point before the first outside one
        new_lo, new_hi = lo, hi
        for p, ins in zip(pts, inside):
            if ins:
                new_lo = p
            else:
                new_hi = p
                break
        lo, hi = new_lo, new_hi
    c_re = MpVal.from_fraction(lo * ct, prec).to_fraction()
    c_im = MpVal.from_fraction(lo * st, prec).to_fraction()
    return c_re, c_im


def make_views() -> None:
    views = {}
    # C1: fixed
    views["c1"] = dict(name="c1", width=240, height=180, depth=1000, cx="-0.75", cy="0",
                       size="3.0", precision=80, aa=1)
    # C2: FP64, 1920x1080 x3 AA, maxiter 20000, width 1e-11, seed 2
    t0 = time.time()
    cx, cy = bisect_fp64(seed=2, depth=20000)
    views["c2"] = dict(name="c2", width=1920, height=1080, depth=20000, cx=hexfloat(Fraction(cx)),
                       cy=hexfloat(Fraction(cy)), size="1e-11", precision=80, aa=3, seed=2)
    print("c2", cx, cy, f"{time.time() - t0:.1f}s")
    # C3: 256-bit, 640x480, width 2^-200, maxiter 50000, seed 3, offset
    t0 = time.time()
    bre, bim = bisect_mpfr(seed=3, depth=50000, prec=256)
    rng = np.random.Generator(np.random.PCG64(1003))
    u1, u2 = (Fraction(float(x)) for x in rng.uniform(-0.5, 0.5, size=2))
    w3 = Fraction(1, 2 ** 200)
    views["c3"] = dict(name="c3", width=640, height=480, depth=50000,
                       cx=hexfloat(MpVal.from_fraction(bre + u1 * w3, 256).to_fraction()),
                       cy=hexfloat(MpVal.from_fraction(bim + u2 * w3, 256).to_fraction()),
                       size=hexfloat(w3), precision=256, aa=1, multi_prec=True, rounding=True,
                       seed=3)
    print("c3", f"{time.time() - t0:.1f}s")
    (GOLD / "views.json").write_text(json.dumps(views, indent=1))
    # C4: perturbation, 1920x1080, width 2^-1000, 1088-bit centre, maxiter 200000, seed 4
    t0 = time.time()
    bre, bim = bisect_mpfr(seed=4, depth=200000, prec=1088)
    views["c4"] = dict(name="c4", width=1920, height=1080, depth=200000, cx=hexfloat(bre),
                       cy=hexfloat(bim), size=hexfloat(Fraction(1, 2 ** 1000)), precision=1088,
                       aa=1, seed=4)
    print("c4", f"{time.time() - t0:.1f}s")
    (GOLD / "views.json").write_text(json.dumps(views, indent=1))


# Centre pool of the serving stream: seeded ray bisection per formula,
# refined to 1100 bits (enough for every precision of the stream,
# ceil(-log2 width) + 64 <= 1064).  The stream draws each request's centre
# from this pool.
SERVE_POOL = {0: range(5000, 5012), 1: range(6000, 6006), 2: range(7000, 7006)}
SERVE_BISECT_DEPTH = 10000
SERVE_PREC = 1100


def make_centres() -> None:
    out = {"bisect_depth": SERVE_BISECT_DEPTH, "prec": SERVE_PREC, "centres": []}
    for fractal, seeds in SERVE_POOL.items():
        for seed in seeds:
            t0 = time.time()
            bre, bim = bisect_mpfr(seed=seed, depth=SERVE_BISECT_DEPTH, prec=SERVE_PREC,
                                   fractal=fractal)
            out["centres"].append(dict(fractal=fractal, seed=seed, cx=hexfloat(bre),
                                       cy=hexfloat(bim)))
            print("centre", fractal, seed, f"{time.time() - t0:.1f}s", flush=True)
            (GOLD / "serve_centres.json").write_text(json.dumps(out, indent=1))


# Colouring fixtures: the reference's own palette_apply / do_anti_aliasing
# (oracle/_ref/libmdzref_io.so) on seeded counts, palettes and settings,
# including the palettes and colour settings of the gallery files.
def make_colour() -> None:
    import ctypes as C
    lib = C.CDLL(str(ROOT / "oracle" / "_ref" / "libmdzref_io.so"))
    from mdz_gb300.mdzfile import load as load_mdz
    rng = np.random.Generator(np.random.PCG64(2024))
    cases = []
    for f in sorted(_gallery().glob("*.mdz")):
        try:
            s = load_mdz(f)
        except Exception:
            continue
        cases.append(dict(palette=s.palette, scale=s.colour_scale, ip=int(s.palette_ip),
                          offset=s.palette_offset, tag=f.stem))
    for k in range(12):
        n = int(rng.integers(2, 257))
        cases.append(dict(palette=[int(x) for x in rng.integers(0, 2 ** 24, n)],
                          scale=float(rng.choice([1.0, 0.25, 0.37, 2.5, 7.125])),
                          ip=int(k % 2), offset=int(rng.integers(0, 256)), tag=f"random{k}"))
    arrays, meta = {}, []
    for i, c in enumerate(cases):
        for aa in (1, 2, 3):
            H, W = 6 * aa, 10 * aa
            raw = rng.integers(0, 5000, (H, W)).astype(np.int32)
            raw[rng.random((H, W)) < 0.15] = 0
            pal = np.asarray(c["palette"], np.uint32)
            out = np.zeros((H // aa, W // aa), np.uint32)
            ok = lib.mdzref_io_colour(raw.ctypes.data_as(C.c_void_p), W, H, aa, c["ip"],
                                      C.c_double(c["scale"]), pal.ctypes.data_as(C.c_void_p),
                                      len(pal), c["offset"], out.ctypes.data_as(C.c_void_p))
            assert ok
            key = f"c{i}_aa{aa}"
            arrays[key + "_raw"] = raw
            arrays[key + "_pal"] = pal
            arrays[key + "_rgb"] = out
            meta.append(dict(key=key, aa=aa, ip=c["ip"], scale=c["scale"], offset=c["offset"],
                             tag=c["tag"]))
    np.savez_compressed(GOLD / "colour.npz", **arrays)
    (GOLD / "colour.json").write_text(json.dumps(meta, indent=1))
    print("colour cases", len(meta))


# --------------------------------------------------------------------------
# Multiprecision fixtures (reference MPFR path at p and 2p)
# --------------------------------------------------------------------------

_RECTS: dict = {}


def mdz_mpfr_c(v: View, prec: int, ix: int, line: int) -> tuple[Fraction, Fraction]:
    """c of pixel (ix, line) exactly as fractal_mpfr_calculate_line computes
    it at `prec` bits (src/fractal.c:159-186) from image_info's rect."""
    from mdz_gb300.views import mdz_rect
    key = (v.width, v.height, v.precision, v.cx, v.cy, v.size)
    if key not in _RECTS:
        _RECTS[key] = mdz_rect(*key)
    r = _RECTS[key]

    def rn(x):
        return MpVal.from_fraction(x, prec).to_fraction()
    W = v.real_width
    width, xmin, ymax = r.width.to_fraction(), r.xmin.to_fraction(), r.ymax.to_fraction()
    t1 = rn(rn(width / W) * line)
    y = rn(ymax - t1)
    x = rn(rn(rn(Fraction(ix, W)) * width) + xmin)
    return x, y


def _gallery() -> Path:
    from oracle.build import ref_root
    root = ref_root()
    if root is None:
        raise SystemExit("make_golden: the MDZ source tree is not on this machine "
                         "(set MDZ_REF_ROOT)")
    return root / "gallery"


def gallery_views(width: int = 64) -> list[View]:
    """The reference's saved deep views (gallery/*.mdz), shrunk to `width`
    pixels across; rect-form files are turned into centre/size exactly."""
    from mdz_gb300.mpval import parse_number
    vs = []
    for f in sorted(_gallery().glob("*.mdz")):
        kv = {}
        for line in f.read_text().splitlines():
            parts = line.split(None, 1)
            if len(parts) == 2 and parts[0] in (
                    "fractal", "family", "depth", "aspect", "precision", "cx", "cy", "size",
                    "xmin", "xmax", "ymax"):
                kv.setdefault(parts[0], parts[1].strip())
            if line.strip() == "palette":
                break
        aspect = float(kv.get("aspect", "1.3333333333333333"))
        if "cx" in kv:
            cx, cy, size = (parse_number(kv[k]) for k in ("cx", "cy", "size"))
        else:
            xmin, xmax, ymax = (parse_number(kv[k]) for k in ("xmin", "xmax", "ymax"))
            size = xmax - xmin
            cx = (xmin + xmax) / 2
            cy = ymax - size / Fraction(aspect) / 2
        if aspect < 1:
            continue
        prec = int(kv.get("precision", "80"))
        H = max(8, int(round(width / aspect)))
        frac = {"mandelbrot": 0, "burning ship": 1, "generalized celtic": 2,
                "mandel-celtic hybrid": 3}[kv.get("fractal", "mandelbrot")]
        if frac != 0 and "family" not in kv:
            frac = 0
        digits = prec // 3 + 10
        vs.append(View(f"gal_{f.stem}", width, H, int(kv["depth"]), _dec(cx, digits),
                       _dec(cy, digits), _dec(size, digits), precision=prec,
                       multi_prec=True, rounding=True, fractal=frac))
    return vs


def _dec(x: Fraction, digits: int) -> str:
    """Decimal string with `digits` significant digits (exact enough for
    parsing at the view's precision)."""
    from decimal import Decimal, getcontext
    getcontext().prec = digits
    return str(Decimal(x.numerator) / Decimal(x.denominator))


def mp_views() -> list[View]:
    c3 = json.loads((GOLD / "views.json").read_text())["c3"]
    vs = gallery_views()
    for fr in range(4):
        vs.append(View(f"mp128_f{fr}", 48, 32, 1500, c3["cx"], c3["cy"], "0x1p-60",
                       precision=128, multi_prec=True, fractal=fr))
    vs.append(View("mp256_c3zoom", 64, 48, 4000, c3["cx"], c3["cy"], "0x1p-180",
                   precision=256, multi_prec=True))
    for fr in (1, 2):
        vs.append(View(f"mp96_shallow_f{fr}", 40, 30, 800, "-0.6", "0.3", "0.05",
                       precision=96, multi_prec=True, fractal=fr))
    vs.append(View("mp_julia", 40, 30, 1000, "0.01", "0.02", "0x1p-50", precision=128,
                   multi_prec=True, family=1, julia_re="-0.8", julia_im="0.156"))
    return vs


def make_mp() -> None:
    """Counts of the reference's MPFR path at the view's precision p, and the
    arbiter: the same pixel c values (p-bit, as fractal_mpfr_calculate_line
    rounds them) iterated with MPFR at 2p."""
    out, meta = {}, {}
    for v in mp_views():
        t0 = time.time()
        ref, _ = O.ref_render(v, threads=THREADS)
        cre, cim = [], []
        for ln in range(v.real_height):
            for ix in range(v.real_width):
                x, y = mdz_mpfr_c(v, v.precision, ix, ln)
                cre.append(hexfloat(x))
                cim.append(hexfloat(y))
        if v.family:
            jre, jim = (x.to_fraction() for x in v.julia())
            p1 = O.points_julia_mpfr(cre, cim, hexfloat(jre), hexfloat(jim), v.depth,
                                     v.precision, v.fractal, THREADS)
            p2 = O.points_julia_mpfr(cre, cim, hexfloat(jre), hexfloat(jim), v.depth,
                                     2 * v.precision, v.fractal, THREADS)
        else:
            p1, _ = O.points_mpfr(cre, cim, v.depth, v.precision, fractal=v.fractal,
                                  threads=THREADS)
            p2, _ = O.points_mpfr(cre, cim, v.depth, 2 * v.precision, fractal=v.fractal,
                                  threads=THREADS)
        p1 = p1.reshape(ref.shape).astype(np.int32)
        p2 = p2.reshape(ref.shape).astype(np.int32)
        assert np.array_equal(p1, ref), f"{v.name}: pixel c restatement differs from reference"
        out[v.name] = ref
        out[v.name + "__2p"] = p2
        meta[v.name] = dict(v.__dict__)
        print(f"{v.name}: confirmed {(ref == p2).mean():.4f} "
              f"iters={pixel_iters(ref, v.depth)} ({time.time() - t0:.1f}s)")
    # config 3 (640x480, 256 bits, width 2^-200, maxiter 50000) on a
    # subsampled pixel grid: every 8th column and row, at p and 2p
    c3 = View.from_dict(json.loads((GOLD / "views.json").read_text())["c3"])
    step = 8
    ixs = list(range(0, c3.real_width, step))
    lns = list(range(0, c3.real_height, step))
    cre, cim = [], []
    for ln in lns:
        for ix in ixs:
            x, y = mdz_mpfr_c(c3, c3.precision, ix, ln)
            cre.append(hexfloat(x))
            cim.append(hexfloat(y))
    for prec, key in ((c3.precision, "c3_sub"), (2 * c3.precision, "c3_sub__2p")):
        t0 = time.time()
        counts, _ = O.points_mpfr(cre, cim, c3.depth, prec, threads=THREADS)
        out[key] = counts.reshape(len(lns), len(ixs)).astype(np.int32)
        print(f"{key}: {time.time() - t0:.1f}s")
    meta["c3_sub"] = dict(c3.__dict__, step=step)
    # the GMP callback: reference's own gxmin/gymax/gwidth (the values its
    # mpfr_to_gmp string conversion leaves, src/my_mpfr_to_str.c:68)
    g = View("gmp_small", 48, 32, 1200, "-0.7436447860", "0.1318252536", "0.00002",
             precision=128, multi_prec=True, rounding=False)
    out["gmp_small"], _ = O.ref_render(g, threads=THREADS)
    d = O.ref_view_dump(g)
    meta["gmp_small"] = dict(g.__dict__, gmp={k: d[k] for k in ("gxmin", "gymax", "gwidth")})
    np.savez_compressed(GOLD / "mp_counts.npz", **out)
    (GOLD / "mp_views.json").write_text(json.dumps(meta, indent=1, default=str))


# --------------------------------------------------------------------------
# Perturbation fixtures (MPFR at twice the centre precision)
# --------------------------------------------------------------------------

def perturb_c(cx: Fraction, cy: Fraction, width: Fraction, W: int, H: int, ix: int, line: int):
    """Pixel c of the perturbation geometry: hs = width / (2 W) rounded to 40
    significant bits (mdzgpu_perturb_spacing), c = centre + ((2 ix - W) hs,
    (H - 2 line) hs)."""
    q = width / (2 * W)
    k = q.numerator.bit_length() - q.denominator.bit_length()
    if Fraction(2) ** k > q:
        k -= 1
    m = q / Fraction(2) ** k                       # [1, 2)
    m = Fraction(round(m * 2 ** 39), 2 ** 39)     # ties to even, 40 bits
    hs = m * Fraction(2) ** k
    return cx + (2 * ix - W) * hs, cy + (H - 2 * line) * hs


def make_perturb() -> None:
    views = json.loads((GOLD / "views.json").read_text())
    out, meta = {}, {}
    # small full frames: around the c3 / c4 centres, around the Misiurewicz
    # point c = i (structure at every scale), and the gallery's Mandelbrot views
    frames = [("p_c3_200", views["c3"]["cx"], views["c3"]["cy"], 64, 48, 6000,
               Fraction(2) ** -200, 256),
              ("p_c4_600", views["c4"]["cx"], views["c4"]["cy"], 48, 36, 8000,
               Fraction(2) ** -600, 704)]
    for wexp, depth in ((-200, 3000), (-600, 6000), (-1000, 8000)):
        frames.append((f"p_mis_i_{-wexp}", "0", "1", 64, 48, depth, Fraction(2) ** wexp,
                       -wexp + 64))
    frames.append(("p_mis_b_1000", "-0.10109636384562", "0.95628651080914", 48, 36, 8000,
                   Fraction(2) ** -1000, 1064))
    for g in gallery_views(48):
        if g.fractal == 0:
            frames.append(("p_" + g.name, g.cx, g.cy, g.width, g.height, g.depth,
                           parse_num(g.size), max(g.precision, 128)))
    for name, scx, scy, W, H, depth, width, prec in frames:
        cx = MpVal.from_fraction(parse_num(scx), prec).to_fraction()
        cy = MpVal.from_fraction(parse_num(scy), prec).to_fraction()
        width = MpVal.from_fraction(width, prec).to_fraction()
        t0 = time.time()
        cre, cim = [], []
        for ln in range(H):
            for ix in range(W):
                x, y = perturb_c(cx, cy, width, W, H, ix, ln)
                cre.append(hexfloat(x))
                cim.append(hexfloat(y))
        c1, m1 = O.points_mpfr(cre, cim, depth, prec, threads=THREADS)
        c2, m2 = O.points_mpfr(cre, cim, depth, 2 * prec, threads=THREADS)
        out[name] = c2.reshape(H, W).astype(np.int32)
        out[name + "__p"] = c1.reshape(H, W).astype(np.int32)
        out[name + "__mag"] = m2.reshape(H, W)
        meta[name] = dict(cx=hexfloat(cx), cy=hexfloat(cy), width=hexfloat(width), W=W, H=H,
                          depth=depth, prec=prec, oracle_prec=2 * prec)
        print(f"{name}: {time.time() - t0:.1f}s confirmed {(c1 == c2).mean():.4f}")
    # config 4: 4096 seeded sample pixels of the full frame, MPFR at 2176 bits
    v = views["c4"]
    cx, cy = parse_num(v["cx"]), parse_num(v["cy"])
    width = parse_num(v["size"])
    W, H, depth = v["width"], v["height"], v["depth"]
    rng = np.random.Generator(np.random.PCG64(4004))
    ix = rng.integers(0, W, 4096)
    ln = rng.integers(0, H, 4096)
    cre, cim = [], []
    for a, b in zip(ix, ln):
        x, y = perturb_c(cx, cy, width, W, H, int(a), int(b))
        cre.append(hexfloat(x))
        cim.append(hexfloat(y))
    t0 = time.time()
    counts, mag = O.points_mpfr(cre, cim, depth, 2176, threads=THREADS)
    print(f"c4 samples at 2176 bits: {time.time() - t0:.1f}s")
    out["c4_ix"], out["c4_line"] = ix.astype(np.int32), ln.astype(np.int32)
    out["c4_counts"], out["c4_mag"] = counts.astype(np.int64), mag
    meta["c4"] = dict(W=W, H=H, depth=depth, oracle_prec=2176, samples=4096, seed=4004)
    np.savez_compressed(GOLD / "perturb.npz", **out)
    (GOLD / "perturb_views.json").write_text(json.dumps(meta, indent=1))


def _fx_log2_abs2(re: int, im: int, F: int) -> float:
    """log2 |x + iy|^2 of fixed-point integers (F fractional bits); -inf at 0."""
    a = re * re + im * im
    if a == 0:
        return -math.inf
    sh = max(0, a.bit_length() - 60)
    return math.log2(a >> sh) + sh - 2 * F


def find_nucleus(cx: Fraction, cy: Fraction, radius: Fraction, maxp: int,
                 F: int = 1120) -> tuple[int, Fraction, Fraction]:
    """The nucleus of a minibrot near c0 = cx + i cy: its period p is the
    first n whose first-order image of the disc |c - c0| < radius,
    Z_n + dZ_n/dc (c - c0), contains 0; the nucleus solves Z_p(c) = 0 by
    Newton's method from c0 (Python integers, F fractional bits)."""
    one = 1 << F
    CR, CI = int(cx * one), int(cy * one)
    zr = zi = dr = di = 0
    lr2 = 2 * (math.log2(radius.numerator) - math.log2(radius.denominator))
    p = 0
    for n in range(1, maxp + 1):
        # dZ' = 2 Z dZ + 1, Z' = Z^2 + C
        dr, di = ((2 * (zr * dr - zi * di)) >> F) + one, (2 * (zr * di + zi * dr)) >> F
        zr, zi = ((zr * zr - zi * zi) >> F) + CR, ((2 * zr * zi) >> F) + CI
        lz2 = _fx_log2_abs2(zr, zi, F)
        if lz2 > 2.0:
            raise RuntimeError(f"centre escapes at {n}")
        if lz2 < lr2 + _fx_log2_abs2(dr, di, F):
            p = n
            break
    if not p:
        raise RuntimeError("no period below maxp")
    cr, ci = CR, CI
    for _ in range(60):
        zr = zi = dr = di = 0
        for _ in range(p):
            dr, di = ((2 * (zr * dr - zi * di)) >> F) + one, (2 * (zr * di + zi * dr)) >> F
            zr, zi = ((zr * zr - zi * zi) >> F) + cr, ((2 * zr * zi) >> F) + ci
        den = dr * dr + di * di
        if den == 0:
            raise RuntimeError("zero derivative")
        # (zr + i zi) / (dr + i di) in units of 2^-F
        qr = ((zr * dr + zi * di) << F) // den
        qi = ((zi * dr - zr * di) << F) // den
        cr, ci = cr - qr, ci - qi
        if abs(qr) <= 4 and abs(qi) <= 4:
            break
    return p, Fraction(cr, one), Fraction(ci, one)


def make_perturb_rebase() -> None:
    """A 2^-1000 frame, maxiter 200000, whose reference orbit passes through
    zero: the view is centred on the nucleus of a minibrot near the
    Misiurewicz point c = i whose size is about the frame's (its period p
    from the first-order image of a disc of radius 2^-500 around i, the
    nucleus by Newton's method), so Z_p is ~0 and every pixel rebases there
    (|Z_p + dz| < |dz|) -- and again at every multiple of p it reaches --
    while the pixels near the cardioid's edge orbit for up to ~2*10^5
    iterations before escaping.  The reference never escapes.  Scored, as
    config 4, on 4096 seeded pixels against MPFR at 2176 bits (counts and
    |z|^2 at escape).  (Around config 4's own centre the dynamics are nearly
    parabolic -- |dZ/dc| only reaches ~2^137 by iteration 200000 -- so a
    2^-1000 frame there is flat: every pixel escapes within one iteration of
    the reference and no pixel rebases.)"""
    W, H, depth, width = 1920, 1080, 200000, Fraction(2) ** -1000
    t0 = time.time()
    p, cx, cy = find_nucleus(Fraction(0), Fraction(1), Fraction(2) ** -500, 20000, F=1200)
    cx = MpVal.from_fraction(cx, 1088).to_fraction()
    cy = MpVal.from_fraction(cy, 1088).to_fraction()
    print(f"nucleus of period {p} ({time.time() - t0:.1f}s)")
    rng = np.random.Generator(np.random.PCG64(9009))
    ix = rng.integers(0, W, 4096)
    ln = rng.integers(0, H, 4096)
    cre, cim = [], []
    for a, b in zip(ix, ln):
        x, y = perturb_c(cx, cy, width, W, H, int(a), int(b))
        cre.append(hexfloat(x))
        cim.append(hexfloat(y))
    t0 = time.time()
    counts, mag = O.points_mpfr(cre, cim, depth, 2176, threads=THREADS)
    print(f"rebase view samples at 2176 bits: {time.time() - t0:.1f}s; counts "
          f"{int(counts.min())}..{int(counts.max())}, {len(np.unique(counts))} distinct, "
          f"{(counts == 0).mean():.3f} not escaping")
    np.savez_compressed(GOLD / "perturb_rebase.npz", ix=ix.astype(np.int32),
                        line=ln.astype(np.int32), counts=counts.astype(np.int64), mag=mag)
    (GOLD / "perturb_rebase.json").write_text(json.dumps(dict(
        cx=hexfloat(cx), cy=hexfloat(cy), width=hexfloat(width), W=W, H=H, depth=depth,
        prec=1088, oracle_prec=2176, samples=4096, seed=9009, period=p), indent=1))


def make_perturb_fold() -> None:
    """Burning ship and celtic frames for the folded perturbation, scored
    against MPFR at twice the precision.  The deep views sit at the serving
    pool's boundary points of each formula.  Near those points the folded
    maps are often chaotic: MPFR at p, 2p and 3p bits then give different
    counts for many pixels, so no computation at the view's precision can
    match pixel by pixel.  Each frame therefore stores the counts at p, 2p
    and 3p bits and a kind: "resolved" (the three agree on >= 99% of
    pixels: pixel-level parity applies) or "chaotic" (the score is the
    agreement rate with 2p, against the reference's own at p)."""
    pool = json.loads((GOLD / "serve_centres.json").read_text())["centres"]
    ship = [c for c in pool if c["fractal"] == 1]
    celtic = [c for c in pool if c["fractal"] == 2]
    P = Fraction(2)
    frames = [
        ("f_ship_shallow", 1, "-1.7626", "-0.0281", 48, 36, 2000, Fraction(1, 100), 64),
        ("f_celtic_shallow", 2, "-0.8", "0.15", 48, 36, 2000, Fraction(1, 5), 64),
        ("f_ship_a300", 1, ship[3]["cx"], ship[3]["cy"], 48, 36, 10000, P ** -300, 364),
        ("f_ship_b700", 1, ship[4]["cx"], ship[4]["cy"], 32, 24, 10000, P ** -700, 764),
        ("f_ship_c300", 1, ship[1]["cx"], ship[1]["cy"], 48, 36, 3000, P ** -300, 364),
        ("f_celtic_a300", 2, celtic[0]["cx"], celtic[0]["cy"], 48, 36, 3000, P ** -300, 364),
        ("f_celtic_b300", 2, celtic[2]["cx"], celtic[2]["cy"], 48, 36, 3000, P ** -300, 364),
        ("f_ship_chaos100", 1, ship[0]["cx"], ship[0]["cy"], 48, 36, 4000, P ** -100, 164),
        ("f_celtic_chaos1000", 2, celtic[2]["cx"], celtic[2]["cy"], 32, 24, 12000, P ** -1000,
         1064),
    ]
    out, meta = {}, {}
    for name, fr, scx, scy, W, H, depth, width, prec in frames:
        cx = MpVal.from_fraction(parse_num(scx), prec).to_fraction()
        cy = MpVal.from_fraction(parse_num(scy), prec).to_fraction()
        width = MpVal.from_fraction(width, prec).to_fraction()
        t0 = time.time()
        cre, cim = [], []
        for ln in range(H):
            for ix in range(W):
                x, y = perturb_c(cx, cy, width, W, H, ix, ln)
                cre.append(hexfloat(x))
                cim.append(hexfloat(y))
        c1, _ = O.points_mpfr(cre, cim, depth, prec, fractal=fr, threads=THREADS)
        c2, m2 = O.points_mpfr(cre, cim, depth, 2 * prec, fractal=fr, threads=THREADS)
        c3, _ = O.points_mpfr(cre, cim, depth, 3 * prec, fractal=fr, threads=THREADS)
        agree = float(((c1 == c2) & (c2 == c3)).mean())
        out[name] = c2.reshape(H, W).astype(np.int32)
        out[name + "__p"] = c1.reshape(H, W).astype(np.int32)
        out[name + "__3p"] = c3.reshape(H, W).astype(np.int32)
        out[name + "__mag"] = m2.reshape(H, W)
        meta[name] = dict(fractal=fr, cx=hexfloat(cx), cy=hexfloat(cy), width=hexfloat(width),
                          W=W, H=H, depth=depth, prec=prec, oracle_prec=2 * prec,
                          kind="resolved" if agree >= 0.99 else "chaotic")
        print(f"{name}: {time.time() - t0:.1f}s distinct counts {len(np.unique(c2))} "
              f"p = 2p = 3p on {agree:.4f} -> {meta[name]['kind']}", flush=True)
    np.savez_compressed(GOLD / "perturb_fold.npz", **out)
    (GOLD / "perturb_fold_views.json").write_text(json.dumps(meta, indent=1))


def julia_boundary_point(fr: int, jre: str, jim: str, a: tuple, b: tuple, bits: int,
                         depth: int) -> tuple:
    """A point of the Julia set's boundary by bisection on the segment a -> b
    (a inside: never escapes within depth; b outside), at `bits` bits; the
    constant (jre, jim) as exact hexadecimal strings."""
    def escapes(z):
        x, y = z
        c = O.points_julia_mpfr([hexfloat(x)], [hexfloat(y)], jre, jim, depth, bits + 64,
                                fractal=fr)
        return int(c[0]) != 0
    lo, hi = (Fraction(a[0]), Fraction(a[1])), (Fraction(b[0]), Fraction(b[1]))
    assert not escapes(lo) and escapes(hi)
    for _ in range(bits):
        mid = ((lo[0] + hi[0]) / 2, (lo[1] + hi[1]) / 2)
        if escapes(mid):
            hi = mid
        else:
            lo = mid
    return lo


def make_perturb_julia() -> None:
    """Julia-family frames (z0 = pixel, c fixed) for the perturbation with a
    view orbit and a critical orbit: centres on the Julia sets' boundaries
    (bisection at depth 10^4), scored against MPFR at 2p, with p and 3p
    stored to classify each view as in make_perturb_fold."""
    P = Fraction(2)
    specs = [
        ("j_basilica_40", 0, "-1", "0", (0, 0), (2, "0.75"), 48, 36, 3000, P ** -40, 104),
        ("j_basilica_200", 0, "-1", "0", (0, 0), (2, "0.75"), 48, 36, 6000, P ** -200, 264),
        ("j_rabbit_600", 0, "-0.122561166876654", "0.744861766619744", (0, 0), ("1.5", "1"),
         32, 24, 8000, P ** -600, 664),
        ("j_ship_100", 1, "-0.5", "-0.5", (0, 0), (0, 2), 48, 36, 4000, P ** -100, 164),
        ("j_celtic_150", 2, "-1", "0.1", (0, 0), (2, "0.125"), 48, 36, 4000, P ** -150, 214),
    ]
    out, meta = {}, {}
    for name, fr, jre, jim, a, b, W, H, depth, width, prec in specs:
        t0 = time.time()
        jr = MpVal.from_fraction(Fraction(jre), prec).to_fraction()
        ji = MpVal.from_fraction(Fraction(jim), prec).to_fraction()
        cx, cy = julia_boundary_point(fr, hexfloat(jr), hexfloat(ji), a, b, prec, 10000)
        cx = MpVal.from_fraction(cx, prec).to_fraction()
        cy = MpVal.from_fraction(cy, prec).to_fraction()
        width = MpVal.from_fraction(width, prec).to_fraction()
        zre, zim = [], []
        for ln in range(H):
            for ix in range(W):
                x, y = perturb_c(cx, cy, width, W, H, ix, ln)
                zre.append(hexfloat(x))
                zim.append(hexfloat(y))
        got = [O.points_julia_mpfr(zre, zim, hexfloat(jr), hexfloat(ji), depth, q, fractal=fr,
                                   threads=THREADS) for q in (prec, 2 * prec, 3 * prec)]
        agree = float(((got[0] == got[1]) & (got[1] == got[2])).mean())
        out[name] = got[1].reshape(H, W).astype(np.int32)
        out[name + "__p"] = got[0].reshape(H, W).astype(np.int32)
        out[name + "__3p"] = got[2].reshape(H, W).astype(np.int32)
        meta[name] = dict(fractal=fr, julia_re=hexfloat(jr), julia_im=hexfloat(ji),
                          cx=hexfloat(cx), cy=hexfloat(cy), width=hexfloat(width), W=W, H=H,
                          depth=depth, prec=prec, oracle_prec=2 * prec,
                          kind="resolved" if agree >= 0.99 else "chaotic")
        print(f"{name}: {time.time() - t0:.1f}s distinct counts {len(np.unique(got[1]))} "
              f"interior {(got[1] == 0).mean():.2f} p = 2p = 3p on {agree:.4f}", flush=True)
    np.savez_compressed(GOLD / "perturb_julia.npz", **out)
    (GOLD / "perturb_julia_views.json").write_text(json.dumps(meta, indent=1))


def variant_boundary_point(a: tuple, b: tuple, bits: int, depth: int) -> tuple:
    """A boundary point of the variant formula's set by bisection on the
    segment a -> b of the c plane (a: never escapes within depth; b escapes)."""
    def escapes(z):
        c, _ = O.points_mpfr([hexfloat(z[0])], [hexfloat(z[1])], depth, bits + 64, fractal=3)
        return int(c[0]) != 0
    lo, hi = (Fraction(a[0]), Fraction(a[1])), (Fraction(b[0]), Fraction(b[1]))
    assert not escapes(lo) and escapes(hi)
    for _ in range(bits):
        mid = ((lo[0] + hi[0]) / 2, (lo[1] + hi[1]) / 2)
        if escapes(mid):
            hi = mid
        else:
            lo = mid
    return lo


def make_perturb_variant() -> None:
    """MDZ's variant (mandel/celtic hybrid: the celtic fold on odd
    iterations) under perturbation: frames around boundary points of its set
    (bisection at depth 10^4), counts by MPFR at p, 2p and 3p bits,
    classified as in make_perturb_fold."""
    P = Fraction(2)
    specs = [
        ("v_a_50", ("-0.5", "0.5"), ("0.25", "0.5"), 48, 36, 12000, P ** -50, 114),
        ("v_a_250", ("-0.5", "0.5"), ("0.25", "0.5"), 48, 36, 12000, P ** -250, 314),
        ("v_b_120", ("-0.25", "0.25"), ("-0.75", "0.125"), 48, 36, 12000, P ** -120, 184),
        ("v_b_500", ("-0.25", "0.25"), ("-0.75", "0.125"), 32, 24, 12000, P ** -500, 564),
    ]
    out, meta = {}, {}
    for name, a, b, W, H, depth, width, prec in specs:
        t0 = time.time()
        cx, cy = variant_boundary_point(a, b, prec, 10000)
        cx = MpVal.from_fraction(cx, prec).to_fraction()
        cy = MpVal.from_fraction(cy, prec).to_fraction()
        width = MpVal.from_fraction(width, prec).to_fraction()
        cre, cim = [], []
        for ln in range(H):
            for ix in range(W):
                x, y = perturb_c(cx, cy, width, W, H, ix, ln)
                cre.append(hexfloat(x))
                cim.append(hexfloat(y))
        got = [O.points_mpfr(cre, cim, depth, q, fractal=3, threads=THREADS)[0]
               for q in (prec, 2 * prec, 3 * prec)]
        agree = float(((got[0] == got[1]) & (got[1] == got[2])).mean())
        out[name] = got[1].reshape(H, W).astype(np.int32)
        out[name + "__p"] = got[0].reshape(H, W).astype(np.int32)
        out[name + "__3p"] = got[2].reshape(H, W).astype(np.int32)
        meta[name] = dict(fractal=3, cx=hexfloat(cx), cy=hexfloat(cy), width=hexfloat(width),
                          W=W, H=H, depth=depth, prec=prec, oracle_prec=2 * prec,
                          kind="resolved" if agree >= 0.99 else "chaotic")
        print(f"{name}: {time.time() - t0:.1f}s distinct counts {len(np.unique(got[1]))} "
              f"interior {(got[1] == 0).mean():.2f} p = 2p = 3p on {agree:.4f}", flush=True)
    np.savez_compressed(GOLD / "perturb_variant.npz", **out)
    (GOLD / "perturb_variant_views.json").write_text(json.dumps(meta, indent=1))


def parse_num(s):
    from mdz_gb300.mpval import parse_number
    return parse_number(s)


def make_abi() -> None:
    """abi_layout.json: offsets of image_info / rthdata from the reference
    headers, as compiled by gcc here (LP64)."""
    import tempfile
    sys.path.insert(0, str(ROOT / "tests"))
    import test_abi_cpu as T
    with tempfile.TemporaryDirectory() as d:
        offs = T.reference_layout(Path(d))
    (GOLD / "abi_layout.json").write_text(json.dumps(
        {"source": "gcc -std=gnu99 on src/image_info.h + src/render_threads.h (LP64)",
         "offsets": offs}))


def main(argv: list[str]) -> None:
    from oracle import build as ob
    ob.build()
    what = argv[1:] or ["fp64"]
    for w in what:
        {"fp64": make_fp64, "views": make_views, "abi": make_abi, "mp": make_mp,
         "perturb": make_perturb, "centres": make_centres, "colour": make_colour,
         "perturb_fold": make_perturb_fold, "perturb_julia": make_perturb_julia,
         "perturb_variant": make_perturb_variant, "c2": make_c2,
         "serve_mdz": make_serve_mdz, "perturb_rebase": make_perturb_rebase,
         "gmp4": make_gmp4}[w]()


if __name__ == "__main__":
    main(sys.argv)
