"""Colouring epilogue, CPU side: the oracle's restatement of palette_apply /
do_anti_aliasing against the reference's own functions (committed outputs in
tests/golden/colour.npz, and the compiled reference itself where it was
built), and the .mdz settings reader against the reference's loader."""
import ctypes as C
import json
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from oracle.build import ref_root

ROOT = Path(__file__).resolve().parents[1]
GOLD = ROOT / "tests" / "golden"
REF_IO = ROOT / "oracle" / "_ref" / "libmdzref_io.so"
_REF_ROOT = ref_root()
GALLERY = _REF_ROOT / "gallery" if _REF_ROOT else ROOT / "oracle" / "_absent"
META = json.loads((GOLD / "colour.json").read_text())
DATA = np.load(GOLD / "colour.npz")


@pytest.mark.parametrize("case", META, ids=[m["key"] for m in META])
def test_oracle_colour_matches_reference_fixtures(case):
    k = case["key"]
    got = O.colour(DATA[k + "_raw"], case["aa"], case["ip"], case["scale"], DATA[k + "_pal"],
                   case["offset"])
    assert np.array_equal(got, DATA[k + "_rgb"])


@pytest.mark.skipif(not REF_IO.exists(), reason="reference colouring library not built here")
def test_oracle_colour_matches_reference_random():
    lib = C.CDLL(str(REF_IO))
    rng = np.random.default_rng(7)
    for _ in range(200):
        aa = int(rng.integers(1, 4))
        H, W = aa * int(rng.integers(1, 9)), aa * int(rng.integers(1, 9))
        raw = rng.integers(0, 100000, (H, W)).astype(np.int32)
        raw[rng.random((H, W)) < 0.2] = 0
        n = int(rng.integers(2, 257))
        pal = rng.integers(0, 2 ** 24, n).astype(np.uint32)
        sc = float(rng.choice([1.0, 0.056874995, 0.37, 2.5, float(rng.random() * 10)]))
        ip, off = int(rng.integers(0, 2)), int(rng.integers(0, 256))
        want = np.zeros((H // aa, W // aa), np.uint32)
        assert lib.mdzref_io_colour(raw.ctypes.data_as(C.c_void_p), W, H, aa, ip,
                                    C.c_double(sc), pal.ctypes.data_as(C.c_void_p), n, off,
                                    want.ctypes.data_as(C.c_void_p))
        assert np.array_equal(O.colour(raw, aa, ip, sc, pal, off), want)


def test_colour_interpolation_quirks():
    """Reference behaviours kept on purpose: interior pixels (count 0) are
    black without supersampling but take palette[0] through the
    interpolating AA path; the interpolation weights the floor colour by
    ceil(v) - v."""
    pal = np.array([0x0000ff, 0x00ff00, 0xff0000, 0x101010], np.uint32)
    raw = np.zeros((2, 2), np.int32)
    assert O.colour(raw, 1, True, 1.0, pal)[0, 0] == 0
    assert O.colour(raw, 2, True, 1.0, pal)[0, 0] == 0x0000ff
    raw1 = np.array([[1]], np.int32)
    # v = 1.5: floor index 1, ceil index 2, weights 0.5 / 0.5
    got = O.colour(raw1, 1, True, 1.5, pal)[0, 0]
    assert got == (0x7f << 8) | (0x7f << 16)


def _ref_load(path, W=0, H=0, aa=0):
    lib = C.CDLL(str(REF_IO))
    buf = C.create_string_buffer(1 << 16)
    pal = (C.c_uint32 * 256)()
    n, off = C.c_int(), C.c_int()
    if lib.mdzref_io_load(str(path).encode(), W, H, aa, buf, len(buf), pal, C.byref(n),
                          C.byref(off)) <= 0:
        return None
    d = dict(line.split(" ", 1) for line in buf.value.decode().splitlines())
    return d, list(pal)[:n.value], off.value


@pytest.mark.skipif(not (REF_IO.exists() and GALLERY.exists()),
                    reason="reference loader or gallery not present here")
@pytest.mark.parametrize("sizes", [(0, 0, 0), (1920, 1080, 3), (640, 0, 1), (0, 300, 2)])
def test_mdzfile_matches_reference_loader(sizes):
    from mdz_gb300.mdzfile import MdzFileError, load
    from mdz_gb300.mpval import parse_number
    W, H, aa = sizes
    n = 0
    for f in sorted(GALLERY.glob("*.mdz")):
        ref = _ref_load(f, W, H, aa)
        if ref is None:
            with pytest.raises(MdzFileError):
                load(f)
            continue
        d, pal, off = ref
        s = load(f)
        v = s.view(W, H, aa)
        r = v.rect()
        for k, mine in (("xmin", r.xmin), ("xmax", r.xmax), ("ymax", r.ymax), ("width", r.width)):
            hexv, prec = d[k].rsplit(" ", 1)
            assert parse_number(hexv) == mine.to_fraction(), (f.name, k)
            assert int(prec) == mine.prec, (f.name, k)
        assert (int(d["depth"]), int(d["user_width"]), int(d["user_height"]), int(d["aa"]),
                int(d["precision"]), int(d["family"]), int(d["fractal"])) == \
            (v.depth, v.width, v.height, v.aa, v.precision, v.family, v.fractal)
        assert (int(d["multi_prec"]), int(d["rounding"]), int(d["palette_ip"])) == \
            (int(v.multi_prec), int(v.rounding), int(s.palette_ip))
        assert float(d["colour_scale"]) == s.colour_scale
        assert pal == s.palette and off == s.palette_offset
        n += 1
    assert n >= 8


def test_mdzfile_round_trip(tmp_path):
    from mdz_gb300.mdzfile import MdzSettings, dumps, load
    pal = [int(x) for x in np.random.default_rng(3).integers(0, 2 ** 24, 200)]
    cases = [
        MdzSettings("a", (0, 1, 2), 0, 1, 25000, 16 / 9, 0.25, True, True, True, 300, True,
                    cx=Fraction(-17626, 10000), cy=Fraction(-281, 10000),
                    size=Fraction(1, 2 ** 200), palette=pal, palette_offset=17),
        MdzSettings("b", (0, 1, 2), 1, 0, 1000, 4 / 3, 1.0, False, False, True, 80, True,
                    cx=Fraction(0), cy=Fraction(0), size=Fraction(3),
                    julia_re=Fraction(-8, 10), julia_im=Fraction(156, 1000), palette=pal[:2]),
        MdzSettings("c", (0, 1, 2), 0, 2, 5000, 1.0, 3.5, False, True, False, 128, False,
                    xmin=Fraction(-2), xmax=Fraction(1, 2), ymax=Fraction(5, 4), palette=pal),
    ]
    from mdz_gb300.mdzfile import MdzSettings as _S  # noqa: F401
    for s in cases:
        p = tmp_path / (s.name + ".mdz")
        p.write_text(dumps(s))
        t = load(p)
        from mdz_gb300.mpval import MpVal
        for field in ("family", "fractal", "depth", "aspect", "colour_scale", "palette_ip",
                      "multi_prec", "rounding", "precision", "centre_form", "palette",
                      "palette_offset"):
            assert getattr(t, field) == getattr(s, field), field
        for field in ("cx", "cy", "size", "xmin", "xmax", "ymax", "julia_re", "julia_im"):
            a = getattr(s, field)
            if a is None or (field.startswith("julia") and s.family == 0):
                continue
            assert getattr(t, field) == MpVal.from_fraction(a, s.precision).to_fraction(), field
        if REF_IO.exists():
            assert _ref_load(p) is not None


@pytest.mark.parametrize("bad,msg", [
    ("not an mdz file\n", "recognisable"),
    ("mdz fractal settings 0.1.2\nsettings\nfamily mandelbrot\nfractal mandelbrot\n"
     "depth 0\n", "depth"),
    ("mdz fractal settings 0.1.2\nsettings\nfamily nope\n", "family"),
])
def test_mdzfile_errors(bad, msg):
    from mdz_gb300.mdzfile import MdzFileError, loads
    with pytest.raises(MdzFileError, match=msg):
        loads(bad)
