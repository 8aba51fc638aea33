"""Colouring epilogue on the GPU (mdzgpu_colour / mdzgpu_colour_device)
against the reference's own palette_apply / do_anti_aliasing (committed
outputs, tests/golden/colour.npz) and the oracle restatement, plus the whole
headless path from a settings file: .mdz -> view -> GPU counts -> GPU
colours, equal to the oracle's render and colouring of the same view."""
import json
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "colour.json").read_text())
DATA = np.load(GOLD / "colour.npz")


@pytest.mark.parametrize("case", META, ids=[m["key"] for m in META])
def test_gpu_colour_matches_reference(renderer, case):
    k = case["key"]
    got = renderer.colour(DATA[k + "_raw"], case["aa"], DATA[k + "_pal"], case["scale"],
                          bool(case["ip"]), case["offset"])
    assert np.array_equal(got, DATA[k + "_rgb"])


def test_gpu_colour_random_vs_oracle(renderer):
    rng = np.random.default_rng(11)
    for _ in range(40):
        aa = int(rng.integers(1, 5))
        H, W = aa * int(rng.integers(1, 70)), aa * int(rng.integers(1, 90))
        raw = rng.integers(0, 200000, (H, W)).astype(np.int32)
        raw[rng.random((H, W)) < 0.2] = 0
        n = int(rng.integers(2, 257))
        pal = rng.integers(0, 2 ** 24, n).astype(np.uint32)
        sc = float(rng.choice([1.0, 0.056874995, 0.37, 2.5, float(rng.random() * 10)]))
        ip, off = bool(rng.integers(0, 2)), int(rng.integers(0, 256))
        got = renderer.colour(raw, aa, pal, sc, ip, off)
        assert np.array_equal(got, O.colour(raw, aa, ip, sc, pal, off))


def test_gpu_colour_device_path(renderer):
    import torch
    rng = np.random.default_rng(5)
    raw = rng.integers(0, 3000, (540, 960)).astype(np.int32)
    pal = rng.integers(0, 2 ** 24, 256).astype(np.uint32)
    d_raw = torch.from_numpy(raw).cuda()
    d_rgb = torch.empty((180, 320), dtype=torch.int32, device="cuda")
    renderer.colour_device(d_raw.data_ptr(), 960, 540, 3, pal, d_rgb.data_ptr(), 0.5, True, 3)
    torch.cuda.synchronize()
    got = d_rgb.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, O.colour(raw, 3, True, 0.5, pal, 3))


def test_settings_file_to_rgb(renderer, tmp_path):
    """A settings file in MDZ's own layout, read as MDZ's headless render
    reads it, rendered on the FP64 path (bit-exact counts) and coloured on
    the GPU with 3x3 supersampling: the RGB image equals the oracle's."""
    from mdz_gb300.mdzfile import MdzSettings, dumps, load
    pal = [int(x) for x in np.random.default_rng(9).integers(0, 2 ** 24, 256)]
    s = MdzSettings("view", (0, 1, 2), 0, 0, 1500, 4 / 3, 0.37, True, False, True, 80, True,
                    cx=Fraction(-74375, 100000), cy=Fraction(1314, 10000),
                    size=Fraction(3, 100), palette=pal, palette_offset=5)
    p = tmp_path / "view.mdz"
    p.write_text(dumps(s))
    t = load(p)
    v = t.view(96, 72, 3)
    xmin, xmax, ymax = v.rect().doubles()
    counts, _ = renderer.render_fp64(v.real_width, v.real_height, v.depth, xmin, xmax, ymax)
    rgb = renderer.colour(counts, v.aa, t.palette, t.colour_scale, t.palette_ip,
                          t.palette_offset)
    want_counts, _ = O.render_fp64(v.real_width, v.real_height, v.depth, xmin, xmax, ymax)
    assert np.array_equal(counts, want_counts)
    want = O.colour(want_counts, v.aa, t.palette_ip, t.colour_scale, t.palette, t.palette_offset)
    assert np.array_equal(rgb, want)
    assert len(np.unique(rgb)) > 20
