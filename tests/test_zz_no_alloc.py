"""The allocation-free multi-limb entry point (mdzgpu_render_mp_noalloc).

Some callers cannot allocate device memory themselves or let the library do
it -- a plugin running under a host application whose allocator owns the
GPU, or a loop that cannot take cudaMalloc's device-wide synchronisation.
For them the library keeps the kernel's scratch in a fixed array per GPU.
This test renders a gallery view and config 3's view through it twice in a
row and checks each result equals the regular entry point's
(mdzgpu_render_mp_device) bit for bit; the output buffers are allocated by
the test, not by the library.  The file sorts last so that a failure here
cannot hide the other tests' results."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MdzGpuError, Renderer, View, native

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "mp_views.json").read_text())


def view_of(name):
    return View.from_dict({k: v for k, v in META[name].items() if k not in ("gmp", "step")})


@pytest.mark.parametrize("name", ["gal_honeytrace", "mp_julia", "c3_sub"])
def test_noalloc_matches_regular_entry_point_twice(name):
    torch = pytest.importorskip("torch")
    v = view_of(name)
    r = v.rect()
    W, H = v.real_width, v.real_height
    jre, jim = v.julia() if v.family else (r.xmin.zero(80), r.xmin.zero(80))
    lib = native.load()
    with Renderer(0) as rend:
        ref_buf = torch.empty((H, W), dtype=torch.int32, device="cuda")
        rend.render_mp_device(W, H, v.depth, r.xmin, r.ymax, r.width, v.precision,
                              ref_buf.data_ptr(), family=v.family, fractal=v.fractal,
                              julia=(jre, jim) if v.family else None)
        torch.cuda.synchronize()
        want = ref_buf.cpu().numpy()
    frame = native.Frame(W, H, v.family, v.fractal, v.depth)
    vals = [x.struct() for x in (r.xmin, r.ymax, r.width, jre, jim)]
    for call in range(2):
        out = torch.full((H, W), -7, dtype=torch.int32, device="cuda")
        rc = lib.mdzgpu_render_mp_noalloc(C.byref(frame), *[C.byref(s) for s, _ in vals],
                                          v.precision, 0, C.c_void_p(out.data_ptr()), None)
        assert rc == 0, native.last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}: {(got != want).sum()} pixels differ"


def test_noalloc_rejects_frames_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    lib = native.load()
    out = torch.empty(16, dtype=torch.int32, device="cuda")
    v = view_of("mp_julia")
    r = v.rect()
    frame = native.Frame(6000, 3000, 0, 0, 100)
    vals = [x.struct() for x in (r.xmin, r.ymax, r.width, r.xmin, r.xmin)]
    rc = lib.mdzgpu_render_mp_noalloc(C.byref(frame), *[C.byref(s) for s, _ in vals], 128, 0,
                                      C.c_void_p(out.data_ptr()), None)
    assert rc == -1  # MDZGPU_ERR_ARG, before any device work
    assert "scratch limit" in native.last_error()


def test_noalloc_rejects_julia_constant_out_of_range_like_regular_entry_point():
    """A Julia constant outside the fixed-point coordinate range (|x| < 4) is
    refused by both entry points with MDZGPU_ERR_RANGE, before any device
    work; the output buffer keeps its contents."""
    torch = pytest.importorskip("torch")
    from mdz_gb300 import MpVal
    lib = native.load()
    v = view_of("mp_julia")
    r = v.rect()
    W, H = 16, 8
    big = MpVal.from_fraction(5, 128)
    jim = MpVal.from_fraction(0, 128)
    frame = native.Frame(W, H, 1, 0, 100)
    vals = [x.struct() for x in (r.xmin, r.ymax, r.width, big, jim)]
    out = torch.full((H, W), -7, dtype=torch.int32, device="cuda")
    rc = lib.mdzgpu_render_mp_noalloc(C.byref(frame), *[C.byref(s) for s, _ in vals], 128, 0,
                                      C.c_void_p(out.data_ptr()), None)
    assert rc == -4, native.last_error()  # MDZGPU_ERR_RANGE
    with Renderer(0) as rend:
        with pytest.raises(MdzGpuError, match="error -4"):
            rend.render_mp_device(W, H, 100, r.xmin, r.ymax, r.width, 128, out.data_ptr(),
                                  family=1, fractal=0, julia=(big, jim))
    torch.cuda.synchronize()
    assert int((out != -7).sum()) == 0
