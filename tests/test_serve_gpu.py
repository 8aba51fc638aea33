"""Serving engine on the GPU (mdzgpu_serve_*).

* A request served alone gives exactly the counts (and |z|^2) of the frame
  API (mdzgpu_render_perturb) -- the per-pixel state is saved and resumed
  between steps, so splitting a pixel's iterations over steps changes
  nothing.
* Each request's result is the same alone and in a mix of requests of
  different size, depth, precision, formula and method submitted while
  others run (bit-exact for both methods), and the mix shares steps.
* The multi-limb method in the serving geometry agrees with MPFR at twice
  the precision on >= 99.9% of pixels (burning ship, celtic, Mandelbrot).
* Admission by memory footprint, slots, cancel and timeout.
"""
import json
import time
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300 import MpVal, hexfloat, parse_number, perturb_pixel_c
from mdz_gb300.serve import RenderRequest, Server, ServeError, footprint

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "perturb_views.json").read_text())


def view_request(name, W=None, H=None, depth=None, **kw):
    m = META[name]
    prec = m["prec"]
    return RenderRequest(W or m["W"], H or m["H"], depth or m["depth"],
                         MpVal.from_fraction(parse_number(m["cx"]), prec),
                         MpVal.from_fraction(parse_number(m["cy"]), prec),
                         MpVal.from_fraction(parse_number(m["width"]), prec), prec, **kw)


def region_request(fractal, cx, cy, span, W, H, depth, prec, **kw):
    return RenderRequest(W, H, depth, MpVal.from_fraction(Fraction(cx), prec),
                         MpVal.from_fraction(Fraction(cy), prec),
                         MpVal.from_fraction(Fraction(span), prec), prec, fractal=fractal,
                         method="multi_limb", **kw)


def mix_requests():
    return [
        view_request("p_gal_polyp", want_mag=True),
        view_request("p_mis_b_1000", W=160, H=120),
        region_request(1, "-1.7626", "-0.0281", "0.01", 160, 120, 2000, 96, want_mag=True),
        region_request(2, "-0.8", "0.15", "0.2", 96, 64, 3000, 300),
        view_request("p_c4_600", W=240, H=180),
        region_request(0, "-0.75", "0.1", "0.05", 64, 48, 4000, 200),
        region_request(1, "-1.7626", "-0.0281", "0.01", 48, 36, 1500, 700),
        view_request("p_gal_honeytrace"),
    ]


@pytest.fixture(scope="module")
def server():
    s = Server(0, arena_bytes=2 << 30, queue_pixels=1 << 21, step_ms=1.0)
    yield s
    s.close()


def run_alone(server, req):
    rid = server.submit(req)
    st = server.wait(rid, 120_000)
    assert st["state"] == "done", (st, req)
    return st


@pytest.mark.parametrize("name", ["p_gal_polyp", "p_mis_i_1000", "p_gal_spiralblues"])
def test_serve_perturb_equals_frame_api(server, renderer, name):
    req = view_request(name, want_mag=True)
    st = run_alone(server, req)
    counts, mag, fst = renderer.render_perturb(req.width, req.height, req.depth, req.cx, req.cy,
                                               req.span, req.precision, want_mag=True)
    assert np.array_equal(req.counts, counts)
    assert np.array_equal(req.mag.view(np.uint32), mag.view(np.uint32))
    assert st["pixel_iters"] == fst["pixel_iters"]
    assert st["escalated_fp64"] == fst["escalated_fp64"]
    assert st["escalated_mp"] == fst["escalated_mp"]


def test_serve_alone_equals_mix(server):
    alone = []
    steps_alone = 0
    for req in mix_requests():
        st = run_alone(server, req)
        steps_alone += st["steps"]
        alone.append((req.counts.copy(), None if req.mag is None else req.mag.copy()))
    before = server.stats()["steps"]
    mix = mix_requests()
    ids = []
    for k, req in enumerate(mix):
        ids.append(server.submit(req))
        if k % 3 == 2:
            time.sleep(0.002)   # later arrivals join requests already running
    sts = [server.wait(i, 120_000) for i in ids]
    steps_mix = server.stats()["steps"] - before
    for k, (st, req) in enumerate(zip(sts, mix)):
        assert st["state"] == "done", (k, st)
        assert np.array_equal(req.counts, alone[k][0]), f"request {k} differs in the mix"
        if req.mag is not None:
            assert np.array_equal(req.mag.view(np.uint32), alone[k][1].view(np.uint32))
    print(f"steps: alone {steps_alone}, mix {steps_mix}")
    assert steps_mix < steps_alone   # the requests shared steps


def test_serve_mix_many_orbits_and_classes(server):
    """Many reference orbits running (their SMs are left to them) while
    multi-limb requests of every word count, one request per class, share
    the steps: every request finishes and equals its result alone."""
    def build():
        reqs = [view_request("p_mis_i_1000", W=64, H=48, depth=60000) for _ in range(10)]
        reqs += [view_request("p_c4_600", W=96, H=72, depth=40000) for _ in range(6)]
        for k, prec in enumerate([64, 120, 180, 250, 330, 450, 560, 700, 820, 1000, 1060]):
            fr = (1, 2, 0)[k % 3]
            reqs.append(region_request(fr, "-1.7626" if fr == 1 else "-0.8" if fr == 2 else
                                       "-0.75", "-0.0281" if fr == 1 else "0.15" if fr == 2
                                       else "0.1", "0.01", 64, 48, 2500, prec))
        return reqs
    alone = []
    for req in build():
        run_alone(server, req)
        alone.append(req.counts.copy())
    mix = build()
    ids = [server.submit(r) for r in mix]
    sts = [server.wait(i, 120_000) for i in ids]
    for k, (st, req) in enumerate(zip(sts, mix)):
        assert st["state"] == "done", (k, st)
        assert np.array_equal(req.counts, alone[k]), f"request {k} differs in the mix"
    words = {st["words"] for st, r in zip(sts, mix) if r.method == "multi_limb"}
    assert len(words) >= 9


@pytest.mark.parametrize("fractal,cx,cy,span,prec", [
    (1, "-1.7626", "-0.0281", "0.01", 128),
    (2, "-0.8", "0.15", "0.2", 256),
    (0, "-0.75", "0.1", "0.05", 96),
])
def test_serve_multi_limb_vs_mpfr_2x(server, fractal, cx, cy, span, prec):
    from oracle import oracle as O
    W, H, depth = 32, 24, 1500
    req = region_request(fractal, cx, cy, span, W, H, depth, prec)
    run_alone(server, req)
    cre, cim = [], []
    for line in range(H):
        for ix in range(W):
            a, b = perturb_pixel_c(req.cx, req.cy, req.span, W, H, ix, line)
            cre.append(hexfloat(a))
            cim.append(hexfloat(b))
    want, _ = O.points_mpfr(cre, cim, depth, 2 * prec, fractal=fractal, threads=8)
    diff = req.counts.ravel() != want
    print(f"formula {fractal}: {int(diff.sum())}/{diff.size} differ from MPFR at {2 * prec} bits")
    assert diff.mean() <= 0.001 or diff.sum() <= 2
    assert len(np.unique(want)) > 10


@pytest.mark.parametrize("fractal,jre,jim,cx,cy,span,prec", [
    (0, "-0.8", "0.156", "0", "0", "1.5", 128),
    (1, "-1.75", "-0.03", "0", "0", "2", 96),
    (2, "-0.9", "0.2", "0.1", "0.1", "1.5", 160),
])
def test_serve_julia_vs_mpfr_2x(server, fractal, jre, jim, cx, cy, span, prec):
    """Julia family (z0 = pixel, c = the constant) through the multi-limb
    slice kernel, picked by the automatic method."""
    from oracle import oracle as O
    W, H, depth = 32, 24, 1500
    jr = MpVal.from_fraction(Fraction(jre), prec)
    ji = MpVal.from_fraction(Fraction(jim), prec)
    req = region_request(fractal, cx, cy, span, W, H, depth, prec)
    req.method = "auto"
    req.family = 1
    req.julia = (jr, ji)
    st = run_alone(server, req)
    assert st["method"] == 2   # multi-limb
    zre, zim = [], []
    for line in range(H):
        for ix in range(W):
            a, b = perturb_pixel_c(req.cx, req.cy, req.span, W, H, ix, line)
            zre.append(hexfloat(a))
            zim.append(hexfloat(b))
    want = O.points_julia_mpfr(zre, zim, hexfloat(jr.to_fraction()), hexfloat(ji.to_fraction()),
                               depth, 2 * prec, fractal=fractal, threads=8)
    diff = req.counts.ravel() != want
    print(f"julia formula {fractal}: {int(diff.sum())}/{diff.size} differ from MPFR at "
          f"{2 * prec} bits")
    assert diff.mean() <= 0.001 or diff.sum() <= 2
    assert len(np.unique(want)) > 10


def test_serve_admission_by_footprint():
    reqs = [view_request("p_c4_600", W=160, H=120) for _ in range(5)]
    dev, host = footprint(reqs[0])
    arena = 2 * dev + dev // 2      # room for two at a time
    with Server(0, max_requests=4, arena_bytes=arena, queue_pixels=1 << 18) as s:
        big = view_request("p_c4_600", W=1920, H=1080)
        with pytest.raises(ServeError):
            s.submit(big)            # can never fit: refused at submission
        ids = [s.submit(r) for r in reqs]
        sts = [s.wait(i, 120_000) for i in ids]
        stats = s.stats()
    assert all(st["state"] == "done" for st in sts)
    assert dev <= stats["device_bytes_peak"] <= arena
    # admitted in arrival order as memory freed up: later requests queued longer
    assert sts[-1]["queue_ms"] > sts[0]["queue_ms"]
    for r in reqs[1:]:
        assert np.array_equal(r.counts, reqs[0].counts)


def test_serve_slots_limit():
    reqs = [region_request(1, "-1.7626", "-0.0281", "0.01", 64, 48, 1000, 96) for _ in range(6)]
    with Server(0, max_requests=2, arena_bytes=256 << 20, queue_pixels=1 << 16) as s:
        ids = [s.submit(r) for r in reqs]
        sts = [s.wait(i, 120_000) for i in ids]
    assert all(st["state"] == "done" for st in sts)
    for r in reqs[1:]:
        assert np.array_equal(r.counts, reqs[0].counts)


def heavy_request(**kw):
    # burning ship, 1088-bit multi-limb, 1920x1080 to depth 10^5: minutes of work
    return region_request(1, "-1.7626", "-0.0281", "1e-3", 1920, 1080, 100_000, 1024, **kw)


def test_serve_cancel_running(server):
    req = heavy_request()
    req.counts = np.full((1080, 1920), -7, np.int32)
    rid = server.submit(req)
    t0 = time.time()
    while server.poll(rid)["steps"] < 2 and time.time() - t0 < 30:
        time.sleep(0.01)
    assert server.poll(rid)["state"] == "running"
    server.cancel(rid)
    st = server.wait(rid, 30_000)
    assert st["state"] == "cancelled"
    assert (req.counts == -7).all()   # the caller's buffer is never written
    # the engine carries on
    small = view_request("p_gal_polyp")
    assert run_alone(server, small)["state"] == "done"


def test_serve_cancel_after_main_pass(server):
    """A cancel that arrives while a request's escalation passes run (its
    steps no longer advance): no further pass, the caller's buffer is never
    written, the engine carries on."""
    m = json.loads((Path(__file__).resolve().parent / "golden" /
                    "perturb_fold_views.json").read_text())["f_ship_a300"]
    prec, W, H = m["prec"], 1280, 720
    req = RenderRequest(W, H, m["depth"], MpVal.from_fraction(parse_number(m["cx"]), prec),
                        MpVal.from_fraction(parse_number(m["cy"]), prec),
                        MpVal.from_fraction(parse_number(m["width"]) * Fraction(W, m["W"]),
                                            prec), prec, fractal=1)
    req.counts = np.full((H, W), -7, np.int32)
    rid = server.submit(req)
    t0 = time.time()
    last, since = -1, time.time()
    while time.time() - t0 < 60:
        st = server.poll(rid)
        if st["state"] != "running" and st["state"] != "queued":
            break
        if st["steps"] != last:
            last, since = st["steps"], time.time()
        elif last > 0 and time.time() - since > 0.05:
            break   # steps stopped: the main pass is over
        time.sleep(0.002)
    server.cancel(rid)
    st = server.wait(rid, 60_000)
    assert st["state"] in ("cancelled", "done"), st
    if st["state"] == "cancelled":
        assert (req.counts == -7).all()
    small = view_request("p_gal_polyp")
    assert run_alone(server, small)["state"] == "done"


def test_serve_timeout(server):
    req = heavy_request(timeout_ms=300.0)
    rid = server.submit(req)
    st = server.wait(rid, 30_000)
    assert st["state"] == "timeout"
    assert server.stats()["timed_out"] >= 1


def test_serve_rejects_bad_requests(server):
    bad = view_request("p_gal_polyp", method="perturbation")
    bad.fractal = 3                     # no perturbation for the hybrid
    with pytest.raises(ServeError):
        server.submit(bad)
    deep = region_request(1, "-1.7626", "-0.0281", "0.01", 16, 16, 100, 4000)
    with pytest.raises(ServeError):
        server.submit(deep)             # beyond the multi-limb kernel's words


def test_serve_latency_stats(server):
    st = server.stats()
    assert st["completed"] > 0
    assert 0 < st["latency_p50_ms"] <= st["latency_p99_ms"] <= st["latency_max_ms"]
    assert st["launches"] > st["steps"] > 0
