"""One render of each GPU path on the seeded views, for profiling and timing.

    python -m mdz_gb300.cases c2 [--frame 480x270] [--repeat 1]
    python -m mdz_gb300.cases c3 | c4 | serve [--requests 4]
    python -m mdz_gb300.cases ship [--frame 480x270]
    python -m mdz_gb300.cases c4mp | wide | colour [--frame WxH] [--depth N]
    python -m mdz_gb300.cases serve --method multi_limb

c1/c2: FP64 kernel (MDZ's double path) on the views' rectangles (c2 without
supersampling unless --aa); c3: the multi-limb kernel at 256 bits; c4: the
perturbation frame (orbit + FP32 pixels + escalation passes); serve: the
first requests of the seeded serving stream through the serving engine;
ship: the burning-ship perturbation on the 2^-300 view of the folded-formula
fixtures (tests/golden/perturb_fold_views.json, f_ship_a300); c4mp: the
one-thread multi-limb kernel at 34 words on a crop of the 2^-1000 view (MDZ
geometry); wide: the warp-cooperative multi-limb kernel at 2176 bits (80
words) around c = i; colour: config 2's FP64 counts on a crop, coloured on
the GPU (3x3 supersampling, interpolated palette).
--frame keeps the view's pixel spacing and crops around its centre; --depth
overrides the view's maxiter (shorter reference orbits for profiling).
Prints one JSON line of the call's statistics per repeat.
"""
from __future__ import annotations

import argparse
import json
import sys
from fractions import Fraction
from pathlib import Path

from . import MpVal, Renderer, View, parse_number

VIEWS = json.loads((Path(__file__).resolve().parents[1] / "tests" / "golden" /
                    "views.json").read_text())


def view(name: str, frame: str | None, aa: bool) -> View:
    d = dict(VIEWS[name])
    if not aa:
        d["aa"] = 1
    if frame:
        w, h = (int(x) for x in frame.lower().split("x"))
        d["size"] = str(parse_number(d["size"]) * Fraction(w, d["width"]))
        d["width"], d["height"] = w, h
    return View.from_dict(d)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["c1", "c2", "c3", "c4", "serve", "ship", "c4mp", "wide",
                                     "colour"])
    ap.add_argument("--method", default="auto", help="serve: request method")
    ap.add_argument("--frame", default=None)
    ap.add_argument("--aa", action="store_true")
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--requests", type=int, default=4)
    ap.add_argument("--depth", type=int, default=0, help="maxiter override (0: the view's)")
    a = ap.parse_args(argv)
    if a.case == "serve":
        from .serve import Server
        from .stream import load_pool, make_stream
        pool = load_pool()
        items = make_stream(a.requests, pool)
        with Server(0, arena_bytes=16 << 30) as srv:
            for _ in range(a.repeat):
                reqs = [it.request(pool) for it in items]
                for rq in reqs:
                    rq.method = a.method
                ids = [srv.submit(rq) for rq in reqs]
                sts = [srv.wait(i) for i in ids]
                print(json.dumps({"requests": len(sts), "states": [s["state"] for s in sts],
                                  "stats": srv.stats()}), flush=True)
        return
    if a.case == "ship":
        m = json.loads((Path(__file__).resolve().parents[1] / "tests" / "golden" /
                        "perturb_fold_views.json").read_text())["f_ship_a300"]
        W, H = (int(x) for x in (a.frame or "480x270").lower().split("x"))
        prec = m["prec"]
        vals = [MpVal.from_fraction(parse_number(m[k]), prec) for k in ("cx", "cy")]
        w = MpVal.from_fraction(parse_number(m["width"]) * Fraction(W, m["W"]), prec)
        with Renderer(0) as r:
            for _ in range(a.repeat):
                _, _, st = r.render_perturb(W, H, m["depth"], vals[0], vals[1], w, prec,
                                            fractal=m["fractal"])
                print(json.dumps(st), flush=True)
        return
    if a.case == "wide":
        W, H = (int(x) for x in (a.frame or "96x64").lower().split("x"))
        v = View("wide", W, H, a.depth or 4000, "0", "1", "0x1p-2100", precision=2176,
                 multi_prec=True, rounding=True)
        rc = v.rect()
        with Renderer(0) as r:
            for _ in range(a.repeat):
                _, st = r.render_mp(W, H, v.depth, rc.xmin, rc.ymax, rc.width, v.precision)
                print(json.dumps(st), flush=True)
        return
    if a.case == "colour":
        import numpy as np
        v = view("c2", a.frame or "640x360", True)
        xmin, xmax, ymax = v.rect().doubles()
        pal = [(i * 2654435761) & 0xffffff for i in range(256)]
        with Renderer(0) as r:
            counts, st = r.render_fp64(v.real_width, v.real_height, v.depth, xmin, xmax, ymax)
            for _ in range(a.repeat):
                rgb = r.colour(counts, v.aa, pal, colour_scale=1.0, interpolate=True)
                print(json.dumps({"rgb_sum": int(np.asarray(rgb, np.uint64).sum())}), flush=True)
        return
    v = view("c4" if a.case == "c4mp" else a.case, a.frame, a.aa)
    if a.depth:
        v.depth = a.depth
    if a.case == "c4mp":
        rc = v.rect()
        with Renderer(0) as r:
            for _ in range(a.repeat):
                _, st = r.render_mp(v.real_width, v.real_height, v.depth, rc.xmin, rc.ymax,
                                    rc.width, v.precision, words=34)
                print(json.dumps(st), flush=True)
        return
    with Renderer(0) as r:
        for _ in range(a.repeat):
            if a.case in ("c1", "c2"):
                xmin, xmax, ymax = v.rect().doubles()
                _, st = r.render_fp64(v.real_width, v.real_height, v.depth, xmin, xmax, ymax)
            elif a.case == "c3":
                rc = v.rect()
                _, st = r.render_mp(v.real_width, v.real_height, v.depth, rc.xmin, rc.ymax,
                                    rc.width, v.precision)
            else:
                prec = v.precision
                cx = MpVal.from_fraction(parse_number(v.cx), prec)
                cy = MpVal.from_fraction(parse_number(v.cy), prec)
                w = MpVal.from_fraction(parse_number(v.size), prec)
                _, _, st = r.render_perturb(v.real_width, v.real_height, v.depth, cx, cy, w,
                                            prec)
            print(json.dumps(st), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
