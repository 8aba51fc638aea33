"""Speed of the oracle restatement against the unmodified reference -- TEST
INFRASTRUCTURE.

The GPU machine has no copy of the reference's sources, so the CPU baseline timed
there is the restatement (oracle/mdz_oracle.c).  This script measures, where
the reference is compiled (oracle/_ref, x86-64), how fast the restatement is
compared with the reference's own rth_* + fractal_*_calculate_line + frac_*
on the same frames and thread count, checks the two produce the same counts,
and writes oracle/port_vs_reference.json:

  * MPFR at 1088 bits on a 32x24 crop around the 2^-1000 view's centre with
    its pixel spacing (maxiter 200000): the deep-zoom CPU baseline;
  * FP64 (long double = double, no FMA) on a 480x270 crop of the
    1920x1080x3x3, width 1e-11 view (maxiter 20000): the FP64 CPU baseline.

Run: python -m oracle.port_vs_reference [--threads N]
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import time
from fractions import Fraction
from pathlib import Path

import numpy as np

from mdz_gb300 import View
from mdz_gb300.mpval import parse_number
from oracle import oracle as O

HERE = Path(__file__).resolve().parent
VIEWS = json.loads((HERE.parent / "tests" / "golden" / "views.json").read_text())


def crop(name: str, w: int, h: int, size: str, **kw) -> View:
    """w x h pixels around the view's centre at its pixel spacing (`size` =
    the crop's real-axis width, given as a string of that exact value)."""
    v = dict(VIEWS[name])
    want = parse_number(v["size"]) * Fraction(w, v["width"] * v.get("aa", 1))
    assert parse_number(size) == want, (size, want)
    return View(name=f"{name}_{w}x{h}", width=w, height=h, depth=v["depth"], cx=v["cx"],
                cy=v["cy"], size=size, precision=v["precision"], **kw)


def its_of(counts: np.ndarray, depth: int) -> int:
    return int(np.where(counts == 0, depth, counts).sum())


def compare(v: View, threads: int, mpfr: bool) -> dict:
    r = v.rect()
    W, H = v.real_width, v.real_height
    t0 = time.perf_counter()
    ref, _ = O.ref_render(v, threads=threads, variant="d")
    t_ref = time.perf_counter() - t0
    t0 = time.perf_counter()
    if mpfr:
        port, _ = O.render_mpfr(W, H, v.depth, v.precision, r.xmin, r.ymax, r.width,
                                threads=threads)
    else:
        xmin, xmax, ymax = r.doubles()
        port, _ = O.render_fp64(W, H, v.depth, xmin, xmax, ymax, threads=threads)
    t_port = time.perf_counter() - t0
    its = its_of(ref, v.depth)
    return {"frame": f"{W}x{H}", "depth": v.depth, "precision": v.precision if mpfr else 53,
            "pixel_iters": its, "identical_counts": bool(np.array_equal(ref, port)),
            "reference_s": t_ref, "port_s": t_port,
            "reference_pixel_iters_per_s": its / t_ref, "port_pixel_iters_per_s": its / t_port,
            "port_over_reference": t_ref / t_port}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    if not O.ref_available():
        raise SystemExit("port_vs_reference: the reference is not compiled here (oracle/_ref)")
    out = {"host": platform.machine(), "threads": args.threads,
           "mpfr_1088": compare(crop("c4", 30, 20, "0x1p-1006", multi_prec=True,
                                     rounding=True),
                                args.threads, True),
           "fp64": compare(crop("c2", 576, 324, "1e-12"), args.threads, False)}
    (HERE / "port_vs_reference.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
