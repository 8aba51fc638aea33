"""The seeded mixed request stream of the serving benchmark.

Each request: size uniform over {240x180, 640x480, 1280x720, 1920x1080};
log2(span) ~ U[-1000, -10] with precision ceil(-log2 span) + 64 bits;
formula Mandelbrot / burning ship / generalized celtic (power 2) with
probabilities 0.7 / 0.2 / 0.1; maxiter log-uniform in [1e3, 1e5]; centre
drawn from a pool of seeded ray-bisection boundary points of that formula
(tests/golden/serve_centres.json, 1100 bits, made by make_golden.py
centres).  Arrivals are a Poisson process: unit exponential gaps, scaled by
the rate chosen at run time.  Everything comes from one numpy PCG64
generator with the seed given.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass
from fractions import Fraction
from pathlib import Path

import numpy as np

from .mpval import MpVal, parse_number
from .serve import RenderRequest

POOL_PATH = Path(__file__).resolve().parents[1] / "tests" / "golden" / "serve_centres.json"
SIZES = [(240, 180), (640, 480), (1280, 720), (1920, 1080)]
FORMULAS = [0, 1, 2]
FORMULA_P = [0.7, 0.2, 0.1]
DEFAULT_SEED = 5005


@dataclass
class StreamItem:
    index: int
    width: int
    height: int
    fractal: int
    depth: int
    log2_span: float
    precision: int
    centre: int          # index into the pool
    gap: float           # unit-mean exponential inter-arrival gap

    def request(self, pool: list[dict], want_mag: bool = False) -> RenderRequest:
        c = pool[self.centre]
        prec = self.precision
        # span = 2^log2_span, its mantissa a double (a dyadic rational)
        e = math.floor(self.log2_span)
        span = Fraction(2.0 ** (self.log2_span - e)) * Fraction(2) ** e
        return RenderRequest(self.width, self.height, self.depth,
                             MpVal.from_fraction(parse_number(c["cx"]), prec),
                             MpVal.from_fraction(parse_number(c["cy"]), prec),
                             MpVal.from_fraction(span, prec), prec, fractal=self.fractal,
                             want_mag=want_mag)


def load_pool(path: Path = POOL_PATH) -> list[dict]:
    return json.loads(Path(path).read_text())["centres"]


def make_stream(n: int, pool: list[dict], seed: int = DEFAULT_SEED) -> list[StreamItem]:
    rng = np.random.Generator(np.random.PCG64(seed))
    by_formula = {f: [i for i, c in enumerate(pool) if c["fractal"] == f] for f in FORMULAS}
    items = []
    for i in range(n):
        W, H = SIZES[int(rng.integers(len(SIZES)))]
        log2_span = float(rng.uniform(-1000.0, -10.0))
        fractal = int(rng.choice(FORMULAS, p=FORMULA_P))
        depth = int(round(10.0 ** float(rng.uniform(3.0, 5.0))))
        choices = by_formula[fractal]
        centre = choices[int(rng.integers(len(choices)))]
        gap = float(rng.exponential(1.0))
        items.append(StreamItem(i, W, H, fractal, depth, log2_span,
                                math.ceil(-log2_span) + 64, centre, gap))
    return items
