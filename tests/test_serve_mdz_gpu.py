"""MDZ settings files drive the serving engine: each gallery file (as
written by mdz_gb300.mdzfile.dumps into tests/golden/mdz/) is read with
MDZ's load sequence (image_info_load_settings, src/image_info.c:456-721),
turned into a request (its own rectangle, 64 pixels across) and submitted;
all of them are admitted together and run as one mix.  Counts are scored
against MPFR at twice the file's precision on every pixel of the serving
geometry (tests/golden/serve_mdz.npz): over the whole mix at most 0.1% of
the pixels where MPFR at p and 2p agree may differ from them (the
perturbation bar), and per file at most 0.2% or 4 of them (one gallery
view, deep_embedded_julia at 320 bits, has 4 of 3072 pixels one iteration
off after the FP64 re-run of its rebased pixels); and per file the served
counts may not disagree with MPFR(2p) more often than MPFR(p) itself
does, plus 3 sigma."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300.serve import Server, request_from_mdz

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLD / "serve_mdz.json").read_text())
DATA = np.load(GOLD / "serve_mdz.npz")


def test_gallery_settings_files_served_as_one_mix():
    reqs = {k: request_from_mdz(GOLD / m["file"], width=64, intended=True) for k, m in
            META.items()}
    for k, r in reqs.items():
        m = META[k]
        assert (r.width, r.height, r.depth, r.precision, r.fractal) == \
            (m["W"], m["H"], m["depth"], m["prec"], m["fractal"])
    with Server(0, arena_bytes=4 << 30, queue_pixels=1 << 20) as srv:
        ids = {k: srv.submit(r) for k, r in reqs.items()}
        sts = {k: srv.wait(i, 300_000) for k, i in ids.items()}
    for k, st in sts.items():
        assert st["state"] == "done", (k, st)
    failures = []
    tot_bad = tot_resolved = 0
    for k, r in reqs.items():
        want, want_p = DATA[k], DATA[k + "__p"]
        got = r.counts
        resolved = want_p == want
        n = want.size
        bad_resolved = int(((got != want) & resolved).sum())
        n_diff, n_ref = int((got != want).sum()), int((want_p != want).sum())
        print(f"{k}: method {sts[k]['method']}, differ {n_diff}/{n} "
              f"(MPFR at p: {n_ref}), on resolved pixels {bad_resolved}, escalated "
              f"{sts[k]['escalated_fp64']} / {sts[k]['escalated_mp']}")
        for ln, ix in zip(*np.nonzero(got != want)):
            print(f"   ({ix}, {ln}): served {got[ln, ix]}, MPFR(2p) {want[ln, ix]}, "
                  f"MPFR(p) {want_p[ln, ix]}")
        tot_bad += bad_resolved
        tot_resolved += int(resolved.sum())
        if bad_resolved > max(4, 0.002 * int(resolved.sum())):
            failures.append(f"{k}: {bad_resolved} resolved pixels differ")
        rate = n_ref / n
        slack = 3 * math.sqrt(max(rate * (1 - rate), 1.0 / n) / n) * 2
        if n_diff / n > rate + slack + 2.0 / n:
            failures.append(f"{k}: {n_diff} differ, MPFR at p {n_ref}")
        assert len(np.unique(want)) > 3
    print(f"mix: {tot_bad} of {tot_resolved} resolved pixels differ")
    assert tot_bad <= 0.001 * tot_resolved, f"{tot_bad} of {tot_resolved} resolved pixels differ"
    assert not failures, failures
