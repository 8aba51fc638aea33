"""Multi-rank path on CPU: world_size-2 gloo ranks render interleaved row
bands of one frame (here with the CPU oracle standing in for each rank's
GPU), gather them to rank 0 and stitch them; the result must equal the
single-rank frame bit for bit."""
import json
import os
import socket
from pathlib import Path

import numpy as np
import pytest

from mdz_gb300.shard import assemble, row_bands

GOLD = Path(__file__).resolve().parent / "golden"


def test_row_bands_cover_frame_once():
    for h, world, band, aa in [(180, 2, 16, 1), (3240, 8, 16, 3), (7, 3, 2, 1), (0, 2, 4, 1)]:
        bands = row_bands(h, world, band, aa)
        rows = sorted(r for rank in bands for r0, n in rank for r in range(r0, r0 + n))
        assert rows == list(range(h))
        for rank in bands:
            for r0, n in rank:
                assert r0 % (band * aa) == 0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mdz_gb300 import View, parse_number
    from oracle import oracle as O
    meta = json.loads((GOLD / "fp64_views.json").read_text())["c1"]
    xmin, xmax, ymax = (float(parse_number(s)) for s in meta["rect"])
    W, H, depth = meta["width"], meta["height"], meta["depth"]
    mine = []
    for r0, n in row_bands(H, world, band=16)[rank]:
        mine.append((r0, O.render_fp64_rows(W, H, r0, n, depth, xmin, xmax, ymax)))
    parts = [None] * world
    dist.all_gather_object(parts, mine)
    if rank == 0:
        q.put(assemble(H, W, parts))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_assemble_the_frame():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    frame = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert np.array_equal(frame, np.load(GOLD / "fp64_counts.npz")["c1"])
