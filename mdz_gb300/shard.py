"""Row sharding of one frame across ranks (one process per GPU).

Pixels are independent, so a frame splits into row bands with no exchange
on the data path; the only communication is gathering each band's counts to
the rank that owns raw_data.  Bands are whole multiples of the
anti-aliasing factor so that every user row (aa real rows,
src/render_threads.c:364-381) lives on one rank, and are interleaved
round-robin so that the expensive rows (near the set) spread over all ranks.
"""
from __future__ import annotations

import numpy as np


def row_bands(height: int, world: int, band: int = 16, aa: int = 1) -> list[list[tuple[int, int]]]:
    """Per rank, the (row0, nrows) bands it renders: bands of `band` user
    rows (band * aa real rows) dealt round-robin."""
    if world < 1 or height < 0 or band < 1 or aa < 1:
        raise ValueError("bad shard arguments")
    step = band * aa
    out: list[list[tuple[int, int]]] = [[] for _ in range(world)]
    for i, r0 in enumerate(range(0, height, step)):
        out[i % world].append((r0, min(step, height - r0)))
    return out


def assemble(height: int, width: int, parts: list[list[tuple[int, np.ndarray]]]) -> np.ndarray:
    """Stitch gathered (row0, rows) pieces back into a full frame."""
    frame = np.full((height, width), -1, np.int32)
    for rank_parts in parts:
        for row0, rows in rank_parts:
            frame[row0:row0 + rows.shape[0]] = rows
    if (frame == -1).any():
        raise ValueError("rows missing from the gathered shards")
    return frame
