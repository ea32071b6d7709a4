"""Splitting the frame hot path across GPUs, one process per GPU.

The reference renders on one GPU (CustomCUDARasterizer/main.cpp:397-399).
The path splits two ways without any exchange inside a frame's kernels:

* a batch of independent scenes is partitioned across ranks by estimated
  cost (`scene_partition`); each rank renders its scenes as its own batch and
  nothing is exchanged;
* one frame is split by bin rows (`row_bands`): every rank sets up and bins
  every triangle with its bin rectangles cut to its rows
  (gbr_set_bin_rows), rasterises and shades only those rows, and the bands
  -- disjoint sets of pixel rows -- are gathered once into the frame
  (`gather_composite`).  The composite equals the one-GPU frame because a
  triangle's pairs in a bin do not depend on the other bins.

Host logic only: the GPU side is the library's; these functions are what a
multi-GPU driver (bench.py under torchrun) calls around it.
"""
from __future__ import annotations

import numpy as np


def row_bands(num_rows: int, world: int, weights=None) -> list:
    """`world` contiguous bands [r0, r1) of bin rows covering [0, num_rows),
    cut where the cumulative weight (e.g. each bin row's pairs in the last
    frame; uniform when None) crosses k/world of the total.  Every band holds
    at least one row when num_rows >= world."""
    if world < 1 or num_rows < 1:
        raise ValueError("need at least one rank and one bin row")
    w = np.ones(num_rows, np.float64) if weights is None else np.asarray(weights, np.float64)
    if len(w) != num_rows or (w < 0).any():
        raise ValueError("one non-negative weight per bin row")
    if w.sum() <= 0:
        w = np.ones(num_rows, np.float64)
    cum = np.cumsum(w)
    cuts = [0]
    for k in range(1, world):
        c = int(np.searchsorted(cum, cum[-1] * k / world, side="left")) + 1
        lo = cuts[-1] + 1 if num_rows >= world else cuts[-1]
        hi = num_rows - (world - k) if num_rows >= world else num_rows
        cuts.append(min(max(c, lo), hi))
    cuts.append(num_rows)
    return [(cuts[k], cuts[k + 1]) for k in range(world)]


def band_pixel_rows(band, bin_h: int, height: int):
    """The pixel rows [y0, y1) of a band of bin rows."""
    r0, r1 = band
    return min(r0 * bin_h, height), min(r1 * bin_h, height)


def composite(parts, height: int, width: int, dtype=np.uint32):
    """The frame from disjoint bands: parts = [(y0, y1, rows[y1-y0, width])]."""
    out = np.zeros((height, width), dtype)
    covered = np.zeros(height, bool)
    for y0, y1, rows in parts:
        if covered[y0:y1].any():
            raise ValueError("bands overlap")
        out[y0:y1] = rows
        covered[y0:y1] = True
    if not covered.all():
        raise ValueError("bands leave pixel rows uncovered")
    return out


def gather_composite(dist, rows: np.ndarray, y0: int, y1: int, height: int, width: int):
    """Every rank's band gathered into the full frame on every rank (one
    all_gather over the process group; bands padded to the tallest)."""
    import torch
    world = dist.get_world_size()
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    hdr = torch.tensor([y0, y1], dtype=torch.int64, device=dev)
    hdrs = [torch.empty_like(hdr) for _ in range(world)]
    dist.all_gather(hdrs, hdr)
    tall = max(int(h[1] - h[0]) for h in hdrs)
    buf = np.zeros((tall, width), rows.dtype)
    buf[: y1 - y0] = rows
    t = torch.from_numpy(buf.view(np.int32) if rows.dtype.itemsize == 4 else buf).to(dev)
    outs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(outs, t)
    parts = []
    for h, o in zip(hdrs, outs):
        a, b = int(h[0]), int(h[1])
        arr = o.cpu().numpy()
        if rows.dtype.itemsize == 4:
            arr = arr.view(rows.dtype)
        parts.append((a, b, arr[: b - a]))
    return composite(parts, height, width, rows.dtype)


def scene_cost(num_triangles: int, width: int, height: int) -> float:
    """Estimated cost of a batch scene: its triangles plus its pixels (the
    setup and binning grow with the first, clearing and shading with the
    second; one pixel counted as a quarter triangle)."""
    return float(num_triangles) + 0.25 * float(width) * float(height)


def scene_partition(costs, world: int) -> list:
    """Scenes dealt to `world` ranks, longest first to the least loaded
    (ties to the lower rank): a list of ascending scene indices per rank.
    The same on every rank for the same costs."""
    if world < 1:
        raise ValueError("need at least one rank")
    costs = [float(c) for c in costs]
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]
