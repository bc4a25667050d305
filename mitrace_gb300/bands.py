"""Row-band split of one image across ranks (one GPU per rank).

The reference parallelises a render over 32x32 tiles pulled from a queue by
worker threads (src/Tracer/Tracer.cpp:728-754 builds the queue, 618-631 run
the workers).  Pixels are independent and the firefly clamp needs all samples
of a pixel on one device, so across GPUs the unit is a band of whole rows:
every rank holds the full scene, renders its contiguous band with
mt_render_rows_device, and the bands are gathered into the image on rank 0.
A pixel's random numbers are keyed by its index, not by the band, so the
assembled image equals the single-GPU render bit for bit.  There is no other
exchange on the data path.

``render_rows(r0, r1, out)`` is the band renderer (the library's on a GPU);
``gather_bands`` works with any torch.distributed backend (NCCL on GPUs, gloo
on CPU).
"""
from __future__ import annotations

from typing import Callable, List, Tuple


def row_bands(height: int, world: int) -> List[Tuple[int, int]]:
    """Contiguous [r0, r1) bands covering rows 0..height-1 exactly once; the
    first height % world ranks take one row more.  A rank whose band would be
    empty (world > height) gets (height, height)."""
    if height < 0 or world < 1:
        raise ValueError("height >= 0 and world >= 1 required")
    base, extra = divmod(height, world)
    bands, r0 = [], 0
    for k in range(world):
        r1 = r0 + base + (1 if k < extra else 0)
        bands.append((r0, r1))
        r0 = r1
    return bands


def gather_bands(band_image, bands: List[Tuple[int, int]], rank: int, group=None, dst: int = 0):
    """band_image: this rank's (rows, W, 3) tensor (its own band's rows).
    Returns the assembled (H, W, 3) image on rank dst, None elsewhere.  Bands
    are padded to the largest band for the collective and cut back after."""
    import torch
    import torch.distributed as dist

    world = len(bands)
    rows_max = max(r1 - r0 for r0, r1 in bands)
    W = band_image.shape[1]
    pad = torch.zeros((rows_max, W, 3), dtype=band_image.dtype, device=band_image.device)
    r0, r1 = bands[rank]
    pad[: r1 - r0] = band_image[: r1 - r0]
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    if rank != dst:
        return None
    H = bands[-1][1]
    img = torch.empty((H, W, 3), dtype=band_image.dtype, device=band_image.device)
    for k, (a, b) in enumerate(bands):
        img[a:b] = parts[k][: b - a]
    return img


def render_and_gather(render_rows: Callable[[int, int, object], None], height: int, width: int, rank: int,
                      world: int, device=None, group=None, dst: int = 0):
    """Renders this rank's band with render_rows(r0, r1, out_full) into a full
    (H, W, 3) buffer (only the band's rows are written) and gathers the bands
    on rank dst."""
    import torch

    bands = row_bands(height, world)
    r0, r1 = bands[rank]
    full = torch.zeros((height, width, 3), dtype=torch.float32, device=device)
    if r1 > r0:
        render_rows(r0, r1, full)
    return gather_bands(full[r0:r1] if r1 > r0 else full[:0], bands, rank, group=group, dst=dst)
