"""Row-band split across ranks (mitrace_gb300.bands), on CPU with the gloo
backend and world size 2: the bands cover the image exactly once, and the
image gathered from two ranks' bands equals the single-rank image bit for bit.
The band renderer here is the oracle's (rows [r0, r1) of RenderBlock's tile
queue with the counter RNG); on GPUs it is mt_render_rows_device."""
import os
import socket

import numpy as np
import pytest

from mitrace_gb300.bands import row_bands


@pytest.mark.parametrize("height,world", [(1080, 1), (1080, 2), (1080, 8), (7, 3), (3, 5), (0, 2), (257, 4)])
def test_bands_cover_every_row_once(height, world):
    b = row_bands(height, world)
    assert len(b) == world
    rows = [r for r0, r1 in b for r in range(r0, r1)]
    assert rows == list(range(height))
    sizes = [r1 - r0 for r0, r1 in b]
    assert max(sizes) - min(sizes) <= 1
    assert all(b[k][1] == b[k + 1][0] for k in range(world - 1))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch
    import torch.distributed as dist

    import mitrace_gb300 as mt
    from mitrace_gb300.bands import render_and_gather
    from oracle import oracle_py as orc

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        scene, cfg = mt.box_room(width=24, height=19, samples=3, seed=8)
        o = orc.OracleScene(mt.PackedScene(scene), cfg)

        def render_rows(r0, r1, out):
            img, _, _ = o.render(orc.RNG_COUNTER, 1, r0, r1)
            out[r0:r1] = torch.from_numpy(img[r0:r1])

        img = render_and_gather(render_rows, cfg.height, cfg.width, rank, world)
        if rank == 0:
            np.save(out_path, img.numpy())
    finally:
        dist.destroy_process_group()


def test_two_rank_gather_equals_single_rank(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp

    import mitrace_gb300 as mt
    from oracle import oracle_py as orc

    out = str(tmp_path / "img.npy")
    tmp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    scene, cfg = mt.box_room(width=24, height=19, samples=3, seed=8)
    ref, _, _ = orc.OracleScene(mt.PackedScene(scene), cfg).render(orc.RNG_COUNTER, 1)
    np.testing.assert_array_equal(got, ref)
    assert ref.max() > 0
