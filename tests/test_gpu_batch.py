"""Batched frames on the GPU: every frame of a mixed batch (lenses, grids, wavelength counts,
light positions) equals the single-frame path's image bit for bit, for each tile size and
rays-per-thread setting, and a CUDA-graph replay reproduces the eager run."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from realflare_gb300 import synthetic  # noqa: E402


@pytest.fixture(scope='module')
def projects():
    return synthetic.batched_projects(6, seed=3, resolution=256, surfaces=(8, 16), grids=(16, 32))


@pytest.fixture(scope='module')
def ghosts(projects):
    from realflare_gb300.batch import ghost_textures

    return ghost_textures(projects)


@pytest.fixture(scope='module')
def single_frame_images(projects, ghosts):
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    tex, offsets, shapes = ghosts
    out = []
    for p, off, (h, w) in zip(projects, offsets, shapes):
        ghost = Image(tensor=tex[off: off + h * w].view(h, w))
        rays = RaytracingTask(cache=False).run(p)
        out.append(RasterizingTask().run(p, rays, ghost).array.copy())
    return out


@pytest.mark.parametrize('tile,rpt', [(32, 1), (16, 2), (32, 4)])
def test_batch_equals_single_frames(projects, ghosts, single_frame_images, tile, rpt):
    from realflare_gb300.batch import BatchRenderer

    r = BatchRenderer(projects, tile_size=tile, rays_per_thread=rpt, ghosts=ghosts, entry_capacity=1024)
    images = r.run()  # the capacity grows from 1024 entries: the overflow path runs first
    torch.cuda.synchronize()
    assert r.entry_count() <= r.capacity
    lit = 0
    for got, want in zip(images, single_frame_images):
        g = got.cpu().numpy()
        assert np.array_equal(g, want)
        lit += int((g[..., :3] > 0).any(-1).sum())
    assert lit > 0


def test_graph_replay_reproduces_the_eager_run(projects, ghosts, single_frame_images):
    from realflare_gb300.batch import BatchRenderer

    r = BatchRenderer(projects, tile_size=32, rays_per_thread=2, ghosts=ghosts)
    r.run()
    r.capture()
    r.image_buffer.fill_(-1.0)
    r.rays.zero_()
    torch.cuda.synchronize()
    r.replay()
    torch.cuda.synchronize()
    for got, want in zip(r.images, single_frame_images):
        assert np.array_equal(got.cpu().numpy(), want)
