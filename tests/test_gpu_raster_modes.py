"""The rasteriser's anti-aliasing and wavelength sub-step modes on the GPU.

``anti_aliasing`` S places S n-rook samples per pixel (``rasterizing.cl:628-633``) and
``wavelength_sub_count`` WS blends each wavelength pair's vertices at WS positions with one
spectrum lookup each (``mix_vertex`` at ``wavelength_sub_pos``, ``rasterizing.cl:606-650``).
The oracle is pinned bit for bit to the reference kernels in these modes
(``tests/test_oracle_pin.py``); here the CUDA raster (single frame, both tile sizes, and
the batched persistent raster) is compared with it.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from helpers import ghost_texture, oracle_pipeline, reduced, rel_l2  # noqa: E402

from realflare_gb300._abi import check, lib  # noqa: E402
from realflare_gb300.constants import light_spectrum  # noqa: E402

STAGE_RTOL = 1e-5
IMAGE_RTOL = 1e-4

# (anti_aliasing, wavelength_sub_count)
MODES = [(1, 2), (1, 8), (2, 1), (4, 1), (4, 8), (8, 2)]
WORKLOADS = {
    'spectral-16': dict(grid=20, resolution=(192, 160), paths=24, wavelengths=4),
    'production-24': dict(grid=14, resolution=(160, 192), paths=20, wavelengths=3),
}


@pytest.fixture(scope='module')
def oracle():
    from oracle.oracle import Oracle

    return Oracle('f32')


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def workload(name, aa, ws):
    w = reduced(name, **WORKLOADS[name])
    w.project.render.anti_aliasing = aa
    w.project.render.wavelength_sub_count = ws
    return w


@pytest.mark.parametrize('tile', [32, 16])
@pytest.mark.parametrize('aa,ws', MODES)
@pytest.mark.parametrize('name', list(WORKLOADS))
def test_raster_mode_matches_oracle(oracle, name, aa, ws, tile):
    from realflare_gb300.tasks import RasterizingTask

    w = workload(name, aa, ws)
    ghost = ghost_texture()
    spec = light_spectrum()
    r = oracle_pipeline(oracle, w, ghost, spec)
    ra = r['raster_args']
    assert ra.sub_steps == aa and ra.wavelength_sub_count == ws
    ra.tile_size = tile
    vtx_d = dev(r['vtx'])
    task = RasterizingTask()
    offsets, entries = task.bin(ra, dev(r['bounds']), vtx_d)
    image = torch.empty((ra.height, ra.width, 4), device='cuda')
    ghost_d, spec_d, masks_d = dev(ghost), dev(spec), dev(r['masks'].view(np.int64))
    check(lib().rf_raster(vtx_d.data_ptr(), offsets.data_ptr(), entries.data_ptr(), ghost_d.data_ptr(),
                          spec_d.data_ptr(), ctypes.byref(ra), image.data_ptr(), stream()), 'rf_raster')
    masks_img = torch.empty_like(image)
    check(lib().rf_raster_masks(vtx_d.data_ptr(), masks_d.data_ptr(), r['masks'].shape[1], ghost_d.data_ptr(),
                                spec_d.data_ptr(), ctypes.byref(ra), masks_img.data_ptr(), stream()),
          'rf_raster_masks')
    torch.cuda.synchronize()
    ref = r['image']
    got = image.cpu().numpy()
    assert (ref[..., :3] != 0).any(-1).mean() > 0.05
    assert ((got[..., :3] != 0).any(-1) == (ref[..., :3] != 0).any(-1)).mean() > 0.9999
    assert rel_l2(got, ref) < STAGE_RTOL
    assert rel_l2(masks_img.cpu().numpy(), ref) < STAGE_RTOL


@pytest.mark.parametrize('aa,ws', [(4, 8), (2, 2)])
def test_render_path_in_mode_matches_oracle(oracle, aa, ws):
    """The task path (trace -> setup -> bin -> ordered raster) at anti-aliasing 4 and 8
    wavelength sub-steps, the reference benchmark's settings."""
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    w = workload('spectral-16', aa, ws)
    ghost = ghost_texture()
    r = oracle_pipeline(oracle, w, ghost, light_spectrum())
    rays = RaytracingTask(cache=False).run(w.project, paths=w.paths)
    got = RasterizingTask().run(w.project, rays, Image(tensor=dev(ghost))).array
    assert rel_l2(got, r['image']) < IMAGE_RTOL


def test_batched_raster_in_modes_equals_single_frames():
    """Batched frames with anti-aliasing and wavelength sub-steps (mixed per frame) equal
    the single-frame path bit for bit."""
    from realflare_gb300 import synthetic
    from realflare_gb300.batch import BatchRenderer, ghost_textures
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    projects = synthetic.batched_projects(6, seed=5, resolution=192, surfaces=(8, 16), grids=(16, 24))
    modes = [(1, 8), (4, 2), (2, 1), (4, 8), (8, 4), (1, 1)]
    for p, (aa, ws) in zip(projects, modes):
        p.render.anti_aliasing = aa
        p.render.wavelength_sub_count = ws
    tex, offs, shapes = ghost_textures(projects)
    images = BatchRenderer(projects, tile_size=32, rays_per_thread=2, ghosts=(tex, offs, shapes)).run()
    torch.cuda.synchronize()
    lit = 0
    for p, img, off, (h, w) in zip(projects, images, offs, shapes):
        ghost = Image(tensor=tex[off: off + h * w].view(h, w))
        want = RasterizingTask().run(p, RaytracingTask(cache=False).run(p), ghost).array
        got = img.cpu().numpy()
        assert np.array_equal(got, want)
        lit += int((got[..., :3] > 0).any(-1).sum())
    assert lit > 0
    assert any(p.render.wavelength_count > 1 and p.render.wavelength_sub_count > 1 for p in projects)
