"""Edge cases of the render path on the GPU, against the oracle: no ghost paths and a lens
without two elements (the reference's trace returns nothing and the rasteriser its cleared
image, ``raytracing.py:164-165``, ``rasterizing.py:318-319``), an image of a few pixels,
and an image wide enough that with 8 samples per pixel the sample coordinates pass 2^14,
where the raster cannot reject records by their bounds and tests every record of a tile at
every pixel."""
from __future__ import annotations

import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from helpers import ghost_texture, oracle_pipeline, reduced, rel_l2  # noqa: E402

from realflare_gb300 import prepare  # noqa: E402
from realflare_gb300.constants import light_spectrum  # noqa: E402

# whole path (trace -> setup -> bin -> raster) against the oracle's, relative L2
IMAGE_RTOL = 1e-4


@pytest.fixture(scope='module')
def oracle():
    from oracle.oracle import Oracle

    return Oracle('f32')


def gpu_image(w, ghost, paths):
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    rays = RaytracingTask(cache=False).run(w.project, paths=paths)
    image = RasterizingTask().run(w.project, rays, Image(tensor=torch.from_numpy(ghost).cuda()))
    return rays, image.array


def test_no_ghost_paths_give_an_empty_image():
    w = reduced('plain-8', grid=8, resolution=(48, 32))
    rays, image = gpu_image(w, ghost_texture(), paths=[])
    assert rays is not None and rays.shape[0] == 0
    assert image.shape == (32, 48, 4)
    assert not np.any(image)


def test_lens_without_two_elements_gives_an_empty_image():
    w = reduced('plain-8', grid=8, resolution=(48, 32))
    model = copy.deepcopy(w.project.flare.lens.lens_model)
    model.lens_elements = []
    w.project.flare.lens.lens_model = model
    assert prepare.trace_inputs(w.project) is None
    rays, image = gpu_image(w, ghost_texture(), paths=None)
    assert rays is None
    assert image.shape == (32, 48, 4)
    assert not np.any(image)


@pytest.mark.parametrize('samples', [1, 8])
def test_image_of_a_few_pixels(oracle, samples):
    w = reduced('plain-8', grid=10, resolution=(7, 5), paths=8)
    w.project.render.anti_aliasing = samples
    ghost = ghost_texture()
    r = oracle_pipeline(oracle, w, ghost, light_spectrum())
    _, got = gpu_image(w, ghost, w.paths)
    assert np.abs(r['image']).sum() > 0
    assert rel_l2(got, r['image']) < IMAGE_RTOL


def test_sample_coordinates_beyond_exact_bounds_rejection(oracle):
    w = reduced('plain-8', grid=12, resolution=(2100, 40), paths=8)
    w.project.render.anti_aliasing = 8
    ghost = ghost_texture()
    ra = prepare.raster_args(w.project, len(w.paths), 1, ghost.shape)
    assert ra.width * ra.sub_steps > 16384  # records are tested at every pixel of their tiles
    r = oracle_pipeline(oracle, w, ghost, light_spectrum())
    _, got = gpu_image(w, ghost, w.paths)
    assert np.abs(r['image']).sum() > 0
    assert ((got[..., :3] != 0).any(-1) == (r['image'][..., :3] != 0).any(-1)).mean() > 0.9999
    assert rel_l2(got, r['image']) < IMAGE_RTOL
