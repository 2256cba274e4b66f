"""The oracle against golden vectors produced by the reference's own kernels
(tests/golden/make_golden.py): the fixtures are intact, and the C oracle reproduces every
array bit for bit from the same inputs."""
from __future__ import annotations

import hashlib
import json
import os

import numpy as np
import pytest

from golden.make_golden import CASES, case_project
from helpers import ghost_texture  # noqa: F401

from realflare_gb300 import prepare
from realflare_gb300.constants import light_spectrum

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    with np.load(os.path.join(HERE, f'{name}.npz')) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope='module')
def oracle():
    from oracle.oracle import Oracle

    return Oracle('f32')


@pytest.mark.parametrize('name', list(CASES))
def test_fixtures_intact(name):
    with open(os.path.join(HERE, 'manifest.json')) as f:
        manifest = json.load(f)[name]
    g = load(name)
    assert set(g) == set(manifest)
    for k, v in g.items():
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == manifest[k], k
    assert (g['image'][..., :3] != 0).any(), 'a golden image must have lit pixels'
    assert np.isfinite(g['rays'][5]).mean() > 0.3


def same(a, b):
    return np.array_equal(a, b) or np.array_equal(np.nan_to_num(a, nan=1e30), np.nan_to_num(b, nan=1e30))


@pytest.mark.parametrize('name', list(CASES))
def test_oracle_reproduces_golden(oracle, name):
    g = load(name)
    w = case_project(name)
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays = oracle.trace(ti.elements, ti.paths, ti.wavelengths, a)
    assert same(rays, g['rays'])
    area, min_area = prepare.quad_constants(w.project)
    bounds, inten = oracle.quad_setup(g['rays'], P, W, G, area, min_area)
    assert same(bounds, g['bounds']) and same(inten, g['intensities'])
    ra = prepare.raster_args(w.project, P, W, g['ghost'].shape)
    vtx = oracle.vertex(g['rays'], g['intensities'], P, W, G, ra.screen_transform, ra.width, ra.height)
    assert same(vtx, g['vertexes'])
    masks = oracle.bin_masks(g['bounds'], ra.screen_transform, ra.width, ra.height, ra.bin_size)
    assert np.array_equal(masks, g['masks'])
    image = oracle.raster(g['vertexes'], g['masks'], g['ghost'], light_spectrum(), ra)
    assert np.array_equal(image, g['image'])
