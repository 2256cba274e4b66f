"""Host logic of the batched form: rf_batch_plan's layout of frames (called through the C
ABI; it is host code, no GPU needed) and the memory grouping of frames."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from realflare_gb300 import build, synthetic
from realflare_gb300._abi import RF_ERR_INVALID_ARG, RF_ERR_NOT_SUPPORTED, RF_OK, SIGNATURES, BatchSizes


@pytest.fixture(scope='module')
def L():
    import os

    if not os.path.exists(build.LIB):
        build.build()
    handle = ctypes.CDLL(build.LIB)
    handle.rf_batch_plan.argtypes = SIGNATURES['rf_batch_plan']
    handle.rf_batch_plan.restype = ctypes.c_int
    return handle


@pytest.fixture(scope='module')
def projects():
    return synthetic.batched_projects(7, seed=5, resolution=200, surfaces=(8, 16), grids=(16, 32))


def inputs(projects):
    from realflare_gb300.batch import _frame_inputs

    return _frame_inputs(projects, [0] * len(projects), [(64, 64)] * len(projects))


@pytest.mark.parametrize('tile,rpt', [(32, 1), (16, 2), (32, 4)])
def test_plan_lays_frames_out_back_to_back(L, projects, tile, rpt):
    inp = inputs(projects)
    z = BatchSizes()
    assert L.rf_batch_plan(inp.frames, len(projects), tile, rpt, ctypes.byref(z)) == RF_OK
    rays = prims = inten = verts = pairs = tb = qb = vb = pb = tiles = pix = 0
    for f in inp.frames:
        P, W, G = f.trace.path_count, f.trace.wavelength_count, f.trace.grid_count
        n, Q, maxW = P * W * G * G, (G - 1) ** 2, max(W - 1, 1)
        assert (f.ray_offset, f.prim_offset, f.inten_offset, f.vertex_offset, f.pair_offset) == (
            rays, prims, inten, verts, pairs)
        assert (f.trace_block, f.quad_block, f.vertex_block, f.pair_block) == (tb, qb, vb, pb)
        assert (f.tile_offset, f.image_offset, f.raster.tile_size) == (tiles, pix, tile)
        ntiles = -(-f.raster.width // tile) * -(-f.raster.height // tile)
        assert f.tile_count == ntiles
        rays += n
        prims += P * Q
        inten += P * Q * W
        verts += n + 1
        pairs += P * Q * maxW
        tb += -(-n // (256 * rpt))
        qb += -(-(P * Q) // 256)
        vb += -(-(n + 1) // 256)
        pb += -(-(P * Q * maxW) // 256)
        tiles += ntiles
        pix += f.raster.width * f.raster.height
        # the light direction as rf_trace normalises it (FP32, no contraction)
        v = -np.array(f.trace.direction[:3], np.float32)
        dd = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
        inv = np.float32(1.0) / np.sqrt(dd)
        assert list(f.direction_n) == [float(v[k] * inv) for k in range(3)]
    assert (z.rays, z.prims, z.intensities, z.vertices, z.pairs) == (rays, prims, inten, verts, pairs)
    assert (z.trace_blocks, z.quad_blocks, z.vertex_blocks, z.pair_blocks, z.tiles) == (tb, qb, vb, pb, tiles)
    assert z.image_pixels == pix and z.frame_count == len(projects)
    assert z.max_sub == 1 and z.max_colors == max(max(f.trace.wavelength_count - 1, 1) for f in inp.frames)
    # texture lookups only when every frame has a ghost texture object
    assert z.ghost_textures == 0
    for k, f in enumerate(inp.frames):
        f.ghost_texture = 1 + k
    assert L.rf_batch_plan(inp.frames, len(projects), tile, rpt, ctypes.byref(z)) == RF_OK
    assert z.ghost_textures == 1
    inp.frames[3].ghost_texture = 0
    assert L.rf_batch_plan(inp.frames, len(projects), tile, rpt, ctypes.byref(z)) == RF_OK
    assert z.ghost_textures == 0


def test_plan_rejects_bad_settings(L, projects):
    z = BatchSizes()
    inp = inputs(projects)
    assert L.rf_batch_plan(inp.frames, len(projects), 8, 1, ctypes.byref(z)) == RF_ERR_NOT_SUPPORTED
    assert L.rf_batch_plan(inp.frames, len(projects), 32, 3, ctypes.byref(z)) == RF_ERR_NOT_SUPPORTED
    inp.frames[2].trace.grid_count = 1
    assert L.rf_batch_plan(inp.frames, len(projects), 32, 1, ctypes.byref(z)) == RF_ERR_INVALID_ARG
    inp = inputs(projects)
    inp.frames[1].raster.sub_steps = 3
    assert L.rf_batch_plan(inp.frames, len(projects), 32, 1, ctypes.byref(z)) == RF_ERR_INVALID_ARG
    assert L.rf_batch_plan(inp.frames, 0, 32, 1, ctypes.byref(z)) == RF_ERR_INVALID_ARG


def test_group_frames_respects_the_memory_budget(projects):
    from realflare_gb300.batch import frame_bytes, group_frames

    sizes = [2 * frame_bytes(p) for p in projects]
    budget = max(sizes) * 2
    groups = group_frames(projects, budget)
    assert [i for g in groups for i in g] == list(range(len(projects)))
    for g in groups:
        assert len(g) == 1 or sum(sizes[i] for i in g) <= budget


def test_batched_requests_follow_the_recipe():
    ps = synthetic.batched_projects(64, seed=0)
    assert {len(p.flare.lens.ghost_paths) for p in ps} == {28, 120, 276}
    assert {p.render.grid_count for p in ps} == {32, 64, 128}
    ws = [p.render.wavelength_count for p in ps]
    assert min(ws) >= 1 and max(ws) <= 16
    assert all(p.render.resolution.width() == 1024 for p in ps)
    xs = np.array([(p.flare.light.position.x(), p.flare.light.position.y()) for p in ps])
    assert np.all(np.abs(xs) <= 1)
