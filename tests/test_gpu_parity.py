"""Parity of every CUDA stage with the C oracle (FP32), on identical inputs.

Integer stages (bin masks, tile lists) must be bit-exact; the quad and vertex setup,
compiled without FMA contraction, must equal the oracle bit for bit; the trace's ray
positions (FMA-free, no transcendental functions) must equal the oracle's; reflectances
and images may differ by FP32 rounding in CUDA's transcendental functions and FMA
contraction of the shading arithmetic: tolerances are stated per test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from helpers import ghost_texture, oracle_pipeline, reduced, rel_l2  # noqa: E402

from realflare_gb300 import prepare  # noqa: E402
from realflare_gb300._abi import check, lib  # noqa: E402
from realflare_gb300.constants import light_spectrum  # noqa: E402

# The image tolerance of the render path (relative L2 over the whole image).
IMAGE_RTOL = 1e-4
# Identical inputs: only FMA contraction and transcendental rounding differ.
STAGE_RTOL = 1e-5

WORKLOADS = {
    'plain-8': dict(),
    'spectral-16-small': dict(name='spectral-16', grid=24, resolution=256, paths=40, wavelengths=5),
    'production-24-small': dict(name='production-24', grid=16, resolution=256, paths=30, wavelengths=4),
    # an image whose sides are not multiples of the 8-pixel blocks or the tiles
    'spectral-16-ragged': dict(name='spectral-16', grid=20, resolution=(203, 117), paths=24, wavelengths=3),
}


def workload(key):
    spec = dict(WORKLOADS[key])
    name = spec.pop('name', key)
    return reduced(name, **spec)


@pytest.fixture(scope='module')
def oracle():
    from oracle.oracle import Oracle

    return Oracle('f32')


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


def gpu_trace(ti):
    L = lib()
    rays = torch.empty((6, ti.ray_count), device='cuda')
    # keep every device input referenced until the kernel has run: a freed temporary's
    # block is handed to the next allocation by torch's caching allocator
    el, pa, wl = dev(ti.elements.view(np.uint8)), dev(ti.paths), dev(ti.wavelengths)
    check(L.rf_trace(el.data_ptr(), pa.data_ptr(), wl.data_ptr(), ctypes.byref(ti.args), rays.data_ptr(), stream()),
          'rf_trace')
    torch.cuda.synchronize()
    return rays.cpu().numpy()


@pytest.mark.parametrize('key', list(WORKLOADS))
def test_trace_positions_exact(oracle, key):
    w = workload(key)
    ti = prepare.trace_inputs(w.project, w.paths)
    ref = oracle.trace(ti.elements, ti.paths, ti.wavelengths, ti.args)
    got = gpu_trace(ti)
    valid_ref, valid_got = ~np.isnan(ref[5]), ~np.isnan(got[5])
    assert (valid_ref == valid_got).mean() == 1.0
    for k in range(5):  # positions, aperture positions, rrel: no transcendentals involved
        same = (ref[k] == got[k]) | (np.isnan(ref[k]) & np.isnan(got[k]))
        assert same.all(), f'plane {k}: {(~same).sum()} rays differ'
    # reflectance goes through sin/cos/tan/asin/acos: CUDA's and libm's differ by ulps
    r, g = ref[5][valid_ref], got[5][valid_ref]
    assert np.allclose(g, r, rtol=2e-5, atol=1e-12)


@pytest.mark.parametrize('key', list(WORKLOADS))
def test_quad_and_vertex_setup_exact(oracle, key):
    w = workload(key)
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays = oracle.trace(ti.elements, ti.paths, ti.wavelengths, a)
    area, min_area = prepare.quad_constants(w.project)
    b_ref, i_ref = oracle.quad_setup(rays, P, W, G, area, min_area)
    L = lib()
    rays_d = dev(rays)
    Q = (G - 1) ** 2
    bounds = torch.empty((P * Q, 4), device='cuda')
    inten = torch.empty((P * Q * W,), device='cuda')
    check(L.rf_quad_setup(rays_d.data_ptr(), P, W, G, area, min_area, bounds.data_ptr(), inten.data_ptr(), stream()),
          'rf_quad_setup')
    ra = prepare.raster_args(w.project, P, W, (64, 64))
    v_ref = oracle.vertex(rays, i_ref, P, W, G, ra.screen_transform, ra.width, ra.height)
    vtx = torch.empty(v_ref.shape, device='cuda')
    i_ref_d = dev(i_ref)
    check(L.rf_vertex(rays_d.data_ptr(), i_ref_d.data_ptr(), P, W, G, ra.screen_transform, ra.width, ra.height,
                      vtx.data_ptr(), stream()), 'rf_vertex')
    torch.cuda.synchronize()
    np.testing.assert_array_equal(bounds.cpu().numpy(), b_ref)
    np.testing.assert_array_equal(inten.cpu().numpy(), i_ref)
    np.testing.assert_array_equal(vtx.cpu().numpy(), v_ref)


@pytest.mark.parametrize('key', list(WORKLOADS))
def test_bin_masks_bit_exact(oracle, key):
    w = workload(key)
    ghost = ghost_texture()
    r = oracle_pipeline(oracle, w, ghost, light_spectrum())
    ra = r['raster_args']
    masks = torch.zeros(r['masks'].shape, dtype=torch.int64, device='cuda')
    bounds_d = dev(r['bounds'])
    check(lib().rf_bin_masks(bounds_d.data_ptr(), r['bounds'].shape[0], ra.screen_transform, ra.width,
                             ra.height, ra.bin_size, masks.data_ptr(), stream()), 'rf_bin_masks')
    torch.cuda.synchronize()
    np.testing.assert_array_equal(masks.cpu().numpy().view(np.uint64), r['masks'])


def gpu_tiles(ra, bounds_d, vtx_d):
    from realflare_gb300.tasks import RasterizingTask

    task = RasterizingTask()
    offsets, entries = task.bin(ra, bounds_d, vtx_d)
    torch.cuda.synchronize()
    return offsets, entries, task


@pytest.mark.parametrize('tile', [32, 16])
@pytest.mark.parametrize('key', list(WORKLOADS))
def test_tile_lists_ordered_and_within_reference_bins(oracle, key, tile):
    w = workload(key)
    ghost = ghost_texture()
    r = oracle_pipeline(oracle, w, ghost, light_spectrum())
    ra = r['raster_args']
    ra.tile_size = tile
    offsets, entries, task = gpu_tiles(ra, dev(r['bounds']), dev(r['vtx']))
    T = task.tile_size
    off = offsets.cpu().numpy().astype(np.int64)
    ent = entries.cpu().numpy().view(np.uint32)[: task.last_entry_count].astype(np.int64)
    ntx = (ra.width + T - 1) // T
    maxW = max(ra.wavelength_count - 1, 1)
    B = ra.bin_size
    bdx = (ra.width + B - 1) // B
    masks = r['masks']
    assert off[0] == 0 and off[-1] == task.last_entry_count
    for t in range(len(off) - 1):
        seg = ent[off[t]: off[t + 1]]
        assert np.all(np.diff(seg) > 0), 'entries of a tile must be strictly increasing'
        if len(seg) == 0:
            continue
        prims = seg // maxW
        tx, ty = t % ntx, t // ntx
        b = (ty * T // B) * bdx + (tx * T // B)
        bits = prims % 255 + 1
        words = masks[b, prims // 255, bits // 64]
        assert np.all((words >> (bits % 64).astype(np.uint64)) & np.uint64(1)), 'entry outside its reference bin'


@pytest.mark.parametrize('tile', [32, 16])
@pytest.mark.parametrize('key', list(WORKLOADS))
def test_raster_matches_oracle(oracle, key, tile):
    w = workload(key)
    ghost = ghost_texture()
    spec = light_spectrum()
    r = oracle_pipeline(oracle, w, ghost, spec)
    ra = r['raster_args']
    ra.tile_size = tile
    bounds_d, vtx_d = dev(r['bounds']), dev(r['vtx'])
    offsets, entries, task = gpu_tiles(ra, bounds_d, vtx_d)
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
    assert np.abs(ref).sum() > 0
    # the same pixels are lit, and values agree to FP32 shading rounding
    assert ((got[..., :3] != 0).any(-1) == (ref[..., :3] != 0).any(-1)).mean() > 0.9999
    assert rel_l2(got, ref) < STAGE_RTOL
    assert rel_l2(masks_img.cpu().numpy(), ref) < STAGE_RTOL
    assert np.all(got[..., 3] == 0)


def order_key(count: np.ndarray) -> np.ndarray:
    """rf_tile_order's key: 255 - (leading-one position * 8 + the next three bits), 255 for 0."""
    c = count.astype(np.int64)
    e = np.where(c > 0, np.floor(np.log2(np.maximum(c, 1))).astype(np.int64), 0)
    m = np.where(c > 0, (c << 3 >> e) & 7, 0)
    return np.where(c > 0, 255 - (e * 8 + m), 255)


@pytest.mark.parametrize('tile', [32, 16])
@pytest.mark.parametrize('key', ['spectral-16-small', 'production-24-small'])
def test_tile_order_and_ordered_raster(oracle, key, tile):
    """rf_tile_order is the stable sort of the tiles by decreasing entry count (3 significant
    bits), and rf_raster_ordered's image equals rf_raster's bit for bit."""
    w = workload(key)
    ghost = ghost_texture()
    spec = light_spectrum()
    r = oracle_pipeline(oracle, w, ghost, spec)
    ra = r['raster_args']
    ra.tile_size = tile
    vtx_d = dev(r['vtx'])
    offsets, entries, task = gpu_tiles(ra, dev(r['bounds']), vtx_d)
    order = task.order(offsets)
    torch.cuda.synchronize()
    off = offsets.cpu().numpy().astype(np.int64)
    tiles = off.size - 1
    got = order.cpu().numpy()[:tiles].astype(np.int64)
    want = np.argsort(order_key(np.diff(off)), kind='stable')
    np.testing.assert_array_equal(got, want)
    assert len(np.unique(np.diff(off))) > 3  # tiles of different weights
    ghost_d, spec_d = dev(ghost), dev(spec)
    images = []
    for ordered in (False, True):
        image = torch.empty((ra.height, ra.width, 4), device='cuda')
        if ordered:
            st = lib().rf_raster_ordered(vtx_d.data_ptr(), offsets.data_ptr(), entries.data_ptr(), order.data_ptr(),
                                         ghost_d.data_ptr(), spec_d.data_ptr(), ctypes.byref(ra), image.data_ptr(),
                                         stream())
        else:
            st = lib().rf_raster(vtx_d.data_ptr(), offsets.data_ptr(), entries.data_ptr(), ghost_d.data_ptr(),
                                 spec_d.data_ptr(), ctypes.byref(ra), image.data_ptr(), stream())
        check(st, 'raster')
        images.append(image)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(images[0].cpu().numpy(), images[1].cpu().numpy())


@pytest.mark.parametrize('key', ['plain-8', 'production-24-small'])
def test_raster_skipped_records_add_nothing(oracle, key):
    """The raster leaves out records whose fragments are all zero (a NaN reflectance; or,
    at one sample per pixel, a convex counter-clockwise quad with every rrel >= 1). With
    rrel raised by 0.5 (many quads outside the housing) and NaN planted in 3 % of the
    reflectances, its image still equals the oracle's, which shades every record."""
    w = workload(key)
    ghost = ghost_texture()
    spec = light_spectrum()
    r = oracle_pipeline(oracle, w, ghost, spec)
    ra = r['raster_args']
    assert ra.sub_steps == 1
    vtx = r['vtx'].copy().reshape(-1, 8)
    n = vtx.shape[0] - 1  # the last slot stays zero
    vtx[:n, 4] += 0.5
    rng = np.random.default_rng(1)
    vtx[:n, 5][rng.random(n) < 0.03] = np.nan
    vtx = vtx.reshape(r['vtx'].shape)
    image_ref = oracle.raster(vtx, r['masks'], ghost, spec, ra)
    vtx_d = dev(vtx)
    offsets, entries, task = gpu_tiles(ra, dev(r['bounds']), vtx_d)
    image = torch.empty((ra.height, ra.width, 4), device='cuda')
    ghost_d, spec_d = dev(ghost), dev(spec)
    check(lib().rf_raster(vtx_d.data_ptr(), offsets.data_ptr(), entries.data_ptr(), ghost_d.data_ptr(),
                          spec_d.data_ptr(), ctypes.byref(ra), image.data_ptr(), stream()), 'rf_raster')
    torch.cuda.synchronize()
    got = image.cpu().numpy()
    assert np.abs(image_ref).sum() > 0
    # quads outside the housing still light pixels through their negative weights
    assert ((got[..., :3] != 0).any(-1) == (image_ref[..., :3] != 0).any(-1)).mean() > 0.9999
    assert rel_l2(got, image_ref) < STAGE_RTOL


@pytest.mark.parametrize('key', list(WORKLOADS))
def test_render_path_matches_oracle(oracle, key):
    """The whole GPU path (trace -> setup -> bin -> raster) against the oracle's."""
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    w = workload(key)
    ghost = ghost_texture()
    r = oracle_pipeline(oracle, w, ghost, light_spectrum())
    rays = RaytracingTask().run(w.project, paths=w.paths)
    image = RasterizingTask().run(w.project, rays, Image(tensor=dev(ghost)))
    got = image.array
    assert rel_l2(got, r['image']) < IMAGE_RTOL


@pytest.mark.parametrize('name', ['plain8_g12_96', 'spectral16_g10_64'])
def test_cuda_path_reproduces_golden_vectors(name):
    """The CUDA stages on the inputs of the reference-generated golden fixtures."""
    import os

    from golden.make_golden import case_project

    with np.load(os.path.join(os.path.dirname(__file__), 'golden', f'{name}.npz')) as z:
        g = {k: z[k] for k in z.files}
    w = case_project(name)
    ti = prepare.trace_inputs(w.project, w.paths)
    got = gpu_trace(ti)
    for k in range(5):
        np.testing.assert_array_equal(np.nan_to_num(got[k], nan=9e9), np.nan_to_num(g['rays'][k], nan=9e9))
    assert (np.isnan(got[5]) == np.isnan(g['rays'][5])).all()
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    ra = prepare.raster_args(w.project, P, W, g['ghost'].shape)
    bounds_d, vtx_d = dev(g['bounds']), dev(g['vertexes'])
    offsets, entries, task = gpu_tiles(ra, bounds_d, vtx_d)
    image = torch.empty((ra.height, ra.width, 4), device='cuda')
    ghost_d, spec_d = dev(g['ghost']), dev(light_spectrum())
    check(lib().rf_raster(vtx_d.data_ptr(), offsets.data_ptr(), entries.data_ptr(), ghost_d.data_ptr(),
                          spec_d.data_ptr(), ctypes.byref(ra), image.data_ptr(), stream()), 'rf_raster')
    torch.cuda.synchronize()
    assert rel_l2(image.cpu().numpy(), g['image']) < STAGE_RTOL
