"""Parity at full size: the spectral 16-surface workload (1024 x 1024, 120 ghosts, 64 x 64
grid, 8 wavelengths) compared whole, the production 24-surface workload (2048 x 2048, 276
ghosts, 128 x 128 grid, 16 wavelengths) on a ghost subset and on sampled pixels of the
whole frame, and the reference's own benchmark project (Nikon AI 50-135 mm, 1920 x 1080,
anti-aliasing 4, 5 wavelengths with 8 sub-steps, 129 x 129 grid, 50 % culling) rendered
through ``Engine.render`` against the reference's own kernels on sampled pixels.

Bars as in ``test_gpu_parity.py``: trace positions, quad setup, vertices and bin masks bit
for bit; reflectances to transcendental rounding; images to relative L2 1e-4 for the
whole path (the GPU's own trace) and 1e-5 for the raster on identical inputs.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from helpers import at_pixels, ghost_texture, kept_paths, reduced, rel_l2, stratified_pixels  # noqa: E402

from realflare_gb300 import prepare  # noqa: E402
from realflare_gb300._abi import check, lib  # noqa: E402
from realflare_gb300.constants import light_spectrum  # noqa: E402

IMAGE_RTOL = 1e-4
STAGE_RTOL = 1e-5


@pytest.fixture(scope='module')
def oracle():
    from oracle.oracle import Oracle

    return Oracle('f32')


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def assert_trace_equal(got, ref):
    """Positions, aperture positions and rrel bit for bit. Reflectances go through CUDA's
    and libm's sin/cos/tan/asin/acos, which differ by an ulp or two; over millions of rays a
    few near grazing incidence (where the Fresnel terms are steep in the angle) amplify that
    beyond 2e-5, so: at most 1 in 10^4 rays beyond 2e-5 relative, every ray within 1e-3, and
    the sum of reflectances (what the image integrates) within 1e-6."""
    valid = ~np.isnan(ref[5])
    assert np.array_equal(valid, ~np.isnan(got[5]))
    for k in range(5):
        same = (ref[k] == got[k]) | (np.isnan(ref[k]) & np.isnan(got[k]))
        assert same.all(), f'plane {k}: {(~same).sum()} rays differ'
    g, r = got[5][valid].astype(np.float64), ref[5][valid].astype(np.float64)
    rel = np.abs(g - r) / np.maximum(np.abs(r), 1e-30)
    stats = (f'{rel.size} rays: max rel {rel.max():.3e}, beyond 2e-5: {(rel > 2e-5).sum()}, '
             f'beyond 1e-4: {(rel > 1e-4).sum()}, sum rel {abs(g.sum() - r.sum()) / abs(r.sum()):.3e}')
    assert (rel > 2e-5).mean() <= 1e-4, stats
    assert rel.max() <= 1e-3, stats
    assert abs(g.sum() - r.sum()) <= 1e-6 * abs(r.sum()), stats


def gpu_stages(project, rays_host, P, W, G):
    """rf_quad_setup, rf_vertex and rf_bin_masks on the oracle's rays."""
    L = lib()
    area, min_area = prepare.quad_constants(project)
    Q = (G - 1) ** 2
    rays_d = dev(rays_host)
    bounds = torch.empty((P * Q, 4), device='cuda')
    inten = torch.empty((P * Q * W,), device='cuda')
    check(L.rf_quad_setup(rays_d.data_ptr(), P, W, G, area, min_area, bounds.data_ptr(), inten.data_ptr(), stream()),
          'rf_quad_setup')
    ra = prepare.raster_args(project, P, W, (64, 64))
    vtx = torch.empty((P * W * G * G + 1, 8), device='cuda')
    check(L.rf_vertex(rays_d.data_ptr(), inten.data_ptr(), P, W, G, ra.screen_transform, ra.width, ra.height,
                      vtx.data_ptr(), stream()), 'rf_vertex')
    B = ra.bin_size
    bins = ((ra.width + B - 1) // B) * ((ra.height + B - 1) // B)
    masks = torch.zeros((bins, (P * Q + 254) // 255, 4), dtype=torch.int64, device='cuda')
    check(L.rf_bin_masks(bounds.data_ptr(), P * Q, ra.screen_transform, ra.width, ra.height, B, masks.data_ptr(),
                         stream()), 'rf_bin_masks')
    torch.cuda.synchronize()
    return bounds.cpu().numpy(), inten.cpu().numpy(), vtx.cpu().numpy(), masks.cpu().numpy().view(np.uint64)


def check_stages(oracle, w, paths):
    """Trace, quad setup, vertices and bin masks of ``paths`` bit-exact against the oracle."""
    from realflare_gb300.tasks import RaytracingTask

    ti = prepare.trace_inputs(w.project, paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    ref = oracle.trace(ti.elements, ti.paths, ti.wavelengths, a)
    got = RaytracingTask(cache=False).run(w.project, paths=paths).tensor.reshape(6, -1).cpu().numpy()
    assert_trace_equal(got, ref)
    area, min_area = prepare.quad_constants(w.project)
    b_ref, i_ref = oracle.quad_setup(ref, P, W, G, area, min_area)
    ra = prepare.raster_args(w.project, P, W, (64, 64))
    v_ref = oracle.vertex(ref, i_ref, P, W, G, ra.screen_transform, ra.width, ra.height)
    m_ref = oracle.bin_masks(b_ref, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    b, i, v, m = gpu_stages(w.project, ref, P, W, G)
    np.testing.assert_array_equal(b, b_ref)
    np.testing.assert_array_equal(i, i_ref)
    np.testing.assert_array_equal(v, v_ref)
    np.testing.assert_array_equal(m, m_ref)
    return ref, v_ref, m_ref


def test_spectral_16_full_size_whole_image(oracle):
    """1024 x 1024, 120 ghosts, 64 x 64 grid, 8 wavelengths: every stage bit-exact and the
    whole image within 1e-4 of the oracle's."""
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    w = reduced('spectral-16')
    assert (w.project.render.resolution.width(), len(w.paths), w.project.render.grid_count,
            len(w.project.render.wavelengths)) == (1024, 120, 64, 8)
    _, vtx, masks = check_stages(oracle, w, w.paths)
    ghost = ghost_texture((256, 256), seed=3)
    ti = prepare.trace_inputs(w.project, w.paths)
    ra = prepare.raster_args(w.project, ti.args.path_count, ti.args.wavelength_count, ghost.shape)
    ref = oracle.raster(vtx, masks, ghost, light_spectrum(), ra)
    rays = RaytracingTask(cache=False).run(w.project, paths=w.paths)
    got = RasterizingTask().run(w.project, rays, Image(tensor=dev(ghost))).array
    assert (ref[..., :3] != 0).any(-1).mean() > 0.05
    assert rel_l2(got, ref) < IMAGE_RTOL


def test_production_24_full_size_subset_and_sampled_pixels(oracle):
    """2048 x 2048, 276 ghosts, 128 x 128 grid, 16 wavelengths, two-layer coatings: every
    stage bit-exact on every 23rd ghost at full grid and wavelength count; the whole frame
    rendered on the GPU and its raster compared with the oracle's on the GPU's own
    vertices at 64 stratified spans of 16 pixels, and the full bin masks bit-exact."""
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    w = reduced('production-24')
    assert (w.project.render.resolution.width(), len(w.paths), w.project.render.grid_count,
            len(w.project.render.wavelengths)) == (2048, 276, 128, 16)
    check_stages(oracle, w, w.paths[::23])

    ghost = ghost_texture((512, 512), seed=5)
    rays = RaytracingTask(cache=False).run(w.project, paths=w.paths)
    task = RasterizingTask()
    got = task.run(w.project, rays, Image(tensor=dev(ghost))).array
    P, W, R = rays.shape
    bounds, _, vertexes = task.setup(w.project, rays)
    ra = prepare.raster_args(w.project, P, W, ghost.shape)
    B = ra.bin_size
    bins = ((ra.width + B - 1) // B) * ((ra.height + B - 1) // B)
    prims = P * (ra.grid_count - 1) ** 2
    masks_d = torch.zeros((bins, (prims + 254) // 255, 4), dtype=torch.int64, device='cuda')
    check(lib().rf_bin_masks(bounds.data_ptr(), prims, ra.screen_transform, ra.width, ra.height, B,
                             masks_d.data_ptr(), task.stream), 'rf_bin_masks')
    torch.cuda.synchronize()
    b_host = bounds[: prims * 4].reshape(prims, 4).cpu().numpy()
    v_host = vertexes[: (P * R * W + 1) * 8].reshape(-1, 8).cpu().numpy()
    masks = oracle.bin_masks(b_host, ra.screen_transform, ra.width, ra.height, B)
    assert np.array_equal(masks_d.cpu().numpy().view(np.uint64), masks)
    del masks_d
    xy = stratified_pixels(ra.width, ra.height, cells=8, span=16, seed=1)
    ref = oracle.raster_pixels(v_host, masks, ghost, light_spectrum(), ra, xy)
    want, have = at_pixels(ref, xy), at_pixels(got, xy)
    assert (want[:, :3] != 0).any(-1).mean() > 0.2
    assert rel_l2(have, want) < STAGE_RTOL


def benchmark_project():
    from realflare_gb300.data import Project, RenderElement, cast

    with open(os.path.join(os.path.dirname(__file__), 'golden', 'nikon_ai_50_135mm.project.json')) as f:
        p = cast(Project, json.load(f))
    p.output.element = RenderElement.FLARE
    return p


def test_reference_benchmark_project_against_reference_kernels():
    """Engine.render of the reference's benchmark project (FLARE element) against the
    reference's own kernels (oracle/_ref) fed the same culled ghosts, integer wavelengths and
    ghost texture, on 4096 stratified pixels; the culled ghost list equals the reference
    probe's."""
    from oracle.oracle import Reference

    if not Reference.available():
        pytest.skip('reference kernels not available (no generated sources)')
    from realflare_gb300.engine import Engine
    from realflare_gb300.tasks import GhostApertureTask, GhostTask, PreprocessTask

    ref_k = Reference()
    p = benchmark_project()
    assert (p.render.anti_aliasing, p.render.wavelength_sub_count, p.render.wavelength_count,
            p.render.grid_count, p.render.cull_percentage) == (4, 8, 5, 129, 0.5)
    kept = kept_paths(p, ref_k.trace)
    assert PreprocessTask().run(p) == kept and len(kept) == 91
    engine = Engine(cache=False)
    assert engine.render(p)
    got = engine.image.array
    ghost = GhostTask().run(p, GhostApertureTask().run(p)).array
    ti = prepare.trace_inputs(p, path_indexes=kept)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays = ref_k.trace(ti.elements, ti.paths, ti.wavelengths.astype(np.int32), a)
    area, min_area = prepare.quad_constants(p)
    bounds, inten = ref_k.prim_shader(rays, P, W, G, area, min_area)
    ra = prepare.raster_args(p, P, W, ghost.shape)
    assert ra.sub_steps == 4 and ra.wavelength_sub_count == 8
    vtx = ref_k.vertex_shader(rays, inten, P, W, G, ra.screen_transform, ra.width, ra.height)
    masks = ref_k.binner(bounds, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    xy = stratified_pixels(ra.width, ra.height, cells=16, span=16, seed=2)
    ref = ref_k.rasterizer_pixels(vtx, masks, ghost, light_spectrum(), ra, xy)
    want, have = at_pixels(ref, xy), at_pixels(got, xy)
    assert (want[:, :3] != 0).any(-1).mean() > 0.2
    assert rel_l2(have, want) < IMAGE_RTOL
