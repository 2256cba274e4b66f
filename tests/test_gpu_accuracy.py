"""Distance of the render from the same algorithm evaluated in double (the FP64 oracle), in
the default mode (the reference's FP32 trace) and with the double-precision ray geometry
of ``rf_trace_accurate``.

The rasteriser truncates vertex positions to integer sample coordinates and special-cases
zero cross products (``rasterizing.cl:95-148,624``): the image is discontinuous in the ray
positions, so the reference's FP32 positions, a few ulps from the double trace's, move some
quad corners across samples. The accurate trace's positions equal the FP64 oracle's rounded
to float, and its image is then within FP32 raster rounding of the FP64 image.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from helpers import at_pixels, ghost_texture, reduced, rel_l2, stratified_pixels  # noqa: E402

from realflare_gb300 import prepare  # noqa: E402
from realflare_gb300._abi import check, lib  # noqa: E402
from realflare_gb300.constants import light_spectrum  # noqa: E402

# the target of the accurate mode: relative L2 image error against the FP64 oracle
FP64_RTOL = 1e-4

REDUCED = {
    'spectral-16': dict(grid=24, resolution=256, paths=40, wavelengths=5),
    'production-24': dict(grid=16, resolution=256, paths=30, wavelengths=4),
}
# measured FP32-mode errors of the reduced cases (the oracle's FP32 build gives 1.23e-3 and
# 2.52e-4): pinned to a band so that a change shows
FP32_BAND = {'spectral-16': (5e-4, 3e-3), 'production-24': (1e-4, 1e-3)}
# and of the full workloads on the sampled pixels (measured 6.8e-4 and 2.1e-2)
FP32_BAND_FULL = {'spectral-16': (2e-4, 3e-3), 'production-24': (5e-3, 8e-2)}


@pytest.fixture(scope='module')
def oracles():
    from oracle.oracle import Oracle

    return Oracle('f32'), Oracle('f64')


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def gpu_rays(ti, accurate):
    L = lib()
    rays = torch.empty((6, ti.ray_count), device='cuda')
    el, pa, wl = dev(ti.elements.view(np.uint8)), dev(ti.paths), dev(ti.wavelengths)
    fn = L.rf_trace_accurate if accurate else L.rf_trace
    check(fn(el.data_ptr(), pa.data_ptr(), wl.data_ptr(), ctypes.byref(ti.args), rays.data_ptr(), stream()), 'trace')
    torch.cuda.synchronize()
    return rays.cpu().numpy()


@pytest.mark.parametrize('name', list(REDUCED))
def test_accurate_trace_positions_equal_the_fp64_trace(oracles, name):
    _, o64 = oracles
    w = reduced(name, **REDUCED[name])
    ti = prepare.trace_inputs(w.project, w.paths)
    ref = o64.trace(ti.elements, ti.paths, ti.wavelengths, ti.args)  # double, rounded to float
    got = gpu_rays(ti, accurate=True)
    valid = ~np.isnan(ref[5])
    assert np.array_equal(valid, ~np.isnan(got[5]))
    for k in range(5):
        same = (ref[k] == got[k]) | (np.isnan(ref[k]) & np.isnan(got[k]))
        assert same.all(), f'plane {k}: {(~same).sum()} rays differ'
    # reflectances: the FP32 coating formulas against the oracle's double ones
    rel = np.abs(got[5][valid] - ref[5][valid]) / np.abs(ref[5][valid])
    assert rel.max() < 1e-4 and np.median(rel) < 1e-6


def render(o, w, rays, ghost):
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    area, min_area = prepare.quad_constants(w.project)
    b, i = o.quad_setup(rays, P, W, G, area, min_area)
    ra = prepare.raster_args(w.project, P, W, ghost.shape)
    v = o.vertex(rays, i, P, W, G, ra.screen_transform, ra.width, ra.height)
    m = o.bin_masks(b, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    return o.raster(v, m, ghost, light_spectrum(), ra)


@pytest.mark.parametrize('name', list(REDUCED))
def test_image_error_against_fp64_in_both_modes(oracles, name):
    """The whole GPU path (trace, setup, binning, raster) in each mode against the FP64
    oracle's image: the accurate mode within 1e-4; the default mode at its measured
    distance (the reference's own FP32 arithmetic)."""
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    _, o64 = oracles
    w = reduced(name, **REDUCED[name])
    ghost = ghost_texture((64, 64))
    ti = prepare.trace_inputs(w.project, w.paths)
    ref = render(o64, w, o64.trace(ti.elements, ti.paths, ti.wavelengths, ti.args), ghost)
    errors = {}
    for accurate in (False, True):
        rays = RaytracingTask(cache=False, accurate=accurate).run(w.project, paths=w.paths)
        got = RasterizingTask().run(w.project, rays, Image(tensor=dev(ghost))).array
        errors[accurate] = rel_l2(got, ref)
    lo, hi = FP32_BAND[name]
    assert errors[True] < FP64_RTOL, errors
    assert lo < errors[False] < hi, errors


@pytest.mark.parametrize('name', ['spectral-16', 'production-24'])
def test_accurate_mode_at_full_size_on_sampled_pixels(oracles, name):
    """The full workloads (1024^2, 120 ghosts, 64^2 grid, 8 wavelengths; 2048^2, 276 ghosts,
    128^2 grid, 16 wavelengths): the accurate GPU image against the FP64 oracle's raster at
    64 stratified spans of 16 pixels, fed the FP64 trace's vertices and bin masks."""
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    _, o64 = oracles
    w = reduced(name)
    ghost = ghost_texture((256, 256), seed=4)
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays64 = o64.trace(ti.elements, ti.paths, ti.wavelengths, a)
    area, min_area = prepare.quad_constants(w.project)
    b, i = o64.quad_setup(rays64, P, W, G, area, min_area)
    ra = prepare.raster_args(w.project, P, W, ghost.shape)
    v = o64.vertex(rays64, i, P, W, G, ra.screen_transform, ra.width, ra.height)
    del rays64, i
    m = o64.bin_masks(b, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    xy = stratified_pixels(ra.width, ra.height, cells=8, span=16, seed=3)
    ref = at_pixels(o64.raster_pixels(v, m, ghost, light_spectrum(), ra, xy), xy)
    del v, m
    errors = {}
    for accurate in (False, True):
        rays = RaytracingTask(cache=False, accurate=accurate).run(w.project, paths=w.paths)
        got = RasterizingTask().run(w.project, rays, Image(tensor=dev(ghost))).array
        errors[accurate] = rel_l2(at_pixels(got, xy), ref)
        del rays
    print(f'{name}: relative L2 against FP64 on {len(xy)} pixels: FP32 trace {errors[False]:.3e}, '
          f'accurate trace {errors[True]:.3e}')
    assert (ref[:, :3] != 0).any(-1).mean() > 0.2
    assert errors[True] < FP64_RTOL, errors
    lo, hi = FP32_BAND_FULL[name]
    assert lo < errors[False] < hi, errors
