"""The C oracle against the reference's own OpenCL kernels compiled for the host
(oracle/_ref, built from the reference checkout or its generated sources): bit-identical
rays, primitive bounds and intensities, vertices, bin masks and images on reduced 8-, 16-
and 24-surface workloads, and the same aperture masks and starburst images."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import ghost_texture, reduced

from realflare_gb300 import prepare
from realflare_gb300.constants import light_spectrum

oracle_mod = pytest.importorskip('oracle.oracle')
if not oracle_mod.reference_available():
    pytest.skip('reference kernels not available (no checkout and no generated sources)',
                allow_module_level=True)

CASES = {
    'plain-8': dict(grid=20, resolution=128),
    'spectral-16': dict(grid=16, resolution=128, paths=24, wavelengths=4),
    # the reference has single-layer coatings only: its lambda0 rule is used here
    'production-24': dict(grid=12, resolution=128, paths=24, wavelengths=5),
}


@pytest.fixture(scope='module')
def pair():
    return oracle_mod.Oracle('f32'), oracle_mod.Reference()


def nan_equal(a, b):
    return np.array_equal(np.nan_to_num(a, nan=7e30), np.nan_to_num(b, nan=7e30))


@pytest.mark.parametrize('name', list(CASES))
def test_oracle_bit_identical_to_reference_kernels(pair, name):
    o, r = pair
    w = reduced(name, **CASES[name])
    w.project.flare.lens.coating_thickness = ()
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays_o = o.trace(ti.elements, ti.paths, ti.wavelengths, a)
    rays_r = r.trace(ti.elements, ti.paths, ti.wavelengths.astype(np.int32), a)
    assert nan_equal(rays_o, rays_r)
    area, min_area = prepare.quad_constants(w.project)
    bo, io = o.quad_setup(rays_r, P, W, G, area, min_area)
    br, ir = r.prim_shader(rays_r, P, W, G, area, min_area)
    assert nan_equal(bo, br) and nan_equal(io, ir)
    ghost = ghost_texture((48, 48), seed=3)
    ra = prepare.raster_args(w.project, P, W, ghost.shape)
    vo = o.vertex(rays_r, ir, P, W, G, ra.screen_transform, ra.width, ra.height)
    vr = r.vertex_shader(rays_r, ir, P, W, G, ra.screen_transform, ra.width, ra.height)
    assert nan_equal(vo, vr)
    mo = o.bin_masks(br, ra.screen_transform, ra.width, ra.height, ra.bin_size)
    mr = r.binner(br, ra.screen_transform, ra.width, ra.height, ra.bin_size, local_size=64)
    assert np.array_equal(mo, mr)
    io_ = o.raster(vr, mr, ghost, light_spectrum(), ra)
    ir_ = r.rasterizer(vr, mr, ghost, light_spectrum(), ra)
    assert np.array_equal(io_, ir_)
    assert (ir_[..., :3] != 0).any()


RASTER_MODES = [(1, 2), (1, 8), (2, 1), (4, 1), (4, 8), (8, 2)]


@pytest.mark.parametrize('aa,ws', RASTER_MODES)
@pytest.mark.parametrize('name', ['plain-8', 'spectral-16'])
def test_oracle_raster_modes_bit_identical_to_reference_kernels(pair, name, aa, ws):
    """Anti-aliasing (n-rook samples, ``rasterizing.cl:628-633``) and wavelength sub-steps
    (``mix_vertex`` at ``wavelength_sub_pos`` with one spectrum lookup per step,
    ``rasterizing.cl:606-650``): the oracle's image equals the reference kernels' bit for bit.
    One wavelength (plain-8) turns the sub-steps off as ``rasterizing.py:390-392`` does."""
    o, r = pair
    kw = dict(grid=20, resolution=128) if name == 'plain-8' else dict(grid=16, resolution=128, paths=24,
                                                                      wavelengths=4)
    w = reduced(name, **kw)
    w.project.flare.lens.coating_thickness = ()
    w.project.render.anti_aliasing = aa
    w.project.render.wavelength_sub_count = ws
    ti = prepare.trace_inputs(w.project, w.paths)
    a = ti.args
    P, W, G = a.path_count, a.wavelength_count, a.grid_count
    rays = r.trace(ti.elements, ti.paths, ti.wavelengths.astype(np.int32), a)
    area, min_area = prepare.quad_constants(w.project)
    bounds, inten = r.prim_shader(rays, P, W, G, area, min_area)
    ghost = ghost_texture((48, 48), seed=3)
    ra = prepare.raster_args(w.project, P, W, ghost.shape)
    assert ra.sub_steps == aa and ra.wavelength_sub_count == (ws if W > 1 else 1)
    vtx = r.vertex_shader(rays, inten, P, W, G, ra.screen_transform, ra.width, ra.height)
    masks = r.binner(bounds, ra.screen_transform, ra.width, ra.height, ra.bin_size, local_size=64)
    img_o = o.raster(vtx, masks, ghost, light_spectrum(), ra)
    img_r = r.rasterizer(vtx, masks, ghost, light_spectrum(), ra)
    assert np.array_equal(img_o, img_r)
    assert (img_r[..., :3] != 0).any()


def test_aperture_and_starburst_match_reference_kernels(pair):
    o, r = pair
    for blades, rot, rnd, soft in [(6, 0.0, 0.0, 0.0), (8, 0.4, 0.3, 0.03)]:
        assert np.array_equal(o.aperture_shape(64, 48, (0.75, 0.6), blades, rot, rnd, soft),
                              r.aperture_shape(64, 48, (0.75, 0.6), blades, rot, rnd, soft))
    base = o.aperture_shape(64, 64, (0.75, 0.75), 8, 0.0, 0.0, 0.0)
    assert np.array_equal(o.aperture_dust(base, (0.75, 0.75), 0.7, 0.3, 0.05, (0.1, 0.2), 0.02),
                          r.aperture_dust(base, (0.75, 0.75), 0.7, 0.3, 0.05, (0.1, 0.2), 0.02))
    spec = oracle_mod.fft_power_spectrum(base, 560e-6, 1000.0).astype(np.float32)
    from realflare_gb300._abi import StarburstArgs

    a = StarburstArgs()
    a.width, a.height, a.spectrum_width, a.spectrum_height, a.spectrum_count = 48, 40, 64, 64, 1
    a.samples, a.blur, a.rotation, a.rotation_weight = 24, 0.02, 0.3, 1.5
    a.vignetting[0], a.vignetting[1] = 0.75, 1.0
    a.intensity = 1e-6
    a.offset[0], a.offset[1] = 0.2, -0.1
    a.scale[0], a.scale[1] = 1.0, 1.2
    assert np.array_equal(o.starburst(spec, light_spectrum(), a), r.starburst(spec, light_spectrum(), a))


def diagram_case(o_or_r, w, diagram_width=384, diagram_height=192):
    """The diagram's trace of a reduced workload (three ghost paths, the diagram's settings)
    and the slice of the centre grid column."""
    from realflare_gb300.data import QSize

    p = w.project
    p.diagram.resolution = QSize(diagram_width, diagram_height)
    p.diagram.grid_count = 9
    p.diagram.grid_length = 30.0
    p.diagram.light_position = 0.3
    dp = prepare.diagram_project(p)
    ti = prepare.trace_inputs(dp, paths=w.paths[:3])
    count = prepare.intersection_count(ti.args.element_count)
    return p, ti, count


@pytest.mark.parametrize('name', ['plain-8', 'spectral-16'])
def test_intersections_and_diagram_match_reference_kernels(pair, name):
    """IntersectionsTask's trace (STORE_INTERSECTIONS) and DiagramTask's two kernels: the
    oracle's records and diagram images equal the reference kernels' (integer wavelengths)."""
    o, r = pair
    w = reduced(name)
    w.project.flare.lens.coating_thickness = ()
    p, ti, count = diagram_case(o, w)
    a = ti.args
    rays_o, inter_o = o.trace_intersections(ti.elements, ti.paths, ti.wavelengths, a, count)
    rays_r, inter_r = r.trace_intersections(ti.elements, ti.paths, ti.wavelengths.astype(np.int32), a, count)
    assert nan_equal(rays_o, rays_r)
    assert np.array_equal(inter_o.view(np.int32), inter_r.view(np.int32))
    hits = inter_r[..., 7].view(np.int32)
    assert hits.sum() > a.element_count * 4  # rays do cross the lens
    G = a.grid_count
    column = (G - 1) // 2
    part = inter_r.reshape(a.path_count, 1, G, G, count, 8)[0, 0, :, column]
    scale = np.float32(prepare.diagram_scale(p))
    res = p.diagram.resolution
    for rec in (None, part):
        img_o = o.diagram(ti.elements, a.aperture_index, scale, rec, res.width(), res.height())
        img_r = r.diagram(ti.elements, a.aperture_index, scale, rec, res.width(), res.height())
        assert np.array_equal(img_o, img_r)
        assert (img_r[..., 2] > 0).sum() > 100  # element profiles
        if rec is not None:
            assert (img_r[..., 0] == 0.25).sum() > 100  # ray segments
