"""Host-side logic: glass catalogue (the reference's own known-answer tests), lens element
construction, ghost paths, wavelengths, synthetic lenses and argument preparation."""
from __future__ import annotations

import math

import numpy as np
import pytest

from realflare_gb300 import glass, lens, prepare, synthetic
from realflare_gb300.constants import LAMBDA_MAX, LAMBDA_MIN, light_spectrum
from realflare_gb300.data import Glass, LensElement, LensModel, Project, QSize, RealflareError, cast


def test_glass_catalogue_known_answers():
    # realflare tests/glass.py:11-53
    glasses = glass.glasses_from_path('$GLASS/schott')
    assert glasses[0] == Glass('BAFN6', 'schott', 1.589, 48.45,
                               [1.36719201, 0.00882820704, 0.10907994, 0.0438731646, 1.02108011, 113.58602])
    closest = glass.closest_glass(tuple(glasses), 1.5, 80, 0)
    assert closest == Glass('N-PK52A', 'schott', 1.497, 81.61,
                            [1.029607, 0.00516800155, 0.1880506, 0.0166658798, 0.736488165, 138.964129])
    assert glass.manufacturers() == {'schott': '$GLASS/schott'}
    assert glass.closest_glass((), 1.5, 60) is None and glass.closest_glass(tuple(glasses), 0, 60) is None


def test_sellmeier_matches_catalogue_nd():
    for g in glass.glasses_from_path('$GLASS/schott')[:40]:
        assert abs(glass.sellmeier(g.coefficients, 587.5618) - g.n) < 2e-3


def test_lens_elements_follow_reference_rules():
    m = LensModel(aperture_index=1, lens_elements=[
        LensElement(radius=50, distance=5, refractive_index=1.6, abbe_nr=40, height=12),
        LensElement(radius=0, distance=3, refractive_index=1.0, height=8),
        LensElement(radius=-40, distance=30, refractive_index=1.0, height=12)])
    el = lens.elements(m, (36, 24), '$GLASS/schott', 0, (550, 0, 600))
    assert len(el) == 4  # + sensor
    assert list(el['center']) == [50, 5, 8 - 40, 38]  # sum(distance before) + radius
    assert el[3]['height'] == pytest.approx(math.hypot(36, 24) / 2)
    assert list(el['coating']) == [550, 0, 600, 0]
    assert not np.isnan(el[0]['coefficients'][0])
    el2 = lens.elements(m, (36, 24), '/nonexistent', 0, ())
    assert np.isnan(el2[0]['coefficients'][0])  # no catalogue: dispersion off (lens.py:61-62)


def test_ray_paths_and_wavelengths():
    m = LensModel(aperture_index=3, lens_elements=[LensElement()] * 8)
    paths = lens.ray_paths(m)
    assert paths == [(1, 0), (2, 0), (2, 1), (5, 4), (6, 4), (6, 5)]
    assert lens.ray_paths(m, (1, 4)) == [(2, 0), (6, 4)]
    assert lens.ray_paths(m, (-1,)) == [(-1, -1)]
    assert len(lens.all_two_bounce_paths(synthetic.make_lens(24, 11))) == 276
    wl = lens.wavelength_array(4)
    assert wl == [LAMBDA_MIN + (i + 0.5) / 4 * (LAMBDA_MAX - LAMBDA_MIN) for i in range(4)]
    assert light_spectrum().shape == (340, 4)


def test_real_lens_models_ghost_counts():
    """The bundled prescriptions (the reference's ``realflare/resources/model``) resolve
    through ``$RES`` and give the reference's ghost counts."""
    counts = {'Canon/ef70-200mm-f2-8l-usm.json': 304, 'Kodak/100mm.json': 25, 'Leica/35mm_1_4.json': 36,
              'Nikon/af_s_28_70mm.json': 157, 'Nikon/ai_50_135mm.json': 182, 'Tronnier/color-heliar.json': 11,
              'Zeiss/zeiss-mp-50-t1-4.json': 127}
    for name, n in counts.items():
        model = lens.model_from_path(lens.decode_path(f'$RES/model/{name}'))
        assert len(lens.ray_paths(model)) == n, name
    p = Project()
    p.flare.lens.lens_model_path = '$RES/model/Nikon/ai_50_135mm.json'
    assert lens.resolve_model(p.flare.lens).aperture_index == 14


def test_model_errors():
    with pytest.raises(RealflareError):
        lens.model_from_path('')
    with pytest.raises(RealflareError):
        lens.model_from_path('/nonexistent/lens.json')


def test_project_cast_and_hash():
    p = cast(Project, {'render': {'resolution': [640, 480], 'grid_count': 17},
                       'flare': {'lens': {'coating': [500, 600], 'sensor_size': [36, 24]}}})
    assert p.render.resolution.width() == 640 and p.render.grid_count == 17
    assert p.flare.lens.coating == (500, 600)
    assert hash(p) == hash(cast(Project, {'render': {'resolution': [640, 480], 'grid_count': 17},
                                          'flare': {'lens': {'coating': [500, 600], 'sensor_size': [36, 24]}}}))


def test_synthetic_lens_acceptance_rule():
    """LENS_SEEDS is the first seed whose ghost rays reach the sensor at >= 40 %."""
    from oracle.oracle import Oracle

    o = Oracle('f32')

    def fraction(n, seed):
        w = synthetic.workload({8: 'plain-8', 16: 'spectral-16', 24: 'production-24'}[n])
        m = synthetic.make_lens(n, seed)
        w.project.flare.lens.lens_model = m
        w.project.flare.lens.coating_thickness = ()
        paths = lens.all_two_bounce_paths(m)
        w.project.render.grid_count = 12
        w.project.render.wavelengths = (550.0,)
        ti = prepare.trace_inputs(w.project, paths)
        r = o.trace(ti.elements, ti.paths, ti.wavelengths, ti.args)
        return np.isfinite(r[5]).mean()

    for n, seed in synthetic.LENS_SEEDS.items():
        assert fraction(n, seed) >= synthetic.ACCEPT_FRACTION
        for s in range(seed):
            assert fraction(n, s) < synthetic.ACCEPT_FRACTION


def test_prepare_arguments():
    w = synthetic.workload('production-24')
    ti = prepare.trace_inputs(w.project)
    assert ti.args.path_count == 276 and ti.args.wavelength_count == 16 and ti.args.grid_count == 128
    assert ti.ray_count == 276 * 16 * 128 * 128
    assert ti.elements['coating_layers'].tolist()[:3] == [2, 2, 2]
    ra = prepare.raster_args(w.project, 276, 16, (256, 256))
    assert ra.screen_transform == pytest.approx(2048 / (math.hypot(36, 24) / 2))
    assert ra.intensity == pytest.approx(1e3)
    w.project.render.anti_aliasing = 3
    with pytest.raises(RealflareError):
        prepare.raster_args(w.project, 276, 16, (256, 256))
    p = Project()
    p.render.resolution = QSize(100, 50)
    d = lens.direction((0.5, -0.5), p.render.resolution, (36, 24), 50)
    assert list(d) == pytest.approx([9.0, -4.5, 50, 1])


def test_light_image_resize_and_sampling():
    """ImageSamplingTask's host arithmetic (preprocessing.py:126-162): bilinear resize with
    half-pixel centres and clamped edges, and the percentile mask keeping the brightest."""
    from realflare_gb300.tasks import ImageSamplingTask, resize_linear

    a = np.arange(4 * 6 * 3, dtype=np.float32).reshape(4, 6, 3)
    assert np.array_equal(resize_linear(a, 6, 4), a)
    half = resize_linear(a, 3, 2)
    # each output pixel is the mean of a 2 x 2 input block at a factor of 2
    assert np.allclose(half[0, 0], a[0:2, 0:2].mean((0, 1)))
    up = resize_linear(a, 12, 8)
    assert np.array_equal(up[0, 0], a[0, 0]) and np.array_equal(up[-1, -1], a[-1, -1])
    img = np.zeros((8, 8, 3), np.float32)
    img[1, 2] = 5.0
    img[6, 6] = 3.0
    img[3, 3] = 1.0
    sd = ImageSamplingTask.sample_data(img, 8, 8, 2)
    assert sd.shape == (8, 8, 4) and np.all(sd[..., 3] == 0)
    lit = np.argwhere(sd[..., :3].sum(-1) > 0)
    assert {tuple(v) for v in lit} == {(1, 2), (6, 6)}


def test_hash_sine_reduction():
    """The noise hash's sine (rf_image.cu hash_sin): Cody-Waite reduction by pi/2 with the
    three-part split in the kernel, emulated exactly here (float32 values, fused
    multiply-adds through float64), then the quadrant; against sin in float64."""
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-2.0**22, 2.0**22, 20000), rng.uniform(-10, 10, 2000),
                        np.float64(np.arange(-50, 50)) * np.pi / 2]).astype(np.float32)
    f = np.float32
    c1, c2, c3 = f(float.fromhex('0x1.921fb6p+0')), f(float.fromhex('-0x1.777a5cp-25')), f(float.fromhex('-0x1.ee59dap-50'))

    def fma(a, b, c):  # exact for these operands: the product fits in 48 bits
        return (np.float64(a) * np.float64(b) + np.float64(c)).astype(np.float32)

    k = np.rint(x * f(float.fromhex('0x1.45f306p-1'))).astype(np.float32)
    r = fma(-k, c1, x)
    r = fma(-k, c2, r)
    r = fma(-k, c3, r)
    q = k.astype(np.int64) & 3
    rs, rc = np.sin(np.float64(r)), np.cos(np.float64(r))
    got = np.select([q == 0, q == 1, q == 2], [rs, rc, -rs], -rc)
    want = np.sin(np.float64(x))
    # x * 2/pi rounds in float32 (a quarter unit at |x| ~ 2^22), so k can be one off and
    # |r| reach 3 pi/4; sincosf stays accurate there, only the quadrant has to match k
    assert np.abs(np.float64(r)).max() < 3 * np.pi / 4
    assert np.abs(got - want).max() < 4e-7


def test_lens_parameter_map_equals_its_direct_form():
    """LensParameters.elements (one matrix-vector product) equals elements_direct (the map
    op by op) in value and in gradient, on parameters away from the lens's own."""
    import torch

    from realflare_gb300 import synthetic
    from realflare_gb300.diff import LensParameters

    w = synthetic.workload('differentiable-16')
    lp = LensParameters(w.project, device='cpu')
    n = len(w.project.flare.lens.lens_model.lens_elements) + 1  # with the sensor
    g = torch.Generator().manual_seed(0)
    base = [t + torch.randn(t.shape, generator=g, dtype=torch.float64) * 0.1 * (t.abs() + 1) for t in lp.tensors()]
    weights = [torch.randn(k, generator=g, dtype=torch.float64) for k in (n, n, n, 3)]
    grads = []
    for fn in (lp.elements, lp.elements_direct):
        ps = [t.clone().requires_grad_(True) for t in base]
        out = fn(*ps, n)
        loss = sum((o * wt).sum() for o, wt in zip(out, weights))
        loss.backward()
        grads.append(([o.detach() for o in out], [p.grad for p in ps]))
    (va, ga), (vb, gb) = grads
    for x, y in zip(va + ga, vb + gb):
        assert torch.allclose(x, y, rtol=1e-12, atol=1e-12)
