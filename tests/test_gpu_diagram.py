"""The lens diagram on the GPU: rf_trace_intersections (the trace with every hit stored) and
rf_diagram (lens profiles, ray paths and normals) against the oracle, and the DIAGRAM render
element through Engine.render.

Hit positions, normals and flags are exact (no transcendental on their path, like the
trace's positions); the incidence angle goes through acos, whose CUDA and libm results
differ by ulps. The diagram image depends on positions and normals only, so it is exact."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip('torch')
pytestmark = pytest.mark.gpu

from helpers import reduced  # noqa: E402

from realflare_gb300 import prepare  # noqa: E402
from realflare_gb300._abi import check, lib  # noqa: E402
from realflare_gb300.data import QSize, RenderElement  # noqa: E402

INCIDENT_ATOL = 2e-6  # radians: a few ulps of acos near pi / 2


@pytest.fixture(scope='module')
def oracle():
    from oracle.oracle import Oracle

    return Oracle('f32')


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


def gpu_trace_intersections(ti, count):
    el, pa, wl = dev(ti.elements.view(np.uint8)), dev(ti.paths), dev(ti.wavelengths)
    n = ti.ray_count
    rays = torch.empty((6, n), device='cuda')
    inter = torch.full((n, count, 8), 7.0, device='cuda')  # the call zeroes it
    plain = torch.empty((6, n), device='cuda')
    L = lib()
    check(L.rf_trace_intersections(el.data_ptr(), pa.data_ptr(), wl.data_ptr(), ctypes.byref(ti.args),
                                   rays.data_ptr(), inter.data_ptr(), count, stream()), 'rf_trace_intersections')
    check(L.rf_trace(el.data_ptr(), pa.data_ptr(), wl.data_ptr(), ctypes.byref(ti.args), plain.data_ptr(),
                     stream()), 'rf_trace')
    torch.cuda.synchronize()
    return rays.cpu().numpy(), inter.cpu().numpy(), plain.cpu().numpy()


def nan_equal(a, b):
    return np.array_equal(np.nan_to_num(a, nan=7e30), np.nan_to_num(b, nan=7e30))


@pytest.mark.parametrize('name,spec', [('plain-8', dict(grid=12)),
                                       ('spectral-16', dict(grid=10, paths=12, wavelengths=3))])
def test_trace_intersections_match_oracle(oracle, name, spec):
    w = reduced(name, **spec)
    ti = prepare.trace_inputs(w.project, w.paths)
    count = prepare.intersection_count(ti.args.element_count)
    rays, inter, plain = gpu_trace_intersections(ti, count)
    assert nan_equal(rays, plain)  # the recorder leaves the rays as rf_trace computes them
    rays_o, inter_o = oracle.trace_intersections(ti.elements, ti.paths, ti.wavelengths, ti.args, count)
    for k in range(5):
        assert nan_equal(rays[k], rays_o[k]), f'plane {k}'
    bits, bits_o = inter.view(np.int32), inter_o.view(np.int32)
    assert np.array_equal(bits[..., 7], bits_o[..., 7])  # the same hits
    for f in (0, 1, 2, 3, 4, 5):  # positions and normals
        assert np.array_equal(bits[..., f], bits_o[..., f]), f'field {f}'
    assert np.allclose(inter[..., 6], inter_o[..., 6], rtol=0, atol=INCIDENT_ATOL)
    assert bits[..., 7].sum() > ti.ray_count * ti.args.element_count // 2


def test_diagram_matches_oracle(oracle):
    w = reduced('plain-8')
    p = w.project
    p.diagram.resolution = QSize(512, 256)
    p.diagram.grid_count = 9
    p.diagram.grid_length = 30.0
    p.diagram.light_position = 0.3
    ti = prepare.trace_inputs(prepare.diagram_project(p), paths=w.paths[4:7])
    a = ti.args
    count = prepare.intersection_count(a.element_count)
    _, inter = oracle.trace_intersections(ti.elements, ti.paths, ti.wavelengths, a, count)
    G = a.grid_count
    part = np.ascontiguousarray(inter.reshape(a.path_count, 1, G, G, count, 8)[1, 0, :, (G - 1) // 2])
    scale = np.float32(prepare.diagram_scale(p))
    el = dev(ti.elements.view(np.uint8))
    for rec in (None, part):
        want = oracle.diagram(ti.elements, a.aperture_index, scale, rec, 512, 256)
        image = torch.empty((256, 512, 4), device='cuda')
        rec_d = dev(rec) if rec is not None else None
        check(lib().rf_diagram(el.data_ptr(), a.element_count, a.aperture_index, float(scale),
                               rec_d.data_ptr() if rec_d is not None else None, G if rec is not None else 0,
                               count, 512, 256, image.data_ptr(), stream()), 'rf_diagram')
        torch.cuda.synchronize()
        got = image.cpu().numpy()
        assert np.array_equal(got, want)
        assert (want[..., 2] > 0).sum() > 100


def test_diagram_render_element(oracle):
    """Engine.render with output.element DIAGRAM (engine.py:189-193) equals the oracle's
    trace-and-draw of the debug ghost's centre column."""
    from realflare_gb300.engine import Engine

    w = reduced('plain-8')
    p = w.project
    p.output.element = RenderElement.DIAGRAM
    p.diagram.resolution = QSize(384, 192)
    p.diagram.grid_count = 8
    p.diagram.grid_length = 30.0
    p.diagram.light_position = -0.2
    p.diagram.debug_ghost = 5
    p.diagram.column_offset = 1
    engine = Engine()
    assert engine.render(p)
    got = engine.image.tensor.cpu().numpy()
    ti = prepare.trace_inputs(prepare.diagram_project(p), path_indexes=(5,))
    a = ti.args
    count = prepare.intersection_count(a.element_count)
    _, inter = oracle.trace_intersections(ti.elements, ti.paths, ti.wavelengths, a, count)
    G = a.grid_count
    part = inter.reshape(a.path_count, 1, G, G, count, 8)[0, 0, :, (G - 1) // 2 + 1]
    want = oracle.diagram(ti.elements, a.aperture_index, np.float32(prepare.diagram_scale(p)), part, 384, 192)
    assert a.path_count == 1
    assert np.array_equal(got, want)
    assert (want[..., 0] == 0.25).sum() > 50
