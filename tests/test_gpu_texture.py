"""Ghost lookups through a texture gather against the texel loads.

The raster reads the four texels of each bilinear ghost lookup with one gather from a
texture object over the ghost texture (border mode: 0 outside) when the library can make
one (``rf_ghost_texture_object``: base and row pitch aligned as the device requires), else
with four bounds-checked loads. Both give the same texels and the same interpolation, so
the images are equal bit for bit; the adjoint's sums over atomics are compared within
rounding.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from helpers import ghost_texture, reduced  # noqa: E402

from realflare_gb300._abi import RF_ERR_INVALID_ARG, check, lib  # noqa: E402


def texture_object(t: torch.Tensor, w: int, h: int) -> int:
    out = ctypes.c_uint64()
    check(lib().rf_ghost_texture_object(t.data_ptr(), w, h, ctypes.byref(out)), 'rf_ghost_texture_object')
    return out.value


def placements(shape=(64, 64)):
    """The same ghost texels at an aligned address and 16 bytes past one."""
    g = torch.from_numpy(ghost_texture(shape)).cuda()
    buf = torch.zeros(g.numel() + 4, device='cuda')
    buf[4:] = g.reshape(-1)
    return g, buf[4:].view(*shape)


def test_texture_objects():
    g, shifted = placements()
    h = texture_object(g, 64, 64)
    assert h != 0 and texture_object(g, 64, 64) == h  # one object per address and size
    assert texture_object(g, 32, 64) not in (0, h)
    assert texture_object(shifted, 64, 64) == 0  # base address not aligned: loads
    odd = torch.zeros(75 * 64, device='cuda')
    assert texture_object(odd, 75, 64) == 0  # row pitch 300 bytes: loads
    # after the cache is forgotten (as after a device reset) the next call makes a new object
    assert lib().rf_ghost_textures_forget() == 0
    h2 = texture_object(g, 64, 64)
    assert h2 not in (0, h) and texture_object(g, 64, 64) == h2
    out = ctypes.c_uint64()
    assert lib().rf_ghost_texture_object(None, 64, 64, ctypes.byref(out)) == RF_ERR_INVALID_ARG
    assert lib().rf_ghost_texture_object(g.data_ptr(), 0, 64, ctypes.byref(out)) == RF_ERR_INVALID_ARG


@pytest.mark.parametrize('aa,ws', [(1, 1), (4, 2)])
def test_raster_gather_equals_loads(aa, ws):
    from realflare_gb300.device import Image
    from realflare_gb300.tasks import RasterizingTask, RaytracingTask

    w = reduced('spectral-16', grid=32, resolution=256, paths=24, wavelengths=4)
    w.project.render.anti_aliasing = aa
    w.project.render.wavelength_sub_count = ws
    g, shifted = placements()
    assert texture_object(g, 64, 64) != 0 and texture_object(shifted, 64, 64) == 0
    rays = RaytracingTask(cache=False).run(w.project, paths=w.paths)
    a = RasterizingTask().run(w.project, rays, Image(tensor=g)).array
    b = RasterizingTask().run(w.project, rays, Image(tensor=shifted)).array
    assert (a[..., :3] > 0).any()
    assert np.array_equal(a, b)


def test_adjoint_gather_matches_loads():
    from realflare_gb300.diff import DifferentiableRenderer

    w = reduced('spectral-16', grid=24, resolution=128, paths=16, wavelengths=3)
    g, shifted = placements()
    grads = []
    for ghost in (g, shifted):
        r = DifferentiableRenderer(w.project, ghost, paths=w.paths)
        params = [t.detach().clone().requires_grad_(True) for t in r.params.tensors()]
        img = r.render(*params)
        (img[..., :3] ** 2).sum().backward()
        grads.append((img.detach().cpu().numpy(), torch.cat([q.grad.reshape(-1) for q in params]).cpu().numpy()))
    (ia, ga), (ib, gb) = grads
    assert np.array_equal(ia, ib)
    assert np.abs(ga).max() > 0
    np.testing.assert_allclose(ga, gb, rtol=1e-4, atol=1e-6 * np.abs(ga).max())
