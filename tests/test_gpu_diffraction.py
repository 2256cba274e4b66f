"""Parity of the diffraction stages (FFT, starburst spectrum and compositor, ghost FRFT,
aperture masks) with numpy FP64 and the C oracle. The FFT stages compute in FP32 against
numpy's FP64 (the reference's own arithmetic for these stages); tolerances are relative L2
over the whole array."""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from helpers import rel_l2  # noqa: E402

from realflare_gb300._abi import StarburstArgs, check, lib  # noqa: E402
from realflare_gb300.constants import light_spectrum  # noqa: E402


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


@pytest.fixture(scope='module')
def oracle():
    from oracle.oracle import Oracle

    return Oracle('f32')


# powers of two (radix-2 passes) and other lengths (Bluestein's chirp-z form): odd, even,
# mixed with a power of two, and the longest row (4095: an 8192-point convolution)
@pytest.mark.parametrize('shape', [(8, 16), (64, 64), (256, 128), (512, 512), (5, 7), (300, 300), (75, 128),
                                   (3, 4095)])
@pytest.mark.parametrize('direction', [-1, 1])
def test_fft2_matches_numpy(shape, direction):
    h, w = shape
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((2, h, w)) + 1j * rng.standard_normal((2, h, w))).astype(np.complex64)
    data = torch.from_numpy(x.view(np.float32).copy()).cuda()
    scratch = torch.empty_like(data)
    scale = 1.0 / math.sqrt(h * w)
    check(lib().rf_fft2(data.data_ptr(), scratch.data_ptr(), 2, w, h, direction, scale, stream()), 'rf_fft2')
    torch.cuda.synchronize()
    got = data.cpu().numpy().view(np.complex64)
    ref = (np.fft.fftn if direction < 0 else np.fft.ifftn)(x.astype(np.complex128), axes=(1, 2), norm='ortho')
    pow2 = all(n & (n - 1) == 0 for n in shape)
    # the chirp-z form rounds through three transforms of twice the length
    assert rel_l2(got.view(np.float32), ref.astype(np.complex64).view(np.float32)) < (2e-6 if pow2 else 1e-5)


def aperture_image(oracle, n=128, blades=8):
    return oracle.aperture_shape(n, n, (0.75, 0.75), blades, 0.0, 0.0, 0.0)


def test_aperture_shape_matches_oracle(oracle):
    for blades, rot, rnd, soft in [(6, 0.0, 0.0, 0.0), (8, 0.3, 0.2, 0.05), (5, -1.0, 0.5, 0.02)]:
        ref = oracle.aperture_shape(96, 80, (0.75, 0.7), blades, rot, rnd, soft)
        img = torch.empty((80, 96), device='cuda')
        check(lib().rf_aperture_shape(img.data_ptr(), 96, 80, 0.75, 0.7, blades, rot, rnd, soft, stream()), 'shape')
        torch.cuda.synchronize()
        got = img.cpu().numpy()
        # pixels on the edge of a hard mask may flip on an ulp of the polygon distance
        assert (np.abs(got - ref) > 1e-3).mean() < 2e-3
        assert rel_l2(got, ref) < 2e-2


def test_aperture_dust_and_noise_dust_match_oracle(oracle):
    base = aperture_image(oracle, 64)
    ref = oracle.aperture_dust(base, (0.75, 0.75), 0.8, 0.2, 0.05, (0.1, -0.2), 0.01)
    img = torch.from_numpy(base.copy()).cuda()
    check(lib().rf_aperture_dust(img.data_ptr(), 64, 64, 0.75, 0.75, 0.8, 0.2, 0.05, 0.1, -0.2, 0.01, stream()),
          'dust')
    torch.cuda.synchronize()
    got = img.cpu().numpy()
    # the dust centres come from the reference's sin-based hash, whose last bits differ
    # between CUDA's sinf and the host libm's (x 43758 amplifies them): the circles move by
    # a fraction of a pixel, so compare coverage statistics, not pixels
    assert abs(got.mean() - ref.mean()) < 0.02 * ref.mean()
    assert (np.abs(got - ref) > 0.5).mean() < 0.15
    noise = np.random.default_rng(3).random((64, 64), dtype=np.float32)
    ref2 = oracle.aperture_noise_dust(base, noise, 1.0, 2.0)
    img2 = torch.from_numpy(base.copy()).cuda()
    scratch = torch.empty((64, 64), device='cuda')
    noise_d = torch.from_numpy(noise).cuda()
    check(lib().rf_aperture_noise_dust(img2.data_ptr(), noise_d.data_ptr(), scratch.data_ptr(), 64, 64, 1.0, 2.0,
                                       stream()), 'noise dust')
    torch.cuda.synchronize()
    assert rel_l2(img2.cpu().numpy(), ref2) < 1e-5


@pytest.mark.parametrize('n', [64, 256, 300])
def test_starburst_spectrum_matches_numpy(oracle, n):
    from oracle.oracle import fft_power_spectrum

    ap = aperture_image(oracle, n)
    lam = [560e-6, 400e-6]
    spectrum = torch.empty((2, n, n), device='cuda')
    scratch = torch.empty((2, 2, n, n, 2), device='cuda')
    arr = (ctypes.c_float * 2)(*lam)
    ap_d = torch.from_numpy(ap).cuda()
    check(lib().rf_starburst_spectrum(ap_d.data_ptr(), n, n, arr, 2, 1000.0, scratch.data_ptr(),
                                      spectrum.data_ptr(), stream()), 'spectrum')
    torch.cuda.synchronize()
    got = spectrum.cpu().numpy()
    for k, l in enumerate(lam):
        ref = fft_power_spectrum(ap, l, 1000.0)
        assert rel_l2(got[k], ref) < 1e-5


@pytest.mark.parametrize('fstop', [0.0, 8.0, 32.0, 64.0, 100.0])
def test_ghost_frft_matches_numpy(oracle, fstop):
    from oracle.oracle import ghost_texture

    n = 64
    ap = aperture_image(oracle, n, 6)
    alpha = 0.15 * (560.0 / 400) * (fstop / 18)
    out = torch.empty((n, n), device='cuda')
    scratch = torch.empty((3, n, n, 2), device='cuda')
    ap_d = torch.from_numpy(ap).cuda()
    check(lib().rf_ghost_frft(ap_d.data_ptr(), n, n, alpha, scratch.data_ptr(), out.data_ptr(), stream()), 'frft')
    torch.cuda.synchronize()
    ref = ghost_texture(ap, fstop, (n, n))
    assert rel_l2(out.cpu().numpy(), ref) < 1e-4


def test_ghost_frft_matches_reference_frft_fixture():
    """rf_ghost_frft against ghost textures computed by the reference's own ``frft.py``
    (``tests/golden/frft_ghost.npz``): every branch of ``frft.normalize``, square and
    non-square apertures."""
    import os

    from golden.make_frft_golden import CASES, key

    with np.load(os.path.join(os.path.dirname(__file__), 'golden', 'frft_ghost.npz')) as z:
        g = {k: z[k] for k in z.files}
    for case, h, w, _, _, fstops in CASES:
        ap_d = torch.from_numpy(g[f'{case}_aperture']).cuda()
        scratch = torch.empty((3, h, w, 2), device='cuda')
        for fstop in fstops:
            out = torch.empty((h, w), device='cuda')
            alpha = 0.15 * (560.0 / 400) * (fstop / 18)
            check(lib().rf_ghost_frft(ap_d.data_ptr(), w, h, alpha, scratch.data_ptr(), out.data_ptr(), stream()),
                  'frft')
            torch.cuda.synchronize()
            assert rel_l2(out.cpu().numpy(), g[key(case, fstop)]) < 1e-4, (case, fstop)


def starburst_args(w, h, sw, sh, samples=16, blur=0.01, rotation=0.2, weight=1.0, vig=(0.75, 1.0)):
    a = StarburstArgs()
    a.width, a.height, a.spectrum_width, a.spectrum_height, a.spectrum_count = w, h, sw, sh, 1
    a.samples, a.blur, a.rotation, a.rotation_weight = samples, blur, rotation, weight
    a.vignetting[0], a.vignetting[1] = vig
    a.intensity = 1e-6
    a.offset[0], a.offset[1] = 0.1, -0.05
    a.scale[0], a.scale[1] = 1.0, 1.0
    a.lambda_first, a.lambda_step = 560.0, 1.0
    return a


def test_starburst_matches_oracle(oracle):
    from oracle.oracle import fft_power_spectrum

    ap = aperture_image(oracle, 64)
    spec = fft_power_spectrum(ap, 560e-6, 1000.0).astype(np.float32)
    a = starburst_args(96, 64, 64, 64, samples=64)
    ref = oracle.starburst(spec, light_spectrum(), a)
    img = torch.empty((64, 96, 4), device='cuda')
    spec_d, light_d = torch.from_numpy(spec).cuda(), torch.from_numpy(light_spectrum()).cuda()
    check(lib().rf_starburst(spec_d.data_ptr(), light_d.data_ptr(), ctypes.byref(a), img.data_ptr(), stream()),
          'starburst')
    torch.cuda.synchronize()
    # the noise hash amplifies sin() rounding of large arguments (x 43758): the jitter of
    # individual samples differs, the sample statistics agree
    got = img.cpu().numpy()
    box = lambda a: a[..., :3].reshape(8, 8, 12, 8, 3).mean(axis=(1, 3))  # 8 x 8 pixel boxes
    assert rel_l2(box(got), box(ref)) < 3e-2
    assert abs(got[..., :3].sum() / ref[..., :3].sum() - 1) < 1e-2


@pytest.mark.parametrize('vignetting', [(0.75, 1.0), (float('nan'), float('nan'))])
def test_starburst_without_jitter_matches_oracle_tightly(oracle, vignetting):
    """blur 0 and rotation 0 (the production settings): the jitter radius and the rotation
    angle are exactly 0, so the noise hash no longer moves samples and the image is
    deterministic up to FP32 rounding (``starburst.cl:1-87``)."""
    from oracle.oracle import fft_power_spectrum

    ap = aperture_image(oracle, 128)
    spec = fft_power_spectrum(ap, 560e-6, 1000.0).astype(np.float32)
    a = starburst_args(160, 96, 128, 128, samples=100, blur=0.0, rotation=0.0, vig=vignetting)
    ref = oracle.starburst(spec, light_spectrum(), a)
    img = torch.empty((96, 160, 4), device='cuda')
    spec_d, light_d = torch.from_numpy(spec).cuda(), torch.from_numpy(light_spectrum()).cuda()
    check(lib().rf_starburst(spec_d.data_ptr(), light_d.data_ptr(), ctypes.byref(a), img.data_ptr(), stream()),
          'starburst')
    torch.cuda.synchronize()
    assert np.abs(ref[..., :3]).sum() > 0
    assert rel_l2(img.cpu().numpy(), ref) < 1e-5


def test_starburst_per_wavelength_spectra_match_oracle(oracle):
    """One power spectrum per rendered wavelength (16 over 390-700 nm, each FFT'd with its own
    wavelength; an extension of ``starburst.py:45-81``, which uses one at 560 nm): each
    sample reads the spectrum of the nearest wavelength. With 120 samples, sample 62 lies
    exactly halfway between spectra 8 and 9 (17 * 62 / 124 = 8.5): the tie is rounded up
    in both implementations."""
    from oracle.oracle import fft_power_spectrum

    n = 64
    ap = aperture_image(oracle, n)
    wl = np.linspace(390.0, 700.0, 16)
    spec = np.stack([fft_power_spectrum(ap, l * 1e-6, 1000.0) for l in wl]).astype(np.float32)
    a = starburst_args(96, 64, n, n, samples=120, blur=0.0, rotation=0.0)
    a.spectrum_count = len(wl)
    a.lambda_first, a.lambda_step = float(wl[0]), float(wl[1] - wl[0])
    ref = oracle.starburst(spec, light_spectrum(), a)
    img = torch.empty((64, 96, 4), device='cuda')
    spec_d, light_d = torch.from_numpy(spec).cuda(), torch.from_numpy(light_spectrum()).cuda()
    check(lib().rf_starburst(spec_d.data_ptr(), light_d.data_ptr(), ctypes.byref(a), img.data_ptr(), stream()),
          'starburst')
    torch.cuda.synchronize()
    # different from the single-spectrum image: the per-wavelength spectra are used
    single = a
    single.spectrum_count = 1
    ref_single = oracle.starburst(spec[7], light_spectrum(), single)
    assert rel_l2(ref, ref_single) > 1e-3
    assert rel_l2(img.cpu().numpy(), ref) < 1e-5
