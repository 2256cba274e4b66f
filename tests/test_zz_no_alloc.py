"""rf_ghost_frft_static: the ghost texture without a caller scratch buffer.

Callers that cannot allocate device memory at render time (a plugin whose host
application owns all device memory, a render loop that must not allocate after start-up)
use this entry point; its scratch is a static device array shared by all calls. The test
calls it through the C ABI several times in a row on different inputs (among them the
largest size, which fills the array to its end, a non-square one and the alpha branch that
flips the spectrum) and compares each result with rf_ghost_frft given a scratch buffer,
and checks that sizes above the static maximum are refused. It runs last (file name) and also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

from realflare_gb300._abi import RF_ERR_INVALID_ARG, RF_OK, lib  # noqa: E402

# the tolerance of the FRFT tests (relative L2); both paths run the same kernels
RTOL = 1e-6


def aperture(h, w, blades, rotation):
    y, x = np.mgrid[-1:1:complex(0, h), -1:1:complex(0, w)]
    angle = np.arctan2(y, x) + rotation
    r = np.hypot(x, y) * np.cos(np.pi / blades) / np.cos((angle % (2 * np.pi / blades)) - np.pi / blades)
    return (r < 0.75).astype(np.float32)


def with_scratch(ap_d, h, w, alpha):
    out = torch.empty((h, w), device='cuda')
    scratch = torch.empty((3, h, w, 2), device='cuda')
    s = int(torch.cuda.current_stream().cuda_stream)
    assert lib().rf_ghost_frft(ap_d.data_ptr(), w, h, alpha, scratch.data_ptr(), out.data_ptr(), s) == RF_OK
    return out


def alpha_of(fstop):
    return 0.15 * (560 / 400) * (fstop / 18)


# (height, width, blades, rotation, alpha): two ordinary calls in a row; the array filled to
# its last element (512 x 512, and 64 x 4096 of the same pixel count, not square); alpha
# 3.2, whose branch flips the spectrum into the third plane and copies it back
CASES = [(256, 256, 6, 0.0, 0.0), (128, 128, 8, 0.3, alpha_of(40)), (512, 512, 8, 0.1, alpha_of(64)),
         (64, 4096, 5, 0.2, alpha_of(8)), (128, 128, 6, 0.0, 3.2)]


def test_static_scratch_matches_caller_scratch_on_two_calls():
    L = lib()
    s = int(torch.cuda.current_stream().cuda_stream)
    for h, w, blades, rot, alpha in CASES:
        ap_d = torch.from_numpy(aperture(h, w, blades, rot)).cuda()
        out = torch.empty((h, w), device='cuda')
        assert L.rf_ghost_frft_static(ap_d.data_ptr(), w, h, alpha, out.data_ptr(), s) == RF_OK
        ref = with_scratch(ap_d, h, w, alpha)
        torch.cuda.synchronize()
        got, want = out.cpu().numpy(), ref.cpu().numpy()
        assert np.isfinite(got).all() and np.linalg.norm(want) > 0
        assert np.linalg.norm(got - want) / np.linalg.norm(want) <= RTOL


def test_static_scratch_rejects_oversize():
    L = lib()
    ap_d = torch.zeros((1024, 1024), device='cuda')
    out = torch.empty((1024, 1024), device='cuda')
    status = L.rf_ghost_frft_static(ap_d.data_ptr(), 1024, 1024, 0.0, out.data_ptr(),
                                    int(torch.cuda.current_stream().cuda_stream))
    assert status == RF_ERR_INVALID_ARG
    assert b'RF_GHOST_FRFT_STATIC_MAX_PIXELS' in L.rf_last_cuda_error()
