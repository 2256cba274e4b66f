"""Generate ``tests/golden/frft_ghost.npz`` from the reference's own FRFT.

The ghost texture of the reference is ``GhostTask.ghost`` (``realflare/api/tasks/ghost.py:
13-36``): fftshift, ``realflare.utils.frft.frft`` (``realflare/utils/frft.py:20-62``),
fftshift, ``np.float32(np.abs(...))`` times ``sqrt(width * height)``. ``ghost.py`` imports
pyopencl and PySide2, so its five lines of arithmetic are restated here; ``frft.py`` itself
is imported from the reference checkout and run unchanged, except that its ``chirp``
(``frft.py:8-17``) sums a generator with ``np.sum``, which numpy 2 no longer accepts: the
shim sums the same arrays with the builtin ``sum``, the arithmetic numpy 1 fell back to.

The apertures are stored with the outputs (polygon masks computed here in numpy; their edge
pixels depend on libm rounding, so the fixture carries them rather than their recipe).
fstop values cover all five branches of ``frft.normalize`` (``frft.py:20-40``): alpha =
0.15 * 560 / 400 * fstop / 18 is 0 and 0.09-0.37 (below 0.5), 0.75 and 1.17 (below 1.5),
1.75 (below 2.5), 3.21 (below 3.5) and 3.85 (above).

Usage: ``python tests/golden/make_frft_golden.py <reference checkout>`` (or set
``REALFLARE_REFERENCE``).
"""
from __future__ import annotations

import hashlib
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, 'frft_ghost.npz')

LAMBDA_MID = 560.0
# (key, height, width, blades, softness, fstops)
CASES = [
    ('s64', 64, 64, 6, 0.05, (0.0, 8.0, 32.0, 64.0, 100.0, 150.0, 275.0, 330.0)),
    ('s256', 256, 256, 8, 0.0, (0.0, 64.0, 275.0)),
    ('r64x128', 64, 128, 5, 0.02, (8.0, 150.0)),
    # lengths that are not powers of two, one odd (numpy's fftshift moves by n // 2)
    ('r75x120', 75, 120, 7, 0.03, (8.0, 150.0, 275.0)),
]


def load_reference_frft(reference: str):
    path = os.path.join(reference, 'realflare', 'utils', 'frft.py')
    spec = importlib.util.spec_from_file_location('reference_frft', path)
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)

    def chirp(shape):
        indices = tuple(slice(-size // 2, size // 2) for size in shape)
        grid = np.mgrid[indices]
        if len(shape) == 1:
            grid = tuple(grid)
        return 1.0j * np.pi * sum(np.fft.fftshift(a) ** 2 / a.shape[i] for i, a in enumerate(grid))

    module.chirp = chirp
    return module


def reference_ghost(frft_module, aperture: np.ndarray, fstop: float) -> np.ndarray:
    h, w = aperture.shape
    alpha = 0.15 * (LAMBDA_MID / 400) * (fstop / 18)
    spectrum = np.fft.fftshift(aperture)
    spectrum = frft_module.frft(spectrum, alpha)
    spectrum = np.fft.fftshift(spectrum)
    array = np.float32(np.abs(spectrum))
    array *= np.sqrt(w * h)
    return array


def polygon(height: int, width: int, blades: int, softness: float) -> np.ndarray:
    y, x = np.mgrid[-1:1:complex(0, height), -1:1:complex(0, width)]
    angle = np.arctan2(y, x)
    sector = 2 * np.pi / blades
    r = np.hypot(x, y) * np.cos(np.pi / blades) / np.cos((angle % sector) - np.pi / blades)
    if softness <= 0:
        return (r < 0.75).astype(np.float32)
    t = np.clip((r - (0.75 - softness)) / (2 * softness), 0, 1)
    return (1 - t * t * (3 - 2 * t)).astype(np.float32)


def key(case: str, fstop: float) -> str:
    return f'{case}_f{int(fstop)}'


def generate(reference: str) -> dict:
    module = load_reference_frft(reference)
    out = {}
    for case, h, w, blades, softness, fstops in CASES:
        ap = polygon(h, w, blades, softness)
        out[f'{case}_aperture'] = ap
        for fstop in fstops:
            out[key(case, fstop)] = reference_ghost(module, ap, fstop)
    return out


def main(reference: str) -> None:
    arrays = generate(reference)
    np.savez_compressed(OUT, **arrays)
    manifest_path = os.path.join(HERE, 'manifest.json')
    with open(manifest_path, encoding='utf-8') as f:
        manifest = json.load(f)
    manifest['frft_ghost'] = {k: hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()
                              for k, v in sorted(arrays.items())}
    with open(manifest_path, 'w', encoding='utf-8') as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
        f.write('\n')
    print(f'{len(arrays)} arrays -> {OUT} ({os.path.getsize(OUT)} bytes)')


if __name__ == '__main__':
    checkout = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('REALFLARE_REFERENCE')
    if not checkout:
        sys.exit('usage: make_frft_golden.py <reference checkout> (or set REALFLARE_REFERENCE)')
    main(checkout)
